"""Seeded random circuits over every gate family the backend dispatches."""
import numpy as np

from qibojit_gb300 import gates as G
from tests.dense import random_unitary


def random_circuit(n, ngates, seed, families=None):
    rng = np.random.default_rng(seed)
    c = G.Circuit(n)
    one = ["H", "X", "Y", "Z", "S", "SDG", "T", "TDG", "SX", "SXDG"]
    one_p = {"RX": 1, "RY": 1, "RZ": 1, "U1": 1, "U2": 2, "U3": 3}
    two_c = ["CNOT", "CZ", "CY", "CH", "CSX", "CSXDG"]
    two_p = {"CRX": 1, "CRY": 1, "CRZ": 1, "CU1": 1, "CU2": 2, "CU3": 3}
    kinds = families or ["one", "one_p", "two_c", "two_p", "swap", "fsim", "gfsim", "toffoli", "ccz",
                         "deutsch", "u1q", "u2q", "u3q", "cu1q", "cu2q", "fanout", "zc"]
    for _ in range(ngates):
        kind = kinds[rng.integers(len(kinds))]
        q = [int(x) for x in rng.permutation(n)]
        ang = list(rng.uniform(0, 2 * np.pi, 3))
        if kind == "one":
            c.add(getattr(G, one[rng.integers(len(one))])(q[0]))
        elif kind == "one_p":
            name = list(one_p)[rng.integers(len(one_p))]
            c.add(getattr(G, name)(q[0], *ang[: one_p[name]]))
        elif kind == "two_c":
            c.add(getattr(G, two_c[rng.integers(len(two_c))])(q[0], q[1]))
        elif kind == "two_p":
            name = list(two_p)[rng.integers(len(two_p))]
            c.add(getattr(G, name)(q[0], q[1], *ang[: two_p[name]]))
        elif kind == "swap":
            c.add(G.SWAP(q[0], q[1]))
        elif kind == "fsim":
            c.add(G.fSim(q[0], q[1], ang[0], ang[1]))
        elif kind == "gfsim":
            c.add(G.GeneralizedfSim(q[0], q[1], random_unitary(2, int(rng.integers(1 << 30))), ang[0]))
        elif kind == "toffoli":
            c.add(G.TOFFOLI(q[0], q[1], q[2]))
        elif kind == "ccz":
            c.add(G.CCZ(q[0], q[1], q[2]))
        elif kind == "deutsch":
            c.add(G.DEUTSCH(q[0], q[1], q[2], ang[0]))
        elif kind == "u1q":
            c.add(G.Unitary(random_unitary(2, int(rng.integers(1 << 30))), q[0]))
        elif kind == "u2q":
            c.add(G.Unitary(random_unitary(4, int(rng.integers(1 << 30))), q[0], q[1]))
        elif kind == "u3q":
            c.add(G.Unitary(random_unitary(8, int(rng.integers(1 << 30))), q[0], q[1], q[2]))
        elif kind == "cu1q":
            c.add(G.Unitary(random_unitary(2, int(rng.integers(1 << 30))), q[0]).controlled_by(q[1], q[2]))
        elif kind == "cu2q":
            c.add(G.Unitary(random_unitary(4, int(rng.integers(1 << 30))), q[0], q[1]).controlled_by(q[2]))
        elif kind == "fanout":
            c.add(G.FanOut(q[0], q[1], q[2]))
        elif kind == "zc":
            c.add(G.Z(q[0]).controlled_by(q[1], q[2], q[3]) if n > 3 else G.Z(q[0]))
    return c
