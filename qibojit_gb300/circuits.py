"""Seeded benchmark circuits (synthetic stand-ins for the reference's workloads).

* ``brickwork(n, depth, seed)``: every layer applies U3(t, p, l) to every qubit with
  angles i.i.d. uniform [0, 2pi), then CZ on disjoint nearest-neighbour pairs
  (2i, 2i+1) on even layers and (2i+1, 2i+2) on odd layers.
* ``qft(n)``: H on qubit q, CU1(pi / 2^(j-q)) from every later qubit j onto q, then
  the qubit-reversal SWAPs (the circuit of qibojit benchmarks/abstract.py:86-104).
* ``hea(n, layers, seed)``: hardware-efficient ansatz, RY(t) RZ(p) on every qubit per
  layer followed by a CNOT ladder q -> q+1.
"""
from __future__ import annotations

import numpy as np

from . import gates as G


def brickwork(n: int, depth: int, seed: int = 1234) -> "G.Circuit":
    rng = np.random.default_rng(seed)
    c = G.Circuit(n)
    for layer in range(depth):
        angles = rng.uniform(0, 2 * np.pi, size=(n, 3))
        for q in range(n):
            c.add(G.U3(q, *angles[q]))
        start = 0 if layer % 2 == 0 else 1
        for q in range(start, n - 1, 2):
            c.add(G.CZ(q, q + 1))
    return c


def qft(n: int) -> "G.Circuit":
    c = G.Circuit(n)
    for i1 in range(n):
        c.add(G.H(i1))
        for i2 in range(i1 + 1, n):
            c.add(G.CU1(i2, i1, theta=np.pi / 2 ** (i2 - i1)))
    for i in range(n // 2):
        c.add(G.SWAP(i, n - i - 1))
    return c


def hea(n: int, layers: int, seed: int = 1234) -> "G.Circuit":
    rng = np.random.default_rng(seed)
    c = G.Circuit(n)
    for _ in range(layers):
        th = rng.uniform(0, 2 * np.pi, size=(n, 2))
        for q in range(n):
            c.add(G.RY(q, theta=th[q, 0]))
            c.add(G.RZ(q, theta=th[q, 1]))
        for q in range(n - 1):
            c.add(G.CNOT(q, q + 1))
    return c


def algorithmic_bytes(gate, n: int, itemsize: int) -> int:
    """Bytes a per-gate pass must move: every touched amplitude read and written once.

    dense (1q/2q/kq) 2*b*2^n; X/CNOT/SWAP/Y touch the amplitudes they permute; Z/U1
    touch 2^(n-1-c) amplitudes, CZ/CU1 2^(n-2) (c = number of controls)."""
    name = type(gate).__name__
    nc = len(gate.control_qubits)
    b = itemsize
    if name in ("Z", "CZ", "CCZ", "U1", "CU1"):
        return 2 * b * (1 << (n - 1 - nc))
    if name in ("X", "CNOT", "TOFFOLI", "Y", "CY"):
        return 2 * b * (1 << (n - nc))
    if name == "SWAP":
        return 2 * b * (1 << (n - 1 - nc))
    return 2 * b * (1 << (n - nc))
