"""Host-side checks of the k-qubit block fuser (``autotune.fuse_blocks``): blocks stay
within k qubits, keep every gate once, and the fused circuit's unitary equals the
original's (the oracle applying each block's dense matrix against the oracle applying
the gates one by one)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from qibojit_gb300 import circuits
from qibojit_gb300 import gates as G
from qibojit_gb300.autotune import fuse_blocks
from qibojit_gb300.fusion import _expand, _target_matrix, matrix_fused
from tests.circuits_random import random_circuit
from tests.dense import random_state


def _oracle_run_gates(gates, n, x):
    ob = O.OracleBackend(nthreads=1)
    s = x.copy()
    for g in gates:
        t, c = list(g.target_qubits), list(g.control_qubits)
        s = ob._multi_qubit_base(s, n, t, _target_matrix(g), ob.qubits_tensor(n, t, c))
    return s


def _oracle_run_blocks(fused, n, x):
    ob = O.OracleBackend(nthreads=1)
    s = x.copy()
    for fg in fused.queue:
        t = list(fg.target_qubits)
        s = ob._multi_qubit_base(s, n, t, matrix_fused(fg), ob.qubits_tensor(n, t))
    return s


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("which", ["brickwork", "random", "qft", "hea"])
def test_fused_blocks_reproduce_the_circuit(k, which):
    n = 9
    c = {"brickwork": lambda: circuits.brickwork(n, 5, 3), "qft": lambda: circuits.qft(n),
         "hea": lambda: circuits.hea(n, 3, 4),
         "random": lambda: random_circuit(n, 80, 11, families=["one", "one_p", "two_c", "two_p", "swap", "fsim",
                                                                 "toffoli", "u2q", "cu1q", "zc", "fanout"])}[which]()
    fused = fuse_blocks(c, k)
    gates = _expand(c.queue)
    inner = [h for fg in fused.queue for h in fg.gates]
    key = lambda g: (type(g).__name__, tuple(g.target_qubits), tuple(g.control_qubits))  # noqa: E731
    assert sorted(map(key, inner)) == sorted(map(key, gates))
    width = max(len(g.qubits) for g in gates)
    assert all(len(fg.target_qubits) <= max(k, width) for fg in fused.queue)
    x = random_state(n, 5)
    np.testing.assert_allclose(_oracle_run_blocks(fused, n, x), _oracle_run_gates(gates, n, x), atol=1e-12)
    if k >= 2:
        assert len(fused.queue) < len(gates)


def test_merge_does_not_reorder_dependent_blocks():
    """k=3: g1 on {0}, g2 on {1,2}, g3 on {2,3} (a new block: {1,2,3} is fine but
    {1,2} then takes g3 only if it is latest on 2 -- it is -> merged), g4 on {0,2}.
    Whatever merges happen, g3 must still follow g2 on qubit 2."""
    c = G.Circuit(4)
    c.add(G.H(0))
    c.add(G.CNOT(1, 2))
    c.add(G.CZ(2, 3))
    c.add(G.CNOT(0, 2))
    for k in (2, 3, 4):
        fused = fuse_blocks(c, k)
        x = random_state(4, 2)
        np.testing.assert_allclose(_oracle_run_blocks(fused, 4, x), _oracle_run_gates(c.queue, 4, x), atol=1e-12)


def test_brickwork_blocks_shrink_with_k():
    """Wider blocks absorb more of the brickwork (the greedy is not monotone in k at
    every step, but k = 5..6 needs well under half the blocks of k = 2)."""
    c = circuits.brickwork(30, 20, 1234)
    counts = [len(fuse_blocks(c, k).queue) for k in range(1, 7)]
    assert counts[0] <= len(c.queue) and counts[1] < counts[0]
    assert max(counts[4:]) < 0.6 * counts[1]
