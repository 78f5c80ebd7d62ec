"""Batched circuits (config: many hardware-efficient-ansatz circuits of uneven size)."""
import numpy as np
import pytest

from qibojit_gb300.batch import BatchedCircuits, hea_batch, hea_circuit, tfim_energy_dense
from tests.circuits_random import random_circuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


@pytest.mark.parametrize("dt,tol", [("complex128", 1e-12), ("complex64", 2e-5)])
def test_hea_batch_matches_single_circuits(backend, dt, tol):
    dtype = dt
    specs = hea_batch(40, seed=5, nmin=8, nmax=15, lmin=2, lmax=5)
    circs = [hea_circuit(n, L, p) for n, L, p in specs]
    batch = BatchedCircuits(backend, circs, dtype)
    st = batch.stats()
    assert st["groups"] <= len(circs)
    batch.run()
    energies = batch.tfim_energies(1.0)
    for i, c in enumerate(circs):
        got = backend.to_numpy(batch.state(i))
        want = backend.to_numpy(backend.execute_circuit(c, backend.zero_state(c.nqubits, dtype=dtype), fuse=False))
        np.testing.assert_allclose(got, want, rtol=0, atol=tol)
        e = tfim_energy_dense(want, c.nqubits, 1.0)
        assert abs(energies[i] - e) < (1e-11 if dtype == "complex128" else 1e-4) * max(1.0, abs(e))


def test_from_hea_matches_gate_objects(backend):
    specs = hea_batch(12, seed=21, nmin=9, nmax=13, lmin=2, lmax=4)
    a = BatchedCircuits(backend, [hea_circuit(n, L, p) for n, L, p in specs], "complex128")
    b = BatchedCircuits.from_hea(backend, specs, "complex128")
    a.run()
    b.run()
    np.testing.assert_allclose(a.tfim_energies(), b.tfim_energies(), atol=1e-13)


def test_batch_graph_replay_is_repeatable(backend):
    specs = hea_batch(64, seed=9, nmin=8, nmax=16, lmin=2, lmax=6)
    batch = BatchedCircuits(backend, [hea_circuit(n, L, p) for n, L, p in specs], "complex64")
    batch.run()                      # eager run + graph capture
    e1 = batch.tfim_energies()
    batch.run()                      # graph replay
    e2 = batch.tfim_energies()
    batch.run()
    e3 = batch.tfim_energies()
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(e2, e3)


def test_batch_of_random_circuits(backend):
    """Arbitrary fusable gates (1-2 targets, controls) in a batch, two structures repeated."""
    from qibojit_gb300 import gates as G

    circs = []
    for k in range(6):
        c = random_circuit(10 + (k % 2), 40, seed=100 + k % 2,
                           families=["one", "one_p", "two_c", "two_p", "swap", "fsim", "u2q", "zc", "ccz", "toffoli"])
        circs.append(c)
    batch = BatchedCircuits(backend, circs, "complex128")
    assert batch.stats()["groups"] == 2
    batch.run()
    for i, c in enumerate(circs):
        want = backend.to_numpy(backend.execute_circuit(c, backend.zero_state(c.nqubits), fuse=False))
        np.testing.assert_allclose(backend.to_numpy(batch.state(i)), want, rtol=0, atol=1e-12)


@pytest.mark.parametrize("dt,tol", [("complex128", 1e-12), ("complex64", 2e-5)])
def test_specialised_batch_matches_single_circuits(backend, dt, tol):
    """sv_batch_specialize: one compiled kernel per group and pass, every circuit's own
    coefficients; states against the per-gate path, energies against the dense formula,
    and the graph recorded after specialising replays the same energies."""
    specs = hea_batch(48, seed=17, nmin=8, nmax=16, lmin=2, lmax=6)
    circs = [hea_circuit(n, L, p) for n, L, p in specs]
    batch = BatchedCircuits(backend, circs, dt)
    batch.run()                      # interpreting kernels, graph recorded
    e0 = batch.tfim_energies(1.0)
    batch.specialize()
    batch.run()                      # specialised, eager, new graph recorded
    e1 = batch.tfim_energies(1.0)
    for i, c in enumerate(circs):
        got = backend.to_numpy(batch.state(i))
        want = backend.to_numpy(backend.execute_circuit(c, backend.zero_state(c.nqubits, dtype=dt), fuse=False))
        np.testing.assert_allclose(got, want, rtol=0, atol=tol)
    np.testing.assert_allclose(e1, e0, atol=1e-11 if dt == "complex128" else 1e-4)
    batch.run()                      # graph replay of the specialised launches
    np.testing.assert_array_equal(batch.tfim_energies(1.0), e1)


def test_specialised_batch_of_random_circuits(backend):
    circs = [random_circuit(10 + (k % 2), 40, seed=300 + k % 2,
                            families=["one", "one_p", "two_c", "two_p", "swap", "fsim", "u2q", "zc", "ccz", "toffoli"])
             for k in range(6)]
    batch = BatchedCircuits(backend, circs, "complex128").specialize()
    batch.run()
    for i, c in enumerate(circs):
        want = backend.to_numpy(backend.execute_circuit(c, backend.zero_state(c.nqubits), fuse=False))
        np.testing.assert_allclose(backend.to_numpy(batch.state(i)), want, rtol=0, atol=1e-12)


@pytest.mark.parametrize("dt,tol", [("complex128", 1e-12), ("complex64", 2e-5)])
def test_persistent_executor_matches_graph(backend, dt, tol):
    """sv_batch_set_executor(SV_BATCH_PERSISTENT): the whole batch in one cooperative
    launch (per-circuit pass ordering through device counters) gives the interpreting
    graph executor's states and energies; circuits of 8 to 15 qubits mix tiles smaller
    than the launch's largest; a second run (recorded or eager) repeats the first."""
    specs = hea_batch(40, seed=23, nmin=8, nmax=15, lmin=2, lmax=6)
    circs = [hea_circuit(n, L, p) for n, L, p in specs]
    batch = BatchedCircuits(backend, circs, dt)
    batch.run()
    want = [backend.to_numpy(batch.state(i)).copy() for i in range(len(circs))]
    e_graph = batch.tfim_energies(1.0)
    batch.set_executor("persistent")
    for _ in range(2):
        batch.run()
        e = batch.tfim_energies(1.0)
        for i in range(len(circs)):
            np.testing.assert_allclose(backend.to_numpy(batch.state(i)), want[i], rtol=0, atol=tol)
        np.testing.assert_allclose(e, e_graph, rtol=0, atol=1e-11 if dt == "complex128" else 1e-5)
    for i, c in enumerate(circs[:6]):
        ref = backend.to_numpy(backend.execute_circuit(c, backend.zero_state(c.nqubits, dtype=dt), fuse=False))
        np.testing.assert_allclose(backend.to_numpy(batch.state(i)), ref, rtol=0, atol=tol)
    batch.set_executor("graph")
    batch.run()
    np.testing.assert_allclose(batch.tfim_energies(1.0), e_graph, rtol=0, atol=1e-12 if dt == "complex128" else 1e-6)
    batch.close()


def test_persistent_executor_random_circuits(backend):
    """Many structures (every fusable gate family), complex128 in double-word and FP64
    arithmetic, against the per-gate path."""
    circs = [random_circuit(9 + (k % 4), 50, seed=500 + k % 5,
                            families=["one", "one_p", "two_c", "two_p", "swap", "fsim", "u2q", "zc", "ccz", "toffoli"])
             for k in range(12)]
    for mode in ("double-word", "fp64"):
        backend.ctx.set_c128_arithmetic(mode)
        try:
            batch = BatchedCircuits(backend, circs, "complex128")
        finally:
            backend.ctx.set_c128_arithmetic("double-word")
        batch.set_executor("persistent").run()
        batch.tfim_energies(1.0)  # synchronises and reports a timed-out wait
        for i, c in enumerate(circs):
            want = backend.to_numpy(backend.execute_circuit(c, backend.zero_state(c.nqubits), fuse=False))
            np.testing.assert_allclose(backend.to_numpy(batch.state(i)), want, rtol=0, atol=1e-12)
        batch.close()


def test_executor_name_is_checked(backend):
    batch = BatchedCircuits(backend, [hea_circuit(8, 2, np.zeros((2, 8, 2)))], "complex64")
    with pytest.raises(ValueError):
        batch.set_executor("threads")
    batch.close()
