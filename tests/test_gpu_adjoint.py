"""Adjoint gradients against parameter shift on the CPU oracle (the reference's kernels
restated), central finite differences in complex128, and complex64 vs complex128."""
import numpy as np
import pytest

from oracle import pyoracle as O
from qibojit_gb300.batch import tfim_energy_dense

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


def oracle_energy(n, layers, p, h=1.0):
    """HEA forward on the CPU oracle kernels, TFIM energy in numpy."""
    ob = O.OracleBackend()
    s = ob.zero_state(n)
    for layer in range(layers):
        for q in range(n):
            t, f = p[layer, q]
            ry = np.array([[np.cos(t / 2), -np.sin(t / 2)], [np.sin(t / 2), np.cos(t / 2)]], dtype=complex)
            rz = np.diag([np.exp(-0.5j * f), np.exp(0.5j * f)])
            s = ob._one_qubit_base(s, n, q, "apply_gate", ry, ob.qubits_tensor(n, [q]))
            s = ob._one_qubit_base(s, n, q, "apply_gate", rz, ob.qubits_tensor(n, [q]))
        for q in range(n - 1):
            s = ob._one_qubit_base(s, n, q + 1, "apply_x", None, ob.qubits_tensor(n, [q + 1], [q]))
    return tfim_energy_dense(s, n, h), s


def test_adjoint_matches_parameter_shift(backend):
    from qibojit_gb300.adjoint import AdjointTFIM

    n, L, nc = 9, 3, 2
    rng = np.random.default_rng(11)
    params = rng.uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    eng = AdjointTFIM(backend, n, L, nc, "complex128", h=1.0, checkpoint_every=2)
    E, G = eng(params)
    for c in range(nc):
        e0, _ = oracle_energy(n, L, params[c])
        assert abs(E[c] - e0) < 1e-11
        for (layer, q, k) in [(0, 0, 0), (0, 8, 1), (1, 3, 0), (2, 5, 1), (2, 0, 0), (1, 6, 1)]:
            pp, pm = params[c].copy(), params[c].copy()
            pp[layer, q, k] += np.pi / 2
            pm[layer, q, k] -= np.pi / 2
            shift = (oracle_energy(n, L, pp)[0] - oracle_energy(n, L, pm)[0]) / 2
            assert abs(G[c, layer, q, k] - shift) < 1e-10, (c, layer, q, k, G[c, layer, q, k], shift)


def test_adjoint_matches_finite_differences(backend):
    from qibojit_gb300.adjoint import AdjointTFIM

    n, L = 9, 2
    rng = np.random.default_rng(12)
    p = rng.uniform(0, 2 * np.pi, size=(1, L, n, 2))
    eng = AdjointTFIM(backend, n, L, 1, "complex128", checkpoint_every=1)
    E, G = eng(p)
    fd = np.zeros_like(p)
    step = 1e-4
    probe = AdjointTFIM(backend, n, L, 1, "complex128", checkpoint_every=1)
    for idx in np.ndindex(p.shape):
        a, b = p.copy(), p.copy()
        a[idx] += step
        b[idx] -= step
        fd[idx] = (probe(a)[0][0] - probe(b)[0][0]) / (2 * step)
    np.testing.assert_allclose(G, fd, atol=1e-7)


@pytest.mark.parametrize("every", [1, 2, 10])
def test_checkpointing_does_not_change_results(backend, every):
    from qibojit_gb300.adjoint import AdjointTFIM

    n, L, nc = 10, 4, 3
    p = np.random.default_rng(13).uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    E1, G1 = AdjointTFIM(backend, n, L, nc, "complex128", checkpoint_every=every)(p)
    E2, G2 = AdjointTFIM(backend, n, L, nc, "complex128", checkpoint_every=L)(p)
    np.testing.assert_allclose(E1, E2, atol=1e-12)
    np.testing.assert_allclose(G1, G2, atol=1e-11)


def test_complex64_gradients_track_complex128(backend):
    from qibojit_gb300.adjoint import AdjointTFIM

    n, L, nc = 12, 5, 4
    p = np.random.default_rng(14).uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    E64, G64 = AdjointTFIM(backend, n, L, nc, "complex64", checkpoint_every=2)(p)
    E128, G128 = AdjointTFIM(backend, n, L, nc, "complex128", checkpoint_every=2)(p)
    np.testing.assert_allclose(E64, E128, atol=2e-5)
    np.testing.assert_allclose(G64, G128, atol=2e-4)


def test_small_circuits_are_rejected(backend):
    from qibojit_gb300.adjoint import AdjointTFIM

    with pytest.raises(ValueError):
        AdjointTFIM(backend, 8, 2, 1, "complex128")(np.zeros((1, 2, 8, 2)))


def test_update_and_autograd(backend):
    import torch

    from qibojit_gb300.adjoint import AdjointTFIM, HEAEnergy

    n, L, nc = 9, 2, 2
    rng = np.random.default_rng(15)
    eng = AdjointTFIM(backend, n, L, nc, "complex128")
    p1 = rng.uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    p2 = rng.uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    eng(p1)
    E2, G2 = eng(p2)  # re-uses plans and memory
    E2b, G2b = AdjointTFIM(backend, n, L, nc, "complex128")(p2)
    np.testing.assert_allclose(E2, E2b, atol=1e-13)
    np.testing.assert_allclose(G2, G2b, atol=1e-13)
    t = torch.tensor(p2, dtype=torch.float64, requires_grad=True)
    loss = HEAEnergy.apply(t, eng).sum()
    loss.backward()
    np.testing.assert_allclose(t.grad.numpy(), G2, atol=1e-13)


def _random_unitary(rng):
    q, r = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("dt", ["complex128", "complex64"])
def test_fixed_complex_gates_inside_adjoint_circuits(backend, dt):
    """A layer of parameter-free complex one-qubit gates (the planner fuses consecutive
    ones into register runs) before every RY/RZ layer: energies and gradients against
    the CPU oracle and parameter shift."""
    import ctypes

    from qibojit_gb300 import _lib
    from qibojit_gb300.fusion import GateOp

    n, L = 9, 2
    rng = np.random.default_rng(16)
    fixed = [[_random_unitary(rng) for _ in range(n)] for _ in range(L)]
    theta = rng.uniform(0, 2 * np.pi, size=(L, n, 2))
    keep = []

    def mat(m):
        buf = np.ascontiguousarray(np.column_stack([m.real.ravel(), m.imag.ravel()]).ravel(), dtype=np.float64)
        keep.append(buf)
        return buf.ctypes.data

    def circuit_ops(p):
        ops, gens, pidx = [], [], []
        for layer in range(L):
            for q in range(n):
                ops.append((0, q, -1, mat(fixed[layer][q])))
                gens.append(0)
                pidx.append(-1)
            for q in range(n):
                t, f = p[layer, q]
                ops.append((0, q, -1, mat(np.array([[np.cos(t / 2), -np.sin(t / 2)], [np.sin(t / 2), np.cos(t / 2)]]))))
                gens.append(2)
                pidx.append((layer * n + q) * 2)
                ops.append((1, q, -1, mat(np.array([np.exp(-0.5j * f), np.exp(0.5j * f)]))))
                gens.append(3)
                pidx.append((layer * n + q) * 2 + 1)
            for q in range(n - 1):
                ops.append((0, q + 1, q, mat(np.array([[0, 1], [1, 0]], dtype=complex))))
                gens.append(0)
                pidx.append(-1)
        arr = (GateOp * len(ops))()
        for k, (kind, t, c, m) in enumerate(ops):
            arr[k].kind, arr[k].ntargets = kind, 1
            arr[k].targets[0] = t
            if c >= 0:
                arr[k].ncontrols = 1
                arr[k].controls[0] = c
            arr[k].matrix = m
        return arr, np.array(gens, dtype=np.int8), np.array(pidx, dtype=np.int32)

    def oracle_energy(p):
        ob = O.OracleBackend()
        s = ob.zero_state(n)
        for layer in range(L):
            for q in range(n):
                s = ob._one_qubit_base(s, n, q, "apply_gate", fixed[layer][q], ob.qubits_tensor(n, [q]))
            for q in range(n):
                t, f = p[layer, q]
                ry = np.array([[np.cos(t / 2), -np.sin(t / 2)], [np.sin(t / 2), np.cos(t / 2)]], dtype=complex)
                rz = np.diag([np.exp(-0.5j * f), np.exp(0.5j * f)])
                s = ob._one_qubit_base(s, n, q, "apply_gate", ry, ob.qubits_tensor(n, [q]))
                s = ob._one_qubit_base(s, n, q, "apply_gate", rz, ob.qubits_tensor(n, [q]))
            for q in range(n - 1):
                s = ob._one_qubit_base(s, n, q + 1, "apply_x", None, ob.qubits_tensor(n, [q + 1], [q]))
        return tfim_energy_dense(s, n, 1.0)

    arr, gens, pidx = circuit_ops(theta)
    nops, nparams = len(gens), L * n * 2
    ptrs = (ctypes.c_void_p * 1)(ctypes.cast(arr, ctypes.c_void_p).value)
    per_layer = 4 * n - 1
    ends = np.array([per_layer, nops], dtype=np.int32)
    lib, h = backend.lib, ctypes.c_void_p()
    _lib.check(lib.sv_adjoint_create(backend.ctx.handle, _lib.DTYPE_CODES[dt], 1, n, ptrs, nops, gens.ctypes.data,
                                     pidx.ctypes.data, nparams, ends.ctypes.data, len(ends), 0, ctypes.byref(h)))
    try:
        E = np.zeros(1)
        G = np.zeros((1, nparams))
        _lib.check(lib.sv_adjoint_run(backend.ctx.handle, h, 1.0, E.ctypes.data, G.ctypes.data))
    finally:
        lib.sv_adjoint_destroy(h)
    tol_e, tol_g = (1e-11, 1e-10) if dt == "complex128" else (2e-5, 2e-4)
    assert abs(E[0] - oracle_energy(theta)) < tol_e
    G = G.reshape(L, n, 2)
    for (layer, q, k) in [(0, 0, 0), (0, 4, 1), (1, 8, 0), (1, 2, 1)]:
        pp, pm = theta.copy(), theta.copy()
        pp[layer, q, k] += np.pi / 2
        pm[layer, q, k] -= np.pi / 2
        shift = (oracle_energy(pp) - oracle_energy(pm)) / 2
        assert abs(G[layer, q, k] - shift) < tol_g, (layer, q, k, G[layer, q, k], shift)


def test_adjoint_n26_l20_against_parameter_shift_and_complex128(backend):
    """The benchmarked configuration (n=26, 20 layers, 1040 parameters per circuit,
    checkpoints every 5 layers): complex64 adjoint gradients and energies against the
    complex128 adjoint on every parameter, and the complex128 adjoint against parameter
    shift on six parameters spread over the circuit (the shifted energies from batched
    complex128 circuits in FP64 arithmetic)."""
    from qibojit_gb300.adjoint import AdjointTFIM
    from qibojit_gb300.batch import BatchedCircuits

    n, L, nc = 26, 20, 2
    p = np.random.default_rng(21).uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    res = {}
    for dt in ("complex64", "complex128"):
        eng = AdjointTFIM(backend, n, L, nc, dt, checkpoint_every=5)
        res[dt] = eng(p)
        eng.close()
    (E64, G64), (E128, G128) = res["complex64"], res["complex128"]
    assert np.abs(E64 - E128).max() < 1e-6
    assert np.abs(G64 - G128).max() < 1e-6
    picks = [(0, 0, 0), (0, 25, 1), (7, 13, 0), (12, 4, 1), (19, 25, 0), (19, 0, 1)]
    specs = []
    for layer, q, k in picks:
        for sgn in (1, -1):
            pp = p[0].copy()
            pp[layer, q, k] += sgn * np.pi / 2
            specs.append((n, L, pp))
    backend.ctx.set_c128_arithmetic("fp64")
    try:
        bat = BatchedCircuits.from_hea(backend, specs, "complex128")
    finally:
        backend.ctx.set_c128_arithmetic("double-word")
    bat.run()
    en = bat.tfim_energies(1.0)
    bat.close()
    for i, (layer, q, k) in enumerate(picks):
        shift = (en[2 * i] - en[2 * i + 1]) / 2
        assert abs(G128[0, layer, q, k] - shift) < 1e-10, (layer, q, k, G128[0, layer, q, k], shift)


@pytest.mark.parametrize("dt,tol", [("complex128", 1e-12), ("complex64", 2e-5)])
@pytest.mark.parametrize("n,L,every", [(9, 3, 2), (12, 4, 1), (14, 5, 5)])
def test_specialised_adjoint_matches_interpreted(backend, dt, tol, n, L, every):
    """sv_adjoint_specialize: forward and reverse-sweep passes compiled with the
    structure and every gradient marker as literals give the interpreting kernels'
    energies and gradients, also after new parameters (sv_adjoint_update)."""
    from qibojit_gb300.adjoint import AdjointTFIM

    nc = 3
    rng = np.random.default_rng(40 + n)
    p1 = rng.uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    p2 = rng.uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    spec = AdjointTFIM(backend, n, L, nc, dt, checkpoint_every=every, specialize=True)
    ref = AdjointTFIM(backend, n, L, nc, dt, checkpoint_every=every)
    for p in (p1, p2):
        Es, Gs = spec(p)
        Er, Gr = ref(p)
        np.testing.assert_allclose(Es, Er, rtol=0, atol=tol)
        np.testing.assert_allclose(Gs, Gr, rtol=0, atol=tol)
    spec.close()
    ref.close()


def test_specialised_adjoint_matches_parameter_shift(backend):
    from qibojit_gb300.adjoint import AdjointTFIM

    n, L, nc = 9, 3, 2
    params = np.random.default_rng(11).uniform(0, 2 * np.pi, size=(nc, L, n, 2))
    eng = AdjointTFIM(backend, n, L, nc, "complex128", h=1.0, checkpoint_every=2, specialize=True)
    E, G = eng(params)
    eng.close()
    for c in range(nc):
        assert abs(E[c] - oracle_energy(n, L, params[c])[0]) < 1e-11
        for (layer, q, k) in [(0, 0, 0), (0, 8, 1), (1, 3, 0), (2, 5, 1)]:
            pp, pm = params[c].copy(), params[c].copy()
            pp[layer, q, k] += np.pi / 2
            pm[layer, q, k] -= np.pi / 2
            shift = (oracle_energy(n, L, pp)[0] - oracle_energy(n, L, pm)[0]) / 2
            assert abs(G[c, layer, q, k] - shift) < 1e-10
