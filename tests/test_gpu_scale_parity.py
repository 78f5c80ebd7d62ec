"""The benchmark configurations against the oracle at (close to) their own sizes.

* Brickwork n=28, depth 20, seed 1234 (the bench circuit's construction two qubits
  smaller): the exact path the bench times (complex64, pass kernels specialised at
  run time on 2^13-amplitude tiles, phase-folded) against the complex128 oracle at
  max-abs <= 1e-5 and normalised infidelity <= 1e-6; the complex128 fused programs
  (interpreted and specialised) against the oracle at max-abs <= 1e-12.
* Adjoint gradients of the batched-gradient configuration (n=26, 20 layers of RY RZ
  plus a CNOT ladder, TFIM h=1): 2 circuits x 4 parameters against parameter shift
  on the oracle (<= 1e-9), 16 more parameters spread over all layers against
  parameter shift on the plain complex128 GPU path, and complex64 against complex128
  (gradients, energies and the final state's infidelity <= 1e-6).
* Circuits pre-fused into qibo-style ``FusedGate`` blocks, through ``execute_circuit``
  fused and per gate, against the oracle applying the component gates one by one.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from qibojit_gb300 import circuits
from qibojit_gb300 import gates as G
from tests.circuits_random import random_circuit
from tests.conftest import PARITY_ATOL
from tests.dense import random_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


def _oracle_gate(ob, state, n, g, cm):
    """One gate of any family on the C oracle (its textbook target matrix with its
    controls, through the oracle's multi-target kernel; U3 and CZ through the kernels
    the reference dispatches them to)."""
    from qibojit_gb300.fusion import _target_matrix

    name = type(g).__name__
    t, c = list(g.target_qubits), list(g.control_qubits)
    if name == "U3" and not c:
        return ob._one_qubit_base(state, n, t[0], "apply_gate", cm.U3(*g.parameters), ob.qubits_tensor(n, t))
    if name == "CZ":
        return ob._one_qubit_base(state, n, t[0], "apply_z", None, ob.qubits_tensor(n, t, c))
    if getattr(g, "name", "") == "fanout":
        for q in t:
            state = ob._one_qubit_base(state, n, q, "apply_x", None, ob.qubits_tensor(n, [q], c))
        return state
    m = _target_matrix(g)
    return ob._multi_qubit_base(state, n, t, m, ob.qubits_tensor(n, t, c))


# ------------------------------------------------------------------ brickwork n=28
N_BW = 28


@pytest.fixture(scope="module")
def brickwork28_oracle(backend):
    circ = circuits.brickwork(N_BW, 20, 1234)
    ob = O.OracleBackend()
    ref = ob.zero_state(N_BW)
    cm = backend.custom_matrices
    for g in circ.queue:
        ref = _oracle_gate(ob, ref, N_BW, g, cm)
    return circ, ref


def _compare(got, ref):
    got = got.astype(np.complex128)
    maxabs = float(np.abs(got - ref).max())
    ip = np.vdot(ref, got)
    fid = abs(ip) ** 2 / (np.vdot(got, got).real * np.vdot(ref, ref).real)
    return maxabs, 1.0 - fid


def test_brickwork28_bench_path_complex64_vs_oracle(backend, brickwork28_oracle):
    import torch

    circ, ref = brickwork28_oracle
    prog = backend.compile(circ, "complex64", specialize=True)
    st = prog.stats()
    assert prog.specialized and st["tile_bits"] == 13 and st["unfused"] == 0
    got = backend.to_numpy(prog.run(backend.zero_state(N_BW, dtype="complex64")))
    maxabs, infid = _compare(got, ref)
    del got
    torch.cuda.empty_cache()
    assert maxabs <= 1e-5, maxabs
    assert infid <= 1e-6, infid


@pytest.mark.parametrize("specialize", [False, True])
def test_brickwork28_complex128_fused_vs_oracle(backend, brickwork28_oracle, specialize):
    import torch

    circ, ref = brickwork28_oracle
    prog = backend.compile(circ, "complex128", specialize=specialize)
    got = backend.to_numpy(prog.run(backend.zero_state(N_BW, dtype="complex128")))
    maxabs, infid = _compare(got, ref)
    del got
    torch.cuda.empty_cache()
    assert maxabs <= PARITY_ATOL["complex128"], maxabs
    assert infid <= 1e-12


# ------------------------------------------------------- adjoint gradients, n=26
N_AD, L_AD = 26, 20


def _hea_gates(n, layers):
    """(kind, qubit, parameter index) in application order; the parameter index of
    RY(layer, q) is (layer*n + q)*2 and of RZ(layer, q) that plus one."""
    out = []
    for layer in range(layers):
        for q in range(n):
            out.append(("ry", q, (layer * n + q) * 2))
            out.append(("rz", q, (layer * n + q) * 2 + 1))
        for q in range(n - 1):
            out.append(("cx", q, -1))
    return out


def _oracle_hea_run(ob, state, n, gates, flat, start, stop):
    for kind, q, p in gates[start:stop]:
        if kind == "ry":
            t = flat[p] / 2
            m = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]], dtype=np.complex128)
            state = ob._one_qubit_base(state, n, q, "apply_gate", m, ob.qubits_tensor(n, [q]))
        elif kind == "rz":
            f = flat[p] / 2
            m = np.diag([np.exp(-1j * f), np.exp(1j * f)])
            state = ob._one_qubit_base(state, n, q, "apply_gate", m, ob.qubits_tensor(n, [q]))
        else:
            state = ob._one_qubit_base(state, n, q + 1, "apply_x", None, ob.qubits_tensor(n, [q + 1], [q]))
    return state


def _tfim_energy(psi, n, h=1.0):
    """E = -sum_i <Z_i Z_{i+1}> - h sum_i <X_i> of a complex128 state (numpy or torch),
    evaluated with plain torch FP64 operations on the GPU (none of the engine's
    kernels): marginals of adjacent bit pairs for ZZ, 2 Re sum conj(a_0) a_1 over
    the pairs split by qubit i for X."""
    import torch

    t = psi if isinstance(psi, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(psi))
    t = t.to("cuda", torch.complex128).reshape(-1)
    p = t.real ** 2 + t.imag ** 2
    e = torch.zeros((), dtype=torch.float64, device="cuda")
    for i in range(n - 1):
        m = p.reshape(2**i, 2, 2, -1).sum(dim=(0, 3))
        e -= m[0, 0] + m[1, 1] - m[0, 1] - m[1, 0]
    for i in range(n):
        a = t.reshape(2**i, 2, -1)
        e -= h * 2 * (a[:, 0, :].conj() * a[:, 1, :]).real.sum()
    return float(e.item())


def _oracle_parameter_shift(n, layers, params, chosen):
    """dE/dtheta_p = (E(theta_p + pi/2) - E(theta_p - pi/2)) / 2 on the oracle, for the
    chosen flat parameter indices; the forward prefix up to the earliest chosen gate is
    computed once and shared by all shifted runs."""
    gates = _hea_gates(n, layers)
    flat = params.reshape(-1)
    pos = {p: j for j, (_, _, p) in enumerate(gates) if p >= 0}
    first = min(pos[p] for p in chosen)
    ob = O.OracleBackend()
    prefix = _oracle_hea_run(ob, ob.zero_state(n), n, gates, flat, 0, first)
    out = {}
    for p in chosen:
        vals = []
        for sign in (+1, -1):
            f = flat.copy()
            f[p] += sign * np.pi / 2
            s = _oracle_hea_run(ob, prefix.copy(), n, gates, f, first, len(gates))
            vals.append(_tfim_energy(s, n, 1.0))
        out[p] = (vals[0] - vals[1]) / 2
    energy = _tfim_energy(_oracle_hea_run(ob, prefix.copy(), n, gates, flat, first, len(gates)), n, 1.0)
    return out, energy


@pytest.fixture(scope="module")
def adjoint26(backend):
    from qibojit_gb300.adjoint import AdjointTFIM

    rng = np.random.default_rng(2026)
    params = rng.uniform(0, 2 * np.pi, size=(2, L_AD, N_AD, 2))
    res = {}
    for dt in ("complex128", "complex64"):
        eng = AdjointTFIM(backend, N_AD, L_AD, 2, dt, h=1.0, checkpoint_every=5)
        E, Gr = eng(params)
        states = [backend.to_numpy(eng.state(c)).astype(np.complex128) for c in range(2)]
        eng.close()
        res[dt] = (E, Gr, states)
    return params, res


def test_adjoint26_vs_oracle_parameter_shift(adjoint26):
    params, res = adjoint26
    E, Gr, _ = res["complex128"]
    # parameters of the last three layers (the shared oracle prefix runs the first 17)
    chosen = [[(L_AD - 1) * N_AD * 2 + 2 * 3, (L_AD - 1) * N_AD * 2 + 2 * 20 + 1,
               (L_AD - 2) * N_AD * 2 + 2 * 11 + 1, (L_AD - 3) * N_AD * 2 + 2 * 25],
              [(L_AD - 1) * N_AD * 2 + 2 * 0 + 1, (L_AD - 2) * N_AD * 2 + 2 * 13,
               (L_AD - 3) * N_AD * 2 + 2 * 7 + 1, (L_AD - 3) * N_AD * 2 + 2 * 18]]
    for c in range(2):
        shifts, e0 = _oracle_parameter_shift(N_AD, L_AD, params[c], chosen[c])
        assert abs(E[c] - e0) < 1e-9, (E[c], e0)
        flat = Gr[c].reshape(-1)
        for p, want in shifts.items():
            assert abs(flat[p] - want) < 1e-9, (c, p, flat[p], want)


def test_adjoint26_vs_gpu_parameter_shift_all_layers(backend, adjoint26):
    """16 parameters from every part of the circuit, against parameter shift on the
    plain complex128 GPU path (fused passes, no adjoint code)."""
    params, res = adjoint26
    E, Gr, _ = res["complex128"]

    def energy(p):
        c = G.Circuit(N_AD)
        for layer in range(L_AD):
            for q in range(N_AD):
                c.add(G.RY(q, theta=float(p[layer, q, 0])))
                c.add(G.RZ(q, theta=float(p[layer, q, 1])))
            for q in range(N_AD - 1):
                c.add(G.CNOT(q, q + 1))
        s = backend.execute_circuit(c, backend.zero_state(N_AD, dtype="complex128"), fuse=True)
        return _tfim_energy(s, N_AD, 1.0)

    rng = np.random.default_rng(7)
    picks = [tuple(int(v) for v in (rng.integers(L_AD), rng.integers(N_AD), rng.integers(2))) for _ in range(16)]
    for (layer, q, k) in picks:
        pp, pm = params[0].copy(), params[0].copy()
        pp[layer, q, k] += np.pi / 2
        pm[layer, q, k] -= np.pi / 2
        want = (energy(pp) - energy(pm)) / 2
        assert abs(Gr[0, layer, q, k] - want) < 1e-9, ((layer, q, k), Gr[0, layer, q, k], want)


def test_adjoint26_complex64_vs_complex128(adjoint26):
    params, res = adjoint26
    E128, G128, S128 = res["complex128"]
    E64, G64, S64 = res["complex64"]
    np.testing.assert_allclose(E64, E128, rtol=0, atol=1e-4)
    assert np.abs(G64 - G128).max() < 1e-3
    for a, b in zip(S64, S128):
        ip = np.vdot(b, a)
        infid = 1 - abs(ip) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
        assert infid <= 1e-6, infid


# ------------------------------------------------------------ qibo-fused circuits
def _fuse_like_qibo(circ, max_qubits):
    """Greedy block fusion in the manner of qibo's Circuit.fuse: consecutive gates join
    the open block while the union of their qubits stays within ``max_qubits``."""
    out = G.Circuit(circ.nqubits)
    block, qs = [], set()
    for g in circ.queue:
        gq = set(g.qubits)
        if block and len(qs | gq) > max_qubits:
            fg = G.FusedGate(*sorted(qs))
            for h in block:
                fg.append(h)
            out.add(fg)
            block, qs = [], set()
        block.append(g)
        qs |= gq
    if block:
        fg = G.FusedGate(*sorted(qs))
        for h in block:
            fg.append(h)
        out.add(fg)
    return out


@pytest.mark.parametrize("n,max_qubits,seed", [(10, 2, 1), (12, 3, 2), (14, 4, 3), (16, 5, 4), (13, 6, 5)])
@pytest.mark.parametrize("fuse", [True, False])
def test_fused_gate_circuits_vs_oracle(backend, n, max_qubits, seed, fuse, dtype):
    base = random_circuit(n, 60, seed, families=["one", "one_p", "two_c", "two_p", "swap", "fsim", "toffoli",
                                                 "u2q", "u3q", "cu1q", "zc", "fanout"])
    fused = _fuse_like_qibo(base, max_qubits)
    assert any(type(g).__name__ == "FusedGate" and len(g.target_qubits) > 1 for g in fused.queue)
    state = random_state(n, seed + 50, dtype)
    backend.set_dtype(dtype)
    got = backend.to_numpy(backend.execute_circuit(fused, backend.cast(state, copy=True), fuse=fuse))
    ob = O.OracleBackend()
    ref = state.astype(np.complex128)
    cm = backend.custom_matrices
    for g in base.queue:
        ref = _oracle_gate(ob, ref, n, g, cm)
    tol = PARITY_ATOL[dtype] * (10 if dtype == "complex64" else 1)
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol)
