"""Gate fusion: circuits compiled into cache-blocked HBM passes by the engine.

The reference leaves fusion to qibo (``Circuit.fuse`` builds ``FusedGate`` objects
whose dense matrix qibojit applies with its multi-qubit kernel, ``cpu.py:535-537``).
Here a circuit is lowered to a list of engine ops (``sv_gate_op``): a gate whose
target matrix is diagonal becomes a diagonal op (its phases), anything else a dense
op on its targets, each with its control qubits.  The engine's planner
(``csrc/sv_fused.cu``) groups them into passes, each applied by one tile kernel
that reads and writes the state once.

``matrix_fused`` gives the dense matrix of a ``FusedGate`` (qibo's ``matrix_fused``)
for callers that use the per-gate multi-qubit kernel instead.
"""
from __future__ import annotations

import ctypes
from typing import Iterable, List, Optional

import numpy as np

from . import _lib

SV_OP_DENSE, SV_OP_DIAG = 0, 1


class GateOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("ntargets", ctypes.c_int32), ("ncontrols", ctypes.c_int32),
                ("targets", ctypes.c_int32 * 10), ("controls", ctypes.c_int32 * 16), ("matrix", ctypes.c_void_p)]


def _target_matrix(gate) -> np.ndarray:
    """Dense matrix of the gate on its target qubits (controls excluded)."""
    if hasattr(gate, "base_matrix"):
        return np.asarray(gate.base_matrix("complex128"), dtype=np.complex128)
    name = type(gate).__name__
    if name == "Unitary":
        return np.asarray(gate.parameters[0], dtype=np.complex128)
    from .matrices import Matrices

    m = Matrices("complex128")
    attr = getattr(m, name)
    return np.asarray(attr(*gate.parameters) if callable(attr) else attr, dtype=np.complex128)


def _expand(gates: Iterable) -> List:
    """Component gates in application order: nested FusedGates flattened and a FanOut
    written as one CNOT per target (its target matrix is the X of each CNOT)."""
    from . import gates as G

    out = []
    for g in gates:
        if type(g).__name__ == "FusedGate":
            out.extend(_expand(g.gates))
        elif getattr(g, "name", "") == "fanout":
            out.extend(G.CNOT(g.control_qubits[0], t) for t in g.target_qubits)
        else:
            out.append(g)
    return out


def lower(gates: Iterable) -> List[tuple]:
    """Gates -> (kind, targets, controls, complex entries) in application order."""
    out = []
    for g in gates:
        name = type(g).__name__
        if name == "FusedGate":
            out.extend(lower(g.gates))
            continue
        if getattr(g, "name", "") == "fanout":
            x = np.array([[0, 1], [1, 0]], dtype=np.complex128)
            for t in g.target_qubits:
                out.append((SV_OP_DENSE, (t,), tuple(g.control_qubits), x.ravel()))
            continue
        m = _target_matrix(g)
        targets = tuple(int(t) for t in g.target_qubits)
        controls = tuple(int(c) for c in g.control_qubits)
        if m.ndim == 2 and np.count_nonzero(m - np.diag(np.diag(m))) == 0:
            out.append((SV_OP_DIAG, targets, controls, np.diag(m).copy()))
        else:
            out.append((SV_OP_DENSE, targets, controls, m.ravel()))
    return out


def lower_density(gates: Iterable, nqubits: int) -> List[tuple]:
    """Gates acting on an n-qubit density matrix rho -> ops on the 2n-qubit vector of the
    row-major rho (cpu.py:452-498): each gate's U on the row qubits q (bit 2n-q-1) and
    conj(U) on the column qubits q + n (bit n-q-1), so the pair is rho -> U rho U^dagger."""
    out = []
    for kind, targets, controls, entries in lower(gates):
        out.append((kind, targets, controls, entries))
        out.append((kind, tuple(q + nqubits for q in targets), tuple(q + nqubits for q in controls),
                    np.conj(entries)))
    return out


class FusedProgram:
    """A circuit planned into fused passes for one state size and dtype (``ops``, when
    given, replaces the lowering of ``gates``)."""

    def __init__(self, ctx: "_lib.Context", gates, nqubits: int, dtype: str = "complex128", tile_bits: int = 0,
                 ops: Optional[List[tuple]] = None):
        lib = ctx.lib
        self.ctx = ctx
        self.nqubits = int(nqubits)
        self.dtype = dtype
        ops = lower(gates) if ops is None else ops
        arr = (GateOp * max(1, len(ops)))()
        self._keep = []
        for i, (kind, targets, controls, entries) in enumerate(ops):
            if len(controls) > 16 or len(targets) > 10:
                raise ValueError("gate has too many targets or controls for the fused engine")
            buf = np.ascontiguousarray(np.column_stack([entries.real, entries.imag]).ravel(), dtype=np.float64)
            self._keep.append(buf)
            arr[i].kind = kind
            arr[i].ntargets = len(targets)
            arr[i].ncontrols = len(controls)
            for k, t in enumerate(targets):
                arr[i].targets[k] = t
            for k, c in enumerate(controls):
                arr[i].controls[k] = c
            arr[i].matrix = buf.ctypes.data
        h = ctypes.c_void_p()
        rc = lib.sv_program_create(ctx.handle, _lib.DTYPE_CODES[dtype], self.nqubits, ctypes.cast(arr, ctypes.c_void_p),
                                   len(ops), int(tile_bits), ctypes.byref(h))
        _lib.check(rc, "sv_program_create")
        self._h = h
        self._lib = lib
        self.ngates = len(ops)
        self._keep = None
        self.specialized = False
        self.runs = 0

    def specialize(self) -> "FusedProgram":
        """Compiles pass kernels with this program's structure as literals (the engine's
        run-time specialiser, ``sv_program_specialize``); later runs launch them."""
        _lib.check(self._lib.sv_program_specialize(self.ctx.handle, self._h), "sv_program_specialize")
        self.specialized = True
        return self

    def stats(self) -> dict:
        a, b, c, d = (ctypes.c_int() for _ in range(4))
        _lib.check(self._lib.sv_program_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                              ctypes.byref(d)))
        return {"passes": a.value, "unfused": b.value, "fused_gates": c.value, "tile_bits": d.value,
                "gates": self.ngates}

    def arith_per_amplitude(self) -> float:
        """Arithmetic lane instructions (FFMA and FMUL) per amplitude of one run as
        planned (``sv_program_arith_per_amplitude``)."""
        v = ctypes.c_double()
        _lib.check(self._lib.sv_program_arith_per_amplitude(self._h, ctypes.byref(v)),
                   "sv_program_arith_per_amplitude")
        return v.value

    def param_bytes(self) -> int:
        """Bytes of the pass parameter blocks one run sends to the device with its
        launches (gate coefficients and the pass layout, as kernel parameters)."""
        st = self.stats()
        if st["passes"] == 0:
            return 0
        ptr, nb = ctypes.c_void_p(), ctypes.c_size_t()
        _lib.check(self._lib.sv_program_pass_params(self._h, 0, ctypes.byref(ptr), ctypes.byref(nb)))
        return st["passes"] * nb.value

    def run(self, state):
        if state.numel() != (1 << self.nqubits):
            raise ValueError("state size does not match the program")
        if str(state.dtype).replace("torch.", "") != self.dtype:
            raise TypeError(f"program was planned for {self.dtype} states")
        if not state.is_cuda or not state.is_contiguous():
            raise ValueError("state must be a contiguous CUDA tensor")
        _lib.check(self._lib.sv_program_run(self.ctx.handle, self._h, ctypes.c_void_p(state.data_ptr())),
                   "sv_program_run")
        self.runs += 1
        return state

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sv_program_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def matrix_fused(gate, dtype: str = "complex128") -> np.ndarray:
    """Dense matrix of a FusedGate on its (sorted) target qubits, qubit[0] most significant."""
    qubits = list(gate.target_qubits)
    k = len(qubits)
    u = np.eye(2**k, dtype=np.complex128)
    for g in _expand(gate.gates):
        m = _target_matrix(g)
        gq = list(g.control_qubits) + list(g.target_qubits)
        nc = len(g.control_qubits)
        full = m
        for _ in range(nc):
            d = full.shape[0]
            c = np.eye(2 * d, dtype=np.complex128)
            c[d:, d:] = full
            full = c
        # embed `full` (on qubits gq, gq[0] most significant) into the fused space
        t = full.reshape((2,) * (2 * len(gq)))
        big = np.eye(2**k, dtype=np.complex128).reshape((2,) * (2 * k))
        axes = [qubits.index(q) for q in gq]
        big = np.tensordot(t, big, axes=(list(range(len(gq), 2 * len(gq))), axes))
        big = np.moveaxis(big, list(range(len(gq))), axes)
        u = big.reshape(2**k, 2**k) @ u
    return u.astype(dtype)
