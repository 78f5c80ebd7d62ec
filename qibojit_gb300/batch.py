"""Batched execution of many circuits of uneven size (variational workloads).

``BatchedCircuits`` lowers every circuit to engine ops (``fusion.lower``) and hands
them to ``sv_batch_create``: circuits with the same gate structure share one fused
plan, each keeps its own parameters, and a run applies all of them as batched
tile-kernel launches recorded once as a CUDA graph.  Energies of the transverse-field
Ising chain are reduced on the device in FP64.

``hea_batch`` generates the hardware-efficient-ansatz workload: per circuit a qubit
count uniform on {10..22} and a layer count uniform on {4..12}; each layer is
RY(t) RZ(p) on every qubit (angles uniform [0, 2pi)) followed by a CNOT ladder
q -> q+1.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np

from . import _lib
from . import gates as G
from .fusion import GateOp, lower


def hea_circuit(n: int, layers: int, params: np.ndarray) -> "G.Circuit":
    """params: (layers, n, 2) angles (RY, RZ)."""
    c = G.Circuit(n)
    for layer in range(layers):
        for q in range(n):
            c.add(G.RY(q, theta=float(params[layer, q, 0])))
            c.add(G.RZ(q, theta=float(params[layer, q, 1])))
        for q in range(n - 1):
            c.add(G.CNOT(q, q + 1))
    return c


def hea_batch(ncirc: int, seed: int = 1234, nmin: int = 10, nmax: int = 22, lmin: int = 4, lmax: int = 12):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ncirc):
        n = int(rng.integers(nmin, nmax + 1))
        layers = int(rng.integers(lmin, lmax + 1))
        params = rng.uniform(0, 2 * np.pi, size=(layers, n, 2))
        out.append((n, layers, params))
    return out


class _DeviceArray:
    """Zero-copy view of engine-owned device memory (``__cuda_array_interface__``)."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


class BatchedCircuits:
    def __init__(self, backend, circuits: Sequence, dtype: str = "complex64", tile_bits: int = 0):
        self.backend = backend
        self.ctx = backend.ctx
        self.lib = backend.lib
        self.dtype = dtype
        self.ncirc = len(circuits)
        nq = (ctypes.c_int32 * self.ncirc)(*[c.nqubits for c in circuits])
        ptrs = (ctypes.c_void_p * self.ncirc)()
        counts = (ctypes.c_int32 * self.ncirc)()
        keep = []
        for i, circ in enumerate(circuits):
            ops = lower(circ.queue)
            arr = (GateOp * max(1, len(ops)))()
            for k, (kind, targets, controls, entries) in enumerate(ops):
                buf = np.ascontiguousarray(np.column_stack([entries.real, entries.imag]).ravel(), dtype=np.float64)
                keep.append(buf)
                arr[k].kind, arr[k].ntargets, arr[k].ncontrols = kind, len(targets), len(controls)
                for j, t in enumerate(targets):
                    arr[k].targets[j] = t
                for j, c in enumerate(controls):
                    arr[k].controls[j] = c
                arr[k].matrix = buf.ctypes.data
            keep.append(arr)
            ptrs[i] = ctypes.cast(arr, ctypes.c_void_p).value
            counts[i] = len(ops)
        h = ctypes.c_void_p()
        _lib.check(self.lib.sv_batch_create(self.ctx.handle, _lib.DTYPE_CODES[dtype], self.ncirc, nq, ptrs, counts,
                                            int(tile_bits), ctypes.byref(h)), "sv_batch_create")
        self._h = h
        self.nqubits = [c.nqubits for c in circuits]

    @classmethod
    def from_hea(cls, backend, specs, dtype: str = "complex64", tile_bits: int = 0):
        """Batch of hardware-efficient-ansatz circuits from ``hea_batch`` specs, with the
        op arrays built directly from the angles (no per-gate Python objects)."""
        self = cls.__new__(cls)
        self.backend, self.ctx, self.lib, self.dtype = backend, backend.ctx, backend.lib, dtype
        self.ncirc = len(specs)
        self.nqubits = [n for n, _, _ in specs]
        nq = (ctypes.c_int32 * self.ncirc)(*self.nqubits)
        ptrs = (ctypes.c_void_p * self.ncirc)()
        counts = (ctypes.c_int32 * self.ncirc)()
        x = np.array([0.0, 0.0, 1.0, 0.0, 1.0, 0.0, 0.0, 0.0])
        keep = [x]
        for i, (n, layers, params) in enumerate(specs):
            th = params[..., 0].reshape(-1) / 2
            ph = params[..., 1].reshape(-1) / 2
            c, s_ = np.cos(th), np.sin(th)
            z = np.zeros_like(c)
            ry = np.ascontiguousarray(np.stack([c, z, -s_, z, s_, z, c, z], axis=-1))
            rz = np.ascontiguousarray(np.stack([np.cos(ph), -np.sin(ph), np.cos(ph), np.sin(ph)], axis=-1))
            keep += [ry, rz]
            nops = layers * (3 * n - 1)
            arr = (GateOp * nops)()
            k = 0
            for layer in range(layers):
                for q in range(n):
                    a = arr[k]
                    a.kind, a.ntargets = 0, 1
                    a.targets[0] = q
                    a.matrix = ry[layer * n + q].ctypes.data
                    b = arr[k + 1]
                    b.kind, b.ntargets = 1, 1
                    b.targets[0] = q
                    b.matrix = rz[layer * n + q].ctypes.data
                    k += 2
                for q in range(n - 1):
                    a = arr[k]
                    a.kind, a.ntargets, a.ncontrols = 0, 1, 1
                    a.targets[0] = q + 1
                    a.controls[0] = q
                    a.matrix = x.ctypes.data
                    k += 1
            keep.append(arr)
            ptrs[i] = ctypes.cast(arr, ctypes.c_void_p).value
            counts[i] = nops
        h = ctypes.c_void_p()
        _lib.check(self.lib.sv_batch_create(self.ctx.handle, _lib.DTYPE_CODES[dtype], self.ncirc, nq, ptrs, counts,
                                            int(tile_bits), ctypes.byref(h)), "sv_batch_create")
        self._h = h
        return self

    def stats(self) -> dict:
        g, p, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        _lib.check(self.lib.sv_batch_stats(self._h, ctypes.byref(g), ctypes.byref(p), ctypes.byref(b)))
        pb, ar = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.sv_batch_pass_bytes(self._h, ctypes.byref(pb)))
        _lib.check(self.lib.sv_batch_arith(self._h, ctypes.byref(ar)))
        return {"groups": g.value, "passes": p.value, "state_bytes": b.value, "pass_bytes": pb.value,
                "arith_instructions": ar.value}

    def run(self) -> None:
        _lib.check(self.lib.sv_batch_run(self.ctx.handle, self._h), "sv_batch_run")

    def specialize(self) -> "BatchedCircuits":
        """Compiles one pass kernel per group and pass with the group's structure as
        literals (``sv_batch_specialize``: seconds, once per structure in the process);
        later runs launch them."""
        _lib.check(self.lib.sv_batch_specialize(self.ctx.handle, self._h), "sv_batch_specialize")
        return self

    def set_executor(self, executor: str) -> "BatchedCircuits":
        """"graph": a launch per group and pass over four streams, recorded as one CUDA
        graph (the default); "persistent": the whole batch in one cooperative launch of
        an interpreting kernel (``sv_batch_set_executor``)."""
        codes = {"graph": 0, "persistent": 1}
        if executor not in codes:
            raise ValueError(f"executor must be one of {sorted(codes)}")
        _lib.check(self.lib.sv_batch_set_executor(self.ctx.handle, self._h, codes[executor]),
                   "sv_batch_set_executor")
        return self

    def tfim_energies(self, h: float = 1.0) -> np.ndarray:
        out = np.zeros(self.ncirc, dtype=np.float64)
        _lib.check(self.lib.sv_batch_tfim_energy(self.ctx.handle, self._h, float(h), out.ctypes.data),
                   "sv_batch_tfim_energy")
        return out

    def state(self, i: int):
        """The state of circuit i as a torch CUDA tensor (a view, valid while the batch lives)."""
        import torch

        p, n = ctypes.c_void_p(), ctypes.c_int()
        _lib.check(self.lib.sv_batch_state(self._h, int(i), ctypes.byref(p), ctypes.byref(n)))
        typestr = "<c16" if self.dtype == "complex128" else "<c8"
        return torch.as_tensor(_DeviceArray(p.value, 1 << n.value, typestr), device="cuda")

    def close(self):
        if getattr(self, "_h", None):
            self.lib.sv_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tfim_energy_dense(state: np.ndarray, n: int, h: float = 1.0) -> float:
    """Reference TFIM energy of a state vector (numpy, FP64)."""
    psi = np.asarray(state, dtype=np.complex128)
    idx = np.arange(1 << n)
    e = 0.0
    p = np.abs(psi) ** 2
    for i in range(n - 1):
        bi = (idx >> (n - 1 - i)) & 1
        bj = (idx >> (n - 2 - i)) & 1
        e -= np.sum(p * (1 - 2 * (bi ^ bj)))
    for i in range(n):
        e -= h * np.real(np.vdot(psi, psi[idx ^ (1 << (n - 1 - i))]))
    return float(e)
