"""Adjoint-method gradients of the transverse-field Ising energy, behind torch.autograd.

``AdjointTFIM`` evaluates, for many hardware-efficient-ansatz circuits of one shape
(n qubits, L layers of RY(t) RZ(p) on every qubit plus a CNOT ladder), the energies
E = <psi|H|psi> with H = -sum_i Z_i Z_{i+1} - h sum_i X_i and all dE/dt in one
forward pass and one reverse sweep per circuit (``sv_adjoint_*`` in the engine): the
forward state is checkpointed every ``checkpoint_every`` layers and restored during
the sweep, and the gradient inner products accumulate in FP64.
``HEAEnergy`` wraps it as a ``torch.autograd.Function``.  Parameters have shape
(ncirc, L, n, 2): [..., 0] the RY angles, [..., 1] the RZ angles.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .fusion import GateOp

SV_OP_DENSE, SV_OP_DIAG = 0, 1
GEN_NONE, GEN_X, GEN_Y, GEN_Z = 0, 1, 2, 3


def _hea_structure(n: int, layers: int):
    """Op list template: (kind, target, control, generator, parameter slot)."""
    ops = []
    for layer in range(layers):
        for q in range(n):
            ops.append(("ry", q, -1, GEN_Y, (layer * n + q) * 2))
            ops.append(("rz", q, -1, GEN_Z, (layer * n + q) * 2 + 1))
        for q in range(n - 1):
            ops.append(("cx", q + 1, q, GEN_NONE, -1))
    return ops


class AdjointTFIM:
    def __init__(self, backend, nqubits: int, layers: int, ncirc: int, dtype: str = "complex64", h: float = 1.0,
                 checkpoint_every: int = 5, tile_bits: int = 0, specialize: bool = False):
        self.backend = backend
        self.ctx = backend.ctx
        self.lib = backend.lib
        self.n, self.layers, self.ncirc, self.dtype, self.h = nqubits, layers, ncirc, dtype, float(h)
        self.template = _hea_structure(nqubits, layers)
        self.nops = len(self.template)
        self.nparams = layers * nqubits * 2
        self.gens = np.array([t[3] for t in self.template], dtype=np.int8)
        self.params_idx = np.array([t[4] for t in self.template], dtype=np.int32)
        per_layer = 3 * nqubits - 1
        ends = [min(k * checkpoint_every, layers) * per_layer for k in range(1, (layers + checkpoint_every - 1)
                                                                            // checkpoint_every + 1)]
        ends[-1] = self.nops
        self.segment_ends = np.array(ends, dtype=np.int32)
        self.tile_bits = int(tile_bits)
        # compile every forward and reverse-sweep pass with the structure as literals
        # (NVRTC) when the engine is created; the interpreting kernels otherwise
        self.specialize = bool(specialize)
        self._h = None

    # op arrays for all circuits (vectorised matrices, then one struct per op)
    def _build(self, params: np.ndarray):
        params = np.asarray(params, dtype=np.float64).reshape(self.ncirc, self.layers, self.n, 2)
        th = params[..., 0].reshape(self.ncirc, -1) / 2
        ph = params[..., 1].reshape(self.ncirc, -1) / 2
        c, s = np.cos(th), np.sin(th)
        ry = np.stack([c, np.zeros_like(c), -s, np.zeros_like(c), s, np.zeros_like(c), c, np.zeros_like(c)], axis=-1)
        rz = np.stack([np.cos(ph), -np.sin(ph), np.cos(ph), np.sin(ph)], axis=-1)
        x = np.array([0.0, 0.0, 1.0, 0.0, 1.0, 0.0, 0.0, 0.0])
        self._keep = [ry, rz, x]
        arrays = (ctypes.c_void_p * self.ncirc)()
        self._arrs = []
        ry = np.ascontiguousarray(ry)
        rz = np.ascontiguousarray(rz)
        for ci in range(self.ncirc):
            arr = (GateOp * self.nops)()
            k_ry = k_rz = 0
            for j, (kind, t, ctl, gen, slot) in enumerate(self.template):
                op = arr[j]
                op.ntargets = 1
                op.targets[0] = t
                if kind == "ry":
                    op.kind = SV_OP_DENSE
                    op.matrix = ry[ci, slot // 2].ctypes.data
                elif kind == "rz":
                    op.kind = SV_OP_DIAG
                    op.matrix = rz[ci, slot // 2].ctypes.data
                else:
                    op.kind = SV_OP_DENSE
                    op.ncontrols = 1
                    op.controls[0] = ctl
                    op.matrix = x.ctypes.data
            self._arrs.append(arr)
            arrays[ci] = ctypes.cast(arr, ctypes.c_void_p).value
        return arrays

    def __call__(self, params: np.ndarray):
        arrays = self._build(params)
        if self._h is None:
            h = ctypes.c_void_p()
            _lib.check(self.lib.sv_adjoint_create(self.ctx.handle, _lib.DTYPE_CODES[self.dtype], self.ncirc, self.n,
                                                  arrays, self.nops, self.gens.ctypes.data,
                                                  self.params_idx.ctypes.data, self.nparams,
                                                  self.segment_ends.ctypes.data, len(self.segment_ends),
                                                  self.tile_bits, ctypes.byref(h)), "sv_adjoint_create")
            self._h = h
            if self.specialize:
                _lib.check(self.lib.sv_adjoint_specialize(self.ctx.handle, self._h), "sv_adjoint_specialize")
        else:
            _lib.check(self.lib.sv_adjoint_update(self.ctx.handle, self._h, arrays, self.nops, self.gens.ctypes.data,
                                                  self.params_idx.ctypes.data), "sv_adjoint_update")
        energies = np.zeros(self.ncirc, dtype=np.float64)
        grads = np.zeros((self.ncirc, self.nparams), dtype=np.float64)
        _lib.check(self.lib.sv_adjoint_run(self.ctx.handle, self._h, self.h, energies.ctypes.data, grads.ctypes.data),
                   "sv_adjoint_run")
        self._arrs = None
        return energies, grads.reshape(self.ncirc, self.layers, self.n, 2)

    def state(self, i: int):
        import torch

        from .batch import _DeviceArray

        p = ctypes.c_void_p()
        _lib.check(self.lib.sv_adjoint_state(self._h, int(i), ctypes.byref(p)))
        typestr = "<c16" if self.dtype == "complex128" else "<c8"
        return torch.as_tensor(_DeviceArray(p.value, 1 << self.n, typestr), device="cuda")

    def close(self):
        if self._h is not None:
            self.lib.sv_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _autograd_function():
    import torch

    class HEAEnergy(torch.autograd.Function):
        """energies = HEAEnergy.apply(params, engine); params (ncirc, L, n, 2) float64."""

        @staticmethod
        def forward(ctx, params, engine):
            energies, grads = engine(params.detach().cpu().numpy())
            ctx.save_for_backward(torch.from_numpy(grads).to(params.device, params.dtype))
            return torch.from_numpy(energies).to(params.device, params.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            (grads,) = ctx.saved_tensors
            return grad_out.reshape(-1, 1, 1, 1) * grads, None

    return HEAEnergy


def __getattr__(name):
    if name == "HEAEnergy":
        return _autograd_function()
    raise AttributeError(name)
