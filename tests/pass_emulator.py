"""Host emulation of a planned program's fused passes, for checking the planner on CPU.

A pass block (``sv_program_pass_params``, laid out as ``sv_pass_layout`` reports) is
what the tile kernel receives.  This module restates the tile kernel's semantics
(``k_fused_pass`` in ``qibojit_gb300/csrc/sv_fused.cu`` and the register ops of
``sv_device.cuh``) with numpy, vectorised over every tile and thread of a phase:

* tile ``t`` covers the global indices ``tile_origin(t) | dep(e)``, ``e`` the local
  index whose bit b sits at global bit ``tile_pos[b]`` (ascending), ``tile_origin``
  inserting zeros at those positions into ``t``;
* in a phase the register slots are local bits ``rb[0..3]``; a thread holds the 16
  amplitudes ``lbase | sum_u bit_u(j) << rb[u]``, ``lbase`` its index deposited into the
  other local bits;
* ops run in order on the 16 registers; sign diagonals collect a negation mask that
  is applied before the next mixing op and at the end of the phase, as the kernel does.

Arithmetic is complex128 on the block's coefficients (complex64 coefficients are
widened exactly), so a complex64 program agrees with the oracle to its coefficients'
rounding and a complex128 program to double rounding."""
from __future__ import annotations

import ctypes

import numpy as np

from qibojit_gb300 import _lib

(FOP_DENSE1, FOP_DENSE2, FOP_DIAG, FOP_SIGN, FOP_D1RUN, FOP_X1, FOP_DENSE1R, FOP_SWAP2, FOP_GRADX, FOP_GRADY,
 FOP_GRADZ, FOP_DIAGR, FOP_D1RUNR, FOP_DENSE1P) = range(14)
FLAG_OMASK, FLAG_TMASK = 1, 2
_MIXING = (FOP_D1RUN, FOP_D1RUNR, FOP_DENSE1, FOP_DENSE1R, FOP_DENSE1P, FOP_X1, FOP_SWAP2, FOP_DENSE2)

_KEYS = ["size", "n", "kt", "nphases", "nops", "ntiles", "tile_pos", "coef_goff", "phases", "ops", "coef",
         "phase_size", "rb", "op_begin", "op_end", "op_size", "type", "u0", "u1", "nd", "tb", "ob", "jmask", "tmask",
         "op_coef", "omask", "rpart", "neg", "flags", "nrun", "ru", "coef_size"]


def layout(lib, dtype: int) -> dict:
    o = (ctypes.c_int64 * 32)()
    _lib.check(lib.sv_pass_layout(dtype, o, 32), "sv_pass_layout")
    return dict(zip(_KEYS, list(o)))


def _read(buf: bytes, off: int, fmt: str, count: int = 1):
    a = np.frombuffer(buf, dtype=np.dtype(fmt), count=count, offset=off)
    return a if count > 1 else a[0].item()


def read_pass(lib, prog, i: int, dtype: int) -> dict:
    """Decodes pass ``i`` of program handle ``prog``."""
    L = layout(lib, dtype)
    p, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
    _lib.check(lib.sv_program_pass_params(prog, i, ctypes.byref(p), ctypes.byref(nbytes)), "sv_program_pass_params")
    buf = ctypes.string_at(p.value, nbytes.value)
    kt = _read(buf, L["kt"], "<i4")
    out = {"n": _read(buf, L["n"], "<i4"), "kt": kt, "ntiles": _read(buf, L["ntiles"], "<i8"),
           "tile_pos": [int(x) for x in _read(buf, L["tile_pos"], "<i4", 14)[:kt]]}
    nph, nops = _read(buf, L["nphases"], "<i4"), _read(buf, L["nops"], "<i4")
    phases = []
    for k in range(nph):
        b = L["phases"] + k * L["phase_size"]
        phases.append(([int(x) for x in _read(buf, b + L["rb"], "u1", 4)], _read(buf, b + L["op_begin"], "<u2"),
                       _read(buf, b + L["op_end"], "<u2")))
    ops = []
    for k in range(nops):
        b = L["ops"] + k * L["op_size"]
        ops.append({"type": _read(buf, b + L["type"], "u1"), "u0": _read(buf, b + L["u0"], "u1"),
                    "u1": _read(buf, b + L["u1"], "u1"), "nd": _read(buf, b + L["nd"], "u1"),
                    "tb": [int(x) for x in _read(buf, b + L["tb"], "i1", 3)],
                    "ob": [int(x) for x in _read(buf, b + L["ob"], "i1", 3)],
                    "jmask": _read(buf, b + L["jmask"], "<u2"), "tmask": _read(buf, b + L["tmask"], "<u4"),
                    "coef": _read(buf, b + L["op_coef"], "<u4"), "omask": _read(buf, b + L["omask"], "<u8"),
                    "rpart": _read(buf, b + L["rpart"], "<u8"), "neg": [int(x) for x in _read(buf, b + L["neg"], "<u2", 8)],
                    "flags": _read(buf, b + L["flags"], "u1"), "nrun": _read(buf, b + L["nrun"], "u1"),
                    "ru": [int(x) for x in _read(buf, b + L["ru"], "u1", 4)]})
    ncoef = (L["size"] - L["coef"]) // L["coef_size"]
    real = np.frombuffer(buf, dtype="<f8" if dtype == _lib.SV_C128 else "<f4", count=2 * ncoef, offset=L["coef"])
    out["coef"] = real[0::2].astype(np.float64) + 1j * real[1::2].astype(np.float64)
    out["phases"], out["ops"] = phases, ops
    return out


def _deposit(values: np.ndarray, positions) -> np.ndarray:
    """Bit b of each value moved to bit positions[b]."""
    out = np.zeros_like(values)
    for b, p in enumerate(positions):
        out |= ((values >> b) & 1) << p
    return out


def run_pass(ps: dict, state: np.ndarray) -> None:
    """Applies one decoded pass to ``state`` (complex128, 2^n entries) in place."""
    n, kt, tile_pos = ps["n"], ps["kt"], ps["tile_pos"]
    outer = [b for b in range(n) if b not in tile_pos]
    tiles = np.arange(ps["ntiles"], dtype=np.int64)
    base_t = _deposit(tiles, outer)
    c = ps["coef"]
    for rb, ob_, oe in ps["phases"]:
        nonreg = [b for b in range(kt) if b not in rb]
        threads = np.arange(1 << (kt - 4), dtype=np.int64)
        lbase_th = _deposit(threads, nonreg)
        # columns: (tile, thread) pairs
        base = np.repeat(base_t, len(threads))
        lbase = np.tile(lbase_th, len(tiles))
        jreg = np.array([sum(((j >> u) & 1) << rb[u] for u in range(4)) for j in range(16)], dtype=np.int64)
        loc = lbase[None, :] | jreg[:, None]
        gidx = base[None, :] | _deposit(loc, tile_pos)
        v = state[gidx]
        neg = np.zeros(v.shape[1], dtype=np.int64)

        def flush():
            nonlocal neg
            for j in range(16):
                m = ((neg >> j) & 1).astype(bool)
                v[j, m] = -v[j, m]
            neg = np.zeros_like(neg)

        for op in ps["ops"][ob_:oe]:
            t = op["type"]
            if t in _MIXING:
                flush()
            if t in (FOP_D1RUN, FOP_D1RUNR):
                for k in range(op["nrun"]):
                    m = c[op["coef"] + 4 * k: op["coef"] + 4 * k + 4]
                    _dense1(v, op["ru"][k], m.real if t == FOP_D1RUNR else m, 0xFFFF, None)
                continue
            if t == FOP_DIAGR:
                v *= c[op["coef"]: op["coef"] + 16][:, None]
                continue
            cond = np.ones(v.shape[1], dtype=bool)
            if op["flags"] & FLAG_OMASK:
                cond &= (base & op["omask"]) == op["omask"]
            if op["flags"] & FLAG_TMASK:
                cond &= (lbase & op["tmask"]) == op["tmask"]
            assert bool(op["flags"] & FLAG_OMASK) == (op["omask"] != 0)
            assert bool(op["flags"] & FLAG_TMASK) == (op["tmask"] != 0)
            m = c[op["coef"]: op["coef"] + 16]
            if t == FOP_DENSE1:
                _dense1(v, op["u0"], m[:4], op["jmask"], cond)
            elif t == FOP_DENSE1R:
                _dense1(v, op["u0"], m[:4].real, op["jmask"], cond)
            elif t == FOP_DENSE1P:
                _pivot1(v, op["u0"], op["u1"], m[0].real, m[1].real, op["jmask"], cond)
            elif t == FOP_X1:
                _perm(v, [(j, j | (1 << op["u0"])) for j in range(16) if not (j >> op["u0"]) & 1], op["jmask"], cond)
            elif t == FOP_SWAP2:
                u0, u1 = op["u0"], op["u1"]
                bits = (1 << u0) | (1 << u1)
                _perm(v, [(j | (1 << u1), j | (1 << u0)) for j in range(16) if not j & bits], op["jmask"], cond)
            elif t == FOP_DENSE2:
                _dense2(v, op["u0"], op["u1"], m, op["jmask"], cond)
            elif t in (FOP_SIGN, FOP_DIAG):
                tp = np.zeros(v.shape[1], dtype=np.int64)
                for i in range(op["nd"]):
                    sh = op["nd"] - 1 - i
                    if op["tb"][i] >= 0:
                        tp |= ((lbase >> op["tb"][i]) & 1) << sh
                    elif op["ob"][i] >= 0:
                        tp |= ((base >> op["ob"][i]) & 1) << sh
                if t == FOP_SIGN:
                    table = np.array(op["neg"], dtype=np.int64)
                    neg = np.where(cond, neg ^ table[tp], neg)
                else:
                    for j in range(16):
                        if not (op["jmask"] >> j) & 1:
                            continue
                        r = (op["rpart"] >> (4 * j)) & 15
                        f = c[op["coef"] + (r | tp)]
                        v[j] = np.where(cond, f * v[j], v[j])
            else:
                raise NotImplementedError(f"op type {t}")
        flush()
        state[gidx] = v


def _mask_pairs(jmask, u):
    return [j for j in range(16) if not (j >> u) & 1 and (jmask >> j) & 1]


def _dense1(v, u, m, jmask, cond):
    for j in _mask_pairs(jmask, u):
        k = j | (1 << u)
        x, y = v[j].copy(), v[k].copy()
        a = m[0] * x + m[1] * y
        b = m[2] * x + m[3] * y
        if cond is None:
            v[j], v[k] = a, b
        else:
            v[j], v[k] = np.where(cond, a, x), np.where(cond, b, y)


def _pivot1(v, u, form, r0, r1, jmask, cond):
    for j in _mask_pairs(jmask, u):
        k = j | (1 << u)
        x, y = v[j].copy(), v[k].copy()
        a = r0 * x + y if form & 1 else r0 * y + x
        b = r1 * x + y if form & 2 else r1 * y + x
        v[j], v[k] = np.where(cond, a, x), np.where(cond, b, y)


def _perm(v, pairs, jmask, cond):
    for a_, b_ in pairs:
        base_j = a_ & b_
        if not (jmask >> base_j) & 1:
            continue
        x, y = v[a_].copy(), v[b_].copy()
        v[a_], v[b_] = np.where(cond, y, x), np.where(cond, x, y)


def _dense2(v, u0, u1, m, jmask, cond):
    bits = (1 << u0) | (1 << u1)
    for j in range(16):
        if j & bits or not (jmask >> j) & 1:
            continue
        idx = [j, j | (1 << u1), j | (1 << u0), j | bits]
        x = [v[i].copy() for i in idx]
        for r in range(4):
            o = m[4 * r] * x[0] + m[4 * r + 1] * x[1] + m[4 * r + 2] * x[2] + m[4 * r + 3] * x[3]
            v[idx[r]] = np.where(cond, o, x[r])


def run_program(lib, prog, dtype: int, state: np.ndarray) -> np.ndarray:
    """All passes of a program without unfused segments, on a copy of ``state``."""
    npasses, nunfused = ctypes.c_int(), ctypes.c_int()
    _lib.check(lib.sv_program_stats(prog, ctypes.byref(npasses), ctypes.byref(nunfused), None, None))
    if nunfused.value:
        raise ValueError("the program has unfused segments")
    out = np.array(state, dtype=np.complex128)
    for i in range(npasses.value):
        run_pass(read_pass(lib, prog, i, dtype), out)
    return out
