"""Host-side planning and run-time specialisation without a GPU.

``sv_program_create`` plans entirely on the host (the context is only carried along),
so every gate family, dtype and tile size can be planned here; the planner's phase
folding, sign merging, run merging and phase packing all run.  ``sv_program_specialize``
generates each pass's CUDA source and compiles it with NVRTC before it needs a device,
so on this machine it must get as far as selecting the device and fail there."""
import ctypes

import numpy as np
import pytest

from qibojit_gb300 import _lib, circuits
from qibojit_gb300.fusion import GateOp, lower
from tests.circuits_random import random_circuit


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def _ops(circ):
    ops = lower(circ.queue)
    arr = (GateOp * max(1, len(ops)))()
    keep = []
    for i, (kind, targets, controls, entries) in enumerate(ops):
        buf = np.ascontiguousarray(np.column_stack([entries.real, entries.imag]).ravel(), dtype=np.float64)
        keep.append(buf)
        arr[i].kind, arr[i].ntargets, arr[i].ncontrols = kind, len(targets), len(controls)
        for k, t in enumerate(targets):
            arr[i].targets[k] = t
        for k, c in enumerate(controls):
            arr[i].controls[k] = c
        arr[i].matrix = buf.ctypes.data
    return arr, len(ops), keep


def _create(lib, circ, dtype, tile_bits):
    arr, nops, keep = _ops(circ)
    ctx = ctypes.create_string_buffer(512)  # never dereferenced by the planner
    h = ctypes.c_void_p()
    rc = lib.sv_program_create(ctypes.addressof(ctx), _lib.DTYPE_CODES[dtype], circ.nqubits,
                               ctypes.cast(arr, ctypes.c_void_p), nops, tile_bits, ctypes.byref(h))
    return rc, h, ctx, keep


def _stats(lib, h):
    a, b, c, d = (ctypes.c_int() for _ in range(4))
    _lib.check(lib.sv_program_stats(h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)))
    return a.value, b.value, c.value, d.value


@pytest.mark.parametrize("dt", ["complex64", "complex128"])
@pytest.mark.parametrize("n,ngates,seed,tile_bits", [(8, 60, 1, 0), (9, 120, 2, 8), (12, 200, 3, 10),
                                                     (16, 300, 4, 0), (22, 400, 5, 12)])
def test_random_circuits_plan(lib, n, ngates, seed, tile_bits, dt):
    circ = random_circuit(n, ngates, seed)
    rc, h, _, _ = _create(lib, circ, dt, tile_bits)
    assert rc == _lib.SV_OK, _lib.last_error()
    try:
        passes, unfused, fused, kt = _stats(lib, h)
        assert passes >= 1 and fused + unfused >= 1 and kt <= n
    finally:
        lib.sv_program_destroy(h)


@pytest.mark.parametrize("dt,tile_bits", [("complex64", 13), ("complex128", 12)])
def test_benchmark_circuits_plan(lib, dt, tile_bits):
    for circ in (circuits.brickwork(30, 20, 1234), circuits.qft(24), circuits.hea(20, 6)):
        rc, h, _, _ = _create(lib, circ, dt, min(tile_bits, circ.nqubits))
        assert rc == _lib.SV_OK, _lib.last_error()
        lib.sv_program_destroy(h)


def test_bad_tile_bits_are_rejected(lib):
    # complex64 tiles hold at most 2^13 amplitudes (512 threads of 16)
    rc, _, _, _ = _create(lib, circuits.brickwork(20, 2, 1), "complex64", 15)
    assert rc == _lib.SV_ERR_ARG


@pytest.mark.parametrize("dt", ["complex64", "complex128"])
@pytest.mark.parametrize("circ", [random_circuit(12, 150, 7), circuits.brickwork(16, 6, 8), circuits.qft(14)],
                         ids=["random", "brickwork", "qft"])
def test_specialised_sources_compile(lib, circ, dt):
    """Phase folding, packing and code generation run, and NVRTC compiles every pass for
    sm_103a; without a GPU the call then stops at device selection."""
    rc, h, ctx, _ = _create(lib, circ, dt, 8)
    assert rc == _lib.SV_OK
    try:
        rc = lib.sv_program_specialize(ctypes.addressof(ctx), h)
        msg = _lib.last_error()
        if rc == _lib.SV_ERR_UNSUPPORTED:
            pytest.skip(msg)
        assert rc == _lib.SV_ERR_CUDA and "cudaSetDevice" in msg, msg
    finally:
        lib.sv_program_destroy(h)


def test_disk_cache_of_compiled_passes(lib, monkeypatch):
    """NVRTC output goes to the on-disk cache: one file per distinct pass source, found
    again (not rewritten) by a later specialisation of the same structure, and a damaged
    file is replaced by a fresh compile."""
    import glob
    import os
    import shutil

    cache = os.path.join(os.path.dirname(_lib.__file__), "_build", "test_disk_cache")
    shutil.rmtree(cache, ignore_errors=True)
    monkeypatch.setenv("QIBOJIT_GB300_CACHE", cache)
    circ = circuits.brickwork(14, 4, 3)

    def specialise():
        rc, h, ctx, _ = _create(lib, circ, "complex64", 10)
        assert rc == _lib.SV_OK
        try:
            rc = lib.sv_program_specialize(ctypes.addressof(ctx), h)
            msg = _lib.last_error()
            if rc == _lib.SV_ERR_UNSUPPORTED:
                pytest.skip(msg)
            assert rc == _lib.SV_ERR_CUDA and "cudaSetDevice" in msg, msg
        finally:
            lib.sv_program_destroy(h)

    try:
        specialise()
        files = sorted(glob.glob(os.path.join(cache, "*.cubin")))
        assert files
        for f in files:
            data = open(f, "rb").read()
            assert data[:8] == b"SVCUBIN1"
            klen = int.from_bytes(data[8:16], "little")
            clen = int.from_bytes(data[16 + klen:24 + klen], "little")
            assert len(data) == 24 + klen + clen and data[24 + klen:28 + klen] == b"\x7fELF"
        stamps = {f: os.stat(f).st_mtime_ns for f in files}
        with open(files[0], "r+b") as fh:  # damage one cubin
            fh.seek(-8, os.SEEK_END)
            fh.truncate()
        specialise()
        again = sorted(glob.glob(os.path.join(cache, "*.cubin")))
        assert again == files
        assert [f for f in files if os.stat(f).st_mtime_ns != stamps[f]] == [files[0]]
        assert not glob.glob(os.path.join(cache, "*.tmp.*"))
    finally:
        shutil.rmtree(cache, ignore_errors=True)
