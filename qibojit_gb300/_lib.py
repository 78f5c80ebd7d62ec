"""ctypes binding of the engine's C ABI (``include/qibojit_gb300.h``).

The shared library is loaded from the package folder; if it is missing, every
entry point raises instead of falling back to any other implementation.  Status
codes map to the exceptions the reference raises for the same conditions
(``src/qibojit/backends/gpu.py:85-91`` ImportError without a device,
``gpu.py:989-993`` ValueError for bad targets, ``gpu.py:733-739`` RuntimeError
when out of memory).
"""
from __future__ import annotations

import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libqibojit_gb300.so")

SV_OK, SV_ERR_ARG, SV_ERR_OOM, SV_ERR_CUDA, SV_ERR_TIMEOUT, SV_ERR_UNSUPPORTED, SV_ERR_NO_DEVICE = range(7)
SV_C128, SV_C64, SV_F64, SV_F32 = range(4)
DTYPE_CODES = {"complex128": SV_C128, "complex64": SV_C64, "float64": SV_F64, "float32": SV_F32}
ONE_KINDS = {"apply_gate": 0, "apply_x": 1, "apply_y": 2, "apply_z": 3, "apply_z_pow": 4}
TWO_KINDS = {"apply_two_qubit_gate": 0, "apply_swap": 1, "apply_fsim": 2}

# every symbol the header declares; tests check the library exports all of them
EXPORTS = (
    "sv_version", "sv_last_error", "sv_device_count", "sv_context_create", "sv_context_destroy",
    "sv_context_set_stream", "sv_context_set_dense_mode", "sv_context_set_c128_arithmetic", "sv_sync", "sv_zero_state", "sv_apply_one_qubit", "sv_apply_two_qubit",
    "sv_apply_multi_qubit", "sv_collapse_state", "sv_probabilities", "sv_density_probabilities", "sv_axpby",
    "sv_measure_frequencies",
    "sv_collapse_state_noalloc", "sv_sample_cdf", "sv_program_create", "sv_program_run", "sv_program_stats", "sv_program_specialize", "sv_program_pass_params", "sv_program_arith_per_amplitude", "sv_pass_layout",
    "sv_program_destroy", "sv_inner_product", "sv_max_abs_diff", "sv_expectation_z",
    "sv_batch_create", "sv_batch_run", "sv_batch_specialize", "sv_batch_set_executor", "sv_batch_tfim_energy", "sv_batch_state", "sv_batch_stats", "sv_batch_pass_bytes", "sv_batch_arith",
    "sv_batch_destroy", "sv_adjoint_create", "sv_adjoint_update", "sv_adjoint_run", "sv_adjoint_specialize", "sv_adjoint_state",
    "sv_adjoint_destroy",
)


class EngineError(RuntimeError):
    """A CUDA-level failure reported by the engine."""


_lock = threading.Lock()
_lib = None

_vp = ctypes.c_void_p
_i32p = ctypes.POINTER(ctypes.c_int32)
_int = ctypes.c_int
_i64 = ctypes.c_int64

_SIGNATURES = {
    "sv_version": ([], _int),
    "sv_last_error": ([], ctypes.c_char_p),
    "sv_device_count": ([], _int),
    "sv_context_create": ([_int, ctypes.POINTER(_vp)], _int),
    "sv_context_destroy": ([_vp], _int),
    "sv_context_set_stream": ([_vp, _vp], _int),
    "sv_context_set_dense_mode": ([_vp, _int], _int),
    "sv_context_set_c128_arithmetic": ([_vp, _int], _int),
    "sv_sync": ([_vp], _int),
    "sv_zero_state": ([_vp, _vp, _int, _int], _int),
    "sv_apply_one_qubit": ([_vp, _vp, _int, _int, _int, _vp, _int, _vp, _int], _int),
    "sv_apply_two_qubit": ([_vp, _vp, _int, _int, _int, _vp, _int, _int, _vp, _int], _int),
    "sv_apply_multi_qubit": ([_vp, _vp, _int, _int, _vp, _vp, _int, _vp, _int], _int),
    "sv_collapse_state": ([_vp, _vp, _int, _int, _vp, _int, _i64, _int], _int),
    "sv_probabilities": ([_vp, _vp, _int, _int, _vp, _int, _vp, _int], _int),
    "sv_density_probabilities": ([_vp, _vp, _int, _int, _vp, _int, _vp, _int], _int),
    "sv_axpby": ([_vp, _int, ctypes.c_int64, _vp, ctypes.c_double, ctypes.c_double, _vp, ctypes.c_double,
                  ctypes.c_double], _int),
    "sv_measure_frequencies": ([_vp, _vp, _vp, _int, _int, _i64, ctypes.c_uint32, _int], _int),
    "sv_collapse_state_noalloc": ([_vp, _vp, _int, _int, _vp, _int, _i64, _int], _int),
    "sv_program_create": ([_vp, _int, _int, _vp, _int, _int, ctypes.POINTER(_vp)], _int),
    "sv_program_run": ([_vp, _vp, _vp], _int),
    "sv_program_stats": ([_vp] + [ctypes.POINTER(_int)] * 4, _int),
    "sv_program_specialize": ([_vp, _vp], _int),
    "sv_sample_cdf": ([_vp, _vp, _int, _int, _vp, ctypes.c_int64, _vp, _vp], _int),
    "sv_program_pass_params": ([_vp, _int, _vp, _vp], _int),
    "sv_program_arith_per_amplitude": ([_vp, _vp], _int),
    "sv_pass_layout": ([_int, _vp, _int], _int),
    "sv_program_destroy": ([_vp], _int),
    "sv_inner_product": ([_vp, _vp, _int, _vp, _int, _int, _vp], _int),
    "sv_max_abs_diff": ([_vp, _vp, _int, _vp, _int, _int, _vp], _int),
    "sv_expectation_z": ([_vp, _vp, _int, _int, _vp, _int, _vp], _int),
    "sv_batch_create": ([_vp, _int, _int, _vp, _vp, _vp, _int, ctypes.POINTER(_vp)], _int),
    "sv_batch_run": ([_vp, _vp], _int),
    "sv_batch_specialize": ([_vp, _vp], _int),
    "sv_batch_set_executor": ([_vp, _vp, _int], _int),
    "sv_batch_tfim_energy": ([_vp, _vp, ctypes.c_double, _vp], _int),
    "sv_batch_state": ([_vp, _int, ctypes.POINTER(_vp), ctypes.POINTER(_int)], _int),
    "sv_batch_stats": ([_vp, ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(ctypes.c_size_t)], _int),
    "sv_batch_pass_bytes": ([_vp, _vp], _int),
    "sv_batch_arith": ([_vp, _vp], _int),
    "sv_batch_destroy": ([_vp], _int),
    "sv_adjoint_create": ([_vp, _int, _int, _int, _vp, _int, _vp, _vp, _int, _vp, _int, _int, ctypes.POINTER(_vp)],
                          _int),
    "sv_adjoint_update": ([_vp, _vp, _vp, _int, _vp, _vp], _int),
    "sv_adjoint_run": ([_vp, _vp, ctypes.c_double, _vp, _vp], _int),
    "sv_adjoint_specialize": ([_vp, _vp], _int),
    "sv_adjoint_state": ([_vp, _int, ctypes.POINTER(_vp)], _int),
    "sv_adjoint_destroy": ([_vp], _int),
}


def load(path: str = LIB_PATH):
    """Loads (once) and returns the engine library; raises ImportError if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise ImportError(
                f"GB300 engine library not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (nvcc, sm_103a)")
        lib = ctypes.CDLL(path)
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def last_error() -> str:
    msg = load().sv_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str = "") -> None:
    if rc == SV_OK:
        return
    msg = last_error()
    text = f"{what}: {msg}" if what else msg
    if rc == SV_ERR_ARG:
        raise ValueError(text)
    if rc == SV_ERR_OOM:
        raise RuntimeError(f"State does not fit in device memory. {text}")
    if rc == SV_ERR_NO_DEVICE:
        raise ImportError(text)
    if rc == SV_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if rc == SV_ERR_TIMEOUT:
        raise TimeoutError(text)
    raise EngineError(text)


def int32_array(values):
    """A ctypes int32 array (host) for qubit lists, or None for an empty list."""
    values = [int(v) for v in values]
    if not values:
        return None, 0
    return (ctypes.c_int32 * len(values))(*values), len(values)


class Context:
    """Owns one ``sv_context`` (device, stream, scratch) for the lifetime of a backend."""

    def __init__(self, device: int = 0, stream: int = 0):
        lib = load()
        h = _vp()
        check(lib.sv_context_create(int(device), ctypes.byref(h)), "sv_context_create")
        self._h = h
        self.lib = lib
        self.device = device
        self.c128_arithmetic = "double-word"
        if stream:
            check(lib.sv_context_set_stream(h, _vp(stream)), "sv_context_set_stream")

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream: int) -> None:
        check(self.lib.sv_context_set_stream(self._h, _vp(stream)), "sv_context_set_stream")

    def sync(self) -> None:
        check(self.lib.sv_sync(self._h), "sv_sync")

    def set_c128_arithmetic(self, mode: str) -> None:
        """'double-word' (FP32 pipe, default) or 'fp64' for the complex128 kernels and passes."""
        codes = {"double-word": 0, "fp64": 1}
        if mode not in codes:
            raise ValueError(f"complex128 arithmetic must be one of {sorted(codes)}")
        check(self.lib.sv_context_set_c128_arithmetic(self._h, codes[mode]), "sv_context_set_c128_arithmetic")
        self.c128_arithmetic = mode

    def set_dense_mode(self, mode: str) -> None:
        """'auto' (tensor cores for complex64 gates with 4..6 targets), 'simt' or 'tensor'."""
        codes = {"auto": 0, "simt": 1, "tensor": 2}
        if mode not in codes:
            raise ValueError(f"dense mode must be one of {sorted(codes)}")
        check(self.lib.sv_context_set_dense_mode(self._h, codes[mode]), "sv_context_set_dense_mode")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.sv_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
