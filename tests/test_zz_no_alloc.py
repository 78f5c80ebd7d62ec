"""The collapse entry point that allocates nothing (``sv_collapse_state_noalloc``).

Some callers cannot call cudaMalloc: a host framework that owns all device memory
through its own pool allocator, or a latency-critical loop that cannot afford an
allocation or the device synchronisation of a later cudaFree.  For them the library
offers one collapse entry point whose reduction scratch is a fixed device array
inside the library.  This test calls it through the C ABI and checks it against the
regular, context-based ``sv_collapse_state`` on the same inputs, within the parity
tolerance the other GPU tests use, on two calls in a row (the second one runs on the
scratch the first one left behind).  The file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import PARITY_ATOL
from tests.dense import random_state

pytestmark = pytest.mark.gpu


def _collapse_both(lib, ctx, state_np, dtype, n, qubits, result, normalize):
    import torch

    from qibojit_gb300 import _lib

    tdt = {"complex128": torch.complex128, "complex64": torch.complex64, "float64": torch.float64,
           "float32": torch.float32}[dtype]
    code = _lib.DTYPE_CODES[dtype]
    a = torch.from_numpy(state_np).to("cuda", tdt)
    b = a.clone()
    q, nq = _lib.int32_array(qubits)
    _lib.check(lib.sv_collapse_state(ctx.handle, a.data_ptr(), code, n, q, nq, result, int(normalize)))
    _lib.check(lib.sv_collapse_state_noalloc(None, b.data_ptr(), code, n, q, nq, result, int(normalize)))
    torch.cuda.synchronize()
    return a.cpu().numpy(), b.cpu().numpy()


def test_noalloc_collapse_matches_context_collapse():
    from qibojit_gb300 import _lib

    lib = _lib.load()
    ctx = _lib.Context(0)
    calls = [("complex128", 20, [0, 1, 2, 3], 11, True), ("complex64", 18, [5, 2, 17], 3, True),
             ("complex128", 12, [7], 0, False), ("float64", 16, [3, 9], 2, True), ("float32", 15, [14], 1, True)]
    for dtype, n, qubits, result, normalize in calls:
        if dtype.startswith("float"):
            x = np.random.default_rng(100 + n).standard_normal(2**n)
            state = (x / np.linalg.norm(x)).astype(dtype)
        else:
            state = random_state(n, 100 + n, dtype)
        want, got = _collapse_both(lib, ctx, state, dtype, n, qubits, result, normalize)
        np.testing.assert_allclose(got, want, rtol=0, atol=PARITY_ATOL[dtype])
        if normalize:
            assert abs((np.abs(got.astype(np.complex128)) ** 2).sum() - 1) < PARITY_ATOL[dtype]
    ctx.close()


def test_noalloc_collapse_rejects_bad_arguments():
    from qibojit_gb300 import _lib

    lib = _lib.load()
    q, nq = _lib.int32_array([0, 0])
    rc = lib.sv_collapse_state_noalloc(None, ctypes.c_void_p(256), _lib.SV_C128, 4, q, nq, 0, 1)
    assert rc == _lib.SV_ERR_ARG
    q, nq = _lib.int32_array([1])
    rc = lib.sv_collapse_state_noalloc(None, ctypes.c_void_p(256), _lib.SV_C128, 4, q, nq, 2, 1)
    assert rc == _lib.SV_ERR_ARG
