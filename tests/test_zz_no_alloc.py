"""b200_vec_dot_static, the dot product that allocates nothing, against b200_vec_dot.

For callers that cannot allocate device memory when they need a reduction; its partial sums live in a fixed array
inside the library.  Collected last (file name) so that a run stopping at the first failure has run everything else.
The comparison tolerance is 1e-12 relative: both accumulate in FP64, in different fixed orders.
"""
import ctypes

import pytest
import torch

from libceed_gb300 import _ffi, mesh

pytestmark = pytest.mark.gpu

F64, F32 = 0, 1


@pytest.fixture(scope="module")
def ctx():
    h = ctypes.c_void_p()
    _ffi.call("b200_ctx_create", 0, ctypes.byref(h))
    yield h
    _ffi.load().b200_ctx_destroy(h)


@pytest.mark.parametrize("prec,dtype", [(F64, torch.float64), (F32, torch.float32)])
@pytest.mark.parametrize("n", [1, 8191, 8192, 1000003])
def test_static_dot_matches_allocating_dot(ctx, prec, dtype, n):
    x = torch.tensor(mesh.uniform(11, n), device="cuda", dtype=dtype)
    y = torch.tensor(mesh.uniform(12, n), device="cuda", dtype=dtype)
    stream = torch.cuda.current_stream()
    _ffi.call("b200_ctx_set_stream", ctx, ctypes.c_void_p(stream.cuda_stream))
    ref = ctypes.c_double()
    _ffi.call("b200_vec_dot", ctx, prec, n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), ctypes.byref(ref))
    out = torch.full((2,), float("nan"), device="cuda", dtype=torch.float64)
    for k in range(2):  # two calls in a row share the static scratch
        _ffi.call("b200_vec_dot_static", prec, n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                  ctypes.c_void_p(out.data_ptr() + 8 * k), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    got = out.cpu().tolist()
    assert abs(got[0] - ref.value) <= 1e-12 * max(1.0, abs(ref.value))
    assert got[0] == got[1]  # fixed order: identical bits on repeat


def test_static_dot_empty_and_limit():
    stream = torch.cuda.current_stream()
    out = torch.full((1,), 5.0, device="cuda", dtype=torch.float64)
    _ffi.call("b200_vec_dot_static", F64, 0, None, None, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    assert out.item() == 0.0
    x = torch.zeros(4, device="cuda", dtype=torch.float64)
    # Beyond the static limit the call is refused before any kernel runs (so the short buffers are never read).
    with pytest.raises(_ffi.B200Error, match="static scratch limit"):
        _ffi.call("b200_vec_dot_static", F64, 134217728 + 1, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
