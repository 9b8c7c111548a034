"""The run-time QFunction compiler (NVRTC, sm_103a) builds the fused kernel template around user sources; no GPU is
needed to compile.  Errors come back with the compiler log."""
import ctypes
import os

import pytest

from libceed_gb300 import _ffi

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "qfunctions", "user-qfunctions.h")
INTERP, GRAD, NONE = 1, 2, 0


def _desc(path, name, sizes, active, ein, eout):
    j = _ffi.JitQFunction()
    j.source_path, j.name = path.encode(), name.encode()
    j.num_inputs = len(sizes)
    for i, s in enumerate(sizes):
        j.input_size[i] = s
    j.active_input, j.eval_in, j.eval_out = active, ein, eout
    return j


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_ffi.LIB_PATH):
        from libceed_gb300 import build

        build.build()
    return _ffi.load()


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("P", [2, 5, 9])
def test_user_qfunctions_compile(lib, prec, P):
    _ffi.call("b200_jit_compile_check", ctypes.byref(_desc(SRC, "DiffusionKappa", [3, 6, 1], 0, GRAD, GRAD)), prec, P)
    _ffi.call("b200_jit_compile_check", ctypes.byref(_desc(SRC, "ScaledMass", [1, 1], 1, INTERP, INTERP)), prec, P)


def test_compile_error_carries_the_log(lib, tmp_path):
    bad = tmp_path / "bad.h"
    bad.write_text("#include <ceed/types.h>\nCEED_QFUNCTION(Broken)(void *ctx, const CeedInt Q, const CeedScalar *const *in, "
                   "CeedScalar *const *out) { return undefined_symbol; }\n")
    with pytest.raises(_ffi.B200Error, match="undefined_symbol"):
        _ffi.call("b200_jit_compile_check", ctypes.byref(_desc(str(bad), "Broken", [1, 1], 0, INTERP, INTERP)), 0, 4)


def test_missing_source(lib):
    with pytest.raises(_ffi.B200Error, match="cannot read"):
        _ffi.call("b200_jit_compile_check", ctypes.byref(_desc("/nonexistent/q.h", "X", [1], 0, INTERP, INTERP)), 0, 4)
