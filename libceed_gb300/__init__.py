"""libceed_gb300: the GB300 (sm_103a) backend `/gpu/cuda/b200` for libCEED's operator-apply path.

`Ceed("/gpu/cuda/b200")` gives the libCEED-style Python API (ceed.py) over the C ABI of
libceed_b200.so (include/ceed-b200.h).  Build the library with `libceed_gb300.build.build()`.
"""
from . import mesh  # noqa: F401  (seeded boxes and values; libceed_gb300.mesh without a separate import)
from ._ffi import B200Error  # noqa: F401
from .ceed import (  # noqa: F401
    COPY_VALUES, EVAL_GRAD, EVAL_INTERP, EVAL_NONE, EVAL_WEIGHT, F32, F64, F64X, GAUSS, GAUSS_LOBATTO, MEM_DEVICE, MEM_HOST, NORM_1,
    NORM_2, NORM_MAX, NOTRANSPOSE, STRIDES_BACKEND, TRANSPOSE, USE_POINTER, Ceed,
)
