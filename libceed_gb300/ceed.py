"""Python face of the `/gpu/cuda/b200` backend, mirroring libCEED's Python binding.

Names, arguments and behaviour follow python/ceed.py, ceed_vector.py, ceed_elemrestriction.py,
ceed_basis.py, ceed_qfunction.py and ceed_operator.py of the reference, so code written against
`libceed.Ceed("/gpu/cuda/...")` reads the same here.  Every compute call goes through the C ABI of
libceed_b200.so (include/ceed-b200.h); device memory and the stream come from PyTorch.  There is no
CPU fallback: a missing library or an unsupported configuration raises.

Layouts (published the way CeedElemRestrictionSetELayout does):
  E-vector [comp][elem][node], Q-vector [eval-dim][comp][elem][qpt], qdata [comp][elem][qpt].
"""
import contextlib
import ctypes
import re

import numpy as np
import torch

from . import basis1d
from ._ffi import B200Error, OpDesc, call, load

# Constants of include/ceed/ceed.h
MEM_HOST, MEM_DEVICE = 0, 1
COPY_VALUES, USE_POINTER, OWN_POINTER = 0, 1, 2
NOTRANSPOSE, TRANSPOSE = 0, 1
EVAL_NONE, EVAL_INTERP, EVAL_GRAD, EVAL_DIV, EVAL_CURL, EVAL_WEIGHT = 0, 1, 2, 4, 8, 16
NORM_1, NORM_2, NORM_MAX = 0, 1, 2
GAUSS, GAUSS_LOBATTO = basis1d.GAUSS, basis1d.GAUSS_LOBATTO
REQUEST_IMMEDIATE = None
STRIDES_BACKEND = "backend"
SCATTER_ATOMIC, SCATTER_DETERMINISTIC = 0, 1
F64, F32, F64X = 0, 1, 2  # F64X: float-float arithmetic on double vectors (fused operator only)

# Gallery QFunctions on the hot path (include/ceed/jit-source/gallery/*.h), plus the kappa-weighted diffusion
# this backend adds for the differentiable operator.  Fields: (name, size, eval mode).
QF_MASS, QF_POISSON, QF_VECMASS, QF_VECPOISSON, QF_POISSON_KAPPA = 0, 1, 2, 3, 4
GALLERY = {
    "MassApply": (QF_MASS, [("u", 1, EVAL_INTERP), ("qdata", 1, EVAL_NONE)], [("v", 1, EVAL_INTERP)]),
    "Poisson3DApply": (QF_POISSON, [("du", 3, EVAL_GRAD), ("qdata", 6, EVAL_NONE)], [("dv", 3, EVAL_GRAD)]),
    "Vector3MassApply": (QF_VECMASS, [("u", 3, EVAL_INTERP), ("qdata", 1, EVAL_NONE)], [("v", 3, EVAL_INTERP)]),
    "Vector3Poisson3DApply": (QF_VECPOISSON, [("du", 9, EVAL_GRAD), ("qdata", 6, EVAL_NONE)], [("dv", 9, EVAL_GRAD)]),
    "Poisson3DApplyKappa": (QF_POISSON_KAPPA, [("du", 3, EVAL_GRAD), ("qdata", 6, EVAL_NONE), ("kappa", 1, EVAL_NONE)],
                            [("dv", 3, EVAL_GRAD)]),
    "Mass3DBuild": ("build_mass", [("dx", 9, EVAL_GRAD), ("weights", 1, EVAL_WEIGHT)], [("qdata", 1, EVAL_NONE)]),
    "Poisson3DBuild": ("build_poisson", [("dx", 9, EVAL_GRAD), ("weights", 1, EVAL_WEIGHT)], [("qdata", 6, EVAL_NONE)]),
}


def _vp(x):
    return ctypes.c_void_p(x)


class Ceed:
    """A device context of the `/gpu/cuda/b200` backend (resource string `/gpu/cuda/b200[:device_id=N]`)."""

    def __init__(self, resource="/gpu/cuda/b200", on_error="store", deterministic=False):
        m = re.match(r"^/gpu/cuda/b200(?::device_id=(\d+))?$", resource)
        if not m:
            raise B200Error("CeedInit", 1, f"resource {resource!r} is not /gpu/cuda/b200[:device_id=N]")
        if not torch.cuda.is_available():
            raise B200Error("CeedInit", -1, "/gpu/cuda/b200 needs a CUDA device; none is visible")
        self.device_id = int(m.group(1) or 0)
        self.resource = resource
        self.device = torch.device("cuda", self.device_id)
        load()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            call("b200_ctx_create", self.device_id, ctypes.byref(h))
        self._ctx = h
        self.deterministic = deterministic
        self.set_stream(torch.cuda.current_stream(self.device))

    # ---- libCEED Ceed methods -------------------------------------------------------------------------------------
    def get_resource(self):
        return self.resource

    def get_preferred_memtype(self):
        return MEM_DEVICE

    def scalar_type(self):
        """numpy name of CeedScalar (python/ceed.py:107-113): double; FP32 vectors are a per-Vector choice here."""
        return "float64"

    def set_deterministic(self, flag=True):
        """CeedSetDeterministic: transposed restrictions and operators use the inverse-offset scatter."""
        self.deterministic = bool(flag)

    def is_deterministic(self):
        return self.deterministic

    def set_stream(self, stream):
        self.stream = stream
        call("b200_ctx_set_stream", self._ctx, _vp(stream.cuda_stream))

    def synchronize(self):
        call("b200_ctx_sync", self._ctx)

    def launch_count(self):
        n = ctypes.c_int64()
        call("b200_ctx_launch_count", self._ctx, ctypes.byref(n))
        return n.value

    def status(self):
        """Read and clear the device status word (B200_STATUS_* bits; 0 when every bounded wait completed)."""
        st = ctypes.c_int()
        call("b200_ctx_status", self._ctx, ctypes.byref(st))
        return st.value

    def fma_peak(self, prec=F64):
        """Measured fused multiply-add rate of the FP64 or FP32 pipe (TFLOP/s), the compute roofline's denominator."""
        t = ctypes.c_double()
        call("b200_fma_peak", self._ctx, prec, ctypes.byref(t))
        return t.value

    def fp64_tensor_peak(self):
        """(DMMA-only, DMMA+DFMA interleaved) FP64 TFLOP/s: whether the FP64 tensor path adds to the FP64 FMA pipe."""
        a, b = ctypes.c_double(), ctypes.c_double()
        call("b200_fp64_tensor_peak", self._ctx, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def gauss_quadrature(self, q):
        return basis1d.gauss_quadrature(q)

    def lobatto_quadrature(self, q):
        return basis1d.lobatto_quadrature(q)

    def Vector(self, size, dtype=torch.float64):
        return Vector(self, size, dtype)

    def ElemRestriction(self, nelem, elemsize, ncomp, compstride, lsize, offsets, memtype=MEM_HOST, cmode=COPY_VALUES):
        return ElemRestriction(self, nelem, elemsize, ncomp, compstride, lsize, offsets)

    def StridedElemRestriction(self, nelem, elemsize, ncomp, lsize, strides):
        return StridedElemRestriction(self, nelem, elemsize, ncomp, lsize, strides)

    def BasisTensorH1(self, dim, ncomp, P1d, Q1d, interp1d, grad1d, qref1d, qweight1d):
        return BasisTensorH1(self, dim, ncomp, P1d, Q1d, interp1d, grad1d, qref1d, qweight1d)

    def BasisTensorH1Lagrange(self, dim, ncomp, P, Q, qmode=GAUSS):
        interp, grad, qref, qw = basis1d.lagrange_1d(P, Q, qmode)
        return BasisTensorH1(self, dim, ncomp, P, Q, interp, grad, qref, qw)

    def QFunctionByName(self, name):
        return QFunctionByName(self, name)

    def QFunction(self, vlength, f, source):
        return QFunction(self, vlength, f, source)

    def QFunctionContext(self):
        return QFunctionContext(self)

    def Operator(self, qf, dqf=None, qdfT=None):
        return Operator(self, qf)

    def CompositeOperator(self):
        return CompositeOperator(self)

    def __del__(self):
        try:
            if getattr(self, "_ctx", None):
                load().b200_ctx_destroy(self._ctx)
                self._ctx = None
        except Exception:
            pass


def _prec(dtype):
    if dtype == torch.float64:
        return F64
    if dtype == torch.float32:
        return F32
    raise B200Error("Vector", 4, f"unsupported scalar type {dtype}")


class Vector:
    """CeedVector with its array in device memory (a torch tensor); host access copies."""

    def __init__(self, ceed, size, dtype=torch.float64):
        self.ceed = ceed
        self.size = int(size)
        self.dtype = dtype
        self.prec = _prec(dtype)
        self.data = torch.empty(self.size, dtype=dtype, device=ceed.device)
        self._host = None      # host array handed out by get_array / get_array_write, written back by restore_array
        self._borrowed = None  # the array given with USE_POINTER, returned by take_array

    def __repr__(self):
        return f"CeedVector length {self.size} ({self.dtype}) on {self.data.device}"

    def __str__(self):
        """Like CeedVectorView: the length, then one value per line."""
        vals = self.get_array_read()
        return "\n".join([f"CeedVector length {self.size}"] + [f"  {float(x):.14g}" for x in vals])

    def __len__(self):
        return self.size

    def get_length(self):
        return self.size

    def ptr(self):
        return _vp(self.data.data_ptr())

    @property
    def __cuda_array_interface__(self):
        """The device array, for CuPy, Numba and other consumers of the CUDA array interface (no copy)."""
        return self.data.__cuda_array_interface__

    def set_array(self, array, memtype=MEM_HOST, cmode=COPY_VALUES):
        """Copy (or, for a device array with USE_POINTER, borrow) the values.  A device array is a torch tensor or any
        object with __cuda_array_interface__ (CuPy, Numba), taken without a copy as python/ceed_vector.py:73-102 does."""
        given = array
        self._borrowed = given if cmode == USE_POINTER else None
        if not isinstance(array, torch.Tensor) and hasattr(array, "__cuda_array_interface__"):
            array = torch.as_tensor(array, device=self.ceed.device)  # a view of the same device memory
        if isinstance(array, torch.Tensor):
            if cmode == USE_POINTER and array.is_cuda and array.dtype == self.dtype and array.numel() == self.size and array.is_contiguous():
                self.data = array
                return
            self.data.copy_(array.reshape(-1).to(self.dtype))
        else:
            a = np.ascontiguousarray(np.asarray(array).reshape(-1))
            if a.size != self.size:
                raise B200Error("CeedVectorSetArray", 2, f"array of {a.size} entries for a vector of {self.size}")
            self.data.copy_(torch.from_numpy(a).to(self.dtype))

    def take_array(self, memtype=MEM_HOST):
        """CeedVectorTakeArray: return the array given with USE_POINTER and forget it (python/ceed_vector.py:105-125).
        A host array given with USE_POINTER was copied to the device, so the vector's current values are copied back
        into it first; a device array was used in place.  The vector holds no valid data afterwards."""
        given = self._borrowed
        if given is None:
            raise B200Error("CeedVectorTakeArray", 5, "no array was set with USE_POINTER")
        if isinstance(given, np.ndarray):
            given[...] = self.data.cpu().numpy().reshape(given.shape)
        else:
            view = given if isinstance(given, torch.Tensor) else torch.as_tensor(given, device=self.ceed.device)
            if view.data_ptr() != self.data.data_ptr():  # copied at set_array (another type or layout): copy back
                view.copy_(self.data.reshape(view.shape))
        self._borrowed = None
        self._host = None
        self.data = torch.empty(self.size, dtype=self.dtype, device=self.ceed.device)
        return given

    def sync_array(self, memtype=MEM_HOST):
        """CeedVectorSyncArray: the device array is always current and host arrays are made on request, so there is
        nothing to move; waits for the work queued on the device array."""
        if self.data.is_cuda:
            self.ceed.synchronize()

    def _host_copy(self):
        h = self.data.cpu().numpy()
        return h if self.data.is_cuda else h.copy()  # always an array of its own, as after a device-to-host copy

    def get_array_read(self, memtype=MEM_HOST):
        """CeedVectorGetArrayRead: the device tensor, or a host copy of it."""
        if memtype == MEM_DEVICE:
            return self.data
        return self._host_copy()

    def get_array(self, memtype=MEM_HOST):
        """CeedVectorGetArray: read/write access.  MEM_DEVICE gives the device tensor itself; MEM_HOST gives a host
        array that restore_array() copies back, so host writes reach the vector as with the reference's host view."""
        if memtype == MEM_DEVICE:
            return self.data
        self._host = self._host_copy()
        return self._host

    def get_array_write(self, memtype=MEM_HOST):
        """CeedVectorGetArrayWrite: write access; restore_array() publishes the values written."""
        return self.get_array(memtype)

    def restore_array(self):
        """CeedVectorRestoreArray: a host array from get_array / get_array_write goes back to the device."""
        if self._host is not None:
            self.data.copy_(torch.from_numpy(self._host).to(self.dtype))
            self._host = None

    def restore_array_read(self):
        """CeedVectorRestoreArrayRead: read access ends; nothing is written back."""

    @contextlib.contextmanager
    def array(self, memtype=MEM_HOST):
        """`with v.array() as a:` read/write access, restored at the end of the block."""
        a = self.get_array(memtype)
        try:
            yield a
        finally:
            self.restore_array()

    @contextlib.contextmanager
    def array_read(self, memtype=MEM_HOST):
        """`with v.array_read() as a:` read access."""
        try:
            yield self.get_array_read(memtype)
        finally:
            self.restore_array_read()

    @contextlib.contextmanager
    def array_write(self, memtype=MEM_HOST):
        """`with v.array_write() as a:` write access, published at the end of the block."""
        a = self.get_array_write(memtype)
        try:
            yield a
        finally:
            self.restore_array()

    def set_value(self, value):
        call("b200_vec_set_value", self.ceed._ctx, self.prec, self.size, self.ptr(), float(value))

    def set_value_strided(self, start, stop, step, value):
        """Entries start, start + step, ... below stop (-1: the length) set to value (CeedVectorSetValueStrided)."""
        call("b200_vec_set_value_strided", self.ceed._ctx, self.prec, self.size, int(start), int(stop), int(step), self.ptr(),
             float(value))

    def copy_strided(self, start, stop, step, vec_copy):
        """vec_copy[i] = self[i] for i = start, start + step, ... below stop (-1: the shorter length)
        (CeedVectorCopyStrided); both vectors hold the same scalar type."""
        if vec_copy.dtype != self.dtype:
            raise B200Error("CeedVectorCopyStrided", 4, f"copy from {self.dtype} into {vec_copy.dtype}")
        call("b200_vec_copy_strided", self.ceed._ctx, self.prec, min(self.size, vec_copy.size), int(start), int(stop), int(step),
             self.ptr(), vec_copy.ptr())

    def norm(self, normtype=NORM_2):
        out = ctypes.c_double()
        call("b200_vec_norm", self.ceed._ctx, self.prec, self.size, self.ptr(), normtype, ctypes.byref(out))
        return out.value

    def dot(self, other):
        out = ctypes.c_double()
        call("b200_vec_dot", self.ceed._ctx, self.prec, self.size, self.ptr(), other.ptr(), ctypes.byref(out))
        return out.value

    def scale(self, alpha):
        call("b200_vec_scale", self.ceed._ctx, self.prec, self.size, self.ptr(), float(alpha))

    def axpy(self, alpha, x):
        call("b200_vec_axpy", self.ceed._ctx, self.prec, self.size, float(alpha), x.ptr(), self.ptr())

    def axpby(self, alpha, beta, x):
        call("b200_vec_axpby", self.ceed._ctx, self.prec, self.size, float(alpha), float(beta), x.ptr(), self.ptr())

    def pointwise_mult(self, x, y):
        call("b200_vec_pointwise_mult", self.ceed._ctx, self.prec, self.size, self.ptr(), x.ptr(), y.ptr())

    def reciprocal(self):
        call("b200_vec_reciprocal", self.ceed._ctx, self.prec, self.size, self.ptr())

    def copy_from(self, other):
        self.data.copy_(other.data.to(self.dtype))


class TransposeElemRestriction:
    """The transpose of a restriction, from E-vectors to L-vectors (python/ceed_elemrestriction.py:459-495)."""

    def __init__(self, elemrestriction):
        self._elemrestriction = elemrestriction

    def __repr__(self):
        return f"<Transpose CeedElemRestriction instance at {hex(id(self))}>"

    def apply(self, u, v, request=REQUEST_IMMEDIATE):
        self._elemrestriction.apply(u, v, tmode=TRANSPOSE, request=request)


class TransposeBasis:
    """The transpose of a basis, from quadrature points to nodes (python/ceed_basis.py:424-460)."""

    def __init__(self, basis):
        self._basis = basis

    def __repr__(self):
        return f"<Transpose CeedBasis instance at {hex(id(self))}>"

    def apply(self, nelem, emode, u, v):
        self._basis.apply(nelem, emode, u, v, tmode=TRANSPOSE)


def _multiplicity(offsets, ncomp, compstride, lsize):
    """E^T (E 1) of an offset restriction (interface/ceed-elemrestriction.c:1722-1737): how many element nodes share
    each L-vector entry, counted on the host from the offsets."""
    off = np.asarray(offsets, dtype=np.int64).reshape(-1)
    mult = np.zeros(lsize)
    for c in range(ncomp):
        mult += np.bincount(off + c * compstride, minlength=lsize)[:lsize]
    return mult


class ElemRestriction:
    """Offset element restriction (CeedElemRestrictionCreate); E-vector layout [comp][elem][node]."""

    def __init__(self, ceed, nelem, elemsize, ncomp, compstride, lsize, offsets):
        self.ceed = ceed
        self.nelem, self.elemsize, self.ncomp, self.compstride, self.lsize = int(nelem), int(elemsize), int(ncomp), int(compstride), int(lsize)
        off = offsets if isinstance(offsets, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(offsets, dtype=np.int32)))
        if off.numel() != self.nelem * self.elemsize:
            raise B200Error("CeedElemRestrictionCreate", 2, f"{off.numel()} offsets for {self.nelem} elements of size {self.elemsize}")
        host = off.cpu().numpy()
        if host.size and (host.min() < 0 or int(host.max()) + (self.ncomp - 1) * self.compstride >= self.lsize):
            raise B200Error("CeedElemRestrictionCreate", 2, "offsets fall outside the L-vector")
        self.offsets_host = host
        self.offsets = off.to(device=ceed.device, dtype=torch.int32).contiguous()
        self._plan = None

    def get_e_layout(self):
        return (1, self.nelem * self.elemsize, self.elemsize)

    def get_l_layout(self):
        """Only strided restrictions have an L-vector layout (interface/ceed-elemrestriction.c:385-400)."""
        raise B200Error("CeedElemRestrictionGetLLayout", 1, "Only strided CeedElemRestriction have strided L-vector layout")

    @property
    def T(self):
        return TransposeElemRestriction(self)

    @property
    def transpose(self):
        return TransposeElemRestriction(self)

    def get_multiplicity(self):
        """L-vector of how many element nodes share each entry (CeedElemRestrictionGetMultiplicity)."""
        mult = Vector(self.ceed, self.lsize)
        mult.set_array(_multiplicity(self.offsets_host, self.ncomp, self.compstride, self.lsize))
        return mult

    def create_vector(self, dtype=torch.float64):
        return Vector(self.ceed, self.lsize, dtype), Vector(self.ceed, self.nelem * self.elemsize * self.ncomp, dtype)

    def plan(self):
        if self._plan is None:
            h = ctypes.c_void_p()
            call("b200_plan_create", self.ceed._ctx, self.nelem, self.elemsize, self.ncomp, self.compstride, self.lsize,
                 self.offsets_host.ctypes.data_as(ctypes.c_void_p), _vp(self.offsets.data_ptr()), ctypes.byref(h))
            self._plan = h
        return self._plan

    def apply(self, u, v, tmode=NOTRANSPOSE, request=REQUEST_IMMEDIATE):
        """NOTRANSPOSE: v = E u.  TRANSPOSE: v += E^T u (atomic, or the deterministic plan when the Ceed asks)."""
        ctx = self.ceed._ctx
        if tmode == NOTRANSPOSE:
            call("b200_rstr_gather", ctx, u.prec, self.nelem, self.elemsize, self.ncomp, self.compstride, self.lsize,
                 _vp(self.offsets.data_ptr()), u.ptr(), v.ptr())
        elif self.ceed.deterministic:
            call("b200_rstr_scatter_det", ctx, self.plan(), u.prec, u.ptr(), v.ptr(), 1)
        else:
            call("b200_rstr_scatter_atomic", ctx, u.prec, self.nelem, self.elemsize, self.ncomp, self.compstride, self.lsize,
                 _vp(self.offsets.data_ptr()), u.ptr(), v.ptr())

    def __del__(self):
        try:
            if self._plan is not None:
                load().b200_plan_destroy(self._plan)
        except Exception:
            pass


class StridedElemRestriction:
    """Strided restriction (CeedElemRestrictionCreateStrided).  STRIDES_BACKEND is the identity on the backend
    layout [comp][elem][node]."""

    def __init__(self, ceed, nelem, elemsize, ncomp, lsize, strides):
        self.ceed = ceed
        self.nelem, self.elemsize, self.ncomp, self.lsize = int(nelem), int(elemsize), int(ncomp), int(lsize)
        self.backend_strides = isinstance(strides, str) and strides == STRIDES_BACKEND
        self.strides = (1, self.nelem * self.elemsize, self.elemsize) if self.backend_strides else tuple(int(s) for s in strides)
        self.offsets = None

    def get_e_layout(self):
        return (1, self.nelem * self.elemsize, self.elemsize)

    def get_l_layout(self):
        """[node, component, element] strides of the L-vector (CeedElemRestrictionGetLLayout); the backend strides
        are this backend's E-layout."""
        return np.array(self.strides, dtype=np.int32)

    @property
    def T(self):
        return TransposeElemRestriction(self)

    @property
    def transpose(self):
        return TransposeElemRestriction(self)

    def get_multiplicity(self):
        """Every L-vector entry of a strided restriction belongs to one element node: all ones."""
        mult = Vector(self.ceed, self.lsize)
        mult.set_array(np.ones(self.lsize))
        return mult

    def create_vector(self, dtype=torch.float64):
        return Vector(self.ceed, self.lsize, dtype), Vector(self.ceed, self.nelem * self.elemsize * self.ncomp, dtype)

    def apply(self, u, v, tmode=NOTRANSPOSE, request=REQUEST_IMMEDIATE):
        s = (ctypes.c_int64 * 3)(*self.strides)
        # (node, comp, elem) strides as the reference: index = node*s0 + comp*s1 + elem*s2
        node_s, comp_s, elem_s = self.strides
        arr = (ctypes.c_int64 * 3)(node_s, comp_s, elem_s)
        name = "b200_rstr_strided_gather" if tmode == NOTRANSPOSE else "b200_rstr_strided_scatter"
        call(name, self.ceed._ctx, u.prec, self.nelem, self.elemsize, self.ncomp, arr, u.ptr(), v.ptr())
        del s


class BasisTensorH1:
    """Tensor-product H1 basis (CeedBasisCreateTensorH1); tables are row-major Q x P."""

    def __init__(self, ceed, dim, ncomp, P1d, Q1d, interp1d, grad1d, qref1d, qweight1d):
        self.ceed = ceed
        self.dim, self.ncomp, self.P1d, self.Q1d = int(dim), int(ncomp), int(P1d), int(Q1d)
        self.interp1d = np.ascontiguousarray(np.asarray(interp1d, dtype=np.float64).reshape(Q1d, P1d))
        self.grad1d = np.ascontiguousarray(np.asarray(grad1d, dtype=np.float64).reshape(Q1d, P1d))
        self.qref1d = np.ascontiguousarray(np.asarray(qref1d, dtype=np.float64))
        self.qweight1d = np.ascontiguousarray(np.asarray(qweight1d, dtype=np.float64))
        h = ctypes.c_void_p()
        call("b200_basis_create", ceed._ctx, self.dim, self.P1d, self.Q1d, self.ncomp, self.interp1d.ctypes.data_as(ctypes.c_void_p),
             self.grad1d.ctypes.data_as(ctypes.c_void_p), self.qweight1d.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
        self._h = h

    @property
    def T(self):
        return TransposeBasis(self)

    @property
    def transpose(self):
        return TransposeBasis(self)

    def get_num_nodes(self):
        return self.P1d ** self.dim

    def get_num_quadrature_points(self):
        return self.Q1d ** self.dim

    def get_interp_1d(self):
        return self.interp1d

    def get_grad_1d(self):
        return self.grad1d

    def get_q_ref_1d(self):
        return self.qref1d

    def get_q_weight_1d(self):
        return self.qweight1d

    def apply(self, nelem, emode, u, v, tmode=NOTRANSPOSE):
        up = u.ptr() if u is not None else _vp(0)
        prec = v.prec
        call("b200_basis_apply", self._h, prec, int(nelem), tmode, emode, 0, up, v.ptr())

    def apply_add(self, nelem, emode, u, v, tmode=TRANSPOSE):
        call("b200_basis_apply", self._h, v.prec, int(nelem), tmode, emode, 1, u.ptr(), v.ptr())

    def __del__(self):
        try:
            load().b200_basis_destroy(self._h)
        except Exception:
            pass


class QFunction:
    """A QFunction given by source (CeedQFunctionCreateInterior): `source` is "path/file.h:Name".  On this backend the
    source is compiled at run time (NVRTC, sm_103a) into the fused operator kernel; `f` (the host function pointer
    other backends call) is not used."""

    def __init__(self, ceed, vlength, f, source):
        if ":" not in source:
            raise B200Error("CeedQFunctionCreateInterior", 3, f"source {source!r} is not \"path/file.h:Name\"")
        self.ceed = ceed
        self.source_path, self.name = source.rsplit(":", 1)
        self.kind = "jit"
        self.inputs, self.outputs = [], []
        self.context = None

    def add_input(self, name, size, emode):
        self.inputs.append((name, size, emode))

    def add_output(self, name, size, emode):
        self.outputs.append((name, size, emode))

    def set_context(self, ctx):
        self.context = ctx


class QFunctionContext:
    """CeedQFunctionContext: bytes copied to device memory for the compiled QFunction."""

    def __init__(self, ceed):
        self.ceed = ceed
        self._bytes = None  # device copy of the context (uint8)
        self._host = None   # host array handed out by get_data, written back by restore_data

    def set_data(self, data, memtype=MEM_HOST, cmode=COPY_VALUES):
        raw = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        self._bytes = torch.from_numpy(raw.copy()).to(self.ceed.device)
        self._host = None

    def get_context_size(self):
        return 0 if self._bytes is None else int(self._bytes.numel())

    def get_data(self, memtype=MEM_HOST):
        """Read/write access to the context as CeedScalar (float64) values (python/ceed_qfunctioncontext.py:99-146):
        the device bytes viewed as doubles, or a host copy that restore_data() writes back."""
        if self._bytes is None:
            raise B200Error("CeedQFunctionContextGetData", 5, "the context holds no data")
        if memtype == MEM_DEVICE:
            return self._bytes.view(torch.float64)
        self._host = self._bytes.cpu().numpy().copy().view(np.float64)
        return self._host

    def restore_data(self):
        """Publish the host array of get_data() (CeedQFunctionContextRestoreData)."""
        if self._host is not None:
            self._bytes.copy_(torch.from_numpy(self._host.view(np.uint8)))
            self._host = None

    @contextlib.contextmanager
    def data(self, *shape, memtype=MEM_HOST):
        """`with ctx.data() as x:` a writable float64 view, optionally reshaped, published at the end of the block
        (python/ceed_qfunctioncontext.py:159-176)."""
        x = self.get_data(memtype=memtype)
        try:
            yield x.reshape(shape) if shape else x
        finally:
            self.restore_data()

    def ptr(self):
        return _vp(self._bytes.data_ptr()) if self._bytes is not None else None


class QFunctionByName:
    """A gallery QFunction (CeedQFunctionCreateInteriorByName)."""

    def __init__(self, ceed, name):
        if name not in GALLERY:
            raise B200Error("CeedQFunctionCreateInteriorByName", -2, f"no gallery QFunction named {name!r} on /gpu/cuda/b200")
        self.ceed, self.name = ceed, name
        self.kind, self.inputs, self.outputs = GALLERY[name]

    def apply(self, q, inputs, outputs):
        """CeedQFunctionApply on Q-vectors (field component k of point i at k*q + i)."""
        if isinstance(self.kind, str):
            raise B200Error("CeedQFunctionApply", -2, f"{self.name} is applied through its setup operator on this backend")
        ins = (ctypes.c_void_p * 3)(*([x.data.data_ptr() for x in inputs] + [0] * (3 - len(inputs))))
        outs = (ctypes.c_void_p * 1)(outputs[0].data.data_ptr())
        call("b200_qf_apply", self.ceed._ctx, outputs[0].prec, self.kind, int(q), ins, outs)


ACTIVE = "active"
NONE = None


class _Field:
    def __init__(self, name, rstr, basis, vec):
        self.name, self.rstr, self.basis, self.vec = name, rstr, basis, vec


class Operator:
    """CeedOperator on tensor-H1 hexahedra.  Apply-type gallery QFunctions run in one fused kernel per apply;
    the gallery build QFunctions run the geometric-factor kernel.  Anything else raises (no CPU fallback)."""

    def __init__(self, ceed, qf):
        self.ceed, self.qf = ceed, qf
        self.fields = {}
        self._fused = {}
        self.elems_per_block = 0
        self.staging = 0
        # "native": the vectors' precision; "float-float": double vectors, FP32-pipe float-float arithmetic (F64X).
        self.arithmetic = "native"

    def set_field(self, name, rstr, basis, vec):
        names = [f[0] for f in list(self.qf.inputs) + list(self.qf.outputs)]
        if name not in names:
            raise B200Error("CeedOperatorSetField", 2, f"QFunction {self.qf.name} has no field {name!r}")
        self.fields[name] = _Field(name, rstr, basis, vec)

    def name(self, name):
        """CeedOperatorSetName (python/ceed_operator.py:112-120)."""
        self._name = str(name)

    def check(self):
        """CeedOperatorCheckReady (interface/ceed-operator.c:1450): every field of the QFunction has been set."""
        missing = [f[0] for f in list(self.qf.inputs) + list(self.qf.outputs) if f[0] not in self.fields]
        if missing:
            raise B200Error("CeedOperatorCheckReady", 3, f"fields not set: {', '.join(missing)}")

    def linear_assemble_diagonal(self, d, request=REQUEST_IMMEDIATE):
        """CeedOperatorLinearAssembleDiagonal: d (an FP64 L-vector) = diag(A), by the diagonal-assembly kernel."""
        from .solver import assemble_diagonal

        if d.dtype != torch.float64:
            raise B200Error("CeedOperatorLinearAssembleDiagonal", 4, "the diagonal is assembled into an FP64 vector")
        assemble_diagonal(self.ceed, self, d)

    def linear_assemble_add_diagonal(self, d, request=REQUEST_IMMEDIATE):
        """CeedOperatorLinearAssembleAddDiagonal: d += diag(A)."""
        tmp = Vector(self.ceed, d.size)
        self.linear_assemble_diagonal(tmp)
        d.axpy(1.0, tmp)

    # ---- the fused path ---------------------------------------------------------------------------------------------
    def _active_input(self):
        return self.fields[self.qf.inputs[0][0]]

    def _fused_op(self, prec):
        key = (prec, self.ceed.deterministic, self.elems_per_block, self.staging)
        if key in self._fused:
            return self._fused[key]
        f = self._active_input()
        rstr, basis = f.rstr, f.basis
        if not isinstance(rstr, ElemRestriction) or not isinstance(basis, BasisTensorH1) or basis.dim != 3:
            raise B200Error("CeedOperatorApply", -2, "fused apply needs an offset restriction and a 3D tensor H1 basis")
        d = OpDesc()
        d.qf, d.prec, d.P_1d, d.Q_1d, d.num_comp = self.qf.kind, prec, basis.P1d, basis.Q1d, rstr.ncomp
        d.scatter = SCATTER_DETERMINISTIC if self.ceed.deterministic else SCATTER_ATOMIC
        d.num_elem, d.l_size, d.comp_stride = rstr.nelem, rstr.lsize, rstr.compstride
        d.offsets = rstr.offsets.data_ptr()
        d.interp_1d = basis.interp1d.ctypes.data
        d.grad_1d = basis.grad1d.ctypes.data
        d.elems_per_block, d.staging = self.elems_per_block, self.staging
        h = ctypes.c_void_p()
        call("b200_op_create", self.ceed._ctx, ctypes.byref(d), ctypes.byref(h))
        op = _FusedOp(self.ceed, h, (basis.interp1d, basis.grad1d))
        self._fused[key] = op
        return op

    def fused(self, prec=F64):
        """The fused kernel object behind this operator (tile control, cost model)."""
        return self._fused_op(prec)

    def _kernel_prec(self, prec):
        if self.arithmetic == "native":
            return prec
        if self.arithmetic == "float-float" and prec == F64:
            return F64X
        raise B200Error("CeedOperatorApply", -2, f"arithmetic {self.arithmetic!r} needs double vectors")

    def _passive(self, name, prec):
        v = self.fields[name].vec
        if v is None or isinstance(v, str):
            raise B200Error("CeedOperatorApply", 3, f"passive field {name!r} needs a vector")
        if v.prec != prec:
            raise B200Error("CeedOperatorApply", 4, f"field {name!r} precision differs from the active vectors")
        return v

    def _jit_op(self, prec):
        key = ("jit", prec, self.ceed.deterministic)
        if key in self._fused:
            return self._fused[key]
        from ._ffi import JitQFunction

        qf = self.qf
        (out_name, out_size, out_mode), = qf.outputs
        act = [i for i, (n, sz, m) in enumerate(qf.inputs) if isinstance(self.fields[n].vec, str)]
        if len(act) != 1 or not isinstance(self.fields[out_name].vec, str):
            raise B200Error("CeedOperatorApply", -2, "compiled QFunctions need exactly one active input and one active output")
        ai = act[0]
        f = self.fields[qf.inputs[ai][0]]
        rstr, basis = f.rstr, f.basis
        if not isinstance(rstr, ElemRestriction) or not isinstance(basis, BasisTensorH1) or basis.dim != 3 or rstr.ncomp != 1:
            raise B200Error("CeedOperatorApply", -2, "compiled QFunctions: one-component field on a 3D tensor H1 basis")
        for i, (n, sz, m) in enumerate(qf.inputs):
            if i != ai and m != EVAL_NONE:
                raise B200Error("CeedOperatorApply", -2, f"passive input {n!r} must use CEED_EVAL_NONE")
        d = OpDesc()
        d.qf, d.prec, d.P_1d, d.Q_1d, d.num_comp = -1, prec, basis.P1d, basis.Q1d, 1
        d.scatter = SCATTER_DETERMINISTIC if self.ceed.deterministic else SCATTER_ATOMIC
        d.num_elem, d.l_size, d.comp_stride = rstr.nelem, rstr.lsize, rstr.compstride
        d.offsets = rstr.offsets.data_ptr()
        d.interp_1d = basis.interp1d.ctypes.data
        d.grad_1d = basis.grad1d.ctypes.data
        j = JitQFunction()
        j.source_path, j.name = qf.source_path.encode(), qf.name.encode()
        j.num_inputs = len(qf.inputs)
        for i, (n, sz, m) in enumerate(qf.inputs):
            j.input_size[i] = sz
        j.active_input = ai
        j.eval_in, j.eval_out = qf.inputs[ai][2], out_mode
        j.include_dirs = None
        h = ctypes.c_void_p()
        call("b200_op_create_jit", self.ceed._ctx, ctypes.byref(d), ctypes.byref(j), ctypes.byref(h))
        op = _FusedOp(self.ceed, h, (basis.interp1d, basis.grad1d))
        op.passive_names = [n for i, (n, sz, m) in enumerate(qf.inputs) if i != ai]
        self._fused[key] = op
        return op

    def _apply(self, u, v, add):
        kind = self.qf.kind
        if kind == "jit":
            op = self._jit_op(u.prec)
            ptrs = [self._passive(n, u.prec).data.data_ptr() for n in op.passive_names]
            arr = (ctypes.c_void_p * max(1, len(ptrs)))(*ptrs)
            ctx = self.qf.context.ptr() if self.qf.context is not None else None
            call("b200_op_apply_jit", op.h, u.ptr(), v.ptr(), arr, ctx, 1 if add else 0)
            return
        if isinstance(kind, str):
            return self._build(u, v, add)
        op = self._fused_op(self._kernel_prec(u.prec))
        qd = self._passive("qdata", u.prec)
        kap = self._passive("kappa", u.prec) if kind == QF_POISSON_KAPPA else None
        call("b200_op_apply", op.h, u.ptr(), v.ptr(), qd.ptr(), kap.ptr() if kap else _vp(0), 1 if add else 0)

    def _build(self, u, v, add):
        dx = self.fields["dx"]
        if add:
            raise B200Error("CeedOperatorApplyAdd", -2, "the geometric-factor setup is applied with CeedOperatorApply")
        rx, bx = dx.rstr, dx.basis
        if not isinstance(rx, ElemRestriction) or rx.elemsize != 8 or rx.ncomp != 3 or bx.P1d != 2 or bx.dim != 3:
            raise B200Error("CeedOperatorApply", -2, "geometric factors need a trilinear coordinate field (P=2, 3 components)")
        out = self.fields["qdata"].rstr
        if not (isinstance(out, StridedElemRestriction) and out.backend_strides):
            raise B200Error("CeedOperatorApply", -2, "qdata must use CEED_STRIDES_BACKEND on this backend")
        if u.prec != F64 or v.prec != F64:
            raise B200Error("CeedOperatorApply", -2, "geometric factors are computed in FP64")
        call("b200_qdata_build", self.ceed._ctx, 1 if self.qf.kind == "build_poisson" else 0, rx.nelem, bx.Q1d,
             bx.interp1d.ctypes.data_as(ctypes.c_void_p), bx.grad1d.ctypes.data_as(ctypes.c_void_p),
             bx.qweight1d.ctypes.data_as(ctypes.c_void_p), _vp(rx.offsets.data_ptr()), rx.compstride, u.ptr(), v.ptr())

    def apply(self, u, v, request=REQUEST_IMMEDIATE):
        """CeedOperatorApply: v = A u."""
        self._apply(u, v, False)

    def apply_add(self, u, v, request=REQUEST_IMMEDIATE):
        """CeedOperatorApplyAdd: v += A u."""
        self._apply(u, v, True)

    def apply_dot(self, u, v):
        """v = A u, returning u . (A u) as the persistent FP32 kernel (staging 7, atomic scatter) sums it during the
        apply (b200_op_apply_dot); raises B200Error for operators whose kernel has no such form."""
        op = self._fused_op(self._kernel_prec(u.prec))
        qd = self._passive("qdata", u.prec)
        nb, n = ctypes.c_int(), ctypes.c_int64()
        call("b200_op_dot_len", op.h, ctypes.byref(nb), ctypes.byref(n))
        if nb.value == 0:
            raise B200Error("b200_op_apply_dot", -2, "u . (A u) during the apply needs the persistent FP32 kernel (staging 7)")
        part = torch.empty(n.value, dtype=torch.float64, device=self.ceed.device)
        call("b200_op_apply_dot", op.h, u.ptr(), v.ptr(), qd.ptr(), _vp(part.data_ptr()))
        total = 0.0
        for x in part[: nb.value].cpu().tolist():  # in block order, as the CG's final pass adds them
            total += x
        return total

    def get_flops_estimate(self):
        """CeedOperatorGetFlopsEstimate: the reference's FLOP model of one apply (b200_flops_estimate)."""
        f = self._active_input()
        kind = self.qf.kind
        if not isinstance(kind, int):
            raise B200Error("CeedOperatorGetFlopsEstimate", -2, "FLOP model available for the gallery apply QFunctions")
        out = ctypes.c_int64()
        call("b200_flops_estimate", kind, f.basis.P1d, f.basis.Q1d, f.rstr.ncomp, f.rstr.nelem, ctypes.byref(out))
        return out.value

    def kappa_grad(self, u, w, g):
        """g[elem][qpt] = grad(w) . D grad(u): the kappa-adjoint of the kappa-weighted diffusion."""
        op = self._fused_op(u.prec)
        qd = self._passive("qdata", u.prec)
        call("b200_op_kappa_grad", op.h, u.ptr(), w.ptr(), qd.ptr(), g.ptr())


class CompositeOperator:
    """CeedCompositeOperator (interface/ceed-operator.c:1297-1450): the sum of sub-operators on the same vectors.
    apply zeroes the output once and adds every sub-operator's fused apply."""

    def __init__(self, ceed):
        self.ceed = ceed
        self.subs = []

    def add_sub(self, op):
        self.subs.append(op)

    def apply(self, u, v, request=REQUEST_IMMEDIATE):
        if not self.subs:
            v.set_value(0.0)
            return
        self.subs[0].apply(u, v)
        for op in self.subs[1:]:
            op.apply_add(u, v)

    def apply_add(self, u, v, request=REQUEST_IMMEDIATE):
        for op in self.subs:
            op.apply_add(u, v)

    def name(self, name):
        self._name = str(name)

    def check(self):
        for op in self.subs:
            op.check()

    def linear_assemble_diagonal(self, d, request=REQUEST_IMMEDIATE):
        """Sum of the sub-operators' diagonals (the interface assembles composites sub-operator by sub-operator)."""
        d.set_value(0.0)
        self.linear_assemble_add_diagonal(d)

    def linear_assemble_add_diagonal(self, d, request=REQUEST_IMMEDIATE):
        for op in self.subs:
            op.linear_assemble_add_diagonal(d)


class _FusedOp:
    def __init__(self, ceed, h, keep):
        self.ceed, self.h, self._keep = ceed, h, keep

    def cost(self):
        b, f = ctypes.c_double(), ctypes.c_double()
        call("b200_op_cost", self.h, ctypes.byref(b), ctypes.byref(f))
        return b.value, f.value

    def tile(self):
        e, t, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("b200_op_get_tile", self.h, ctypes.byref(e), ctypes.byref(t), ctypes.byref(s))
        return e.value, t.value, s.value

    def set_tile(self, elems_per_block, staging=0):
        call("b200_op_set_tile", self.h, int(elems_per_block), int(staging))

    def __del__(self):
        try:
            load().b200_op_destroy(self.h)
        except Exception:
            pass
