"""ctypes view of the CPU oracle (oracle/ceed_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle restates libCEED's serial reference backend
(`/cpu/self/ref/serial`) for tensor-H1 hexahedral operator apply; the test suite,
the smoke check and the CPU-baseline leg of the benchmark use it as the checker.
The product package never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libceed_oracle.so")

GAUSS, GAUSS_LOBATTO = 0, 1
NOTRANSPOSE, TRANSPOSE = 0, 1
EVAL_NONE, EVAL_INTERP, EVAL_GRAD, EVAL_WEIGHT = 0, 1, 2, 16
QF_MASS, QF_POISSON, QF_VMASS, QF_VPOISSON, QF_POISSON_KAPPA = 0, 1, 2, 3, 4

_lib = None


def build():
    """Compile the oracle library (seconds); no reference sources needed."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(HERE, f) for f in ("ceed_oracle.c", "ceed_oracle_blocked.c", "ceed_oracle.h")]
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(f) for f in srcs):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_uniform.restype = ctypes.c_double
        _lib.orc_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _OrcOperator(ctypes.Structure):
    _fields_ = [
        ("qf", ctypes.c_int), ("P", ctypes.c_int), ("Q", ctypes.c_int), ("num_comp", ctypes.c_int),
        ("num_elem", ctypes.c_int64), ("comp_stride", ctypes.c_int64), ("l_size", ctypes.c_int64),
        ("offsets", ctypes.c_void_p), ("interp_1d", ctypes.c_void_p), ("grad_1d", ctypes.c_void_p),
        ("qdata", ctypes.c_void_p), ("kappa", ctypes.c_void_p),
    ]


def fill_uniform(seed, n, lo=-1.0, hi=1.0):
    x = np.empty(n, dtype=np.float64)
    lib().orc_fill_uniform(ctypes.c_uint64(seed), ctypes.c_int64(n), ctypes.c_double(lo), ctypes.c_double(hi), _p(x))
    return x


def lagrange_1d(P, Q, quad_mode=GAUSS):
    interp = np.zeros(Q * P)
    grad = np.zeros(Q * P)
    qref = np.zeros(Q)
    qw = np.zeros(Q)
    rc = lib().orc_h1_lagrange_1d(P, Q, quad_mode, _p(interp), _p(grad), _p(qref), _p(qw))
    assert rc == 0
    return interp.reshape(Q, P), grad.reshape(Q, P), qref, qw


def collocated_grad(P, Q, interp, grad):
    colo = np.zeros(Q * Q)
    interp = np.ascontiguousarray(interp, dtype=np.float64)
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    assert lib().orc_collocated_grad(P, Q, _p(interp), _p(grad), _p(colo)) == 0
    return colo.reshape(Q, Q)


def box_vertices(nx, ny, nz, noise, seed):
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    c = np.zeros(3 * nv)
    lib().orc_box_vertices(nx, ny, nz, ctypes.c_double(noise), ctypes.c_uint64(seed), _p(c))
    return c


def box_offsets(nx, ny, nz, P, ncomp_interlaced=1):
    off = np.zeros(nx * ny * nz * P ** 3, dtype=np.int32)
    lib().orc_box_offsets(nx, ny, nz, P, ncomp_interlaced, _p(off))
    return off


def rstr_gather(offsets, elem_size, num_comp, comp_stride, l_vec):
    ne = offsets.size // elem_size
    e = np.zeros(ne * num_comp * elem_size)
    lib().orc_rstr_gather(ctypes.c_int64(ne), elem_size, num_comp, ctypes.c_int64(comp_stride), _p(offsets), _p(l_vec), _p(e))
    return e


def rstr_scatter_add(offsets, elem_size, num_comp, comp_stride, e_vec, l_vec):
    ne = offsets.size // elem_size
    lib().orc_rstr_scatter_add(ctypes.c_int64(ne), elem_size, num_comp, ctypes.c_int64(comp_stride), _p(offsets), _p(e_vec), _p(l_vec))
    return l_vec


def basis_apply(dim, P, Q, num_comp, interp, grad, qweight, num_elem, t_mode, eval_mode, u):
    qc = dim if eval_mode == EVAL_GRAD else 1
    nn, nq = P ** dim, Q ** dim
    if eval_mode == EVAL_WEIGHT:
        n_out = nq
    elif t_mode == NOTRANSPOSE:
        n_out = nq * num_comp * qc
    else:
        n_out = nn * num_comp
    v = np.zeros(num_elem * n_out)
    interp = np.ascontiguousarray(interp, dtype=np.float64)
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    qweight = np.ascontiguousarray(qweight, dtype=np.float64)
    up = _p(u) if u is not None else None
    rc = lib().orc_basis_apply(dim, P, Q, num_comp, _p(interp), _p(grad), _p(qweight), ctypes.c_int64(num_elem), t_mode,
                               eval_mode, up, _p(v))
    assert rc == 0
    return v


def qdata_build(n, Q, poisson, coords, quad_mode=GAUSS):
    ne = n ** 3
    qd = np.zeros(ne * Q ** 3 * (6 if poisson else 1))
    assert lib().orc_qdata_build(n, n, n, Q, quad_mode, 1 if poisson else 0, _p(coords), _p(qd)) == 0
    return qd


def operator_apply(qf, P, Q, num_comp, offsets, comp_stride, l_size, interp, grad, qdata, u, kappa=None, v=None, add=False,
                   blocked=False):
    """v = A u (add: v += A u).  blocked: the /cpu/self/opt/blocked form (ceed_oracle_blocked.c), the CPU baseline."""
    interp = np.ascontiguousarray(interp, dtype=np.float64)
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    op = _OrcOperator(qf, P, Q, num_comp, offsets.size // P ** 3, comp_stride, l_size, _p(offsets), _p(interp), _p(grad),
                      _p(qdata), _p(kappa) if kappa is not None else None)
    if v is None:
        v = np.zeros(l_size)
    fn = lib().orc_operator_apply_blocked if blocked else lib().orc_operator_apply
    assert fn(ctypes.byref(op), _p(u), _p(v), 1 if add else 0) == 0
    return v


def kappa_grad(P, Q, offsets, l_size, interp, grad, qdata, u, w):
    interp = np.ascontiguousarray(interp, dtype=np.float64)
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    op = _OrcOperator(QF_POISSON_KAPPA, P, Q, 1, offsets.size // P ** 3, l_size, l_size, _p(offsets), _p(interp), _p(grad),
                      _p(qdata), None)
    g = np.zeros(offsets.size // P ** 3 * Q ** 3)
    assert lib().orc_kappa_grad(ctypes.byref(op), _p(u), _p(w), _p(g)) == 0
    return g


class BoxProblem:
    """Everything the oracle needs for one box-mesh operator: mesh, basis, offsets, qdata and a random input."""

    def __init__(self, n, degree, ncomp=1, poisson=True, noise=0.05, seed=1, kappa=False):
        self.n, self.P, self.Q, self.ncomp = n, degree + 1, degree + 2, ncomp
        self.poisson = poisson
        P, Q = self.P, self.Q
        self.num_elem = n ** 3
        nd = n * degree + 1
        self.num_nodes = nd ** 3
        self.l_size = self.num_nodes * ncomp
        self.comp_stride = self.num_nodes if ncomp == 1 else 1
        self.coords = box_vertices(n, n, n, noise, seed)
        self.offsets = box_offsets(n, n, n, P, ncomp)
        self.interp, self.grad, self.qref, self.qweight = lagrange_1d(P, Q)
        self.qdata = qdata_build(n, Q, poisson, self.coords)
        self.u = fill_uniform(seed + 1, self.l_size)
        self.kappa = None
        if kappa:
            self.kappa = np.exp(0.5 * fill_uniform(seed + 2, self.num_elem * Q ** 3))
        if kappa:
            self.qf = QF_POISSON_KAPPA
        elif poisson:
            self.qf = QF_POISSON if ncomp == 1 else QF_VPOISSON
        else:
            self.qf = QF_MASS if ncomp == 1 else QF_VMASS

    def apply(self, u=None, kappa=None, blocked=False):
        u = self.u if u is None else u
        kap = kappa if kappa is not None else self.kappa
        return operator_apply(self.qf, self.P, self.Q, self.ncomp, self.offsets, self.comp_stride, self.l_size, self.interp,
                              self.grad, self.qdata, np.ascontiguousarray(u), kappa=kap, blocked=blocked)
