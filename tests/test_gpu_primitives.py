"""Vector BLAS-1, reductions, standalone basis and gallery QFunctions on the GPU."""
import os

import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from oracle import oracle as orc
from tests.conftest import GOLDEN, relinf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ceed():
    return lc.Ceed("/gpu/cuda/b200")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_vector_ops(ceed, dtype):
    n = 100003
    x0, y0 = lc.mesh.uniform(1, n), lc.mesh.uniform(2, n)
    tol = 1e-14 if dtype == torch.float64 else 1e-6
    x, y = ceed.Vector(n, dtype), ceed.Vector(n, dtype)
    x.set_array(x0)
    y.set_array(y0)
    xs, ys = x.get_array_read().astype(np.float64), y.get_array_read().astype(np.float64)
    assert abs(x.norm(lc.NORM_2) - np.linalg.norm(xs)) < tol * np.linalg.norm(xs)
    assert abs(x.norm(lc.NORM_1) - np.sum(np.abs(xs))) < tol * np.sum(np.abs(xs))
    assert x.norm(lc.NORM_MAX) == np.max(np.abs(xs))
    assert abs(x.dot(y) - xs @ ys) < 1e-12 * n
    y.axpy(0.5, x)
    assert relinf(y.get_array_read(), ys + 0.5 * xs) < tol
    y.axpby(2.0, -1.0, x)
    assert relinf(y.get_array_read(), 2.0 * xs - (ys + 0.5 * xs)) < 10 * tol
    w = ceed.Vector(n, dtype)
    w.pointwise_mult(x, x)
    assert relinf(w.get_array_read(), xs * xs) < tol
    w.scale(-3.0)
    assert relinf(w.get_array_read(), -3.0 * xs * xs) < tol
    w.set_value(4.0)
    w.reciprocal()
    assert np.all(w.get_array_read() == 0.25)
    # Reductions are bit-reproducible run to run.
    assert len({x.norm() for _ in range(5)}) == 1


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("start,stop,step", [(0, -1, 1), (3, -1, 7), (5, 1000, 3), (17, 17, 2), (0, 4099, 4099), (4098, -1, 1),
                                             (2, -1, 10**12)])
def test_vector_strided(ceed, dtype, start, stop, step):
    """CeedVectorSetValueStrided / CopyStrided (interface/ceed-vector.c:300, :412): exactly the entries
    start, start + step, ... below stop change; stop = -1 means the length (the shorter one for the copy)."""
    n = 4099
    x0, y0 = lc.mesh.uniform(3, n), lc.mesh.uniform(4, n + 5)
    x, y = ceed.Vector(n, dtype), ceed.Vector(n + 5, dtype)
    x.set_array(x0)
    y.set_array(y0)
    xs, ys = x.get_array_read().copy(), y.get_array_read().copy()
    end = n if stop == -1 else stop
    want = xs.copy()
    want[start:end:step] = -2.5
    x.set_value_strided(start, stop, step, -2.5)
    assert np.array_equal(x.get_array_read(), want)
    want_y = ys.copy()
    want_y[start:end:step] = want[start:end:step]
    x.copy_strided(start, stop, step, y)
    assert np.array_equal(y.get_array_read(), want_y)


def test_vector_strided_rejects_bad_ranges(ceed):
    """Out-of-range stop or start and a non-positive step are refused before any kernel runs, vector unchanged."""
    n = 64
    x = ceed.Vector(n)
    x.set_value(1.0)
    for start, stop, step in [(0, n + 1, 1), (0, -2, 1), (-1, -1, 1), (10, 5, 1), (0, -1, 0), (0, -1, -3)]:
        with pytest.raises(lc.B200Error):
            x.set_value_strided(start, stop, step, 7.0)
        with pytest.raises(lc.B200Error):
            x.copy_strided(start, stop, step, ceed.Vector(n))
    assert np.all(x.get_array_read() == 1.0)


class _ForeignDeviceArray:
    """A device array known only through __cuda_array_interface__, as CuPy and Numba arrays present themselves."""

    def __init__(self, t):
        self._owner = t
        self.__cuda_array_interface__ = t.__cuda_array_interface__


def test_vector_cuda_array_interface(ceed):
    """Zero-copy device arrays both ways (python/ceed_vector.py:73-102, :159-170): USE_POINTER borrows a foreign
    array, COPY_VALUES copies it, and the vector exports its own array."""
    t = torch.arange(10, dtype=torch.float64, device="cuda")
    v = ceed.Vector(10)
    v.set_array(_ForeignDeviceArray(t), lc.MEM_DEVICE, lc.USE_POINTER)
    v.scale(2.0)
    torch.cuda.synchronize()
    assert t.cpu().tolist() == [2.0 * i for i in range(10)]
    assert v.__cuda_array_interface__["data"][0] == t.data_ptr()
    w = ceed.Vector(10)
    w.set_array(_ForeignDeviceArray(t), lc.MEM_DEVICE, lc.COPY_VALUES)
    w.set_value(0.0)
    torch.cuda.synchronize()
    assert t.cpu().tolist() == [2.0 * i for i in range(10)]
    assert np.all(w.get_array_read() == 0.0)


def test_empty_vectors(ceed):
    v = ceed.Vector(0)
    v.set_value(1.0)
    assert v.norm() == 0.0


@pytest.mark.parametrize("mode", ["interp", "grad"])
def test_basis_apply_matches_reference(ceed, mode):
    g = np.load(os.path.join(GOLDEN, "basis.npz"))
    P, Q, nc = 4, 5, 2
    em = lc.EVAL_INTERP if mode == "interp" else lc.EVAL_GRAD
    qc = 3 if mode == "grad" else 1
    b = ceed.BasisTensorH1Lagrange(3, nc, P, Q, lc.GAUSS)
    u = ceed.Vector(P ** 3 * nc)
    u.set_array(g[f"bapply_{mode}_u"])
    v = ceed.Vector(Q ** 3 * nc * qc)
    b.apply(1, em, u, v, lc.NOTRANSPOSE)
    assert relinf(v.get_array_read(), g[f"bapply_{mode}_v"]) < 1e-13
    ut = ceed.Vector(Q ** 3 * nc * qc)
    ut.set_array(g[f"bapply_{mode}_ut"])
    vt = ceed.Vector(P ** 3 * nc)
    b.apply(1, em, ut, vt, lc.TRANSPOSE)
    assert relinf(vt.get_array_read(), g[f"bapply_{mode}_vt"]) < 1e-13
    b.apply_add(1, em, ut, vt, lc.TRANSPOSE)
    assert relinf(vt.get_array_read(), 2 * g[f"bapply_{mode}_vt"]) < 1e-13
    w = ceed.Vector(Q ** 3)
    b.apply(1, lc.EVAL_WEIGHT, None, w)
    assert np.array_equal(w.get_array_read(), g["bapply_weight"])


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_basis_multi_element_against_oracle(ceed, dim):
    P, Q, nc, ne = 3, 5, 1, 7
    interp, grad, qref, qw = orc.lagrange_1d(P, Q)
    b = ceed.BasisTensorH1Lagrange(dim, nc, P, Q, lc.GAUSS)
    for mode, qc in ((lc.EVAL_INTERP, 1), (lc.EVAL_GRAD, dim)):
        uu = lc.mesh.uniform(9, ne * P ** dim)
        u = ceed.Vector(uu.size)
        u.set_array(uu)
        v = ceed.Vector(ne * Q ** dim * qc)
        b.apply(ne, mode, u, v)
        want = orc.basis_apply(dim, P, Q, nc, interp, grad, qw, ne, orc.NOTRANSPOSE, mode, uu)
        # oracle layout [elem][d][qpt]; backend [d][elem][qpt]
        want = want.reshape(ne, qc, Q ** dim).transpose(1, 0, 2).reshape(-1)
        assert relinf(v.get_array_read(), want) < 1e-13


def test_gallery_qfunction_apply(ceed):
    n = 1000
    qf = ceed.QFunctionByName("Poisson3DApply")
    du, qd = lc.mesh.uniform(3, 3 * n), lc.mesh.uniform(4, 6 * n)
    a, b, out = ceed.Vector(3 * n), ceed.Vector(6 * n), ceed.Vector(3 * n)
    a.set_array(du)
    b.set_array(qd)
    qf.apply(n, [a, b], [out])
    D = qd.reshape(6, n)
    M = np.array([[D[0], D[5], D[4]], [D[5], D[1], D[3]], [D[4], D[3], D[2]]])  # [3][3][n]
    ug = du.reshape(3, n)
    want = np.einsum("ijn,in->jn", M, ug).reshape(-1)
    assert relinf(out.get_array_read(), want) < 1e-14


def test_pipe_probes_report_positive_rates(ceed):
    # The compute-roofline denominators: FP64 and FP32 FMA rates, and the FP64 tensor-core (DMMA) rate alone and
    # interleaved with DFMA in every warp.
    assert ceed.fma_peak(lc.F64) > 0 and ceed.fma_peak(lc.F32) > 0
    dmma, mixed = ceed.fp64_tensor_peak()
    assert dmma > 0 and mixed > 0
