"""CG and mixed-precision iterative refinement on the GPU; the final residual is re-checked with the oracle."""
import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300 import mesh
from libceed_gb300.smoke_case import build_poisson
from libceed_gb300.solver import cg_solve
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem():
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(6, 3, noise=0.05, seed=21)
    o64 = build_poisson(ceed, box)
    o32 = build_poisson(ceed, box, dtype=torch.float32)
    m = mesh.box_mask(box.n, box.degree)
    xs = mesh.smooth_field(box.n, box.degree, seed=5) * m
    mask = ceed.Vector(box.l_size)
    mask.set_array(m)
    xv = ceed.Vector(box.l_size)
    xv.set_array(xs)
    b = ceed.Vector(box.l_size)
    o64["op"].apply(xv, b)
    bh = m * (b.get_array_read() + mesh.uniform(99, box.l_size, -1e-3, 1e-3))
    b.set_array(bh)
    pb = orc.BoxProblem(6, 3, seed=21)
    return ceed, box, o64, o32, mask, b, m, bh, pb


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("graph", [False, True])
def test_cg_reaches_tolerance(problem, mixed, graph):
    ceed, box, o64, o32, mask, b, m, bh, pb = problem
    x = ceed.Vector(box.l_size)
    st = cg_solve(ceed, o64["op"], o64["qdata"], mask, b, x, mixed=mixed, op32=o32["op"], qdata32=o32["qdata"], rtol=1e-10,
                  use_graph=graph, check_every=10)
    assert st["converged"] and st["rel_residual"] <= 1e-10
    if mixed:
        assert st["outer"] >= 2
    # Independent check of the residual with the CPU oracle.
    xh = x.get_array_read()
    r = m * (bh - pb.apply(m * xh))
    assert np.linalg.norm(r) / np.linalg.norm(bh) < 2e-10


def test_float_float_cg_matches_fp64(problem):
    """CG on the float-float operator (FP64 vectors and Krylov arithmetic, F64X apply) reaches the FP64 tolerance and
    the oracle-checked residual, in about the FP64 iteration count."""
    ceed, box, o64, o32, mask, b, m, bh, pb = problem
    x64, xff = ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    s64 = cg_solve(ceed, o64["op"], o64["qdata"], mask, b, x64, rtol=1e-10, check_every=10)
    o64["op"].arithmetic = "float-float"
    try:
        sff = cg_solve(ceed, o64["op"], o64["qdata"], mask, b, xff, rtol=1e-10, check_every=10)
    finally:
        o64["op"].arithmetic = "native"
    assert sff["converged"] and sff["rel_residual"] <= 1e-10
    assert abs(sff["iterations"] - s64["iterations"]) <= max(3, s64["iterations"] // 20)
    r = m * (bh - pb.apply(m * xff.get_array_read()))
    assert np.linalg.norm(r) / np.linalg.norm(bh) < 2e-10


def test_graph_and_eager_agree(problem):
    """With the deterministic scatter, graph-captured and eager solves run the same kernels in the same order."""
    _, box, _, _, _, _, m, bh, _ = problem
    ceed = lc.Ceed("/gpu/cuda/b200", deterministic=True)
    o64 = build_poisson(ceed, box)
    mask, b = ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    mask.set_array(m)
    b.set_array(bh)
    xs = []
    for graph in (False, True, True):
        x = ceed.Vector(box.l_size)
        cg_solve(ceed, o64["op"], o64["qdata"], mask, b, x, use_graph=graph, check_every=10, rtol=1e-8)
        xs.append(x.get_array_read())
    assert np.array_equal(xs[0], xs[1]) and np.array_equal(xs[1], xs[2])


@pytest.mark.parametrize("qf", ["Poisson3DApply", "MassApply"])
@pytest.mark.parametrize("n,degree,epb", [(3, 1, 4), (3, 3, 4), (4, 4, 6), (2, 6, 1), (2, 7, 1)])
def test_apply_dot_matches_dot_of_output(qf, n, degree, epb):
    """u . (A u) summed inside the persistent FP32 kernel equals the FP64 dot of u with the kernel's own output, and the
    output equals the plain apply's.  27 elements in batches of 4 leave inactive teams in the last batch, and every case
    launches more blocks than batches (blocks without a batch write 0)."""
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(n, degree, noise=0.05, seed=3)
    o = build_poisson(ceed, box, dtype=torch.float32, qf_name=qf)
    o["op"].fused(lc.F32).set_tile(epb, 7)
    u = ceed.Vector(box.l_size, torch.float32)
    u.set_array(mesh.uniform(17, box.l_size, -1.0, 1.0))
    v, v_ref = ceed.Vector(box.l_size, torch.float32), ceed.Vector(box.l_size, torch.float32)
    d = o["op"].apply_dot(u, v)
    o["op"].apply(u, v_ref)
    uh, vh, vr = u.get_array_read().astype(np.float64), v.get_array_read().astype(np.float64), v_ref.get_array_read()
    assert np.allclose(vh, vr, rtol=1e-5, atol=1e-5 * np.abs(vr).max())
    want = float(uh @ vh)
    assert d > 0 and abs(d - want) <= 2e-5 * abs(want)


def test_apply_dot_unavailable_without_persistent_kernel():
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(3, 3, noise=0.05, seed=3)
    o = build_poisson(ceed, box, dtype=torch.float32)
    o["op"].fused(lc.F32).set_tile(4, 5)
    u, v = ceed.Vector(box.l_size, torch.float32), ceed.Vector(box.l_size, torch.float32)
    u.set_value(1.0)
    with pytest.raises(lc.B200Error):
        o["op"].apply_dot(u, v)


@pytest.mark.parametrize("jacobi", [False, True])
def test_cg_fused_pdot_matches_separate(problem, jacobi):
    """Mixed CG on the persistent FP32 kernel: p.(A p) summed inside the apply or in a separate pass over p and A p
    gives the same convergence (iteration counts within a few) and the oracle-checked residual."""
    from libceed_gb300.solver import jacobi_preconditioner

    ceed, box, o64, o32, mask, b, m, bh, pb = problem
    o32["op"].fused(lc.F32).set_tile(4, 7)
    try:
        pre = jacobi_preconditioner(ceed, o64["op"], mask) if jacobi else None
        stats = {}
        for fused in (True, False):
            x = ceed.Vector(box.l_size)
            st = cg_solve(ceed, o64["op"], o64["qdata"], mask, b, x, mixed=True, op32=o32["op"], qdata32=o32["qdata"], rtol=1e-10,
                          check_every=10, jacobi=pre, fused_pdot=fused)
            assert st["converged"] and st["rel_residual"] <= 1e-10
            r = m * (bh - pb.apply(m * x.get_array_read()))
            assert np.linalg.norm(r) / np.linalg.norm(bh) < 2e-10
            stats[fused] = st
        assert abs(stats[True]["iterations"] - stats[False]["iterations"]) <= max(5, stats[False]["iterations"] // 20)
        # One kernel fewer per iteration (the pass over p and A p).
        assert stats[True]["launches"] < stats[False]["launches"]
    finally:
        o32["op"].fused(lc.F32).set_tile(0, 0)
