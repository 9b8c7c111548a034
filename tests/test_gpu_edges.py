"""Edge cases of the fused apply: ragged last element batches for every staging, elements-per-block and kernel
family (against the reference's golden vectors), and operators with no elements (Apply zeroes the output,
ApplyAdd leaves it), as the reference's restriction and operator tests cover empty and partial blocks."""
import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from tests.conftest import relinf
from tests.gpu_cases import setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ceed():
    return lc.Ceed("/gpu/cuda/b200")


@pytest.fixture(scope="module")
def ceed_det():
    return lc.Ceed("/gpu/cuda/b200", deterministic=True)


@pytest.mark.parametrize("case", ["poisson_n3_p4", "mass_n8_p3"])
@pytest.mark.parametrize("staging", [1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("epb", [2, 4, 5, 7])
@pytest.mark.parametrize("family", ["f64", "f32", "f64x"])
def test_ragged_last_block(ceed, ceed_det, case, staging, epb, family):
    """27 or 512 elements in batches of 2, 4, 5 or 7: the last batch is partial."""
    if family == "f64x" and staging == 3:
        pytest.skip("float-float kernels: no persistent pipelined variant")
    if family != "f32" and staging == 7:
        pytest.skip("the persistent bulk-copy kernel is FP32")
    dt = torch.float32 if family == "f32" else torch.float64
    for c in (ceed, ceed_det):
        kind, box, g, objs = setup(c, case, dtype=dt)
        op = objs["op"]
        op.elems_per_block, op.staging = epb, staging
        if family == "f64x":
            op.arithmetic = "float-float"
        u = c.Vector(box.l_size, dt)
        u.set_array(box.u())
        v = c.Vector(box.l_size, dt)
        v.set_value(7.0)
        op.apply(u, v)
        assert relinf(v.get_array_read(), g["v"]) < (5e-5 if family == "f32" else 1e-12)
        assert c.status() == 0


@pytest.mark.parametrize("qf", ["Poisson3DApply", "MassApply"])
@pytest.mark.parametrize("det", [False, True])
def test_operator_without_elements(ceed, ceed_det, qf, det):
    c = ceed_det if det else ceed
    P, Q, n = 5, 6, 10
    poisson = qf.startswith("Poisson")
    ru = c.ElemRestriction(0, P ** 3, 1, 1, n, np.zeros(0, np.int32))
    rq = c.StridedElemRestriction(0, Q ** 3, 6 if poisson else 1, 0, lc.STRIDES_BACKEND)
    bu = c.BasisTensorH1Lagrange(3, 1, P, Q, lc.GAUSS)
    op = c.Operator(c.QFunctionByName(qf))
    fin, fout = ("du", "dv") if poisson else ("u", "v")
    op.set_field(fin, ru, bu, "active")
    op.set_field("qdata", rq, None, c.Vector(0))
    op.set_field(fout, ru, bu, "active")
    u, v = c.Vector(n), c.Vector(n)
    u.set_value(1.0)
    v.set_value(3.0)
    op.apply(u, v)
    assert np.all(v.get_array_read() == 0.0)
    v.set_value(3.0)
    op.apply_add(u, v)
    assert np.all(v.get_array_read() == 3.0)


@pytest.mark.parametrize("staging", [1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("epb", [1, 3])
@pytest.mark.parametrize("family", ["f64", "f32", "f64x"])
def test_kappa_even_q_every_staging(ceed, staging, epb, family):
    """kappa-weighted diffusion at degree 4 (Q = 6: every element's qdata and kappa start on 16 bytes, so the bulk-copy
    staging copies element by element into padded slabs) against the oracle, for every staging."""
    from libceed_gb300 import mesh
    from libceed_gb300.smoke_case import build_poisson
    from oracle import oracle as orc

    if family == "f64x" and staging == 3:
        pytest.skip("float-float kernels: no persistent pipelined variant")
    if family != "f32" and staging == 7:
        pytest.skip("the persistent bulk-copy kernel is FP32")
    dt = torch.float32 if family == "f32" else torch.float64
    pb = orc.BoxProblem(3, 4, poisson=True, noise=0.05, seed=4104, kappa=True)
    box = mesh.Box(3, 4, noise=0.05, seed=4104)
    u0 = box.u()
    ref = pb.apply(u0)
    objs = build_poisson(ceed, box, dtype=dt, qf_name="Poisson3DApplyKappa")
    kap = ceed.Vector(box.num_elem * box.Q ** 3, dt)
    kap.set_array(pb.kappa)
    op = objs["op"]
    op.set_field("kappa", objs["rq"], None, kap)
    op.elems_per_block, op.staging = epb, staging
    if family == "f64x":
        op.arithmetic = "float-float"
    u = ceed.Vector(box.l_size, dt)
    u.set_array(u0)
    v = ceed.Vector(box.l_size, dt)
    op.apply(u, v)
    assert relinf(v.get_array_read(), ref) < (5e-5 if family == "f32" else 1e-12)
    assert ceed.status() == 0


def test_bounded_wait_gives_up_and_context_survives(ceed):
    """A bounded mbarrier wait that nothing completes gives up, sets the status bit the host reads, and leaves the
    context usable: the next apply still matches the reference."""
    from libceed_gb300._ffi import call

    ceed.status()
    call("b200_wait_selftest", ceed._ctx, 256)
    assert ceed.status() == 1  # B200_STATUS_COPY_TIMEOUT, cleared by the read
    assert ceed.status() == 0
    kind, box, g, objs = setup(ceed, "poisson_n3_p4")
    u = ceed.Vector(box.l_size)
    u.set_array(box.u())
    v = ceed.Vector(box.l_size)
    objs["op"].apply(u, v)
    assert relinf(v.get_array_read(), g["v"]) < 1e-12
    assert ceed.status() == 0
