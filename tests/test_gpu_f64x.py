"""Float-float fused apply (B200_F64X): double vectors, FP32-pipe arithmetic carrying ~48 significant bits.

Parity bar: 1e-12 relative l-infinity against the reference's golden vectors, the FP64 bar.  Also checked against the
native FP64 kernel on a larger random problem, for both scatters and both qdata stagings.
"""
import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300 import mesh
from libceed_gb300.smoke_case import build_poisson
from tests.conftest import relinf
from tests.gpu_cases import setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ceed():
    return lc.Ceed("/gpu/cuda/b200")


@pytest.fixture(scope="module")
def ceed_det():
    return lc.Ceed("/gpu/cuda/b200", deterministic=True)


@pytest.mark.parametrize("case", ["poisson_n6_p1", "poisson_n4_p2", "poisson_n3_p3", "poisson_n3_p4", "poisson_n2_p5", "poisson_n2_p6",
                                  "poisson_n2_p7", "poisson_n2_p8", "mass_n8_p3"])
@pytest.mark.parametrize("staging", [1, 2, 4, 5, 6])
@pytest.mark.parametrize("epb", [0, 3])
def test_float_float_apply_matches_reference(ceed, ceed_det, case, staging, epb):
    for c in (ceed, ceed_det):
        kind, box, g, objs = setup(c, case)
        op = objs["op"]
        op.arithmetic = "float-float"
        op.elems_per_block, op.staging = epb, staging
        u = c.Vector(box.l_size)
        u.set_array(box.u())
        v = c.Vector(box.l_size)
        v.set_value(5.0)
        op.apply(u, v)
        assert relinf(v.get_array_read(), g["v"]) < 1e-12
        assert op.fused(lc.F64X).tile()[2] == staging
        assert c.status() == 0


@pytest.mark.parametrize("p", [2, 4, 6])
@pytest.mark.parametrize("qf", ["Poisson3DApply", "MassApply"])
def test_float_float_matches_native_fp64(ceed, p, qf):
    box = mesh.Box(12, p, noise=0.05, seed=77 + p)
    objs = build_poisson(ceed, box, dtype=torch.float64, qf_name=qf)
    op = objs["op"]
    u = ceed.Vector(box.l_size)
    u.set_array(mesh.uniform(5 + p, box.l_size) - 0.5)
    v64, vxx = ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    op.apply(u, v64)
    op.arithmetic = "float-float"
    vxx.set_value(0.0)
    op.apply_add(u, vxx)
    a, b = v64.get_array_read(), vxx.get_array_read()
    assert relinf(b, a) < 1e-12
    assert not np.array_equal(a, b)  # a different arithmetic really ran


def test_float_float_deterministic_is_bit_reproducible(ceed_det):
    kind, box, g, objs = setup(ceed_det, "poisson_n3_p4")
    objs["op"].arithmetic = "float-float"
    u = ceed_det.Vector(box.l_size)
    u.set_array(box.u())
    outs = []
    for _ in range(3):
        v = ceed_det.Vector(box.l_size)
        objs["op"].apply(u, v)
        outs.append(v.get_array_read())
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


@pytest.mark.parametrize("case", ["vpoisson_n4_p2", "vpoisson_n3_p4", "vmass_n3_p4", "kappa_n3_p3"])
@pytest.mark.parametrize("staging", [1, 2, 4, 5, 6])
def test_float_float_vector_and_kappa_match_reference(ceed, ceed_det, case, staging):
    for c in (ceed, ceed_det):
        kind, box, g, objs = setup(c, case)
        op = objs["op"]
        op.arithmetic = "float-float"
        op.staging = staging
        u = c.Vector(box.l_size)
        u.set_array(box.u())
        v = c.Vector(box.l_size)
        op.apply(u, v)
        assert relinf(v.get_array_read(), g["v"]) < 1e-12
        assert c.status() == 0


def test_float_float_unsupported_raise(ceed):
    kind, box, g, objs = setup(ceed, "poisson_n3_p3", dtype=torch.float32)
    objs["op"].arithmetic = "float-float"
    u32 = ceed.Vector(box.l_size, torch.float32)
    with pytest.raises(lc.B200Error):
        objs["op"].apply(u32, ceed.Vector(box.l_size, torch.float32))
