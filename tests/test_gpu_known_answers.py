"""Known answers of the reference's examples, through the fused GPU operator in every arithmetic family.

* Volume (examples/ceed/ex1-volume.c:262-272): 1^T M 1 = 1 for the unit box.  Tolerance 1e-13 for FP64, 1e-12 for
  float-float, ex1's own 1e-5 for FP32.
* Surface area (examples/ceed/ex2-surface.c:248-290): sum |A (x + y + z)| = 6 within ex2's 3D tolerance of 1e-1, and
  equal to the oracle's sum within 1e-12 relative in FP64 and 1e-10 relative in float-float (its ~48-bit arithmetic
  leaves about 1e-15 on each of the 35,937 entries, most of which are zero in exact arithmetic; measured 9.7e-12).
* Energy of linear fields: (x+y+z)^T A (x+y+z) = 3 and x^T A y = 0 (exact Galerkin identities on this mesh).
  Tolerance 1e-12 for FP64, 1e-11 for float-float, 1e-4 for FP32 (vectors rounded to FP32).
"""
import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300 import mesh
from libceed_gb300.smoke_case import build_poisson
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

FAMILIES = ["f64", "f64_det", "f64x", "f32"]
VOL_TOL = {"f64": 1e-13, "f64_det": 1e-13, "f64x": 1e-12, "f32": 1e-5}
ENERGY_TOL = {"f64": 1e-12, "f64_det": 1e-12, "f64x": 1e-11, "f32": 1e-4}
SURFACE_TOL = {"f64": 1e-12, "f64_det": 1e-12, "f64x": 1e-10}


@pytest.fixture(scope="module")
def ceeds():
    return {"atomic": lc.Ceed("/gpu/cuda/b200"), "det": lc.Ceed("/gpu/cuda/b200", deterministic=True)}


def _apply(ceeds, family, box, qf_name, u):
    dtype = torch.float32 if family == "f32" else torch.float64
    ceed = ceeds["det" if family == "f64_det" else "atomic"]
    objs = build_poisson(ceed, box, dtype=dtype, qf_name=qf_name)
    if family == "f64x":
        objs["op"].arithmetic = "float-float"
    uv, vv = ceed.Vector(box.l_size, dtype), ceed.Vector(box.l_size, dtype)
    uv.set_array(u)
    objs["op"].apply(uv, vv)
    return uv.get_array_read().astype(np.float64), vv.get_array_read().astype(np.float64)


@pytest.mark.parametrize("family", FAMILIES)
@pytest.mark.parametrize("n,p", [(3, 1), (3, 3), (2, 5)])
def test_volume(ceeds, family, n, p):
    box = mesh.Box(n, p, noise=0.1, seed=80 + p)
    _, v = _apply(ceeds, family, box, "MassApply", np.ones(box.l_size))
    assert abs(v.sum() - 1.0) < VOL_TOL[family]


@pytest.mark.parametrize("family", FAMILIES)
@pytest.mark.parametrize("n,p", [(3, 3), (2, 5)])
def test_linear_fields_energy(ceeds, family, n, p):
    box = mesh.Box(n, p, noise=0.05, seed=90 + p)
    xyz = box.node_coords()
    s, v = _apply(ceeds, family, box, None, xyz.sum(axis=1))
    assert abs(s @ v - 3.0) < ENERGY_TOL[family]
    _, vy = _apply(ceeds, family, box, None, xyz[:, 1])
    assert abs(xyz[:, 0] @ vy) < ENERGY_TOL[family]


@pytest.mark.parametrize("family", FAMILIES)
def test_surface_area(ceeds, family):
    box = mesh.Box(8, 4, noise=0.05, seed=71)
    u = box.node_coords().sum(axis=1)
    _, v = _apply(ceeds, family, box, None, u)
    area = np.abs(v).sum()
    assert abs(area - 6.0) < 1e-1
    if family != "f32":
        want = np.abs(orc.BoxProblem(8, 4, poisson=True, noise=0.05, seed=71).apply(u)).sum()
        assert abs(area - want) < SURFACE_TOL[family] * want
