"""QFunctions given as source, compiled at run time (NVRTC, sm_103a) into the fused operator kernel."""
import os

import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300.smoke_case import build_poisson
from tests.conftest import relinf
from tests.gpu_cases import golden, parse

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "qfunctions", "user-qfunctions.h")


@pytest.fixture(scope="module", params=[False, True], ids=["atomic", "det"])
def ceed(request):
    return lc.Ceed("/gpu/cuda/b200", deterministic=request.param)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_user_kappa_diffusion(ceed, dtype):
    kind, box = parse("kappa_n3_p3")
    g = golden("kappa_n3_p3")
    objs = build_poisson(ceed, box, dtype=dtype)  # qdata from the Poisson3DBuild setup
    qf = ceed.QFunction(1, None, SRC + ":DiffusionKappa")
    qf.add_input("du", 3, lc.EVAL_GRAD)
    qf.add_input("qdata", 6, lc.EVAL_NONE)
    qf.add_input("kappa", 1, lc.EVAL_NONE)
    qf.add_output("dv", 3, lc.EVAL_GRAD)
    kap = ceed.Vector(box.num_elem * box.Q ** 3, dtype)
    kap.set_array(g["kappa"])
    op = ceed.Operator(qf)
    op.set_field("du", objs["ru"], objs["bu"], "active")
    op.set_field("qdata", objs["rq"], None, objs["qdata"])
    op.set_field("kappa", objs["rq"], None, kap)
    op.set_field("dv", objs["ru"], objs["bu"], "active")
    u, v = ceed.Vector(box.l_size, dtype), ceed.Vector(box.l_size, dtype)
    u.set_array(box.u())
    op.apply(u, v)
    assert relinf(v.get_array_read(), g["v"]) < (1e-12 if dtype == torch.float64 else 5e-5)


def test_user_scaled_mass_with_context(ceed):
    kind, box = parse("mass_n8_p3")
    g = golden("mass_n8_p3")
    objs = build_poisson(ceed, box, qf_name="MassApply")
    qf = ceed.QFunction(1, None, SRC + ":ScaledMass")
    qf.add_input("qdata", 1, lc.EVAL_NONE)  # passive input first: the active field need not be input 0
    qf.add_input("u", 1, lc.EVAL_INTERP)
    qf.add_output("v", 1, lc.EVAL_INTERP)
    ctx = ceed.QFunctionContext()
    ctx.set_data(np.array([2.5]))
    qf.set_context(ctx)
    op = ceed.Operator(qf)
    op.set_field("qdata", objs["rq"], None, objs["qdata"])
    op.set_field("u", objs["ru"], objs["bu"], "active")
    op.set_field("v", objs["ru"], objs["bu"], "active")
    u, v = ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    u.set_array(box.u())
    op.apply(u, v)
    assert relinf(v.get_array_read(), 2.5 * g["v"]) < 1e-12


def test_bad_source_reports_the_compiler_log(ceed, tmp_path):
    bad = tmp_path / "bad.h"
    bad.write_text("#include <ceed/types.h>\nCEED_QFUNCTION(Broken)(void *ctx, const CeedInt Q, const CeedScalar *const *in, "
                   "CeedScalar *const *out) { return undefined_symbol; }\n")
    kind, box = parse("mass_n8_p3")
    objs = build_poisson(ceed, box, qf_name="MassApply")
    qf = ceed.QFunction(1, None, str(bad) + ":Broken")
    qf.add_input("u", 1, lc.EVAL_INTERP)
    qf.add_input("qdata", 1, lc.EVAL_NONE)
    qf.add_output("v", 1, lc.EVAL_INTERP)
    op = ceed.Operator(qf)
    op.set_field("u", objs["ru"], objs["bu"], "active")
    op.set_field("qdata", objs["rq"], None, objs["qdata"])
    op.set_field("v", objs["ru"], objs["bu"], "active")
    u, v = ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    with pytest.raises(lc.B200Error, match="NVRTC"):
        op.apply(u, v)
