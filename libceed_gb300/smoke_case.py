"""A small end-to-end case through the libCEED-style API: box mesh -> qdata setup -> fused Poisson apply."""
import numpy as np
import torch

from . import mesh
from .ceed import EVAL_GRAD, GAUSS, STRIDES_BACKEND, Ceed


def build_poisson(ceed, box, dtype=torch.float64, qf_name=None):
    """Create the setup and apply operators of a Poisson (or mass) problem on `box`; returns a dict of objects."""
    P, Q, ne, nc = box.P, box.Q, box.num_elem, box.ncomp
    poisson = qf_name is None or "Poisson" in qf_name
    qf_name = qf_name or ("Poisson3DApply" if nc == 1 else "Vector3Poisson3DApply")
    nqd = 6 if poisson else 1
    rx = ceed.ElemRestriction(ne, 8, 3, box.num_vertices, 3 * box.num_vertices, box.vertex_offsets())
    ru = ceed.ElemRestriction(ne, P ** 3, nc, box.comp_stride, box.l_size, box.offsets())
    rq = ceed.StridedElemRestriction(ne, Q ** 3, nqd, nqd * ne * Q ** 3, STRIDES_BACKEND)
    bx = ceed.BasisTensorH1Lagrange(3, 3, 2, Q, GAUSS)
    bu = ceed.BasisTensorH1Lagrange(3, nc, P, Q, GAUSS)
    X = ceed.Vector(3 * box.num_vertices)
    X.set_array(box.coords())
    qdata = ceed.Vector(nqd * ne * Q ** 3)
    build = ceed.Operator(ceed.QFunctionByName("Poisson3DBuild" if poisson else "Mass3DBuild"))
    build.set_field("dx", rx, bx, "active")
    build.set_field("weights", None, bx, None)
    build.set_field("qdata", rq, None, "active")
    build.apply(X, qdata)
    if dtype != torch.float64:
        q32 = ceed.Vector(qdata.size, dtype)
        q32.copy_from(qdata)
        qdata = q32
    op = ceed.Operator(ceed.QFunctionByName(qf_name))
    fin, fout = ("du", "dv") if poisson else ("u", "v")
    op.set_field(fin, ru, bu, "active")
    op.set_field("qdata", rq, None, qdata)
    op.set_field(fout, ru, bu, "active")
    return dict(op=op, qdata=qdata, ru=ru, rq=rq, bu=bu, build=build, X=X)


def run_poisson(n=3, degree=3, device="cuda:0", seed=11, family="f64"):
    """Apply the Poisson operator to the seeded input; returns v on the host.  family: "f64" (FP64 kernels), "f64x"
    (float-float kernels on the same double vectors) or "f32" (FP32 vectors and kernels)."""
    ceed = Ceed("/gpu/cuda/b200:device_id=" + str(torch.device(device).index or 0))
    box = mesh.Box(n, degree, noise=0.05, seed=seed)
    dt = torch.float32 if family == "f32" else torch.float64
    objs = build_poisson(ceed, box, dtype=dt)
    if family == "f64x":
        objs["op"].arithmetic = "float-float"
    u = ceed.Vector(box.l_size, dt)
    u.set_array(box.u())
    v = ceed.Vector(box.l_size, dt)
    objs["op"].apply(u, v)
    return v.get_array_read().astype("float64")
