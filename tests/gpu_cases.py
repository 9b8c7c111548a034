"""Shared set-up of the GPU parity tests: the golden cases rebuilt through the libCEED-style API."""
import os

import numpy as np
import torch

from libceed_gb300 import mesh
from libceed_gb300.smoke_case import build_poisson
from tests.conftest import GOLDEN

CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f not in ("basis.npz", "blocked.npz"))

QF_OF_KIND = {"mass": "MassApply", "poisson": "Poisson3DApply", "vpoisson": "Vector3Poisson3DApply", "vmass": "Vector3MassApply",
              "kappa": "Poisson3DApplyKappa"}


def parse(case):
    kind, n, p = case.split("_")
    n, p = int(n[1:]), int(p[1:])
    seeds = {"mass": 1001, "poisson": 2000 + p, "vpoisson": 3000 + p, "vmass": 3100 + p, "kappa": 4000 + p}
    noise = 0.1 if kind == "mass" else 0.05
    ncomp = 3 if kind.startswith("v") else 1
    return kind, mesh.Box(n, p, ncomp=ncomp, noise=noise, seed=seeds[kind])


def golden(case):
    return np.load(os.path.join(GOLDEN, case + ".npz"))


def ref_layout_to_backend(a, num_elem, ncomp, size):
    """[elem][comp][node] (reference CPU E-layout) -> [comp][elem][node] (this backend)."""
    return np.ascontiguousarray(a.reshape(num_elem, ncomp, size).transpose(1, 0, 2).reshape(-1))


def setup(ceed, case, dtype=torch.float64):
    kind, box = parse(case)
    g = golden(case)
    objs = build_poisson(ceed, box, dtype=dtype, qf_name=QF_OF_KIND[kind])
    if kind == "kappa":
        kap = ceed.Vector(box.num_elem * box.Q ** 3, dtype)
        kap.set_array(g["kappa"])  # [elem][qpt] is also this backend's layout for one component
        objs["op"].set_field("kappa", objs["rq"], None, kap)
        objs["kappa"] = kap
    return kind, box, g, objs
