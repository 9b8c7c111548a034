"""Diagonal assembly of the fused operators and Jacobi-preconditioned CG."""
import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300 import mesh
from libceed_gb300.smoke_case import build_poisson
from libceed_gb300.solver import assemble_diagonal, cg_solve, jacobi_preconditioner
from oracle import oracle as orc
from tests.conftest import relinf

pytestmark = pytest.mark.gpu


def _oracle_diag(pb):
    d = np.zeros(pb.l_size)
    for i in range(pb.l_size):
        e = np.zeros(pb.l_size)
        e[i] = 1.0
        d[i] = pb.apply(e)[i]
    return d


@pytest.mark.parametrize("det", [False, True])
@pytest.mark.parametrize("kind,n,p", [("poisson", 2, 3), ("poisson", 2, 4), ("mass", 3, 2), ("poisson", 3, 1)])
def test_diagonal_matches_oracle(det, kind, n, p):
    ceed = lc.Ceed("/gpu/cuda/b200", deterministic=det)
    box = mesh.Box(n, p, noise=0.05, seed=31)
    objs = build_poisson(ceed, box, qf_name=None if kind == "poisson" else "MassApply")
    d = ceed.Vector(box.l_size)
    assemble_diagonal(ceed, objs["op"], d)
    pb = orc.BoxProblem(n, p, poisson=kind == "poisson", noise=0.05, seed=31)
    assert relinf(d.get_array_read(), _oracle_diag(pb)) < 1e-12


def test_vector_diagonal_repeats_per_component():
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(2, 2, ncomp=3, noise=0.05, seed=32)
    objs = build_poisson(ceed, box)
    d = ceed.Vector(box.l_size)
    assemble_diagonal(ceed, objs["op"], d)
    ds = d.get_array_read().reshape(-1, 3)
    box1 = mesh.Box(2, 2, noise=0.05, seed=32)
    pb = orc.BoxProblem(2, 2, poisson=True, noise=0.05, seed=32)
    want = _oracle_diag(pb)
    for c in range(3):
        assert relinf(ds[:, c], want) < 1e-12


@pytest.mark.parametrize("mixed", [False, True])
def test_jacobi_pcg(mixed):
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(6, 3, noise=0.05, seed=21)
    o64 = build_poisson(ceed, box)
    o32 = build_poisson(ceed, box, dtype=torch.float32)
    m = mesh.box_mask(box.n, box.degree)
    mask, b = ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    mask.set_array(m)
    bh = m * mesh.uniform(5, box.l_size)
    b.set_array(bh)
    inv = jacobi_preconditioner(ceed, o64["op"], mask)
    res = {}
    for pc in (None, inv):
        x = ceed.Vector(box.l_size)
        res[pc is None] = cg_solve(ceed, o64["op"], o64["qdata"], mask, b, x, mixed=mixed, op32=o32["op"], qdata32=o32["qdata"], rtol=1e-10,
                                   jacobi=pc, check_every=10)
        assert res[pc is None]["converged"]
        pb = orc.BoxProblem(6, 3, seed=21)
        r = m * (bh - pb.apply(m * x.get_array_read()))
        assert np.linalg.norm(r) / np.linalg.norm(bh) < 2e-10
    assert res[False]["iterations"] < res[True]["iterations"]  # the preconditioner pays


def test_composite_operator_sums_sub_operators():
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(3, 3, noise=0.05, seed=41)
    a = build_poisson(ceed, box)
    m = build_poisson(ceed, box, qf_name="MassApply")
    comp = ceed.CompositeOperator()
    comp.add_sub(a["op"])
    comp.add_sub(m["op"])
    u, v, va, vm = (ceed.Vector(box.l_size) for _ in range(4))
    u.set_array(box.u())
    comp.apply(u, v)
    a["op"].apply(u, va)
    m["op"].apply(u, vm)
    assert relinf(v.get_array_read(), va.get_array_read() + vm.get_array_read()) < 1e-14
