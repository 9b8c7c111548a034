"""Host-side logic of the Python mirror beyond Vector (python/ceed_elemrestriction.py, ceed_basis.py,
ceed_qfunctioncontext.py, ceed_operator.py), on CPU with a stand-in context: no kernel is called.

Multiplicity is pinned to the oracle's restatement of the reference's E^T (E 1) (bitwise: integer counts).
"""
import types

import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300 import ceed as cm
from libceed_gb300 import mesh
from oracle import oracle as orc


@pytest.fixture
def host_ceed():
    return types.SimpleNamespace(device=torch.device("cpu"), deterministic=False)


@pytest.mark.parametrize("n,p,ncomp", [(2, 1, 1), (3, 2, 1), (2, 3, 3)])
def test_multiplicity_matches_oracle_transpose_of_ones(host_ceed, n, p, ncomp):
    P = p + 1
    off = mesh.box_offsets(n, n, n, P, ncomp)
    nodes = (n * p + 1) ** 3
    lsize, compstride = nodes * ncomp, (nodes if ncomp == 1 else 1)
    r = cm.ElemRestriction(host_ceed, n ** 3, P ** 3, ncomp, compstride, lsize, off)
    got = r.get_multiplicity().get_array_read()
    want = orc.rstr_scatter_add(off, P ** 3, ncomp, compstride, np.ones(n ** 3 * ncomp * P ** 3), np.zeros(lsize))
    assert np.array_equal(got, want)
    assert got.max() == 8 and got.min() == 1  # interior vertices are shared by 8 hexahedra, corners by one


def test_layouts(host_ceed):
    r = cm.ElemRestriction(host_ceed, 2, 8, 1, 12, 12, np.arange(16, dtype=np.int32) % 12)
    with pytest.raises(lc.B200Error, match="strided"):
        r.get_l_layout()
    s = cm.StridedElemRestriction(host_ceed, 3, 4, 2, 24, [1, 4, 8])
    assert s.get_l_layout().tolist() == [1, 4, 8]
    assert cm.StridedElemRestriction(host_ceed, 3, 4, 2, 24, lc.STRIDES_BACKEND).get_l_layout().tolist() == [1, 12, 4]
    assert np.all(s.get_multiplicity().get_array_read() == 1.0)
    lvec, evec = s.create_vector()
    assert (lvec.size, evec.size) == (24, 24)


def test_transposes_apply_in_transpose_mode(host_ceed):
    seen = []
    fake_rstr = types.SimpleNamespace(apply=lambda u, v, tmode, request: seen.append(("rstr", tmode)))
    cm.TransposeElemRestriction(fake_rstr).apply("u", "v")
    fake_basis = types.SimpleNamespace(apply=lambda nelem, emode, u, v, tmode: seen.append(("basis", nelem, emode, tmode)))
    cm.TransposeBasis(fake_basis).apply(5, lc.EVAL_GRAD, "u", "v")
    assert seen == [("rstr", lc.TRANSPOSE), ("basis", 5, lc.EVAL_GRAD, lc.TRANSPOSE)]
    r = cm.ElemRestriction(host_ceed, 1, 8, 1, 8, 8, np.arange(8, dtype=np.int32))
    assert isinstance(r.T, cm.TransposeElemRestriction) and r.transpose._elemrestriction is r


def test_qfunction_context_data(host_ceed):
    ctx = cm.QFunctionContext(host_ceed)
    with pytest.raises(lc.B200Error):
        ctx.get_data()
    ctx.set_data(np.array([1.5, 2.0, -3.0]))
    assert ctx.get_context_size() == 24 and ctx.ptr() is not None
    with ctx.data() as x:
        x[1] = 7.0
    assert ctx.get_data().tolist() == [1.5, 7.0, -3.0]
    ctx.restore_data()
    with ctx.data(3, 1) as x:
        assert x.shape == (3, 1)
        x[2, 0] = 0.25
    assert ctx.get_data().tolist() == [1.5, 7.0, 0.25]


def test_operator_check_and_name(host_ceed):
    op = cm.Operator(host_ceed, cm.QFunctionByName(host_ceed, "MassApply"))
    op.name("mass")
    with pytest.raises(lc.B200Error, match="u, qdata, v"):
        op.check()
    for f in ("u", "qdata", "v"):
        op.set_field(f, None, None, "active")
    op.check()
    comp = cm.CompositeOperator(host_ceed)
    comp.add_sub(op)
    comp.check()


def test_diagonal_assembly_plumbing(host_ceed, monkeypatch):
    """linear_assemble_(add_)diagonal route to the diagonal-assembly kernel's wrapper and add with AXPY."""
    import libceed_gb300.solver as solver

    def fake_assemble(ceed, op, d):
        d.data.copy_(torch.full((d.size,), float(op.tag)))

    monkeypatch.setattr(solver, "assemble_diagonal", fake_assemble)
    monkeypatch.setattr(cm.Vector, "axpy", lambda self, a, x: self.data.add_(a * x.data))
    monkeypatch.setattr(cm.Vector, "set_value", lambda self, value: self.data.fill_(value))
    ops = []
    for tag in (2.0, 3.0):
        op = cm.Operator(host_ceed, cm.QFunctionByName(host_ceed, "MassApply"))
        op.tag = tag
        ops.append(op)
    d = cm.Vector(host_ceed, 4)
    d.set_array(np.ones(4))
    ops[0].linear_assemble_diagonal(d)
    assert d.get_array_read().tolist() == [2.0] * 4
    ops[1].linear_assemble_add_diagonal(d)
    assert d.get_array_read().tolist() == [5.0] * 4
    comp = cm.CompositeOperator(host_ceed)
    for op in ops:
        comp.add_sub(op)
    comp.linear_assemble_diagonal(d)
    assert d.get_array_read().tolist() == [5.0] * 4
    with pytest.raises(lc.B200Error, match="FP64"):
        ops[0].linear_assemble_diagonal(cm.Vector(host_ceed, 4, torch.float32))


def test_scalar_type():
    assert cm.Ceed.scalar_type(None) == "float64"


def test_multiplicity_known_answer(host_ceed):
    """The reference's tests/t209-elemrestriction.c: 3 elements of 4 nodes sharing one node with each neighbour."""
    ne = 3
    ind = np.array([[3 * e + k for k in range(4)] for e in range(ne)], dtype=np.int32).reshape(-1)
    r = cm.ElemRestriction(host_ceed, ne, 4, 1, 1, 3 * ne + 1, ind)
    want = [1 + (1 if 0 < i < 3 * ne and i % 3 == 0 else 0) for i in range(3 * ne + 1)]
    assert r.get_multiplicity().get_array_read().tolist() == want


def test_transpose_known_answer_on_oracle():
    """The reference's tests/t206-elemrestriction.c on the oracle's scatter: 5 two-node elements, 2 components with
    component stride num_elem + 1; y[i] = i * mult and y[i + ne + 1] = (10 + i) * mult."""
    ne, P, nc = 5, 2, 2
    ind = np.array([[e, e + 1] for e in range(ne)], dtype=np.int32).reshape(-1)
    x = np.zeros(ne * nc * P)
    for i in range(P):  # node
        for j in range(nc):  # component
            for k in range(ne):  # element; the oracle's E-layout is [elem][comp][node]
                x[i + P * j + P * nc * k] = 10 * j + (2 * k + i + 1) // 2
    y = orc.rstr_scatter_add(ind, P, nc, ne + 1, x, np.zeros(nc * (ne + 1)))
    for i in range(ne + 1):
        mult = 2 if 0 < i < ne else 1
        assert y[i] == i * mult and y[i + ne + 1] == (10 + i) * mult


def test_cg_solve_passes_each_option_to_its_field(monkeypatch):
    """solver.cg_solve builds b200_cg_opts positionally; every keyword must land in the field of the same meaning."""
    from libceed_gb300 import solver

    seen = {}

    def call(name, *args):
        assert name == "b200_cg_solve"
        seen["opts"] = args[-2]._obj
        stats = args[-1]._obj
        stats.iterations, stats.outer, stats.converged, stats.rel_residual = 42, 3, 1, 5e-11

    monkeypatch.setattr(solver, "call", call)
    vec = types.SimpleNamespace(ptr=lambda: None, size=10, data=types.SimpleNamespace(data_ptr=lambda: 0x1000))
    op = types.SimpleNamespace(fused=lambda prec: types.SimpleNamespace(h="h"), _kernel_prec=lambda prec: prec)
    out = solver.cg_solve(types.SimpleNamespace(_ctx=None), op, vec, vec, vec, vec, mixed=True, op32=op, qdata32=vec, rtol=1e-9,
                          inner_rtol=2e-3, max_it=777, max_outer=11, use_graph=False, check_every=13, jacobi=vec, fused_pdot=False)
    o = seen["opts"]
    assert (o.rtol, o.max_it, o.mixed, o.inner_rtol, o.max_outer, o.use_graph, o.check_every, o.jacobi, o.separate_pdot) == (
        1e-9, 777, 1, 2e-3, 11, 0, 13, 0x1000, 1)
    assert out["iterations"] == 42 and out["outer"] == 3 and out["converged"] is True and out["rel_residual"] == 5e-11
