"""Pin the CPU oracle (oracle/ceed_oracle.c) to vectors produced by the reference libCEED.

The fixtures in tests/golden/ come from the reference's own `/cpu/self/ref/serial`
backend driven through the libCEED API (tests/golden/make_golden.py).  These tests
need no GPU.
"""
import hashlib
import os

import numpy as np
import pytest

from libceed_gb300 import mesh
from oracle import oracle as orc
from tests.conftest import GOLDEN, relinf

CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f not in ("basis.npz", "blocked.npz"))


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _problem(case):
    kind, n, p = case.split("_")
    n, p = int(n[1:]), int(p[1:])
    seeds = {"mass": 1001, "poisson": 2000 + p, "vpoisson": 3000 + p, "vmass": 3100 + p, "kappa": 4000 + p}
    noise = 0.1 if kind == "mass" else 0.05
    return orc.BoxProblem(n, p, ncomp=3 if kind.startswith("v") else 1, poisson=kind not in ("mass", "vmass"), noise=noise,
                          seed=seeds[kind], kappa=kind == "kappa")


@pytest.fixture(scope="module")
def basis_gold():
    return np.load(os.path.join(GOLDEN, "basis.npz"))


@pytest.mark.parametrize("P", range(2, 11))
def test_basis_tables_match_reference(basis_gold, P):
    Q = P + 1
    interp, grad, qref, qw = orc.lagrange_1d(P, Q, orc.GAUSS)
    tag = f"basis_P{P}_Q{Q}_gauss_"
    # Same recurrences as the reference: bitwise equal.
    assert np.array_equal(interp.ravel(), basis_gold[tag + "interp"])
    assert np.array_equal(grad.ravel(), basis_gold[tag + "grad"])
    assert np.array_equal(qref, basis_gold[tag + "qref"])
    assert np.array_equal(qw, basis_gold[tag + "qweight"])
    # Collocated gradient through the same Householder pseudoinverse: bitwise equal.
    colo = orc.collocated_grad(P, Q, interp, grad)
    assert np.array_equal(colo.ravel(), basis_gold[tag + "colograd"])


def test_lobatto_tables_match_reference(basis_gold):
    interp, grad, qref, qw = orc.lagrange_1d(4, 4, orc.GAUSS_LOBATTO)
    assert np.array_equal(qref, basis_gold["basis_P4_Q4_lobatto_qref"])
    assert np.array_equal(qw, basis_gold["basis_P4_Q4_lobatto_qweight"])
    assert np.allclose(interp.ravel(), basis_gold["basis_P4_Q4_lobatto_interp"], atol=1e-15)
    assert np.allclose(grad.ravel(), basis_gold["basis_P4_Q4_lobatto_grad"], atol=1e-13)


@pytest.mark.parametrize("mode", ["interp", "grad"])
def test_basis_apply_matches_reference(basis_gold, mode):
    P, Q, nc = 4, 5, 2
    interp, grad, qref, qw = orc.lagrange_1d(P, Q)
    em = orc.EVAL_INTERP if mode == "interp" else orc.EVAL_GRAD
    u = orc.fill_uniform(100 + (mode == "grad"), P ** 3 * nc)
    ut = orc.fill_uniform(200 + (mode == "grad"), Q ** 3 * nc * (3 if mode == "grad" else 1))
    assert np.array_equal(u, basis_gold[f"bapply_{mode}_u"])
    v = orc.basis_apply(3, P, Q, nc, interp, grad, qw, 1, orc.NOTRANSPOSE, em, u)
    vt = orc.basis_apply(3, P, Q, nc, interp, grad, qw, 1, orc.TRANSPOSE, em, ut)
    assert relinf(v, basis_gold[f"bapply_{mode}_v"]) < 1e-13
    assert relinf(vt, basis_gold[f"bapply_{mode}_vt"]) < 1e-13
    w = orc.basis_apply(3, P, Q, 1, interp, grad, qw, 1, orc.NOTRANSPOSE, orc.EVAL_WEIGHT, None)
    assert np.array_equal(w, basis_gold["bapply_weight"])


@pytest.mark.parametrize("case", CASES)
def test_operator_matches_reference(case):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    pb = _problem(case)
    # Inputs regenerate bit-for-bit.
    assert _sha(pb.coords) == str(g["sha_coords"])
    assert _sha(pb.offsets) == str(g["sha_offsets"])
    assert _sha(pb.u) == str(g["sha_u"])
    # Geometric factors from the gallery build QFunction: same arithmetic in the same order, bitwise equal.
    assert np.array_equal(pb.qdata, g["qdata"])
    # Operator apply: the reference's operations in the reference's order, bitwise equal (the bar is 1e-12 relative).
    if "kappa" in g:
        pb.kappa = g["kappa"]
    v = pb.apply()
    assert np.array_equal(v, g["v"])
    if "egather" in g:
        e = orc.rstr_gather(pb.offsets, pb.P ** 3, pb.ncomp, pb.comp_stride, pb.u)
        assert np.array_equal(e, g["egather"])  # gathers are bit-exact
        l = orc.rstr_scatter_add(pb.offsets, pb.P ** 3, pb.ncomp, pb.comp_stride, e, np.zeros(pb.l_size))
        assert np.array_equal(l, g["escatter"])  # element-order scatter: bit-exact
    if "kgrad" in g:
        # kappa = exp(g) is stored: libm exp may differ in the last bit across hosts.
        assert np.max(np.abs(pb.kappa - g["kappa"])) < 1e-15 * np.max(g["kappa"])
        pb.kappa = g["kappa"]
        assert relinf(pb.apply(), g["v"]) < 1e-12
        f = orc.fill_uniform(4003 + 3, pb.l_size)
        assert _sha(f) == str(g["sha_f"])
        w = pb.apply() - f
        kg = orc.kappa_grad(pb.P, pb.Q, pb.offsets, pb.l_size, pb.interp, pb.grad, pb.qdata, pb.u, w)
        assert relinf(kg, g["kgrad"]) < 1e-12


@pytest.mark.parametrize("case", CASES)
def test_blocked_port_matches_reference_blocked(case):
    """The CPU baseline (the /cpu/self/opt/blocked restatement) against the reference's own opt/blocked backend on the
    same inputs: bitwise equal; and within rounding of the serial form (only the scatter's order of additions within a
    block of eight elements differs)."""
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    gb = np.load(os.path.join(GOLDEN, "blocked.npz"))
    pb = _problem(case)
    if "kappa" in g:
        pb.kappa = g["kappa"]
    vb = pb.apply(blocked=True)
    assert np.array_equal(vb, gb[case])
    assert relinf(vb, pb.apply()) < 1e-14


def test_poisson_constant_nullspace():
    """A 1 = 0 for the diffusion operator (the reference's t522 check), on the oracle."""
    pb = orc.BoxProblem(3, 4, poisson=True, seed=7)
    v = pb.apply(np.ones(pb.l_size))
    assert np.max(np.abs(v)) < 1e-13


@pytest.mark.parametrize("n,p", [(3, 1), (3, 3), (2, 5), (4, 2)])
def test_volume_known_answer(n, p):
    """1^T M 1 is the volume of the domain (examples/ceed/ex1-volume.c:262-272; exact volume 1 for the unit box, whose
    boundary vertices are never perturbed).  Gauss points Q = P + 1 integrate the trilinear map's det J exactly, so
    the bound is rounding, far inside ex1's 1e-5."""
    pb = orc.BoxProblem(n, p, poisson=False, noise=0.1, seed=70 + p)
    assert abs(pb.apply(np.ones(pb.l_size)).sum() - 1.0) < 1e-13


def test_surface_known_answer():
    """sum |A (x + y + z)| is the surface area (examples/ceed/ex2-surface.c:248-290), 6 for the unit box, within
    ex2's 3D tolerance of 1e-1; edge nodes between faces of opposite normal sign cancel, so the gap shrinks with h."""
    box = mesh.Box(8, 4, noise=0.05, seed=71)
    pb = orc.BoxProblem(8, 4, poisson=True, noise=0.05, seed=71)
    v = pb.apply(box.node_coords().sum(axis=1))
    assert abs(np.abs(v).sum() - 6.0) < 1e-1


@pytest.mark.parametrize("n,p", [(3, 1), (3, 3), (2, 5)])
def test_linear_fields_energy_identity(n, p):
    """For fields linear in physical space (exactly representable on the trilinear mesh), a^T A b = grad a . grad b
    times the volume: (x+y+z)^T A (x+y+z) = 3, x^T A y = 0.  Exact up to rounding, so it pins the node coordinates
    and the Poisson qdata together."""
    box = mesh.Box(n, p, noise=0.05, seed=72)
    pb = orc.BoxProblem(n, p, poisson=True, noise=0.05, seed=72)
    xyz = box.node_coords()
    s = xyz.sum(axis=1)
    assert abs(s @ pb.apply(s) - 3.0) < 1e-12
    assert abs(xyz[:, 0] @ pb.apply(xyz[:, 1])) < 1e-12


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("P", [2, 4, 6, 9])
def test_basis_grad_adjoint(dim, P):
    """<G^T 1, u> = sum(G u), the reference's tests/t314-basis.c identity (its FP64 tolerance 1e-10), on the oracle's
    tensor gradient with Gauss points Q = P + 1."""
    Q = P + 1
    interp, grad, _, qw = orc.lagrange_1d(P, Q)
    u = mesh.uniform(314 + P, P ** dim)
    gu = orc.basis_apply(dim, P, Q, 1, interp, grad, qw, 1, orc.NOTRANSPOSE, orc.EVAL_GRAD, u)
    gt1 = orc.basis_apply(dim, P, Q, 1, interp, grad, qw, 1, orc.TRANSPOSE, orc.EVAL_GRAD, np.ones(dim * Q ** dim))
    assert abs(gt1 @ u - gu.sum()) < 1e-10


@pytest.mark.parametrize("dim", [1, 3])
@pytest.mark.parametrize("P", [2, 3, 5, 8])
def test_basis_interp_polynomial_exact(dim, P):
    """Interpolating a polynomial of degree P - 1 per direction from the Gauss-Lobatto nodes to the Gauss points is
    exact (the reference's tests/t311-basis.c, 1D, 100 machine epsilons; 1e-13 here, which also covers 3D)."""
    from libceed_gb300 import basis1d

    Q = P + 1
    interp, grad, qref, qw = orc.lagrange_1d(P, Q)
    nodes, _ = basis1d.lobatto_quadrature(P)
    c = mesh.uniform(311 + P, dim * P)

    def poly(x, d):  # sum_k c[d, k] x^k, degree P - 1
        return sum(c[d * P + k] * x ** k for k in range(P))

    def tensor(points):  # values at the tensor grid of `points`, x fastest
        vals = np.ones(1)
        for d in range(dim):
            vals = np.multiply.outer(poly(points, d), vals) if d else poly(points, 0)
        return np.asarray(vals).reshape(-1)

    got = orc.basis_apply(dim, P, Q, 1, interp, grad, qw, 1, orc.NOTRANSPOSE, orc.EVAL_INTERP, tensor(nodes))
    assert np.max(np.abs(got - tensor(qref))) < 1e-13
