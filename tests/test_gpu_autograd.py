"""torch.autograd binding of y = A(kappa) u: gradients against the reference-backend gradient (golden vectors),
against the oracle, and against central finite differences (h = 1e-6), all in FP64."""
import numpy as np
import pytest
import torch

import libceed_gb300 as lc
from libceed_gb300 import mesh
from libceed_gb300.autograd import KappaDiffusion, gaussian_field_kappa, kappa_diffusion
from oracle import oracle as orc
from tests.conftest import relinf
from tests.gpu_cases import golden, parse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    ceed = lc.Ceed("/gpu/cuda/b200")
    kind, box = parse("kappa_n3_p3")
    g = golden("kappa_n3_p3")
    dop = KappaDiffusion(ceed, box)
    return ceed, box, g, dop


def _loss(dop, u, kappa, f):
    y = kappa_diffusion(u, kappa, dop)
    return 0.5 * torch.sum((y - f) ** 2)


def test_gradients_match_reference(setup):
    ceed, box, g, dop = setup
    u = torch.tensor(box.u(), device="cuda", requires_grad=True)
    kappa = torch.tensor(g["kappa"], device="cuda", requires_grad=True)
    f = torch.tensor(mesh.uniform(4003 + 3, box.l_size), device="cuda")
    loss = _loss(dop, u, kappa, f)
    loss.backward()
    # dL/dkappa against the gradient assembled on the reference's /cpu/self/ref/serial backend.
    assert relinf(kappa.grad.cpu().numpy(), g["kgrad"]) < 1e-12
    # dL/du = A(kappa)^T (A(kappa) u - f) = A(kappa) w; check with the oracle.
    pb = orc.BoxProblem(box.n, box.degree, poisson=True, noise=0.05, seed=4003, kappa=True)
    pb.kappa = g["kappa"]
    w = pb.apply(box.u()) - f.cpu().numpy()
    assert relinf(u.grad.cpu().numpy(), pb.apply(w)) < 1e-12


def test_central_finite_differences(setup):
    ceed, box, g, dop = setup
    u0 = torch.tensor(box.u(), device="cuda")
    k0 = torch.tensor(g["kappa"], device="cuda")
    f = torch.tensor(mesh.uniform(17, box.l_size), device="cuda")
    u = u0.clone().requires_grad_(True)
    k = k0.clone().requires_grad_(True)
    _loss(dop, u, k, f).backward()
    h = 1e-6
    for seed in (1, 2):
        du = torch.tensor(mesh.uniform(100 + seed, box.l_size), device="cuda")
        dk = torch.tensor(mesh.uniform(200 + seed, k0.numel()), device="cuda")
        with torch.no_grad():
            fd_u = (_loss(dop, u0 + h * du, k0, f) - _loss(dop, u0 - h * du, k0, f)) / (2 * h)
            fd_k = (_loss(dop, u0, k0 + h * dk, f) - _loss(dop, u0, k0 - h * dk, f)) / (2 * h)
        an_u = torch.dot(u.grad, du)
        an_k = torch.dot(k.grad, dk)
        assert abs(fd_u.item() - an_u.item()) < 1e-6 * abs(an_u.item())
        assert abs(fd_k.item() - an_k.item()) < 1e-6 * abs(an_k.item())


def test_fp32_gradients_close_to_fp64():
    ceed = lc.Ceed("/gpu/cuda/b200")
    box = mesh.Box(4, 3, noise=0.05, seed=8)
    kap = gaussian_field_kappa(box, seed=3)
    assert np.all(kap > 0)
    grads = {}
    for dt in (torch.float64, torch.float32):
        dop = KappaDiffusion(ceed, box, dtype=dt)
        u = torch.tensor(box.u(), device="cuda", dtype=dt, requires_grad=True)
        k = torch.tensor(kap, device="cuda", dtype=dt, requires_grad=True)
        f = torch.tensor(mesh.uniform(9, box.l_size), device="cuda", dtype=dt)
        _loss(dop, u, k, f).backward()
        grads[dt] = (u.grad.double().cpu().numpy(), k.grad.double().cpu().numpy())
    assert relinf(grads[torch.float32][0], grads[torch.float64][0]) < 1e-4
    assert relinf(grads[torch.float32][1], grads[torch.float64][1]) < 1e-4
