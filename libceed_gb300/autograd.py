"""torch.autograd binding of the variable-coefficient diffusion operator y = A(kappa) u.

A(kappa) = sum_e E^T G^T diag(kappa) D G E: the Poisson operator with the geometric factors D scaled by a
per-quadrature-point coefficient kappa (the "Poisson3DApplyKappa" pointwise kernel).  The backward pass is
hand-written: A is symmetric, so dL/du = A(kappa) (dL/dy) is one more fused apply; dL/dkappa at each quadrature
point is grad(w) . D grad(u) with w = dL/dy, computed by one fused kernel that recomputes both gradients from the
L-vectors (no E-vector or quadrature data is stored by the forward pass).
"""
import torch

from . import mesh
from .ceed import F32, F64, USE_POINTER
from .smoke_case import build_poisson


class KappaDiffusion:
    """y = A(kappa) u on a box mesh; u, kappa and y are CUDA tensors (float64 or float32)."""

    def __init__(self, ceed, box, dtype=torch.float64):
        self.ceed, self.box, self.dtype = ceed, box, dtype
        objs = build_poisson(ceed, box, dtype=dtype, qf_name="Poisson3DApplyKappa")
        self.op, self.qdata, self.rq = objs["op"], objs["qdata"], objs["rq"]
        self._objs = objs
        self.n_q = box.num_elem * box.Q ** 3
        self._kappa = ceed.Vector(self.n_q, dtype)
        self.op.set_field("kappa", self.rq, None, self._kappa)
        self._u = ceed.Vector(box.l_size, dtype)
        self._w = ceed.Vector(box.l_size, dtype)
        self._y = ceed.Vector(box.l_size, dtype)
        self._g = ceed.Vector(self.n_q, dtype)
        self.prec = F64 if dtype == torch.float64 else F32

    def _bind(self, vec, t):
        vec.set_array(t.detach().contiguous(), cmode=USE_POINTER)

    def apply(self, u, kappa):
        self._bind(self._u, u)
        self._bind(self._kappa, kappa)
        y = torch.empty_like(u)
        self._bind(self._y, y)
        self.op.apply(self._u, self._y)
        return y

    def kappa_grad(self, u, w, kappa):
        self._bind(self._u, u)
        self._bind(self._w, w)
        self._bind(self._kappa, kappa)
        g = torch.empty_like(kappa)
        self._bind(self._g, g)
        self.op.kappa_grad(self._u, self._w, self._g)
        return g


class KappaDiffusionFunction(torch.autograd.Function):
    """autograd.Function for y = A(kappa) u with the hand-written adjoint described in the module docstring."""

    @staticmethod
    def forward(ctx, u, kappa, dop):
        ctx.dop = dop
        ctx.save_for_backward(u, kappa)
        return dop.apply(u, kappa)

    @staticmethod
    def backward(ctx, gy):
        u, kappa = ctx.saved_tensors
        dop = ctx.dop
        gy = gy.contiguous()
        gu = dop.apply(gy, kappa) if ctx.needs_input_grad[0] else None
        gk = dop.kappa_grad(u, gy, kappa) if ctx.needs_input_grad[1] else None
        return gu, gk, None


def kappa_diffusion(u, kappa, dop):
    """y = A(kappa) u, differentiable in u and kappa."""
    return KappaDiffusionFunction.apply(u, kappa, dop)


def gaussian_field_kappa(box, seed, modes=64, sigma=0.5):
    """kappa = exp(g) at every quadrature point, g a sum of `modes` seeded Fourier modes with standard deviation
    sigma, evaluated at the reference positions of the Gauss points.  Layout [elem][qpt] (float64 numpy)."""
    import numpy as np

    from .basis1d import gauss_quadrature

    qx, _ = gauss_quadrature(box.Q)
    n = box.n
    # Gauss point positions in [0,1] along one axis, per element: (e + (q+1)/2) / n
    e = np.arange(n)[:, None]
    pos = ((e + 0.5 * (qx[None, :] + 1.0)) / n).reshape(-1)  # index e*Q + q
    r = mesh.uniform(seed, 5 * modes, 0.0, 1.0)
    amp = sigma * np.sqrt(2.0 / modes)
    ez, ey, ex = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    qz, qy, qx_ = np.meshgrid(np.arange(box.Q), np.arange(box.Q), np.arange(box.Q), indexing="ij")
    X = pos[(ex.reshape(-1, 1) * box.Q + qx_.reshape(1, -1))]
    Y = pos[(ey.reshape(-1, 1) * box.Q + qy.reshape(1, -1))]
    Z = pos[(ez.reshape(-1, 1) * box.Q + qz.reshape(1, -1))]
    g = np.zeros_like(X)
    for k in range(modes):
        kx, ky, kz = 1 + int(4 * r[5 * k]), 1 + int(4 * r[5 * k + 1]), 1 + int(4 * r[5 * k + 2])
        phase = 2 * np.pi * r[5 * k + 3]
        g += amp * np.cos(np.pi * (kx * X + ky * Y + kz * Z) + phase)
    return np.exp(g).reshape(-1)
