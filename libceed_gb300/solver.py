"""Conjugate-gradient solves on fused operators (C ABI b200_cg_solve).

FP64 CG, or FP32 CG inside FP64 iterative refinement (defect correction), with homogeneous Dirichlet
conditions through a mask; iteration blocks run as CUDA graphs.  There is no solver in libCEED itself:
the reference benchmarks CG through PETSc KSPCG around CeedOperatorApply (examples/petsc/bps.c).
"""
import ctypes

from ._ffi import CGOpts, CGStats, call
from .ceed import F32, F64


def cg_solve(ceed, op, qdata64, mask, b, x, mixed=False, op32=None, qdata32=None, rtol=1e-10, inner_rtol=1e-4, max_it=20000,
             max_outer=30, use_graph=True, check_every=25, jacobi=None, fused_pdot=True):
    """Solve m A(m x) = m b from x = 0; returns a dict of iteration counts, final FP64 residual and device seconds.
    jacobi: a Vector holding the masked inverse diagonal (see jacobi_preconditioner) for Jacobi-preconditioned CG.
    fused_pdot: in mixed mode, let a persistent FP32 operator sum p.(A p) during its apply (False: a separate pass)."""
    o = CGOpts(rtol, max_it, 1 if mixed else 0, inner_rtol, max_outer, 1 if use_graph else 0, check_every,
               jacobi.data.data_ptr() if jacobi is not None else None, 0 if fused_pdot else 1)
    s = CGStats()
    f64 = op.fused(op._kernel_prec(F64))  # F64X kernels when op.arithmetic == "float-float" (same double vectors)
    f32 = op32.fused(F32).h if mixed else None
    call("b200_cg_solve", ceed._ctx, f64.h, f32, qdata64.ptr(), qdata32.ptr() if mixed else None, mask.ptr(), b.ptr(), x.ptr(),
         b.size, ctypes.byref(o), ctypes.byref(s))
    return dict(iterations=s.iterations, outer=s.outer, converged=bool(s.converged), rel_residual=s.rel_residual,
                seconds=s.seconds, launches=s.launches)


def assemble_diagonal(ceed, op, diag):
    """CeedOperatorLinearAssembleDiagonal for a fused mass or diffusion operator: diag (FP64 Vector, L-vector size)."""
    import ctypes as ct

    from .ceed import QF_MASS, QF_POISSON, QF_POISSON_KAPPA, QF_VECMASS, QF_VECPOISSON

    f = op._active_input()
    r, b = f.rstr, f.basis
    kind = op.qf.kind
    if kind not in (QF_MASS, QF_POISSON, QF_POISSON_KAPPA, QF_VECMASS, QF_VECPOISSON):
        raise ValueError("diagonal assembly covers the mass and diffusion operators")
    poisson = kind in (QF_POISSON, QF_POISSON_KAPPA, QF_VECPOISSON)
    qd = op._passive("qdata", F64)
    kap = op._passive("kappa", F64) if kind == QF_POISSON_KAPPA else None
    plan = r.plan() if ceed.deterministic else None
    call("b200_assemble_diagonal", ceed._ctx, 1 if poisson else 0, b.P1d, b.Q1d, r.nelem, r.ncomp, r.compstride, r.lsize,
         b.interp1d.ctypes.data_as(ct.c_void_p), b.grad1d.ctypes.data_as(ct.c_void_p), ct.c_void_p(r.offsets.data_ptr()), qd.ptr(),
         kap.ptr() if kap is not None else None, diag.ptr(), plan)


def jacobi_preconditioner(ceed, op, mask):
    """Masked inverse diagonal m / diag(A) as a Vector, for cg_solve(jacobi=...)."""
    d = ceed.Vector(mask.size)
    assemble_diagonal(ceed, op, d)
    inv = ceed.Vector(mask.size)
    inv.data.copy_(mask.data / d.data.clamp_min(1e-300))
    return inv
