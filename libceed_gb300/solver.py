"""Conjugate-gradient solves on fused operators (C ABI b200_cg_solve).

FP64 CG, or FP32 CG inside FP64 iterative refinement (defect correction), with homogeneous Dirichlet
conditions through a mask; iteration blocks run as CUDA graphs.  There is no solver in libCEED itself:
the reference benchmarks CG through PETSc KSPCG around CeedOperatorApply (examples/petsc/bps.c).
"""
import ctypes

from ._ffi import CGOpts, CGStats, call
from .ceed import F32, F64


def cg_solve(ceed, op, qdata64, mask, b, x, mixed=False, op32=None, qdata32=None, rtol=1e-10, inner_rtol=1e-4, max_it=20000,
             max_outer=30, use_graph=True, check_every=25):
    """Solve m A(m x) = m b from x = 0; returns a dict of iteration counts, final FP64 residual and device seconds."""
    o = CGOpts(rtol, max_it, 1 if mixed else 0, inner_rtol, max_outer, 1 if use_graph else 0, check_every)
    s = CGStats()
    f64 = op.fused(F64)
    f32 = op32.fused(F32).h if mixed else None
    call("b200_cg_solve", ceed._ctx, f64.h, f32, qdata64.ptr(), qdata32.ptr() if mixed else None, mask.ptr(), b.ptr(), x.ptr(),
         b.size, ctypes.byref(o), ctypes.byref(s))
    return dict(iterations=s.iterations, outer=s.outer, converged=bool(s.converged), rel_residual=s.rel_residual,
                seconds=s.seconds, launches=s.launches)
