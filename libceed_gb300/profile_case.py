"""A small, self-contained fused-apply case for profilers (ncu) and quick timing.

    python -m libceed_gb300.profile_case --degree 4 --prec f64 --n 32 --reps 3 [--det] [--epb E --staging S] [--dot]

--prec f64x runs the float-float kernels on the same double vectors.

Builds the Poisson operator of an n^3 box (qdata of n=32 at degree 4: 340 MB in FP64, larger than L2), applies it
`reps` times and prints the mean device time.  The fused kernel is `k_op_apply`.
"""
import argparse

import torch

import libceed_gb300 as lc
from libceed_gb300 import mesh
from libceed_gb300.smoke_case import build_poisson


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--prec", choices=["f64", "f32", "f64x"], default="f64")
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--det", action="store_true")
    ap.add_argument("--mass", action="store_true")
    ap.add_argument("--ncomp", type=int, default=1)
    ap.add_argument("--epb", type=int, default=0)
    ap.add_argument("--staging", type=int, default=0)
    ap.add_argument("--cg", action="store_true", help="time the FP64 and FP32-refined CG solves of the box instead")
    ap.add_argument("--dot", action="store_true", help="time apply_dot (v = A u and u . A u, persistent FP32 kernel) instead")
    a = ap.parse_args()
    if a.cg:
        return cg_case(a)
    dt = torch.float32 if a.prec == "f32" else torch.float64
    ceed = lc.Ceed("/gpu/cuda/b200", deterministic=a.det)
    box = mesh.Box(a.n, a.degree, ncomp=a.ncomp, noise=0.05, seed=1)
    qf = ("Vector3MassApply" if a.ncomp == 3 else "MassApply") if a.mass else None
    objs = build_poisson(ceed, box, dtype=dt, qf_name=qf)
    op = objs["op"]
    op.elems_per_block, op.staging = a.epb, a.staging
    if a.prec == "f64x":
        op.arithmetic = "float-float"
    u = ceed.Vector(box.l_size, dt)
    u.set_array(box.u())
    v = ceed.Vector(box.l_size, dt)
    run = lambda: op.apply(u, v)  # noqa: E731
    if a.dot:
        import ctypes

        from libceed_gb300._ffi import call

        f32 = op.fused(lc.F32)
        nb, nd = ctypes.c_int(), ctypes.c_int64()
        call("b200_op_dot_len", f32.h, ctypes.byref(nb), ctypes.byref(nd))
        part = torch.empty(max(nd.value, 1), dtype=torch.float64, device=ceed.device)
        qd = objs["qdata"]
        run = lambda: call("b200_op_apply_dot", f32.h, u.ptr(), v.ptr(), qd.ptr(), ctypes.c_void_p(part.data_ptr()))  # noqa: E731
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.reps
    fused = op.fused({"f64": lc.F64, "f32": lc.F32, "f64x": lc.F64X}[a.prec])
    b, f = fused.cost()
    print(f"degree {a.degree} {a.prec} n={a.n}{' apply_dot' if a.dot else ''} dof={box.l_size} tile={fused.tile()} {ms:.4f} ms/apply "
          f"{box.l_size / ms / 1e6:.3f} GDoF/s {b / ms / 1e6:.1f} GB/s(alg) {f / ms / 1e9:.3f} TFLOP/s alg_bytes={b:.0f}")


def cg_case(a):
    """FP64 CG and FP32 CG with FP64 refinement on the n^3 Poisson box with Dirichlet faces (smooth x*, b = A x*),
    rtol 1e-10, graphs of 25 iterations: the solver kernels for a launch list."""
    from libceed_gb300.solver import cg_solve

    ceed = lc.Ceed("/gpu/cuda/b200", deterministic=a.det)
    box = mesh.Box(a.n, a.degree, noise=0.05, seed=3)
    o64 = build_poisson(ceed, box)
    o32 = build_poisson(ceed, box, dtype=torch.float32)
    m = mesh.box_mask(a.n, a.degree)
    mask, xv, b = ceed.Vector(box.l_size), ceed.Vector(box.l_size), ceed.Vector(box.l_size)
    mask.set_array(m)
    xv.set_array(mesh.smooth_field(a.n, a.degree, seed=7) * m)
    o64["op"].apply(xv, b)
    b.set_array(m * b.get_array_read())
    for mixed in (False, True):
        x = ceed.Vector(box.l_size)
        st = cg_solve(ceed, o64["op"], o64["qdata"], mask, b, x, mixed=mixed, op32=o32["op"], qdata32=o32["qdata"], rtol=1e-10,
                      use_graph=True, check_every=25)
        print(f"{'FP32+refinement' if mixed else 'FP64'} CG degree {a.degree} n={a.n} dof={box.l_size}: {st['iterations']} iterations, "
              f"{st['outer']} outer, {st['seconds'] * 1e3:.2f} ms, {st['seconds'] * 1e3 / max(st['iterations'], 1):.4f} ms/iteration, "
              f"rel. residual {st['rel_residual']:.2e}")


if __name__ == "__main__":
    main()
