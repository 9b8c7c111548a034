"""Autotuner of the fused operator's launch shape.

For each (dim, P, Q, components, precision, QFunction, scatter) it sweeps the elements per block
(1 up to what threads and shared memory allow), the thread-to-element mapping (Q^2-thread line slabs or
Q^3-thread points) and, for the line mapping, the qdata staging (registers, shared memory, pipelined,
bulk copy, persistent bulk copy one batch ahead (FP32), or none: qdata read in the pointwise stage),
times each candidate on the device (b200_op_time: CUDA events over repeated applies on the real
problem), keeps the fastest, and records it in a JSON cache (CEED_B200_TUNE_CACHE, default
~/.cache/libceed_b200/tune.json) so later operators with the same key start from the tuned tile.
The reference instead sizes blocks by an occupancy-and-waste heuristic
(backends/cuda-gen/ceed-cuda-gen-operator.c:40-97).
"""
import ctypes
import json
import os

from ._ffi import call
from .ceed import F32, F64, F64X, QF_POISSON_KAPPA

STAGE_NAMES = {1: "registers", 2: "shared", 3: "pipelined", 4: "point3d", 5: "bulkcopy", 6: "late", 7: "persistent"}
STAGE_CODES = {v: k for k, v in STAGE_NAMES.items()}


def cache_path():
    return os.environ.get("CEED_B200_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "libceed_b200", "tune.json"))


def _key(op, prec):
    f = op._active_input()
    b, r = f.basis, f.rstr
    pname = {F64: "f64", F32: "f32", F64X: "f64x"}[prec]
    return f"dim{b.dim}_P{b.P1d}_Q{b.Q1d}_nc{r.ncomp}_{pname}_{op.qf.name}_{'det' if op.ceed.deterministic else 'atomic'}"


def load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache):
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(op, u, v, reps=5, candidates=None, use_cache=True, log=None):
    """Sweep the launch shape of `op` on vectors u, v; set and return the best {epb, staging, ms, key, sweep}."""
    prec = op._kernel_prec(u.prec)
    fused = op.fused(prec)
    key = _key(op, prec)
    cache = load_cache() if use_cache else {}
    qd = op._passive("qdata", u.prec)
    kap = op._passive("kappa", u.prec) if op.qf.kind == QF_POISSON_KAPPA else None
    sweep = []
    for stage in (1, 2, 3, 4, 5, 6, 7):
        m = ctypes.c_int()
        call("b200_op_tile_limits", fused.h, stage, ctypes.byref(m))
        epbs = candidates or sorted({e for e in (1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 14, 16, 20, 24, 28, 32) if e <= m.value})
        for epb in epbs:
            if epb > m.value:
                continue
            fused.set_tile(epb, stage)
            ms = ctypes.c_double()
            call("b200_op_time", fused.h, u.ptr(), v.ptr(), qd.ptr(), kap.ptr() if kap else None, reps, ctypes.byref(ms))
            sweep.append({"epb": epb, "staging": STAGE_NAMES[stage], "ms": round(ms.value, 5)})
            if log:
                log(f"{key} epb={epb} staging={STAGE_NAMES[stage]} {ms.value:.4f} ms")
    best = min(sweep, key=lambda r: r["ms"])
    stage = STAGE_CODES[best["staging"]]
    fused.set_tile(best["epb"], stage)
    op.elems_per_block, op.staging = best["epb"], stage
    op._fused[(prec, op.ceed.deterministic, best["epb"], stage)] = fused
    result = {"key": key, "epb": best["epb"], "staging": best["staging"], "ms": best["ms"], "sweep": sweep}
    if use_cache:
        cache[key] = {"epb": best["epb"], "staging": best["staging"], "ms": best["ms"]}
        save_cache(cache)
    return result


def apply_cached(op, prec=F64):
    """Set `op` to its cached tile, if the cache has its key; returns the entry or None."""
    entry = load_cache().get(_key(op, prec))
    if entry:
        op.elems_per_block = entry["epb"]
        op.staging = STAGE_CODES[entry["staging"]]
    return entry


# Box sizes of the per-degree workload (~16-18 M DoF for scalar fields).
BOX_N = {1: 256, 2: 128, 3: 85, 4: 64, 5: 52, 6: 43, 7: 37, 8: 32}


def sweep_main(argv=None):
    """Tile sweep of the scalar Poisson and mass operators over degrees and kernel families; one JSON line per
    (degree, QFunction, family) with the best tile and the best rate of every staging.  Needs a GPU.

        python -m libceed_gb300.tune --degrees 1,2,3,4,5,6,7,8 [--families f64,f32,f64x] [--qfunctions Poisson3DApply,MassApply]
    """
    import argparse

    import torch

    from . import mesh
    from .ceed import Ceed
    from .smoke_case import build_poisson

    ap = argparse.ArgumentParser()
    ap.add_argument("--degrees", default="1,2,3,4,5,6,7,8")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--families", default="f64,f32,f64x", help="comma-separated subset of f64, f32, f64x")
    ap.add_argument("--qfunctions", default="Poisson3DApply,MassApply")
    a = ap.parse_args(argv)
    families = a.families.split(",")
    ceed = Ceed("/gpu/cuda/b200")
    for p in [int(x) for x in a.degrees.split(",")]:
        box = mesh.Box(BOX_N[p], p, noise=0.05, seed=5)
        for qf in a.qfunctions.split(","):
            for tag, dt, arith in (("f64", torch.float64, "native"), ("f32", torch.float32, "native"), ("f64x", torch.float64, "float-float")):
                if tag not in families:
                    continue
                objs = build_poisson(ceed, box, dtype=dt, qf_name=qf)
                op = objs["op"]
                op.arithmetic = arith
                u = ceed.Vector(box.l_size, dt)
                u.set_array(box.u())
                v = ceed.Vector(box.l_size, dt)
                r = autotune(op, u, v, reps=a.reps, use_cache=False)
                by = {}
                for x in r["sweep"]:
                    if x["staging"] not in by or x["ms"] < by[x["staging"]]["ms"]:
                        by[x["staging"]] = x
                print(json.dumps(dict(degree=p, qfunction=qf, family=tag, dof=box.l_size,
                                      best=dict(epb=r["epb"], staging=r["staging"], gdofs=round(box.l_size / r["ms"] / 1e6, 3)),
                                      per_staging={k: [x["epb"], round(box.l_size / x["ms"] / 1e6, 3)] for k, x in by.items()},
                                      status=ceed.status())), flush=True)
                del objs, op, u, v
                torch.cuda.empty_cache()


if __name__ == "__main__":
    sweep_main()
