"""Regenerate the golden fixtures in this folder from the reference libCEED.

Builds the reference's interface, `/cpu/self/ref/serial` backend and gallery straight
from the reference sources (oracle/Makefile `ref` target, REF=<reference checkout>),
runs oracle/ref_harness.c through the public libCEED API, and packs the arrays into
small .npz files:

  basis.npz        1D tables (interp, grad, qref, qweight, collocated grad) for P=2..10, Q=P+1
                   Gauss, and P=Q=4 Gauss-Lobatto; standalone 3D basis applies (P=4, Q=5, 2 comps)
  blocked.npz      v = A u of every operator case on the reference's /cpu/self/opt/blocked backend
  <case>.npz       operator cases: qdata from the gallery build QFunction, v = A u, and for a few
                   cases the restriction gather/scatter; inputs are stored as SHA-256 digests
                   (tests regenerate them with the oracle's generators and check the digest)

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")

FULL_ARRAYS = {"mass_n8_p3", "vpoisson_n4_p2", "poisson_n3_p4", "kappa_n3_p3"}  # keep gather/scatter for these


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    subprocess.run(["make", "-s", "-C", ORACLE, "ref", f"REF={ref}"], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([os.path.join(ORACLE, "_ref", "ref_harness"), tmp], check=True)
        arrays = {}
        with open(os.path.join(tmp, "manifest.txt")) as f:
            for line in f:
                name, dtype, count = line.split()
                a = np.fromfile(os.path.join(tmp, name + ".bin"), dtype=np.float64 if dtype == "f64" else np.int32)
                assert a.size == int(count)
                arrays[name] = a
    basis = {k: v for k, v in arrays.items() if k.startswith("basis_") or k.startswith("bapply_")}
    np.savez_compressed(os.path.join(HERE, "basis.npz"), **basis)
    cases = sorted({k.rsplit("_", 1)[0] for k in arrays if k.endswith("_qdata")})
    for case in cases:
        out = {}
        for key in ("qdata", "v", "kgrad", "kappa", "flops"):
            if case + "_" + key in arrays:
                out[key] = arrays[case + "_" + key]
        if case in FULL_ARRAYS:
            out["egather"] = arrays[case + "_egather"]
            out["escatter"] = arrays[case + "_escatter"]
        for key in ("coords", "offsets", "u", "f"):
            if case + "_" + key in arrays:
                out["sha_" + key] = np.array(digest(arrays[case + "_" + key]))
        np.savez_compressed(os.path.join(HERE, case + ".npz"), **out)
    print("wrote", len(cases) + 1, "fixtures to", HERE)
    write_blocked()


def write_blocked():
    """blocked.npz: v = A u of every operator case on the reference's /cpu/self/opt/blocked backend (the CPU baseline's
    algorithm), from the same harness and inputs; needs the reference build of main()."""
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([os.path.join(ORACLE, "_ref", "ref_harness"), tmp, "/cpu/self/opt/blocked"], check=True)
        out = {}
        with open(os.path.join(tmp, "manifest.txt")) as f:
            for line in f:
                name, dtype, count = line.split()
                if name.endswith("_v") and not name.startswith("bapply_"):
                    out[name[:-2]] = np.fromfile(os.path.join(tmp, name + ".bin"), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "blocked.npz"), **out)
    print("wrote blocked.npz with", len(out), "cases")


if __name__ == "__main__":
    main()
