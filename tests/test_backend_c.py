"""The libCEED C backend `/gpu/cuda/b200` compiles against the reference headers, links into a libCEED build, and
CeedInit("/gpu/cuda/b200") reaches its init through CeedRegister.  Needs the reference sources (skipped otherwise);
on a host without a GPU the init must fail loudly with the CUDA error, never fall back."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_backend_builds_and_registers():
    import torch

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    from libceed_gb300 import build

    build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "libceed_gb300", "backend"), f"REF={REF}"], check=True)
    exe = os.path.join(ROOT, "libceed_gb300", "backend", "_build", "t-b200-poisson")
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, CEED_ERROR_HANDLER="exit"))
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode != 0
        assert "CeedInit_B200" in r.stdout + r.stderr and "b200_ctx_create" in r.stdout + r.stderr
