"""The C ABI library loads on a host without a GPU and exports every entry point include/ceed-b200.h declares."""
import ctypes
import os
import re

import pytest

from libceed_gb300 import _ffi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", h)).read(), flags=re.S)
            names |= set(re.findall(r"^\s*(?:int|const char \*)\s*(b200_\w+)\s*\(", text, flags=re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_ffi.LIB_PATH):
        from libceed_gb300 import build

        build.build()
    return _ffi.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_parser_sees_every_declaration():
    assert {d[0] for d in _ffi.declarations()} == _declared()


def test_calls_fail_loudly_without_a_device(lib):
    """With no GPU the context cannot be created; the call reports an error instead of falling back."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    with pytest.raises(_ffi.B200Error):
        _ffi.call("b200_ctx_create", 0, ctypes.byref(h))


def test_ceed_refuses_without_gpu():
    import torch

    import libceed_gb300 as ceed

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(ceed.B200Error):
        ceed.Ceed("/gpu/cuda/b200")
    with pytest.raises(ceed.B200Error):
        ceed.Ceed("/cpu/self/ref/serial")


def test_flops_estimate_matches_reference_model():
    """b200_flops_estimate restates CeedOperatorGetFlopsEstimate; the golden fixtures hold the reference's values."""
    import ctypes

    import numpy as np

    from libceed_gb300._ffi import call
    from tests.conftest import GOLDEN
    from tests.gpu_cases import CASES, parse

    from libceed_gb300 import ceed as lcc

    qf_of = {"mass": lcc.QF_MASS, "poisson": lcc.QF_POISSON, "vmass": lcc.QF_VECMASS, "vpoisson": lcc.QF_VECPOISSON}
    checked = 0
    for case in CASES:
        g = np.load(f"{GOLDEN}/{case}.npz")
        if "flops" not in g.files:
            continue
        kind, box = parse(case)
        out = ctypes.c_int64()
        call("b200_flops_estimate", qf_of[kind], box.P, box.Q, box.ncomp, box.num_elem, ctypes.byref(out))
        assert out.value == int(g["flops"][0]), case
        checked += 1
    assert checked >= 10


def test_struct_mirrors_match_the_header(tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's field offsets and sizes."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "ceed-b200.h"', "int main(void) {"]
    want = {}
    for cname, py in _ffi._STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        want[(cname, "sizeof")] = ctypes.sizeof(py)
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
            want[(cname, fname)] = getattr(py, fname).offset
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    assert got == want


@pytest.mark.parametrize("name", ["b200_vec_set_value_strided", "b200_vec_copy_strided"])
def test_strided_range_checks_on_the_host(lib, name):
    """The strided entry points check the range as CeedVectorSetValueStrided / CopyStrided do
    (interface/ceed-vector.c:300-325, :412-425) before touching the context or a device pointer, so a null context
    serves here: bad ranges give B200_ERROR_ACCESS (5), an empty range succeeds without a launch."""
    fn = getattr(lib, name)
    tail = (None, 1.0) if name == "b200_vec_set_value_strided" else (None, None)
    n = 100
    for start, stop, step in [(0, n + 1, 1), (0, -2, 1), (-1, -1, 1), (10, 5, 1), (0, -1, 0), (0, -1, -4)]:
        assert fn(None, 0, n, start, stop, step, *tail) == 5, (start, stop, step)
        assert "must be" in lib.b200_last_error().decode()
    assert fn(None, 0, -1, 0, -1, 1, *tail) == 2  # negative length: B200_ERROR_DIMENSION
    for start, stop in [(7, 7), (n, -1), (0, 0)]:
        assert fn(None, 0, n, start, stop, 3, *tail) == 0
