"""ctypes binding of libceed_b200.so, generated from the declarations in include/ceed-b200.h.

The library is the only compute path: if it is missing or cannot load, every call raises
`B200Error`; nothing falls back to the CPU.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "ceed-b200.h")
LIB_PATH = os.path.join(HERE, "lib", "libceed_b200.so")


class B200Error(RuntimeError):
    """A libceed_b200 call returned a nonzero status (CeedErrorType)."""

    def __init__(self, func, code, message):
        super().__init__(f"{func} failed with status {code}: {message}")
        self.func, self.code, self.message = func, code, message


class OpDesc(ctypes.Structure):
    """b200_op_desc (include/ceed-b200.h)."""

    _fields_ = [
        ("qf", ctypes.c_int), ("prec", ctypes.c_int), ("P_1d", ctypes.c_int), ("Q_1d", ctypes.c_int),
        ("num_comp", ctypes.c_int), ("scatter", ctypes.c_int), ("num_elem", ctypes.c_int64), ("l_size", ctypes.c_int64),
        ("comp_stride", ctypes.c_int64), ("offsets", ctypes.c_void_p), ("interp_1d", ctypes.c_void_p),
        ("grad_1d", ctypes.c_void_p), ("elems_per_block", ctypes.c_int), ("staging", ctypes.c_int),
    ]


class CGOpts(ctypes.Structure):
    """b200_cg_opts (include/ceed-b200.h)."""

    _fields_ = [
        ("rtol", ctypes.c_double), ("max_it", ctypes.c_int), ("mixed", ctypes.c_int), ("inner_rtol", ctypes.c_double),
        ("max_outer", ctypes.c_int), ("use_graph", ctypes.c_int), ("check_every", ctypes.c_int), ("jacobi", ctypes.c_void_p),
        ("separate_pdot", ctypes.c_int),
    ]


class CGStats(ctypes.Structure):
    """b200_cg_stats (include/ceed-b200.h)."""

    _fields_ = [
        ("iterations", ctypes.c_int), ("outer", ctypes.c_int), ("converged", ctypes.c_int), ("rel_residual", ctypes.c_double),
        ("seconds", ctypes.c_double), ("launches", ctypes.c_int64),
    ]


class JitQFunction(ctypes.Structure):
    """b200_jit_qfunction (include/ceed-b200.h)."""

    _fields_ = [
        ("source_path", ctypes.c_char_p), ("name", ctypes.c_char_p), ("num_inputs", ctypes.c_int),
        ("input_size", ctypes.c_int * 8), ("active_input", ctypes.c_int), ("eval_in", ctypes.c_int), ("eval_out", ctypes.c_int),
        ("include_dirs", ctypes.c_char_p),
    ]


_STRUCTS = {"b200_op_desc": OpDesc, "b200_cg_opts": CGOpts, "b200_cg_stats": CGStats, "b200_jit_qfunction": JitQFunction}
_SCALARS = {
    "int": ctypes.c_int, "int64_t": ctypes.c_int64, "size_t": ctypes.c_size_t, "double": ctypes.c_double,
    "int32_t": ctypes.c_int32,
}


def _ctype(decl):
    """ctypes type of one parameter declaration such as `const int64_t strides[3]` or `b200_ctx *ctx`."""
    decl = decl.strip()
    pointer = "*" in decl or "[" in decl
    words = [w for w in re.findall(r"[A-Za-z_]\w*", decl) if w not in ("const", "struct")]
    base = words[0] if words else "void"
    if pointer:
        if base in _STRUCTS:
            return ctypes.POINTER(_STRUCTS[base])
        return ctypes.c_void_p
    if base in ("b200_ctx", "b200_basis", "b200_plan", "b200_op", "b200_cg"):
        return ctypes.c_void_p
    return _SCALARS[base]


def declarations():
    """(name, restype, [argtypes]) for every function declared in include/ceed-b200.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = []
    for m in re.finditer(r"^\s*(int|const char \*)\s*(b200_\w+)\s*\(([^)]*)\)\s*;", text, flags=re.M):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        argtypes = [] if args.strip() in ("", "void") else [_ctype(a) for a in args.split(",")]
        out.append((name, ctypes.c_char_p if "char" in ret else ctypes.c_int, argtypes))
    return out


_lib = None
_load_error = None


def load():
    """Load the library (once) and attach argtypes; raises B200Error when it is missing."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise B200Error("load", -1, f"{LIB_PATH} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError as exc:  # pragma: no cover - depends on the host
        _load_error = str(exc)
        raise B200Error("load", -1, _load_error) from exc
    for name, restype, argtypes in declarations():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _lib = lib
    return lib


def call(name, *args):
    """Call a status-returning entry point and raise B200Error on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.b200_last_error()
        raise B200Error(name, rc, msg.decode() if msg else "")
    return rc
