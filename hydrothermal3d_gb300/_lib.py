"""ctypes binding of libht3d.so, generated from include/ht3d.h.

The header is the single source of truth: every ``ht3d_*`` prototype in it is
bound with matching argument and return types.  Loading fails loudly when the
CUDA library has not been built -- there is no CPU fallback.
"""
import ctypes
import os
import re

_PKG = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(_PKG), "include", "ht3d.h")
LIBPATH = os.path.join(_PKG, "libht3d.so")

_ARG_TYPES = {
    "int": ctypes.c_int,
    "long long": ctypes.c_longlong,
    "double": ctypes.c_double,
    "unsigned long long": ctypes.c_ulonglong,
}
_RET_TYPES = {
    "int": ctypes.c_int,
    "const char*": ctypes.c_char_p,
    "unsigned long long": ctypes.c_ulonglong,
    "double": ctypes.c_double,
}

_PROTO = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_ ]*?\**)\s*\b(ht3d_[A-Za-z0-9_]+)\s*\(([^;]*?)\)\s*;", re.M | re.S)


def _strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", " ", src)


def _ctype_of_param(p: str):
    p = " ".join(p.split())
    if p in ("void", ""):
        return None
    if "*" in p:
        return ctypes.c_void_p
    # drop the parameter name
    toks = p.split()
    base = " ".join(toks[:-1]) if len(toks) > 1 else toks[0]
    base = base.replace("const ", "")
    if base not in _ARG_TYPES:
        raise TypeError(f"unsupported parameter type in ht3d.h: {p!r}")
    return _ARG_TYPES[base]


def parse_header(path: str = HEADER):
    """Return {name: (restype, [argtypes])} for every prototype in ht3d.h."""
    with open(path) as f:
        src = _strip_comments(f.read())
    protos = {}
    for m in _PROTO.finditer(src):
        ret = " ".join(m.group(1).split()).replace(" *", "*")
        name = m.group(2)
        params = [q for q in (x.strip() for x in m.group(3).split(",")) if q]
        args = [t for t in (_ctype_of_param(q) for q in params) if t is not None]
        if ret not in _RET_TYPES:
            raise TypeError(f"unsupported return type {ret!r} for {name}")
        protos[name] = (_RET_TYPES[ret], args)
    return protos


_lib = None


def load():
    """Load libht3d.so and bind every header prototype (cached)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise ImportError(
            f"{LIBPATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA library is required; there is no CPU fallback)")
    lib = ctypes.CDLL(LIBPATH)
    for name, (res, args) in parse_header().items():
        fn = getattr(lib, name)  # AttributeError -> header/library mismatch
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
