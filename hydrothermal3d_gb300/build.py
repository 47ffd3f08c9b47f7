"""Build libht3d.so (sm_103a) in-tree with nvcc.

Every translation unit under ``csrc/`` is compiled in parallel for one
architecture (``-gencode arch=compute_103a,code=sm_103a``) and linked into
``hydrothermal3d_gb300/libht3d.so``.  The granular, reference-shaped kernels
and the plain FP64 fused paths are compiled with ``-fmad=false`` so their
FP64 rounding follows the reference's statement order exactly (Julia does not
contract a*b+c); the mixed-precision paths keep FMA contraction.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libht3d.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FP contraction either (aarch64 g++ would fuse a*b+c by default,
# changing the DYREL parameters h1/h2 in the last bit)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3", "-Xcompiler",
          "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", INCLUDE]
# translation units that restate reference kernels statement by statement
NO_FMA = {"kernels_dimless.cu", "kernels_dim.cu", "dyrel_fp64.cu", "step.cu", "weno.cu", "noalloc.cu", "ensemble.cu",
          "postprocess.cu"}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(f) for f in files)


def _compile(nvcc, src, extra):
    obj = os.path.join(OBJ, src[:-3] + ".o")
    flags = list(COMMON) + list(extra)
    if src in NO_FMA:
        flags.append("-fmad=false")
    cmd = [nvcc, *ARCH, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile and link libht3d.so; returns its path."""
    if not force and not os.environ.get("HT3D_NVCC_FLAGS") and os.path.exists(LIB) and \
            os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    # HT3D_NVCC_FLAGS: extra nvcc flags for every translation unit (e.g. -D
    # switches for experiments or -G for debugging); a rebuild is forced
    env_flags = os.environ.get("HT3D_NVCC_FLAGS", "").split()
    if env_flags:
        extra += env_flags
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            print(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
