"""In-tree build of libstrouhal_gb300.so for sm_103a (nvcc, no cmake).

Every translation unit is compiled in parallel, then linked into
strouhal_gb300/_lib/libstrouhal_gb300.so. The kernels are compiled with
-fmad=false: the step's arithmetic contract is that no multiply-add is fused
except the one the reference writes explicitly (Kernels.metal:181).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIBNAME = "libstrouhal_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, object name, extra flags). The step and row-staged kernels are
# compiled once per arithmetic: the reference's expressions as written
# (STRO_ARITH=0) and the fused-multiply-add collision (STRO_ARITH=1).
SOURCES = [
    ("lbm_step.cu", "lbm_step.o", ["-DSTRO_ARITH=0"]),
    ("lbm_step.cu", "lbm_step_fused.o", ["-DSTRO_ARITH=1"]),
    ("lbm_rows.cu", "lbm_rows.o", ["-DSTRO_ARITH=0"]),
    ("lbm_rows.cu", "lbm_rows_fused.o", ["-DSTRO_ARITH=1"]),
    ("lbm_pair.cu", "lbm_pair.o", ["-DSTRO_ARITH=0"]),
    ("lbm_pair.cu", "lbm_pair_fused.o", ["-DSTRO_ARITH=1"]),
    ("lbm_probe.cu", "lbm_probe.o", []),
    ("lbm_batch.cu", "lbm_batch.o", []),
    ("lbm_adjoint.cu", "lbm_adjoint.o", []),
    ("runtime.cu", "runtime.o", []),
    ("batch.cu", "batch.o", []),
    ("adjoint.cu", "adjoint.o", []),
    ("voxel.cu", "voxel.o", []),
    ("sha256.cpp", "sha256.o", []),
    ("uq.cpp", "uq.o", []),
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _flags(verbose_ptxas=False):
    # -ffp-contract=off for the host compiler as well: host-side arithmetic
    # (statistics, mesh generation) must not depend on the host's FMA choices
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _headers():
    return [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))] + [
        os.path.join(INCLUDE, "strouhal_c.h")]


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(entry, verbose_ptxas):
    src, objname, extra = entry
    obj = os.path.join(BUILD, objname)
    deps = [src, __file__] + _headers()
    if not verbose_ptxas and not _stale(obj, deps):
        return obj, ""
    cmd = [nvcc()] + _flags(verbose_ptxas) + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose_ptxas=False, jobs=None):
    """Compile and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [(os.path.join(CSRC, s), o, x) for s, o, x in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=jobs or len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs = [o for o, _ in results]
    out = lib_path()
    if verbose_ptxas:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if _stale(out, objs):
        tmp = out + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
