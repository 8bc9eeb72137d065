"""Build recipe for the CPU oracle — test infrastructure only.

Builds
  oracle/_build/liblbm_oracle.so   the scalar restatement (lbm_oracle.cpp),
                                   with OpenMP when the compiler has it;
  oracle/_ref/libref_metal.so      the reference's own Kernels.metal compiled
                                   as C++ through ref_shim/, only when the
                                   reference tree is present (it is read in
                                   place, never copied).

Both use -ffp-contract=off so that no multiply-add is fused behind the
source's back (g++ contracts by default on aarch64), and no fast-math. The
restatement is built at -O3 (its FP64 adjoint's dual-number lanes vectorise);
optimisation levels do not change IEEE results without fast-math.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-Wall"]
DEFAULT_REF = "/root/reference"


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs if os.path.exists(s))


def oracle_lib_path():
    return os.path.join(HERE, "_build", "liblbm_oracle.so")


def ref_lib_path():
    return os.path.join(HERE, "_ref", "libref_metal.so")


def build_oracle(force=False):
    src = os.path.join(HERE, "lbm_oracle.cpp")
    out = oracle_lib_path()
    if not force and _newer(out, [src, __file__]):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["g++"] + CXXFLAGS + ["-O3", "-fopenmp", "-o", out, src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:  # no libgomp: build single-threaded
        cmd = ["g++"] + CXXFLAGS + ["-O3", "-Wno-unknown-pragmas", "-o", out, src]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
    return out


def build_ref(ref_root=None, force=False):
    """Compile the reference kernel source as C++; returns None when absent."""
    ref_root = ref_root or os.environ.get("STRO_REFERENCE_ROOT", DEFAULT_REF)
    metal = os.path.join(ref_root, "Sources", "StrouhalCore", "Kernels.metal")
    if not os.path.exists(metal):
        return None
    drv = os.path.join(HERE, "ref_metal_driver.cpp")
    shim = os.path.join(HERE, "ref_shim", "metal_stdlib")
    out = ref_lib_path()
    if not force and _newer(out, [drv, shim, metal, __file__]):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = (["g++"] + CXXFLAGS + ["-Wno-attributes", "-I", os.path.join(HERE, "ref_shim"),
                                 "-I", os.path.dirname(metal), "-o", out, drv])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shim build failed:\n" + r.stderr)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
