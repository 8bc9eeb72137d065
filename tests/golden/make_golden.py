"""Generate tests/golden/reference_cases.npz from the reference's own kernels.

Runs the reference's unmodified Sources/StrouhalCore/Kernels.metal, compiled
as C++ through oracle/ref_shim (oracle/_ref/libref_metal.so), on small seeded
lattices that cover every feature of the step: periodic SRT/TRT, solid walls,
a ramped moving lid, parabolic and uniform inflow walls, the outlet sponge,
Noble-Torczynski cells, Smagorinsky LES, the uniform Guo force, the
momentum-exchange force probe, the moments probe and the field initialiser —
in FP32 and FP16 storage. Inputs and outputs are stored so that tests can
check the oracle and the GPU against the reference where the reference tree
is absent.

Usage (needs the reference tree; writes next to this file):
    python tests/golden/make_golden.py [/path/to/reference]
"""
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle, pyoracle as po  # noqa: E402

CASES = [
    # name, precision kind, dims, collision, features
    dict(name="periodic_trt_f32", kind=0, dims=(6, 5, 4), omega=1.6, omegaMinus=1.25, steps=5),
    dict(name="periodic_srt_f16_tgv", kind=1, dims=(8, 6, 4), omega=1.9, steps=6, init=(2, 0.05)),
    dict(name="cavity_lid_trt_f32", kind=0, dims=(8, 7, 3), omega=1.3, omegaMinus=1.05,
         lid=(0.1, 0.0, 0.0), ramp=4, walls="cavity", steps=6, probe=((1, 6), (1, 5))),
    dict(name="channel_all_f32", kind=0, dims=(12, 8, 3), omega=1.45, omegaMinus=1.2, uin=0.06,
         ramp=5, walls="channel", eps=True, sponge=(6.0, 4.0, 0.9), force=(2e-5, -1e-5, 5e-6),
         cSmago=0.01, steps=6, probe=((2, 9), (1, 6))),
    dict(name="channel_all_f16", kind=1, dims=(12, 8, 3), omega=1.45, omegaMinus=1.2, uin=0.06,
         ramp=5, walls="channel", eps=True, sponge=(6.0, 4.0, 0.9), force=(2e-5, -1e-5, 5e-6),
         cSmago=0.01, steps=6, probe=((2, 9), (1, 6))),
    dict(name="channel_uniform_srt_f32", kind=0, dims=(10, 6, 4), omega=1.7, uin=0.04,
         walls="channel", uniform=True, eps=True, steps=4, probe=((1, 8), (1, 4))),
]


def flags_for(case):
    nx, ny, nz = case["dims"]
    kind = case.get("walls")
    if kind is None:
        return None

    def fn(x, y, z):
        if kind == "cavity":
            if y == ny - 1:
                return po.LID
            if x == 0 or x == nx - 1 or y == 0:
                return po.SOLID
            return po.FLUID
        if y == 0 or y == ny - 1:
            return po.SOLID
        if x == 0 or x == nx - 1:
            return po.INFLOW
        if (x, y) == (nx // 2, ny // 2):
            return po.SOLID
        return po.FLUID

    return po.flags_from(fn, nx, ny, nz)


def run_case(case, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = case["dims"]
    N = nx * ny * nz
    fl = flags_for(case)
    sim = po.OracleSim(nx, ny, nz, omega=case["omega"], omegaMinus=case.get("omegaMinus"),
                       lid=case.get("lid", (0, 0, 0)), uin=case.get("uin", 0.0),
                       rampSteps=case.get("ramp", 0), force=case.get("force", (0, 0, 0)),
                       cSmago=case.get("cSmago", 0.0), wantsForces="probe" in case, flags=fl,
                       kind=case["kind"], backend="ref")
    sim.inflowUniform = case.get("uniform", False)
    if "sponge" in case:
        sim.sponge = case["sponge"]
    eps = None
    if case.get("eps"):
        eps = np.zeros(N, np.float32)
        fluid = np.flatnonzero(sim.flags == po.FLUID)
        pick = rng.choice(fluid, size=max(3, len(fluid) // 6), replace=False)
        eps[pick] = rng.uniform(0.05, 0.95, pick.size).astype(np.float32)
        sim.setSolidFractions(eps)
    if "init" in case:
        sim.initField(*case["init"])
    else:
        sim.f[:] = (rng.standard_normal((19, N)) * 0.01).astype(sim.f.dtype)
    f0 = sim.f.copy()
    sim.run(case["steps"])
    out = {"f0": f0, "f1": sim.f.copy(), "flags": fl if fl is not None else np.zeros(0, np.uint8),
           "eps": eps if eps is not None else np.zeros(0, np.float32)}
    if sim.stepsDone % 2 == 0:
        out["moments"] = sim.probeMoments()
    if "probe" in case:
        (x0, x1), (y0, y1) = case["probe"]
        out["force"] = sim.probeForce((x0, x1), (y0, y1))
        out["f2"] = sim.f.copy()
    return out


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    if build_oracle.build_ref(ref_root) is None:
        raise SystemExit("reference tree not found")
    arrays = {}
    meta = []
    for k, case in enumerate(CASES):
        res = run_case(case, seed=1000 + k)
        for key, val in res.items():
            arrays["%s/%s" % (case["name"], key)] = val
        meta.append(case)
    # initField of the reference (sinf/cosf of the host libm) for modes 1 and 2
    for kind in (0, 1):
        for mode in (1, 2):
            nx, ny, nz = 10, 8, 6
            sim = po.OracleSim(nx, ny, nz, omega=1.2, kind=kind, backend="ref")
            sim.initField(mode, 0.07)
            arrays["init_k%d_m%d/f" % (kind, mode)] = sim.f.copy()
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    path = os.path.join(HERE, "reference_cases.npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
