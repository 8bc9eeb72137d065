"""Error of each observable against the FP64 oracle, per storage precision.

Test infrastructure: used by tests/test_gpu_gates.py (small lattices) and run
as a script for the records gated in tests/test_gate_records.py:

    python tests/precision_observables.py tgv --n 256 --steps 200 --out tests/records/precision_tgv256.json
    python tests/precision_observables.py cylinder --D 20 --steps 20000 --out tests/records/precision_cylinder.json

Observables (Sources/strouhal/Cases.swift):
- kinetic energy E = sum |u|^2 / (2 N u0^2) (1239-1245);
- the library's dissipation reduction sum 2 nu S:S, S from the non-equilibrium
  stress, against the same sum over the FP64 state;
- the reference's dissipation eps = -dE/dt* by central differences of the
  sampled energy (1254-1270), as a series;
- drag and lift coefficients of the force probe (Sim.swift:359-372,
  Cases.swift:884-885) on a cylinder channel with velocity walls and a
  Noble-Torczynski disk;
- the DDFs themselves, normwise.
The GPU runs FP32 arithmetic over FP16 or FP32 storage; the oracle runs the
same step in FP64 from the same initial state (the GPU's, exactly).
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

RUNS = (("fp16s", None), ("fp32", 3.0 / 16.0))  # FP16-storage SRT, FP32-storage TRT


def _series_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def tgv(sg, po, gpu, n, steps, every, threads=None, u0=0.05, runs=RUNS, ddf_every=True):
    """Taylor-Green vortex at Re 1600 on an n^3 periodic lattice, sampled every
    `every` steps (even) for `steps` steps, for each (precision, Lambda)."""
    threads = threads or os.cpu_count() or 1
    L = n / (2.0 * math.pi)
    tau = 3.0 * u0 * L / 1600.0 + 0.5
    tc = L / u0
    out = {"lattice": [n, n, n], "u0": u0, "tau": tau, "steps": steps, "every": every,
           "oracle_threads": threads, "runs": []}
    for precision, lam in runs:
        t0 = time.perf_counter()
        wp, wm = sg.trtOmegas(tau, lam)
        g = sg.Simulation(gpu, precision=precision, nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm)
        g.initField(2, u0)
        o = po.OracleSim(n, n, n, omega=wp, omegaMinus=wm, kind=po.KIND_F64, threads=threads)
        o.f[:] = g.downloadState().astype(np.float64)  # the same initial state, exactly
        norm = 2.0 * n ** 3 * u0 * u0
        rows = []
        while True:
            ke_g, ds_g = g.kineticEnergySum(), g.dissipationSum()
            ke_o, ds_o = o.observables()
            row = {"step": g.stepsDone, "t_star": g.stepsDone / tc, "E_gpu": ke_g / norm,
                   "E_fp64": ke_o / norm, "diss_gpu": ds_g, "diss_fp64": ds_o}
            if ddf_every or g.stepsDone >= steps:
                d = g.downloadState().astype(np.float64)
                d -= o.f
                row["ddf_rel"] = float(np.linalg.norm(d) / np.linalg.norm(o.f))
                del d
            rows.append(row)
            if g.stepsDone >= steps:
                break
            g.run(every)
            o.run(every)
        g.close()
        t = np.array([r["t_star"] for r in rows])
        eg = np.array([r["E_gpu"] for r in rows])
        eo = np.array([r["E_fp64"] for r in rows])
        eps_g = -(eg[2:] - eg[:-2]) / (t[2:] - t[:-2])
        eps_o = -(eo[2:] - eo[:-2]) / (t[2:] - t[:-2])
        run = {"precision": precision, "lambda": lam, "rows": rows,
               "err": {"kinetic_energy": max(abs(r["E_gpu"] - r["E_fp64"]) / r["E_fp64"]
                                             for r in rows),
                       "dissipation_sum": max(abs(r["diss_gpu"] - r["diss_fp64"]) /
                                              abs(r["diss_fp64"]) for r in rows),
                       "eps_dEdt": _series_rel(eps_g, eps_o) if len(rows) > 2 else None,
                       "ddf_final": rows[-1]["ddf_rel"]},
               "seconds": time.perf_counter() - t0}
        out["runs"].append(run)
    return out


def cylinder(sg, po, gpu, D, steps, every, threads=None, uin_max=0.06, nz=3, ramp=None,
             runs=(("fp32", 3.0 / 16.0), ("fp16s", 3.0 / 16.0))):
    """The DFG 2D-2 channel of the cylinder configuration at diameter D
    (22D + 2 by 4.1D + 2 by nz, TRT, Re 100, NT disk from 16 x 16 subcell
    sampling, parabolic velocity walls at both ends, 3D sponge): C_D and C_L of
    the force probe every `every` steps, GPU against the FP64 oracle."""
    threads = threads or os.cpu_count() or 1
    nx = 22 * D + 2
    ny = int(4.1 * D) + 2
    umean = uin_max * 2.0 / 3.0
    cx = cy = 0.5 + 2.0 * D
    ramp = ramp if ramp is not None else int(24000 * D / 64)
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = sg.Cell.solid
    fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = sg.Cell.inflow
    fl = fl.reshape(-1)
    eps = np.tile(sg.diskSolidFractions(nx, ny, cx, cy, D / 2.0), nz)
    box = ((int(cx) - D // 2 - 3, int(cx) + D // 2 + 3), (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3))
    cnorm = 2.0 / (umean * umean * D * nz)
    out = {"lattice": [nx, ny, nz], "D": D, "steps": steps, "every": every, "ramp": ramp,
           "oracle_threads": threads, "runs": []}
    for precision, lam in runs:
        t0 = time.perf_counter()
        wp, wm = sg.trtOmegas(3.0 * (umean * D / 100.0) + 0.5, lam)
        kw = dict(nx=nx, ny=ny, nz=nz, omega=wp, omegaMinus=wm, uin=uin_max, rampSteps=ramp,
                  wantsForces=True)
        g = sg.Simulation(gpu, precision=precision, flags=fl, **kw)
        o = po.OracleSim(flags=fl, kind=po.KIND_F64, threads=threads, **kw)
        sp = (float(nx - 1 - 3 * D), float(3 * D), 1.0)
        g.sponge = o.sponge = sp
        g.setSolidFractions(eps)
        o.setSolidFractions(eps)
        rows = []
        while g.stepsDone + every <= steps:
            g.run(every - 2)
            o.run(every - 2)
            fg = g.probeForce(*box)
            fo = o.probeForce(*box)
            rows.append({"step": g.stepsDone, "cd_gpu": cnorm * fg[0], "cl_gpu": cnorm * fg[1],
                         "cd_fp64": cnorm * fo[0], "cl_fp64": cnorm * fo[1]})
        d = g.downloadState().astype(np.float64) - o.f
        ddf = float(np.linalg.norm(d) / np.linalg.norm(o.f))
        g.close()
        cd_scale = max(abs(r["cd_fp64"]) for r in rows)
        run = {"precision": precision, "lambda": lam, "rows": rows,
               "err": {"drag_coefficient": max(abs(r["cd_gpu"] - r["cd_fp64"]) / abs(r["cd_fp64"])
                                               for r in rows),
                       "lift_coefficient_over_max_cd": max(abs(r["cl_gpu"] - r["cl_fp64"])
                                                           for r in rows) / cd_scale,
                       "lift_series": _series_rel([r["cl_gpu"] for r in rows],
                                                  [r["cl_fp64"] for r in rows]),
                       "max_abs_cl_fp64": max(abs(r["cl_fp64"]) for r in rows),
                       "ddf_final": ddf},
               "seconds": time.perf_counter() - t0}
        out["runs"].append(run)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("case", choices=("tgv", "cylinder"))
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--D", type=int, default=20)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import strouhal_gb300 as sg
    from oracle import build_oracle, pyoracle as po

    build_oracle.build_oracle()
    gpu = sg.GPU(0)
    t0 = time.perf_counter()
    if a.case == "tgv":
        res = tgv(sg, po, gpu, a.n, a.steps, a.every, ddf_every=False)
        cmd = "python tests/precision_observables.py tgv --n %d --steps %d --every %d" % (
            a.n, a.steps, a.every)
    else:
        res = cylinder(sg, po, gpu, a.D, a.steps, a.every)
        cmd = "python tests/precision_observables.py cylinder --D %d --steps %d --every %d" % (
            a.D, a.steps, a.every)
    res["command"] = cmd
    res["elapsed_seconds"] = time.perf_counter() - t0
    for r in res["runs"]:
        print(json.dumps({"precision": r["precision"], "err": r["err"], "s": r["seconds"]}),
              flush=True)
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(res, fh)
    gpu.close()


if __name__ == "__main__":
    main()
