"""Adjoint checks on crops of the cylinder (C3) and sphere-wake (C5) lattices.

Test infrastructure: used by tests/test_gpu_adjoint_crop.py (short windows)
and run as a script for the long-window records gated in
tests/test_gate_records.py:

    python tests/adjoint_crops.py sphere --window 2000 --out tests/records/adjoint_crop_sphere.json
    python tests/adjoint_crops.py cylinder --window 2000 --out tests/records/adjoint_crop_cylinder.json

Three comparisons per crop, all on the same initial state (a GPU spin-up):

1. the GPU adjoint (FP32 reverse pass) against the FP64 host adjoint taken
   about the GPU's own forward trajectory (the oracle's FP32-arithmetic step
   over FP32 or FP16 storage is the library's step value for value, so both
   linearise about the same stored states): checks the reverse arithmetic;
2. the FP64 host adjoint about the FP64 trajectory against FP64 central
   differences of the oracle's forward: checks the differentiation;
3. the GPU adjoint against those FP64 central differences directly.

Geometry (Sources/StrouhalCore/CaseSetups.swift:29-64 and 95-134):
- sphere crop: the 64^3 box around the C5 sphere (D = 48, 8^3 subcell
  Noble-Torczynski fractions), uniform-inflow velocity walls at x = 0 and
  x = 63, periodic y and z, Smagorinsky Cs^2 = 0.01, Re 300 (tau 0.524), an
  outlet sponge 16 cells wide, and a small random per-cell Guo force field
  (C5 differentiates drag with respect to that field);
- cylinder crop: the first 4D + 2 = 258 columns of the C3 channel (D = 64,
  centre 2D + 0.5 from the inlet corner, solid walls at y = 0 and y = 263,
  parabolic-inflow velocity walls at x = 0 and x = 257), TRT Lambda = 3/16,
  Re 100, NT disk from 16 x 16 subcell sampling; its initial state is cropped
  from a spin-up of the full 1410 x 264 x 3 lattice.
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


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ------------------------------------------------------------------ sphere crop
SPHERE = dict(n=64, D=48, u=0.05, re=300.0, cs2=0.01, sponge_w=16.0)


def sphere_crop(sg, po, gpu, precision, spinup=400, ramp=200, seed=11, field_scale=2e-6):
    """GPU simulation and FP64 oracle mirror of the sphere crop after `spinup`
    GPU steps. Returns (sim, oracle, f0, t0, box, eps, ffield, flags)."""
    n, D = SPHERE["n"], SPHERE["D"]
    nu = SPHERE["u"] * D / SPHERE["re"]
    wp, _ = sg.trtOmegas(3.0 * nu + 0.5, None)
    fl = np.zeros((n, n, n), np.uint8)
    fl[:, :, 0] = fl[:, :, -1] = sg.Cell.inflow
    fl = fl.reshape(-1)
    kw = dict(nx=n, ny=n, nz=n, omega=wp, uin=SPHERE["u"], rampSteps=ramp,
              cSmago=SPHERE["cs2"], wantsForces=True)
    g = sg.Simulation(gpu, precision=precision, flags=fl, **kw)
    o = po.OracleSim(flags=fl, kind=po.KIND_F64, **kw)
    g.inflowUniform = o.inflowUniform = True
    sp = (float(n - 1 - SPHERE["sponge_w"]), SPHERE["sponge_w"], 1.0)
    g.sponge = o.sponge = sp
    eps = sg.sphereSolidFractions(n, n, n, n / 2.0, n / 2.0, n / 2.0, D / 2.0, 8)
    g.setSolidFractions(eps)
    o.setSolidFractions(eps)
    rng = np.random.default_rng(seed)
    ff = (rng.standard_normal((3, n ** 3)) * field_scale).astype(np.float32)
    ff[:, rng.random(n ** 3) < 0.25] = 0.0  # some cells without a field force
    g.setForceField(ff)
    o.setForceField(ff)
    g.run(spinup)
    f0 = g.downloadState()
    t0 = g.stepsDone
    o.stepsDone = t0
    box = ((4, n - 5), (4, n - 5))
    return g, o, f0, t0, box, eps, ff, fl


# ---------------------------------------------------------------- cylinder crop
CYL = dict(D=64, uin_max=0.06, nz=3, ramp=24000)


def cylinder_crop(sg, po, gpu, precision, spinup=30000):
    """The first 4D + 2 columns of the C3 channel, state cropped from a
    `spinup`-step GPU run of the full lattice."""
    D, nz = CYL["D"], CYL["nz"]
    nxf = 22 * D + 2
    ny = int(4.1 * D) + 2
    umean = CYL["uin_max"] * 2.0 / 3.0
    wp, wm = sg.trtOmegas(3.0 * (umean * D / 100.0) + 0.5, 3.0 / 16.0)
    cx = cy = 0.5 + 2.0 * D

    def flags(nx):
        f = np.zeros((nz, ny, nx), np.uint8)
        f[:, 0, :] = f[:, -1, :] = sg.Cell.solid
        f[:, 1:-1, 0] = f[:, 1:-1, -1] = sg.Cell.inflow
        return f.reshape(-1)

    kw = dict(ny=ny, nz=nz, omega=wp, omegaMinus=wm, uin=CYL["uin_max"], rampSteps=CYL["ramp"],
              wantsForces=True)
    full = sg.Simulation(gpu, precision=precision, nx=nxf, flags=flags(nxf), **kw)
    full.setSolidFractions(np.tile(sg.diskSolidFractions(nxf, ny, cx, cy, D / 2.0), nz))
    full.sponge = (float(nxf - 1 - 3 * D), float(3 * D), 1.0)
    full.run(spinup)
    t0 = full.stepsDone
    fs = full.downloadState().reshape(19, nz, ny, nxf)
    full.close()
    nx = 4 * D + 2
    fl = flags(nx)
    f0 = np.ascontiguousarray(fs[:, :, :, :nx]).reshape(19, -1)
    f0[:, fl != 0] = 0  # the crop's outlet column becomes a velocity wall
    eps = np.tile(sg.diskSolidFractions(nx, ny, cx, cy, D / 2.0), nz)
    g = sg.Simulation(gpu, precision=precision, nx=nx, flags=fl, **kw)
    o = po.OracleSim(nx=nx, flags=fl, kind=po.KIND_F64, **kw)
    g.setSolidFractions(eps)
    o.setSolidFractions(eps)
    g.uploadState(f0)
    g.stepsDone = t0
    o.stepsDone = t0
    box = ((int(cx) - D // 2 - 3, int(cx) + D // 2 + 3), (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3))
    return g, o, f0, t0, box, eps, None, fl


# ------------------------------------------------------------------ the checks
def run_checks(sg, o, g, f0, box, eps, ff, window, precision, fd_eps=8, fd_force=8, seed=5,
               threads=None, h_eps=2.0 ** -12, h_force=2.0 ** -16, fd_solid=2,
               h_solid=2.0 ** -22):
    """The three comparisons; returns a dict of errors and timings."""
    out = {"window": window, "precision": precision, "cells": int(g.cells)}
    ck = max(1, int(math.ceil(math.sqrt(window))))
    traj = "fp32" if precision == "fp32" else "fp16"
    t = time.perf_counter()
    adj = sg.Adjoint(g, window, box, checkpoints=ck)
    J = adj.forward()
    ge, gf = adj.backward()
    st = adj.stats()
    adj.close()
    out["gpu_seconds"] = {"forward": st["forward_s"], "recompute": st["recompute_s"],
                          "adjoint": st["adjoint_s"], "wall": time.perf_counter() - t}
    out["checkpoints"] = ck
    out["J_gpu"] = J
    t = time.perf_counter()
    Jt, get, gft = o.adjointForce(window, box, trajectory=traj, f0=f0, threads=threads,
                                  checkpoint=ck)
    out["host_seconds_same_trajectory"] = time.perf_counter() - t
    nt = eps != 0
    out["J_same_trajectory"] = Jt
    out["J_rel_err"] = abs(J - Jt) / max(abs(Jt), 1e-300)
    out["grad_eps_rel_err"] = rel(ge[nt], get[nt])
    surf, full = nt & (eps < 1), eps == 1
    out["grad_eps_rel_err_surface"] = rel(ge[surf], get[surf])
    out["grad_eps_rel_err_solid"] = rel(ge[full], get[full]) if full.any() else None
    out["grad_eps_zero_off_nt"] = bool(np.all(ge[~nt] == 0))
    out["grad_force_rel_err"] = rel(gf, gft)
    t = time.perf_counter()
    J64, ge64, gf64 = o.adjointForce(window, box, trajectory="fp64", f0=f0, threads=threads,
                                     checkpoint=ck)
    out["host_seconds_fp64"] = time.perf_counter() - t
    out["J_fp64"] = J64
    out["gpu_vs_fp64_adjoint"] = {"grad_eps": rel(ge[nt], ge64[nt]),
                                  "grad_force": rel(gf, gf64)}
    # central differences of the FP64 forward on cells of large gradient
    rng = np.random.default_rng(seed)
    fd = []
    t = time.perf_counter()
    e_cand = np.flatnonzero((eps > 0.05) & (eps < 0.95))
    if fd_eps and e_cand.size:
        mag = np.abs(ge64[e_cand])
        e_cand = e_cand[mag >= 0.1 * mag.max()]
        for n in rng.choice(e_cand, size=min(fd_eps, e_cand.size), replace=False):
            vals = []
            for sgn in (1.0, -1.0):
                e = eps.copy()
                e[n] = np.float32(e[n] + sgn * h_eps)
                o.setSolidFractions(e)
                vals.append(o.adjointForce(window, box, grads=False, f0=f0, threads=threads)[0])
            o.setSolidFractions(eps)
            h = float(np.float32(eps[n] + h_eps)) - float(np.float32(eps[n] - h_eps))
            d = (vals[0] - vals[1]) / h
            fd.append({"param": "eps", "cell": int(n), "fd": d, "fp64_adjoint": float(ge64[n]),
                       "gpu_adjoint": float(ge[n])})
    # Fully solid cells (eps = 1): eps > 1 is outside the model (the blend
    # factor B exceeds 1 and the cell amplifies its non-equilibrium), so the
    # difference there is one-sided, second order: (3 J(1) - 4 J(1-h) + J(1-2h)) / 2h.
    # Its step is far smaller: below eps = 1 the cell's frozen non-equilibrium
    # relaxes at a rate of about B'(1) h omega per step (B'(1) = (1 + tw) / tw,
    # 14 at tau = 0.577), so J is linear in h only while the window times that
    # rate is small; h = 2^-22 keeps it below 1e-2 for 2,000 steps.
    full_cand = np.flatnonzero(eps == 1)
    if fd_solid and full_cand.size:
        mag = np.abs(ge64[full_cand])
        for n in full_cand[np.argsort(-mag)][:fd_solid]:
            vals = []
            for k in (1, 2):
                e = eps.copy()
                e[n] = np.float32(1.0 - k * h_solid)
                o.setSolidFractions(e)
                vals.append(o.adjointForce(window, box, grads=False, f0=f0, threads=threads)[0])
            o.setSolidFractions(eps)
            d = (3.0 * J64 - 4.0 * vals[0] + vals[1]) / (2.0 * h_solid)
            fd.append({"param": "eps_solid", "cell": int(n), "fd": d,
                       "fp64_adjoint": float(ge64[n]), "gpu_adjoint": float(ge[n])})
    if fd_force and ff is not None:
        mag = np.sqrt((gf64 ** 2).sum(0))
        f_cand = np.flatnonzero(mag >= 0.1 * mag.max())
        for n in rng.choice(f_cand, size=min(fd_force, f_cand.size), replace=False):
            k = int(np.argmax(np.abs(gf64[:, n])))
            vals = []
            for sgn in (1.0, -1.0):
                f = ff.copy()
                f[k, n] = np.float32(f[k, n] + sgn * h_force)
                o.setForceField(f)
                vals.append(o.adjointForce(window, box, grads=False, f0=f0, threads=threads)[0])
            o.setForceField(ff)
            h = float(np.float32(ff[k, n] + h_force)) - float(np.float32(ff[k, n] - h_force))
            d = (vals[0] - vals[1]) / h
            fd.append({"param": "force%d" % k, "cell": int(n), "fd": d,
                       "fp64_adjoint": float(gf64[k, n]), "gpu_adjoint": float(gf[k, n])})
    out["host_seconds_fd"] = time.perf_counter() - t
    for r in fd:
        r["fp64_adjoint_rel_err"] = abs(r["fp64_adjoint"] - r["fd"]) / abs(r["fd"])
        r["gpu_adjoint_rel_err"] = abs(r["gpu_adjoint"] - r["fd"]) / abs(r["fd"])
    out["fd"] = fd
    out["fd_worst_fp64_adjoint"] = max((r["fp64_adjoint_rel_err"] for r in fd), default=None)
    out["fd_worst_gpu_adjoint"] = max((r["gpu_adjoint_rel_err"] for r in fd), default=None)
    ok = np.isfinite(ge).all() and np.isfinite(gf).all()
    out["finite"] = bool(ok)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("crop", choices=("sphere", "cylinder"))
    ap.add_argument("--window", type=int, default=2000)
    ap.add_argument("--spinup", type=int, default=None)
    ap.add_argument("--precision", default=None)
    ap.add_argument("--fd", type=int, default=8)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import strouhal_gb300 as sg
    from oracle import build_oracle, pyoracle as po

    build_oracle.build_oracle()
    gpu = sg.GPU(0)
    t0 = time.perf_counter()
    res = {"crop": a.crop, "runs": []}
    precs = [a.precision] if a.precision else (["fp16s", "fp32"] if a.crop == "sphere"
                                               else ["fp32"])
    for prec in precs:
        if a.crop == "sphere":
            g, o, f0, _, box, eps, ff, _ = sphere_crop(sg, po, gpu, prec,
                                                       spinup=a.spinup or 2000, ramp=1000)
        else:
            g, o, f0, _, box, eps, ff, _ = cylinder_crop(sg, po, gpu, prec,
                                                         spinup=a.spinup or 150000)
        r = run_checks(sg, o, g, f0, box, eps, ff, a.window, prec, fd_eps=a.fd, fd_force=a.fd)
        r["lattice"] = [g.nx, g.ny, g.nz]
        g.close()
        res["runs"].append(r)
        print(json.dumps({k: v for k, v in r.items() if k != "fd"}), flush=True)
    res["host_threads"] = os.cpu_count()
    res["elapsed_seconds"] = time.perf_counter() - t0
    res["command"] = "python tests/adjoint_crops.py %s --window %d" % (a.crop, a.window)
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(res, fh)
    gpu.close()


if __name__ == "__main__":
    main()
