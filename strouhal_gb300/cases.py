"""Case runners over the C ABI for the workloads the step is judged on.

Each function restates a host-side procedure of the reference's gate suite
(Sources/strouhal/Cases.swift, Sources/StrouhalCore/CaseSetups.swift) on top
of strouhal_gb300.Simulation and returns plain measurements (dicts of floats
and lists). The thresholds and published reference values the reference
compares against are applied by the tests, not here.

    python -m strouhal_gb300.cases <name> [--out results.json]

names: poiseuille, tg_order, cavity, dfg2, dfg2_adjoint, tgv, sphere,
sphere_adjoint, ladder.
"""
import argparse
import hashlib
import json
import math
import os
import time

import numpy as np

import strouhal_gb300 as sg


# --------------------------------------------------------------- Poiseuille
def poiseuille(gpu, H=64, precision="fp32"):
    """Body-force channel with TRT Lambda=3/16 (Cases.swift:286-317): max
    |u - u_exact| / u_max over the profile after 6 diffusive times."""
    tau = 0.8
    nu = (tau - 0.5) / 3.0
    umax = 0.05
    F = 8.0 * nu * umax / (H * H)
    wp, wm = sg.trtOmegas(tau, 3.0 / 16.0)
    ny = H + 2
    flags = np.zeros((1, ny, 16), np.uint8)
    flags[:, 0, :] = flags[:, -1, :] = sg.Cell.solid
    s = sg.Simulation(gpu, precision=precision, nx=16, ny=ny, nz=1, omega=wp, omegaMinus=wm,
                      force=(F, 0.0, 0.0), flags=flags.reshape(-1))
    steps = (int(6.0 * H * H / nu) + 1) & ~1
    s.run(steps)
    m = s.probeMoments()
    errs = []
    for j in range(1, H + 1):
        yd = j - 0.5
        exact = F / (2.0 * nu) * yd * (H - yd)
        errs.append(abs(float(m[j * 16 + 8, 0]) - exact) / umax)
    s.close()
    return {"H": H, "steps": steps, "max_err": max(errs), "wall_err": max(errs[0], errs[-1]),
            "center_err": max(errs[H // 2 - 1], errs[H // 2])}


# ------------------------------------------------------- Taylor-Green order
def tg_order(gpu, sizes=(32, 64, 128), u0base=0.20, precision="fp32"):
    """2-D Taylor-Green decay under diffusive scaling (Cases.swift:329-370)."""
    nu = 0.02
    wp, wm = sg.trtOmegas(3.0 * nu + 0.5, 0.25)
    errors = []
    for N in sizes:
        u0 = u0base * 32.0 / N
        k = 2.0 * math.pi / N
        steps = int(math.log(2.0) / (2.0 * nu * k * k)) & ~1
        s = sg.Simulation(gpu, precision=precision, nx=N, ny=N, nz=1, omega=wp, omegaMinus=wm)
        s.initField(1, u0)
        s.run(steps)
        m = s.probeMoments().reshape(N, N, 4)
        decay = math.exp(-2.0 * nu * k * k * steps)
        xa = (np.arange(N) + 0.5)[None, :]
        ya = (np.arange(N) + 0.5)[:, None]
        ue = u0 * decay * np.sin(k * xa) * np.cos(k * ya)
        ve = -u0 * decay * np.cos(k * xa) * np.sin(k * ya)
        du = m[:, :, 0].astype(np.float64) - ue
        dv = m[:, :, 1].astype(np.float64) - ve
        errors.append(math.sqrt(float(np.sum(du * du + dv * dv)) / (2 * N * N)) / (u0 * decay))
        s.close()
    orders = [math.log2(errors[i - 1] / errors[i]) for i in range(1, len(errors))]
    return {"sizes": list(sizes), "errors": errors, "orders": orders, "min_order": min(orders)}


# ------------------------------------------------------------------- cavity
def cavity(gpu, n=128, re=100.0, steps=20000, lam=None, ulid=0.1, ramp=5000, nz=3,
           precision="fp32"):
    """Lid-driven cavity: n x n interior, 1-cell frame, lid at the top moving
    +x, periodic z (Cases.swift:167-215 set-up). Returns the centreline
    profiles u(y)/u_lid on the vertical and v(x)/u_lid on the horizontal
    centreline (each averaged over the two centre columns / rows, z = 0), at
    physical coordinates (i - 0.5)/n, plus the digest and mass drift."""
    nx = ny = n + 2
    nu = ulid * n / re
    wp, wm = sg.trtOmegas(3.0 * nu + 0.5, lam)
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = flags[:, 0, :] = sg.Cell.solid
    flags[:, -1, :] = sg.Cell.lid
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=wp, omegaMinus=wm,
                      lid=(ulid, 0.0, 0.0), rampSteps=ramp, flags=flags.reshape(-1))
    m0 = s.massSum()
    t0 = time.perf_counter()
    s.run(steps)
    wall = time.perf_counter() - t0
    m = s.probeMoments().reshape(nz, ny, nx, 4)[0]
    c0, c1 = n // 2, n // 2 + 1
    u = [(float(m[j, c0, 0]) + float(m[j, c1, 0])) / 2.0 / ulid for j in range(1, n + 1)]
    v = [(float(m[c0, i, 1]) + float(m[c1, i, 1])) / 2.0 / ulid for i in range(1, n + 1)]
    out = {"n": n, "re": re, "steps": steps, "srt": lam is None, "coords": [(i - 0.5) / n
                                                                            for i in range(1, n + 1)],
           "u_centerline": u, "v_centerline": v, "digest": s.stateDigest,
           "mass_drift": s.massSum() - m0, "gpu_seconds": s.gpuSeconds, "wall_seconds": wall}
    s.close()
    return out


def _lid_cavity_sim(gpu, n, nz, re, ulid, lam, ramp, flags, lid=None, precision="fp32"):
    nu = ulid * n / re
    wp, wm = sg.trtOmegas(3.0 * nu + 0.5, lam)
    return sg.Simulation(gpu, precision=precision, nx=n + 2, ny=n + 2, nz=nz, omega=wp,
                         omegaMinus=wm, lid=lid if lid is not None else (ulid, 0.0, 0.0),
                         rampSteps=ramp, flags=flags.reshape(-1))


def cavity_zperiodic(gpu, n=128, nz=8, re=400.0, steps=120000, ulid=0.1, lam=0.25, ramp=5000):
    """3-D lattice, 2-D physics (Cases.swift:642-686): the cavity periodic in z
    must reproduce the 2-D solution and stay z-uniform. Records the vertical
    centreline u(y)/u_lid of slice z = 0 and the largest |u_x| difference of
    any interior cell from its z = 0 counterpart."""
    N = n + 2
    flags = np.zeros((nz, N, N), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = flags[:, 0, :] = sg.Cell.solid
    flags[:, -1, :] = sg.Cell.lid
    s = _lid_cavity_sim(gpu, n, nz, re, ulid, lam, ramp, flags)
    s.run(steps)
    m = s.probeMoments().reshape(nz, N, N, 4)
    ux = m[:, 1:n + 1, 1:n + 1, 0]
    zdev = float(np.max(np.abs(ux[1:] - ux[:1]))) if nz > 1 else 0.0
    c0, c1 = n // 2, n // 2 + 1
    u = [(float(m[0, j, c0, 0]) + float(m[0, j, c1, 0])) / 2.0 / ulid for j in range(1, n + 1)]
    out = {"n": n, "nz": nz, "re": re, "steps": steps, "lambda": lam, "u_centerline": u,
           "max_z_dev": zdev, "finite": bool(np.all(np.isfinite(m))),
           "digest": s.stateDigest, "gpu_seconds": s.gpuSeconds}
    s.close()
    return out


def cavity_cubic(gpu, n=64, re=400.0, steps=120000, ulid=0.1, lam=0.25, ramp=5000):
    """Cubic cavity, full 3-D flow (Cases.swift:688-728): stable, and mirror
    symmetric about the mid-z plane. Records the RMS of u_x(z) - u_x(n+1-z) over
    the interior in units of u_lid and the mid-plane centreline minimum."""
    N = n + 2
    flags = np.zeros((N, N, N), np.uint8)  # (z, y, x)
    flags[0, :, :] = flags[-1, :, :] = sg.Cell.solid
    flags[:, 0, :] = flags[:, -1, :] = sg.Cell.solid
    flags[:, :, 0] = flags[:, :, -1] = sg.Cell.solid
    flags[1:n + 1, -1, 1:n + 1] = sg.Cell.lid
    s = _lid_cavity_sim(gpu, n, N, re, ulid, lam, ramp, flags)
    s.run(steps)
    m = s.probeMoments().reshape(N, N, N, 4)
    ux = m[1:n + 1, 1:n + 1, 1:n + 1, 0].astype(np.float64)
    asym = float(np.sqrt(np.mean((ux - ux[::-1]) ** 2)) / ulid)
    umin = float(min(0.0, np.min(m[n // 2, 1:n + 1, n // 2, 0].astype(np.float64) / ulid)))
    out = {"n": n, "re": re, "steps": steps, "lambda": lam, "asym_rms": asym,
           "centerline_umin": umin, "finite": bool(np.all(np.isfinite(m))),
           "digest": s.stateDigest, "gpu_seconds": s.gpuSeconds}
    s.close()
    return out


def rotation(gpu, n=64, re=100.0, steps=60000, ulid=0.1, lam=0.25, ramp=2000):
    """Rotation / anisotropy (Cases.swift:730-765): a cavity whose lid is the
    +x face moving +y must give the standard cavity (lid on +y moving +x)
    transposed. Records the RMS of the transposed-field difference in u_lid."""
    N = n + 2
    fa = np.zeros((1, N, N), np.uint8)
    fa[0, :, 0] = fa[0, :, -1] = fa[0, 0, :] = sg.Cell.solid
    fa[0, -1, :] = sg.Cell.lid
    fb = np.zeros((1, N, N), np.uint8)
    fb[0, 0, :] = fb[0, -1, :] = fb[0, :, 0] = sg.Cell.solid
    fb[0, :, -1] = sg.Cell.lid
    a = _lid_cavity_sim(gpu, n, 1, re, ulid, lam, ramp, fa)
    b = _lid_cavity_sim(gpu, n, 1, re, ulid, lam, ramp, fb, lid=(0.0, ulid, 0.0))
    a.run(steps)
    b.run(steps)
    ma = a.probeMoments().reshape(N, N, 4)[1:n + 1, 1:n + 1].astype(np.float64)  # [y, x]
    mb = b.probeMoments().reshape(N, N, 4)[1:n + 1, 1:n + 1].astype(np.float64)
    mbt = np.transpose(mb, (1, 0, 2))  # mbt[y, x] = b at (x, y) swapped: cell (y, x) of b
    du = ma[..., 0] - mbt[..., 1]
    dv = ma[..., 1] - mbt[..., 0]
    rms = float(np.sqrt(np.sum(du * du + dv * dv) / (2 * n * n)) / ulid)
    out = {"n": n, "re": re, "steps": steps, "lambda": lam, "transposed_rms": rms,
           "finite": bool(np.all(np.isfinite(ma)) and np.all(np.isfinite(mb))),
           "gpu_seconds": a.gpuSeconds + b.gpuSeconds}
    a.close()
    b.close()
    return out


def mass_drift(gpu, n=128, re=100.0, steps=50000, ulid=0.1, lam=0.25, ramp=5000):
    """Lid mass drift (Cases.swift:787-799): the moving-lid bounce-back with
    rho_w = 1 does not conserve mass exactly; |sum(rho - 1)| after 50,000 steps
    of the 2-D cavity (TRT, Lambda = 1/4) must stay bounded."""
    N = n + 2
    flags = np.zeros((1, N, N), np.uint8)
    flags[0, :, 0] = flags[0, :, -1] = flags[0, 0, :] = sg.Cell.solid
    flags[0, -1, :] = sg.Cell.lid
    s = _lid_cavity_sim(gpu, n, 1, re, ulid, lam, ramp, flags)
    m0 = s.massSum()
    s.run(steps)
    drift = s.massSum() - m0
    out = {"n": n, "re": re, "steps": steps, "lambda": lam, "mass_drift": drift,
           "per_step_cell": abs(drift) / steps / (n * n), "digest": s.stateDigest,
           "gpu_seconds": s.gpuSeconds}
    s.close()
    return out


def dfg1(gpu, D=40, max_steps=240000, uin_max=0.075, upstream_d=2.0, curved=True):
    """Schaefer-Turek DFG 2D-1, Re 20, steady (Cases.swift:440-536): C_D against
    the spectral 5.57953523384, probed every 4,000 steps until it settles
    (three successive relative changes below 1e-5 after three flow-throughs)."""
    nx = int((20.0 + upstream_d) * D) + 2
    ny = int(4.1 * D) + 2
    u_mean = uin_max * 2.0 / 3.0
    nu = u_mean * D / 20.0
    wp, wm = sg.trtOmegas(3.0 * nu + 0.5, 3.0 / 16.0)
    cx, cy = 0.5 + upstream_d * D, 0.5 + 2.0 * D
    flags = np.zeros((ny, nx), np.uint8)
    if not curved:
        yy, xx = np.mgrid[0:ny, 0:nx]
        flags[(xx - cx) ** 2 + (yy - cy) ** 2 <= D * D / 4.0] = sg.Cell.solid
    flags[:, 0] = flags[:, -1] = sg.Cell.inflow
    flags[0, :] = flags[-1, :] = sg.Cell.solid
    s = sg.Simulation(gpu, precision="fp32", nx=nx, ny=ny, nz=1, omega=wp, omegaMinus=wm,
                      uin=uin_max, rampSteps=4000, wantsForces=True, flags=flags.reshape(-1))
    if curved:
        s.setSolidFractions(sg.diskSolidFractions(nx, ny, cx, cy, D / 2.0))
    box = ((int(cx) - D // 2 - 3, int(cx) + D // 2 + 3), (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3))
    flow_through = int(nx / u_mean)
    cd = cl = 0.0
    prev, settled = float("inf"), 0
    while s.stepsDone < max_steps:
        s.run(4000 - 2)  # the probe takes two more
        f = s.probeForce(*box)
        cd = float(2.0 * f[0] / (u_mean * u_mean * D))
        cl = float(2.0 * f[1] / (u_mean * u_mean * D))
        if s.stepsDone > 3 * flow_through:
            settled = settled + 1 if abs(cd - prev) / abs(cd) < 1e-5 else 0
            if settled >= 3:
                break
        prev = cd
    out = {"D": D, "curved": curved, "uin_max": uin_max, "steps": s.stepsDone, "cd": cd,
           "cl": cl, "cd_ref": 5.57953523384, "cd_err": abs(cd - 5.57953523384) / 5.57953523384,
           "digest": s.stateDigest, "gpu_seconds": s.gpuSeconds}
    s.close()
    return out


def ghia_rms(rec, table_u, table_v):
    """Centreline RMS against a table of (coordinate, value) pairs, linear
    interpolation between the two bracketing nodes (Cases.swift:220-270)."""
    n = rec["n"]

    def interp(coord, vals):
        sx = coord * n + 0.5
        k0 = min(max(int(math.floor(sx)), 1), n - 1)
        frac = sx - k0
        return vals[k0 - 1] * (1 - frac) + vals[k0] * frac

    d = [interp(y, rec["u_centerline"]) - r for y, r in table_u]
    d += [interp(x, rec["v_centerline"]) - r for x, r in table_v]
    return math.sqrt(sum(x * x for x in d) / len(d)), max(abs(x) for x in d)


# ------------------------------------------------------------ DFG 2D-2 (C3)
def dfg2(gpu, D=64, uin_max=0.06, nz=3, transient=None, sample_cycles=22, stride=26,
         sponge_d=3, sponge_tau=1.0, ramp=24000, precision="fp32", max_steps=None, tune=True):
    """Cylinder channel with Noble-Torczynski walls (Cases.swift:840-951,
    CaseSetups.swift:29-65): C_D and C_L sampled every `stride` steps by the
    two-step force probe, Strouhal number from the upward zero crossings of
    C_L, peaks and cycle means over complete cycles. The transient and the
    samples run as one sampled submission (the same steps and probes as
    run(stride - 2) + probeForce per sample, bit for bit)."""
    nx = 22 * D + 2
    ny = int(4.1 * D) + 2
    umean = uin_max * 2.0 / 3.0
    nu = umean * D / 100.0
    wp, wm = sg.trtOmegas(3.0 * nu + 0.5, 3.0 / 16.0)
    cx = cy = 0.5 + 2.0 * D
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, 0, :] = flags[:, -1, :] = sg.Cell.solid
    flags[:, 1:-1, 0] = flags[:, 1:-1, -1] = sg.Cell.inflow
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=wp, omegaMinus=wm,
                      uin=uin_max, rampSteps=ramp, wantsForces=True, flags=flags.reshape(-1))
    s.setSolidFractions(np.tile(sg.diskSolidFractions(nx, ny, cx, cy, D / 2.0), nz))
    s.sponge = (float(nx - 1 - sponge_d * D), float(sponge_d * D), sponge_tau)
    box_x = (int(cx) - D // 2 - 3, int(cx) + D // 2 + 3)
    box_y = (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3)
    if transient is None:
        transient = (int(60000 * 0.075 / uin_max) + 1) & ~1
    if tune:
        s.autotune(steps=200)  # kernel variant, launch shape and split (state restored)
    t0 = time.perf_counter()
    period = D / (0.30 * umean)
    samples = int(period * sample_cycles / stride) + 64
    if max_steps is not None:
        samples = min(samples, max(1, (max_steps - transient) // stride))
    norm = umean * umean * D * nz  # force per unit depth: the z extent holds nz cells
    forces, at = s.runSampled(transient, samples * stride, stride, box_x, box_y)
    cd = [float(v) for v in 2.0 * forces[:, 0] / norm]
    cl = [float(v) for v in 2.0 * forces[:, 1] / norm]
    t = [int(v) for v in at]
    wall = time.perf_counter() - t0
    stats = cycle_stats(t, cd, cl, D, umean)
    out = {"D": D, "nx": nx, "ny": ny, "nz": nz, "uin_max": uin_max, "steps": s.stepsDone,
           "stride": stride, "t": t, "cd": cd, "cl": cl, "digest": s.stateDigest,
           "gpu_seconds": s.gpuSeconds, "wall_seconds": wall,
           "glups": nx * ny * nz * s.stepsDone / max(s.gpuSeconds, 1e-30) / 1e9,
           "variant": s.variant, "block": list(s.block), "path": s.lastPath,
           "cells": nx * ny * nz}
    out.update(stats)
    s.close()
    return out


def cycle_stats(t, cd, cl, D, umean):
    """Strouhal number, peaks and batch-mean C_D over complete C_L cycles."""
    cross = []
    for k in range(1, len(cl)):
        if cl[k - 1] < 0 <= cl[k]:
            frac = -cl[k - 1] / (cl[k] - cl[k - 1])
            cross.append(t[k - 1] + frac * (t[k] - t[k - 1]))
    cycles = max(len(cross) - 1, 0)
    st, maxcd, maxcl, means = 0.0, 0.0, float("-inf"), []
    if cycles >= 2:
        st = D / ((cross[-1] - cross[0]) / cycles * umean)
        for c in range(cycles):
            sel = [k for k in range(len(cl)) if cross[c] <= t[k] < cross[c + 1]]
            if sel:
                maxcd = max(maxcd, max(cd[k] for k in sel))
                maxcl = max(maxcl, max(cl[k] for k in sel))
                means.append(sum(cd[k] for k in sel) / len(sel))
    mean, ci = 0.0, 0.0
    if len(means) >= 4:
        mean = sum(means) / len(means)
        sd = math.sqrt(sum((m - mean) ** 2 for m in means) / (len(means) - 1))
        ci = 1.96 * sd / math.sqrt(len(means))
    return {"strouhal": st, "max_cd": maxcd, "max_cl": maxcl, "mean_cd": mean,
            "mean_cd_ci95": ci, "cycles": cycles}


# --------------------------------------------------------------- TGV (C2)
def tgv(gpu, n=256, u0=0.05, t_end=20.0, precision="fp16s", lam=None, log_every=100,
        re=1600.0, collision="reference"):
    """3-D Taylor-Green vortex at Re=1600 (Cases.swift:1217-1282, with the
    logging cadence of the workload): kinetic energy E = sum|u|^2/(2 N u0^2)
    and the strain-rate dissipation every `log_every` steps, dissipation also
    as -dE/dt* by central differences, peak refined by a parabola. A run that
    goes non-finite stops and reports the time. collision="kbc" runs the KBC
    collision instead of SRT / TRT."""
    L = n / (2.0 * math.pi)
    nu = u0 * L / re
    tau = 3.0 * nu + 0.5
    wp, wm = sg.trtOmegas(tau, lam)
    s = sg.Simulation(gpu, precision=precision, nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm)
    s.collision = collision
    s.initField(2, u0)
    s.autotune(steps=10)
    tc = L / u0
    total = int(round(t_end * tc))
    total -= total % log_every
    N = s.cells
    times, E, eps_s = [], [], []
    nonfinite = None
    t0 = time.perf_counter()
    while True:
        ke = s.kineticEnergySum()
        ds = s.dissipationSum()
        times.append(s.stepsDone / tc)
        E.append(ke / (2.0 * N * u0 * u0))
        eps_s.append(ds * L / (N * u0 ** 3))
        if not math.isfinite(ke):
            nonfinite = times[-1]
            break
        if s.stepsDone >= total:
            break
        s.run(log_every)
    wall = time.perf_counter() - t0
    eps_fd = [-(E[j + 1] - E[j - 1]) / (times[j + 1] - times[j - 1]) for j in range(1, len(E) - 1)]
    t_fd = times[1:-1]
    peak_t, peak_e = float("nan"), float("nan")
    if len(eps_fd) >= 3:
        k = int(np.argmax(eps_fd))
        peak_t, peak_e = t_fd[k], eps_fd[k]
        if 0 < k < len(eps_fd) - 1:
            y0, y1, y2 = eps_fd[k - 1], eps_fd[k], eps_fd[k + 1]
            den = y0 - 2 * y1 + y2
            if abs(den) > 1e-12:
                dd = 0.5 * (y0 - y2) / den
                peak_t = t_fd[k] + dd * (t_fd[1] - t_fd[0])
                peak_e = y1 - 0.25 * (y0 - y2) * dd
    out = {"n": n, "u0": u0, "tau": tau, "precision": precision,
           "collision": ("KBC" if collision == "kbc" else
                         "SRT" if lam is None else "TRT Lambda=%g" % lam), "steps": s.stepsDone,
           "steps_per_tstar": tc, "t": times, "E": E, "eps_strain": eps_s, "t_fd": t_fd,
           "eps_fd": eps_fd, "peak_t": peak_t, "peak_eps": peak_e, "nonfinite_at": nonfinite,
           "gpu_seconds": s.gpuSeconds, "wall_seconds": wall,
           "glups": N * s.stepsDone / max(s.gpuSeconds, 1e-30) / 1e9, "variant": s.variant}
    s.close()
    return out


# ------------------------------------------------------------- sphere (C5)
def sphere_sim(gpu, nx=512, ny=256, nz=256, D=48, center=(128.0, 128.0, 128.0), u=0.05,
               re=300.0, cs=0.1, ramp=8000, sponge=True, precision="fp16s", sub=8,
               arithmetic="reference"):
    """The C5 lattice: uniform-inflow velocity walls at x = 0 and x = nx-1,
    periodic y and z, NT sphere from sub^3 subcell sampling, Smagorinsky
    cSmago = Cs^2, a zero Guo force field, outlet sponge one diameter wide."""
    nu = u * D / re
    wp, _ = sg.trtOmegas(3.0 * nu + 0.5, None)
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = sg.Cell.inflow
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=wp, uin=u,
                      rampSteps=ramp, cSmago=cs * cs, wantsForces=True, flags=flags.reshape(-1),
                      arithmetic=arithmetic)
    s.inflowUniform = True
    cx, cy, cz = center
    s.setSolidFractions(sg.sphereSolidFractions(nx, ny, nz, cx, cy, cz, D / 2.0, sub))
    s.setForceField(np.zeros((3, nx * ny * nz), np.float32))
    if sponge:
        s.sponge = (float(nx - 1 - D), float(D), 1.0)
    return s


def sphere(gpu, nx=512, ny=256, nz=256, D=48, center=(128.0, 128.0, 128.0), u=0.05, re=300.0,
           cs=0.1, steps=50000, probe_every=500, ramp=8000, sponge=True, precision="fp16s",
           sub=8, tune=True, arithmetic="reference"):
    """3-D sphere wake with LES (workload set-up from CaseSetups.swift:95-134):
    uniform-inflow velocity walls at x = 0 and x = nx-1, periodic y and z,
    Noble-Torczynski sphere from 8^3 subcell sampling, Smagorinsky
    cSmago = Cs^2, Guo force field present and zero. Drag coefficient
    2 F_x / (u^2 pi D^2 / 4) every `probe_every` steps."""
    s = sphere_sim(gpu, nx, ny, nz, D, center, u, re, cs, ramp, sponge, precision, sub,
                   arithmetic)
    cx, cy, cz = center
    bx = (int(cx) - D // 2 - 3, int(cx) + D // 2 + 3)
    byr = (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3)
    area = u * u * math.pi * D * D / 4.0
    if tune:
        s.autotune(steps=10)  # launch shape and bulk/boundary split (state restored)
    t, cd = [], []
    t0 = time.perf_counter()
    while s.stepsDone + probe_every <= steps:
        s.run(probe_every - 2)
        f = s.probeForce(bx, byr)
        t.append(s.stepsDone)
        cd.append(2.0 * f[0] / area)
    wall = time.perf_counter() - t0
    out = {"nx": nx, "ny": ny, "nz": nz, "D": D, "re": re, "steps": s.stepsDone, "t": t,
           "cd": cd, "finite": s.checkFinite(), "gpu_seconds": s.gpuSeconds,
           "wall_seconds": wall, "glups": s.cells * s.stepsDone / max(s.gpuSeconds, 1e-30) / 1e9,
           "variant": s.variant, "block": list(s.block), "arithmetic": s.arithmetic}
    s.close()
    return out


# ---------------------------------------------------------- ladder (C4)
def ladder_instances(count=32, seed=1234, edges=(32, 48, 64, 96, 128, 160),
                     machs=(0.05, 0.025), t_star=5.0):
    """Seed-fixed TGV rungs: (edge, u0, steps, log_every)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(edges))
        u0 = float(rng.choice(machs))
        L = n / (2.0 * math.pi)
        tc = L / u0
        steps = int(round(t_star * tc)) & ~1
        log_every = max(2, int(tc * 0.1) & ~1)
        out.append((n, u0, steps, log_every))
    return out


def ladder(gpu, count=32, seed=1234, precision="fp32",
           modes=("persistent", "rounds", "streams", "sequential"), t_star=5.0, tune=True,
           edges=(32, 48, 64, 96, 128, 160), tune_rounds=40):
    """32 periodic TGV instances of uneven size and Mach number, FP32 SRT,
    Re = 1600, 5 convective times each, kinetic-energy traces every 0.1 t*;
    wall time of the batched launch against instance-after-instance.
    `edges` is the set the lattice edges are drawn from; the fused modes'
    tile shape is autotuned over `tune_rounds` rounds (states restored)."""
    inst = ladder_instances(count, seed, edges=tuple(edges), t_star=t_star)
    results = {"instances": [{"n": n, "u0": u0, "steps": k, "log_every": le}
                             for n, u0, k, le in inst],
               "cell_updates": sum(n ** 3 * k for n, _, k, _ in inst)}
    traces = {}
    for mode in modes:
        sims = []
        for n, u0, k, le in inst:
            L = n / (2.0 * math.pi)
            wp, wm = sg.trtOmegas(3.0 * u0 * L / 1600.0 + 0.5, None)
            s = sg.Simulation(gpu, precision=precision, nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm)
            s.initField(2, u0)
            sims.append(s)
        b = sg.Batch(gpu, sims, mode=mode)
        tuned = None
        if tune and mode not in ("sequential", "streams"):  # those keep each lattice's shape
            chosen, bx, by, _ = b.autotune(rounds=tune_rounds)  # tile shape (and mode), states restored
            b.mode = mode
            tuned = [bx, by]
        t0 = time.perf_counter()
        tr = b.run([k for _, _, k, _ in inst], [le for _, _, _, le in inst])
        wall = time.perf_counter() - t0
        results[mode] = {"wall_seconds": wall, "gpu_seconds": b.gpuSeconds, "path": b.lastPath,
                         "tile": tuned,
                         "glups": results["cell_updates"] / wall / 1e9,
                         "digests": [s.stateDigest[:16] for s in sims]}
        traces[mode] = tr
        b.close()
        for s in sims:
            s.close()
    if "sequential" in modes:
        seq = results["sequential"]["wall_seconds"]
        for m in modes:
            if m == "sequential":
                continue
            results[m]["speedup_vs_sequential"] = seq / results[m]["wall_seconds"]
            results[m]["identical_states"] = results[m]["digests"] == results["sequential"]["digests"]
            results[m]["max_trace_rel_diff"] = max(
                float(np.max(np.abs(x - y) / np.maximum(np.abs(y), 1e-300)))
                for x, y in zip(traces[m], traces["sequential"]))
    results["traces"] = {m: [list(map(float, t)) for t in traces[m]] for m in traces}
    return results


# ------------------------------------------------------ colormap buffer
def render(gpu, nx=512, ny=256, nz=256, D=48, steps=200, repeats=5, out_png=None):
    """Headless |u| colormap (colorize, Kernels.metal:465-500) of the sphere
    wake's mid slice after `steps` steps: device time of the render kernel,
    whole-call time (with the image read back), and the image's SHA-256.
    With out_png the image is written as an 8-bit PNG (no graphics API)."""
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = sg.Cell.inflow
    nu = 0.05 * D / 300.0
    wp, _ = sg.trtOmegas(3.0 * nu + 0.5, None)
    s = sg.Simulation(gpu, precision="fp16s", nx=nx, ny=ny, nz=nz, omega=wp, uin=0.05,
                      rampSteps=100, cSmago=0.01, flags=flags.reshape(-1))
    s.inflowUniform = True
    s.setSolidFractions(sg.sphereSolidFractions(nx, ny, nz, 128.0, ny / 2.0, nz / 2.0, D / 2.0, 8))
    s.run(steps)
    dev, wall = [], []
    img = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        img, sec = s.renderSlice(nz // 2, 0.08, timing=True)
        wall.append(time.perf_counter() - t0)
        dev.append(sec)
    s.close()
    if out_png:
        _write_png(out_png, img)
    return {"lattice": [nx, ny, nz], "slice": nz // 2, "pixels": nx * ny,
            "kernel_seconds": min(dev), "call_seconds": min(wall),
            "digest": hashlib.sha256(img.tobytes()).hexdigest()}


def _write_png(path, img):
    """8-bit RGB PNG of an (h, w, 4) float image in [0, 1] (zlib, no imaging library)."""
    import struct
    import zlib

    rgb = np.clip(np.rint(img[..., :3].astype(np.float32) * 255.0), 0, 255).astype(np.uint8)
    h, w = rgb.shape[:2]
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag, data):
        c = struct.pack(">I", len(data)) + tag + data
        return c + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
                 + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


# ------------------------------------------------------ STL voxelizer
def stl_voxelize(gpu, nx=512, ny=256, nz=256, D=48, segments=256, rings=128, repeats=3):
    """meshSolidFractions (StlVoxels.swift:52-117) on the GPU for the sphere
    wake's body: a lat-long sphere STL of diameter D cells centred at
    (128, ny/2, nz/2) of the 512x256x256 lattice. Reports the device time of
    the ray kernel, the end-to-end call time (host bucketing and transfers
    included), and the volume against the analytic sphere."""
    mesh = sg.StlMesh(sg.sphereSTLData(1.0, segments, rings))
    off = np.array([128.0, ny / 2.0, nz / 2.0], np.float32)
    scale = D / 2.0
    dev, wall = [], []
    eps = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        eps, sec = sg.meshSolidFractions(gpu, mesh, nx, ny, nz, scale, off, timing=True)
        wall.append(time.perf_counter() - t0)
        dev.append(sec)
    ana = sg.sphereSolidFractions(nx, ny, nz, 128.0, ny / 2.0, nz / 2.0, D / 2.0)
    vol, vol_a = float(eps.astype(np.float64).sum()), float(ana.astype(np.float64).sum())
    return {"lattice": [nx, ny, nz], "triangles": int(len(mesh.triangles)),
            "kernel_seconds": min(dev), "call_seconds": min(wall),
            "volume": vol, "volume_analytic": vol_a, "volume_rel_err": abs(vol - vol_a) / vol_a,
            "digest": hashlib.sha256(eps.tobytes()).hexdigest()}


# ------------------------------------------------------------ adjoints
def _dfg2_sim(gpu, D, uin_max, nz, precision, ramp, sponge_d=3, sponge_tau=1.0):
    nx = 22 * D + 2
    ny = int(4.1 * D) + 2
    umean = uin_max * 2.0 / 3.0
    wp, wm = sg.trtOmegas(3.0 * (umean * D / 100.0) + 0.5, 3.0 / 16.0)
    cx = cy = 0.5 + 2.0 * D
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, 0, :] = flags[:, -1, :] = sg.Cell.solid
    flags[:, 1:-1, 0] = flags[:, 1:-1, -1] = sg.Cell.inflow
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=wp, omegaMinus=wm,
                      uin=uin_max, rampSteps=ramp, wantsForces=True, flags=flags.reshape(-1))
    eps = np.tile(sg.diskSolidFractions(nx, ny, cx, cy, D / 2.0), nz)
    s.setSolidFractions(eps)
    s.sponge = (float(nx - 1 - sponge_d * D), float(sponge_d * D), sponge_tau)
    box = ((int(cx) - D // 2 - 3, int(cx) + D // 2 + 3), (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3))
    return s, eps, box, umean


def dfg2_adjoint(gpu, D=64, uin_max=0.06, nz=3, total=200000, window=10000, checkpoints=20,
                 fd_cells=8, fd_h=0.02, seed=7, precision="fp32", ramp=24000, tune=False,
                 fd_steps=(1.0, 0.5)):
    """Adjoint of the time-averaged C_D over the last `window` steps of the
    cylinder run with respect to the solid-fraction field (20 checkpoints),
    compared with central differences of the same FP32 forward on `fd_cells`
    random boundary cells with 0 < eps < 1, at step sizes fd_h * fd_steps (the
    spread between those shows what FP32 differences can resolve). Also times
    forward and backward."""
    s, eps, box, umean = _dfg2_sim(gpu, D, uin_max, nz, precision, ramp)
    if tune:
        s.autotune(steps=200)  # the forward's kernel and launch shape (state restored)
    s.run(total - window)
    start = s.downloadState()
    t_start = s.stepsDone
    norm = 2.0 / (umean * umean * D * nz)  # C_D = norm * F_x
    adj = sg.Adjoint(s, window, box, checkpoints=checkpoints)
    t0 = time.perf_counter()
    J = adj.forward()
    t1 = time.perf_counter()
    ge, _ = adj.backward()
    t2 = time.perf_counter()
    st = adj.stats()
    adj.close()
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero((eps > 0.05) & (eps < 0.95))
    cells = rng.choice(cand, size=min(fd_cells, cand.size), replace=False)
    fd = []
    for n in cells:
        ests = []
        for scale in fd_steps:
            h = fd_h * scale
            vals = []
            for sgn in (1.0, -1.0):
                e = eps.copy()
                e[n] = np.float32(e[n] + sgn * h)
                s.setSolidFractions(e)
                s.uploadState(start)
                s.stepsDone = t_start
                a2 = sg.Adjoint(s, window, box, checkpoints=1)
                vals.append(a2.forward())
                a2.close()
            h_eff = float(np.float32(eps[n] + h)) - float(np.float32(eps[n] - h))
            ests.append((vals[0] - vals[1]) / h_eff * norm)
        fd.append({"cell": int(n), "eps": float(eps[n]), "adjoint": float(ge[n]) * norm,
                   "fd": ests[0], "fd_steps": list(fd_steps), "fd_all": ests})
    s.setSolidFractions(eps)
    fwd_step = st["forward_s"] / window
    out = {"D": D, "window": window, "checkpoints": checkpoints, "mean_cd": J * norm,
           "fd": fd, "forward_seconds": st["forward_s"], "recompute_seconds": st["recompute_s"],
           "adjoint_seconds": st["adjoint_s"], "wall_forward": t1 - t0, "wall_backward": t2 - t1,
           "adjoint_step_over_forward_step": st["adjoint_s"] / window / fwd_step,
           "backward_over_forward": (st["recompute_s"] + st["adjoint_s"]) / st["forward_s"]}
    s.close()
    return out


def sphere_adjoint(gpu, nx=512, ny=256, nz=256, D=48, u=0.05, re=300.0, cs=0.1, spinup=4000,
                   window=2000, checkpoints=45, precision="fp16s", tune=False):
    """Adjoint of the mean drag over `window` steps of the sphere wake with
    respect to the Guo force field, sqrt(window) checkpoints: gradient
    statistics and the forward / backward device time."""
    nu = u * D / re
    wp, _ = sg.trtOmegas(3.0 * nu + 0.5, None)
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = sg.Cell.inflow
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=wp, uin=u,
                      rampSteps=min(8000, spinup), cSmago=cs * cs, wantsForces=True,
                      flags=flags.reshape(-1))
    s.inflowUniform = True
    cx, cy, cz = 128.0, ny / 2.0, nz / 2.0
    s.setSolidFractions(sg.sphereSolidFractions(nx, ny, nz, cx, cy, cz, D / 2.0, 8))
    s.setForceField(np.zeros((3, nx * ny * nz), np.float32))
    s.sponge = (float(nx - 1 - D), float(D), 1.0)
    box = ((int(cx) - D // 2 - 3, int(cx) + D // 2 + 3), (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3))
    if tune:
        s.autotune(steps=10)  # the forward's kernel and launch shape (state restored)
    s.run(spinup)
    adj = sg.Adjoint(s, window, box, checkpoints=checkpoints)
    J = adj.forward()
    _, gf = adj.backward()
    st = adj.stats()
    adj.close()
    area = u * u * math.pi * D * D / 4.0
    mag = np.sqrt((gf.astype(np.float64) ** 2).sum(0))
    out = {"lattice": [nx, ny, nz], "window": window, "checkpoints": checkpoints,
           "mean_cd": 2.0 * J / area, "grad_norm": float(np.linalg.norm(mag)),
           "grad_max_cell": int(np.argmax(mag)), "grad_finite": bool(np.isfinite(gf).all()),
           "forward_seconds": st["forward_s"], "recompute_seconds": st["recompute_s"],
           "adjoint_seconds": st["adjoint_s"],
           "adjoint_step_over_forward_step": st["adjoint_s"] / st["forward_s"],
           "backward_over_forward": (st["recompute_s"] + st["adjoint_s"]) / st["forward_s"]}
    s.close()
    return out


# ------------------------------------------------------------ credibility ladder
def credibility(gpu, resolutions=(32, 48, 64), base_mach=0.075, steps_factor=1.0,
                precision="fp32", report=None,
                modes=("sequential", "concurrent", "batched", "streams"), autotune=True):
    """The DFG 2D-2 credibility run (mean C_D; three resolutions and a half-Mach
    anchor at the finest) with the four checks the reference's credibility gate
    makes (Sources/strouhal/Cases.swift:1103-1160): a finite calibrated bar in
    the validated domain, a bar that reaches the published mean C_D 3.18 (within
    0.05), a ladder of every resolution, and a refusal out of the domain
    (Re 250000). Each mode in `modes` runs the whole ladder: the final lattices
    must be bitwise equal across modes, the QoIs equal (sequential, concurrent,
    streams) or equal to FP64 rounding (batched: box sums folded per tile)."""
    from . import credibility as cr
    case = cr.StreetLadder(baseMach=base_mach, precision=precision, stepsFactor=steps_factor)
    runs = {}
    for mode in modes:
        runs[mode] = cr.Ladder.credibility(gpu, case, "mean C_D", list(resolutions), mode=mode,
                                           autotune=autotune)
    first = runs[modes[0]]
    b = first.budget
    far = cr.ValidationDomain.classify(250000.0, 0.09, 48, "bluff body in channel")
    far_budget = cr.UncertaintyBudget("C_D", 1.0, 0.01, 0.01, 0.01, far)
    gates = {
        "calibrated_bar_in_domain": bool(math.isfinite(b.combined) and b.combined > 0),
        "bar_covers_published_mean_cd": bool(abs(b.value - 3.18) <= b.combined + 0.05),
        "ladder_recorded": len(first.rungs) == len(resolutions),
        "out_of_domain_refuses": bool(far.isOutside and math.isnan(far_budget.combined)),
    }
    md = cr.report_markdown(first, [
        "cavity (2-D, z-periodic, cubic), rotation, lid mass drift, Poiseuille, Taylor-Green "
        "order, DFG 2D-1 / 2D-2 and sphere gates: "
        "tests/test_gate_records.py over tests/records/",
        "every step kernel against the oracle: tests/test_gpu_parity.py"])
    if report:
        with open(report, "w") as fh:
            fh.write(md)
    gates["report_written"] = bool(report is None or os.path.exists(report))
    out = {"resolutions": list(resolutions), "base_mach": base_mach,
           "steps_factor": steps_factor, "precision": precision,
           "value": b.value, "u_num": b.uNum, "u_stat": b.uStat, "u_ma": b.uMa,
           "combined": b.combined, "headline": b.headline,
           "verdict": b.verdict.kind, "anchor": b.verdict.anchor,
           "observed_order": first.num.observedOrder,
           "stat_batches": first.stat.batches, "stat_lag1": first.stat.lag1,
           "mach_baseline": first.mach.baseline, "mach_half": first.mach.halfMach,
           "rungs": [[r.cellsPerFeature, r.value, r.stat] for r in first.rungs],
           "digest": first.digest, "cell_updates": first.cellUpdates, "gates": gates,
           "report_chars": len(md)}
    for mode, r in runs.items():
        out[mode + "_wall_seconds"] = r.wallSeconds
        out[mode + "_gpu_seconds"] = r.gpuSeconds
        out[mode + "_path"] = r.path
        # the final lattices bitwise equal; the QoIs equal (batched: to FP64 rounding)
        out[mode + "_digest_equal"] = r.digest == first.digest
        out[mode + "_max_rel_diff"] = max(
            [abs(a.value - b.value) / abs(b.value) for a, b in zip(r.rungs, first.rungs)] +
            [abs(r.mach.halfMach - first.mach.halfMach) / abs(first.mach.halfMach)])
    # every variant's sampled tail, for re-deriving the budget with the oracle's statistics
    out["series"] = first.series
    return out


CASES = {"poiseuille": poiseuille, "tg_order": tg_order, "cavity": cavity,
         "cavity_zperiodic": cavity_zperiodic, "cavity_cubic": cavity_cubic,
         "rotation": rotation, "mass_drift": mass_drift, "dfg1": dfg1, "dfg2": dfg2,
         "dfg2_adjoint": dfg2_adjoint, "tgv": tgv, "sphere": sphere,
         "sphere_adjoint": sphere_adjoint, "ladder": ladder, "stl_voxelize": stl_voxelize,
         "render": render, "credibility": credibility}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("name", choices=sorted(CASES))
    ap.add_argument("--out", default=None)
    ap.add_argument("--set", action="append", default=[],
                    help="key=value overrides of the case function's arguments")
    a = ap.parse_args(argv)
    kw = {}
    for item in a.set:
        k, v = item.split("=", 1)
        try:
            kw[k] = json.loads(v)
        except ValueError:
            kw[k] = v
    gpu = sg.GPU(0)
    t0 = time.perf_counter()
    res = CASES[a.name](gpu, **kw)
    res["case"] = a.name
    # the case and its overrides; where the output went is not part of the workload
    res["command"] = " ".join(["python -m strouhal_gb300.cases", a.name] +
                              ["--set " + item for item in a.set])
    res["elapsed_seconds"] = time.perf_counter() - t0
    text = json.dumps(res)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(text)
    summary = {k: v for k, v in res.items() if not isinstance(v, (list, dict))}
    print(json.dumps(summary))
    gpu.close()


if __name__ == "__main__":
    main()
