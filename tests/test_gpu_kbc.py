"""The KBC collision on the GPU: DDFs EQUAL in value to the oracle's KBC for
both storages and arithmetics, every geometry feature it supports and the
bulk / boundary split; the refusals; and the transitional Taylor-Green
vortex at Re 1600 on 128^3 (u0 = 0.1), where the reference measured its TRT
going non-finite at t* = 5.4 (Sources/strouhal/Cases.swift:1290-1302): KBC
stays finite through the decay."""
import math

import numpy as np
import pytest

import strouhal_gb300 as sg

pytestmark = pytest.mark.gpu

PREC = {0: "fp32", 1: "fp16s"}


def flags_walls(po, nx, ny, nz):
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = po.SOLID
    fl[:, -1, :] = po.LID
    fl[:, 1:-1, 0] = po.INFLOW
    fl[:, 1:-1, -1] = po.OUTFLOW
    fl[:, 6:8, 10:12] = po.SOLID
    return fl.reshape(-1)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("arith", ["reference", "fused"])
@pytest.mark.parametrize("geometry", ["periodic", "walls"])
@pytest.mark.parametrize("split", [True, False, "columns", "merged", "pair"])
def test_kbc_matches_oracle(gpu, oracle, kind, arith, geometry, split):
    po = oracle
    nx, ny, nz = 35, 16, 5
    N = nx * ny * nz
    rng = np.random.default_rng(11 + kind + 2 * (arith == "fused") + 4 * (geometry == "walls"))
    flags = flags_walls(po, nx, ny, nz) if geometry == "walls" else None
    kw = dict(omega=1.6, omegaMinus=1.6, lid=(0.04, 0.0, 0.01), uin=0.03, rampSteps=6,
              force=(2e-5, -1e-5, 0.0), wantsForces=True)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=nx, ny=ny, nz=nz, flags=flags,
                      arithmetic=arith, **kw)
    o = po.OracleSim(nx, ny, nz, flags=flags, kind=kind, arithmetic=arith, **kw)
    g.collision = o.collision = "kbc"
    assert g.collision == "kbc"
    g.outflowMode = o.outflowMode = "pressure"
    g.sponge = o.sponge = (24.0, 8.0, 0.9)
    ff = (rng.standard_normal((3, N)) * 1e-5).astype(np.float32)
    ff[:, rng.choice(N, N // 3, replace=False)] = 0.0  # cells with zero total force
    ff[0] -= 2e-5
    ff[1] += 1e-5
    g.setForceField(ff)
    o.setForceField(ff)
    g.setBlockSplit(split)
    g.block = (32, 2)
    f0 = (rng.standard_normal((19, N)) * 0.01).astype(o.f.dtype)
    o.f[:] = f0
    g.uploadState(f0)
    for chunk in (1, 4, 3):
        g.run(chunk)
        o.run(chunk)
        assert np.array_equal(g.downloadState(), o.f), (chunk, g.stepsDone)
        # KBC has no pair form: "pair" runs the merged one-cell lists
        assert g.lastPath in ("cell", "split", "split-merged")
    if geometry == "walls":
        box = ((2, 30), (1, 14))
        fg, fo = g.probeForce(*box), o.probeForce(*box)
        assert np.allclose(fg, fo, rtol=1e-12, atol=1e-12), (fg, fo)
        assert np.array_equal(g.downloadState(), o.f)
    g.close()


def test_kbc_runs_on_one_cell_kernels_only(gpu, oracle):
    """Variants 1-3 have no KBC kernels: a KBC lattice runs the one-cell
    kernel whatever variant is asked for, and the autotuner keeps variant 0."""
    po = oracle
    n = 64
    g = sg.Simulation(gpu, precision="fp16s", nx=n, ny=n, nz=4, omega=1.9)
    o = po.OracleSim(n, n, 4, 1.9, kind=1)
    g.collision = o.collision = "kbc"
    o.initField(1, 0.05)
    g.uploadState(o.f)
    for variant in (1, 2, 3):
        g.variant = variant
        g.run(2)
        o.run(2)
        assert g.lastPath == "cell"
        assert np.array_equal(g.downloadState(), o.f)
    g.autotune(steps=4)
    assert g.variant == 0
    g.close()


def test_kbc_refusals(gpu):
    fl = np.zeros(16 * 8 * 2, np.uint8)
    s = sg.Simulation(gpu, nx=16, ny=8, nz=2, omega=1.5, cSmago=0.01, wantsForces=True, flags=fl)
    with pytest.raises(sg.StrouhalError):
        s.collision = "kbc"  # LES is the reference collision's subgrid model
    s.cSmago = 0.0
    eps = np.zeros(s.cells, np.float32)
    eps[5] = 0.5
    s.setSolidFractions(eps)
    with pytest.raises(sg.StrouhalError):
        s.collision = "kbc"  # no Noble-Torczynski cells
    s.setSolidFractions(np.zeros(s.cells, np.float32))
    s.collision = "kbc"
    with pytest.raises(sg.StrouhalError):
        s.cSmago = 0.01
    with pytest.raises(sg.StrouhalError):
        s.setSolidFractions(eps)
    with pytest.raises(sg.StrouhalError):
        sg.Batch(gpu, [s])
    with pytest.raises(sg.StrouhalError):
        sg.Adjoint(s, 4, ((1, 8), (1, 6)))
    s.close()


def _tgv_finite_until(gpu, collision, lam, t_end, n=128, u0=0.1):
    L = n / (2.0 * math.pi)
    tau = 3.0 * u0 * L / 1600.0 + 0.5
    wp, wm = sg.trtOmegas(tau, lam)
    s = sg.Simulation(gpu, nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm)
    s.collision = collision
    s.initField(2, u0)
    tc = L / u0
    chunk = int(tc / 2) & ~1
    E0 = s.kineticEnergySum()
    E = [E0]
    while s.stepsDone < t_end * tc:
        s.run(chunk)
        E.append(s.kineticEnergySum())
        if not math.isfinite(E[-1]):
            t = s.stepsDone / tc
            s.close()
            return t, E
    s.close()
    return None, E


def test_kbc_carries_the_transitional_tgv_that_trt_loses(gpu):
    t_trt, _ = _tgv_finite_until(gpu, "reference", 0.25, 8.0)
    assert t_trt is not None and t_trt < 8.0  # the reference measured t* = 5.4
    t_kbc, E = _tgv_finite_until(gpu, "kbc", None, 14.0)
    assert t_kbc is None
    assert all(b <= a for a, b in zip(E, E[1:]))  # the energy only decays
    assert 0.15 < E[-1] / E[0] < 0.45  # about 0.3 of it is left at t* = 14 in the DNS
