"""Outflow walls on the GPU against the oracle: the reference's dormant wall
and the pressure wall (STRO_OUTFLOW_PRESSURE) must give DDFs EQUAL in value
to the oracle's, for both storages and arithmetics, with and without the
bulk / boundary split, in batches, and over a full plane-Poiseuille run."""
import numpy as np
import pytest

import strouhal_gb300 as sg

pytestmark = pytest.mark.gpu

PREC = {0: "fp32", 1: "fp16s"}


def channel_flags(po, nx, ny, nz):
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, 1:-1, 0] = po.INFLOW
    fl[:, 1:-1, -1] = po.OUTFLOW
    fl[:, 5:7, 9:11] = po.SOLID
    return fl.reshape(-1)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("mode", ["dormant", "pressure"])
@pytest.mark.parametrize("arith", ["reference", "fused"])
@pytest.mark.parametrize("split", [True, False, "columns"])
def test_outflow_matches_oracle(gpu, oracle, kind, mode, arith, split):
    po = oracle
    nx, ny, nz = 33, 14, 4
    rng = np.random.default_rng(5 + kind + 2 * (mode == "pressure") + 4 * (arith == "fused"))
    flags = channel_flags(po, nx, ny, nz)
    kw = dict(omega=1.45, omegaMinus=1.1, uin=0.04, rampSteps=5, cSmago=0.01, wantsForces=True)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=nx, ny=ny, nz=nz, flags=flags,
                      arithmetic=arith, **kw)
    o = po.OracleSim(nx, ny, nz, flags=flags, kind=kind, arithmetic=arith, **kw)
    g.outflowMode = o.outflowMode = mode
    assert g.outflowMode == mode
    g.sponge = o.sponge = (20.0, 10.0, 0.9)
    eps = np.zeros(nx * ny * nz, np.float32)
    idx = rng.choice(nx * ny * nz, 60, replace=False)
    eps[idx] = rng.uniform(0.05, 0.95, idx.size).astype(np.float32)
    g.setSolidFractions(eps)
    o.setSolidFractions(eps)
    g.setBlockSplit(split)
    g.block = (32, 2)
    f0 = (rng.standard_normal((19, nx * ny * nz)) * 0.01).astype(o.f.dtype)
    o.f[:] = f0
    g.uploadState(f0)
    for chunk in (1, 4, 3):
        g.run(chunk)
        o.run(chunk)
        assert np.array_equal(g.downloadState(), o.f), (chunk, g.stepsDone)
    box = ((20, 32), (1, 12))  # includes the outflow column
    fg, fo = g.probeForce(*box), o.probeForce(*box)
    assert np.allclose(fg, fo, rtol=1e-12, atol=1e-12), (fg, fo)
    assert np.array_equal(g.downloadState(), o.f)
    g.close()


def test_pressure_outflow_poiseuille_run_equals_oracle(gpu, oracle):
    """8,000 steps of a 96 x 18 channel, parabolic inlet, pressure outflow: the
    GPU state equals the FP32 oracle's bit for bit, and the profile next to the
    outlet is Poiseuille."""
    po = oracle
    nx, ny, H, tau, u_in = 96, 18, 16, 0.8, 0.05
    fl = np.zeros((1, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, 1:-1, 0] = po.INFLOW
    fl[:, 1:-1, -1] = po.OUTFLOW
    wp, wm = sg.trtOmegas(tau, 3.0 / 16.0)
    kw = dict(omega=wp, omegaMinus=wm, uin=u_in, rampSteps=1000, flags=fl.reshape(-1))
    g = sg.Simulation(gpu, nx=nx, ny=ny, nz=1, **kw)
    o = po.OracleSim(nx, ny, 1, kind=po.KIND_F32, threads=4, **kw)
    g.outflowMode = o.outflowMode = "pressure"
    g.run(8000)
    o.run(8000)
    assert np.array_equal(g.downloadState(), o.f)
    m = g.probeMoments().reshape(ny, nx, 4)
    yd = np.arange(ny) - 0.5
    prof = np.maximum(4.0 * u_in * yd * (H - yd) / H ** 2, 0.0)[1:-1]
    assert np.abs(m[1:-1, nx - 2, 0] - prof).max() < 2e-3
    g.close()


@pytest.mark.parametrize("mode", ["persistent", "rounds"])
def test_pressure_outflow_in_a_batch(gpu, mode):
    """Batched steps with pressure outflow walls equal single-lattice steps."""
    from oracle import pyoracle as po

    sims, solo = [], []
    for nx in (40, 64):
        for lst in (sims, solo):
            s = sg.Simulation(gpu, nx=nx, ny=14, nz=2, omega=1.3, omegaMinus=1.0, uin=0.04,
                              rampSteps=10, flags=channel_flags(po, nx, 14, 2))
            s.outflowMode = "pressure"
            lst.append(s)
    for s in solo:
        s.run(30)
    b = sg.Batch(gpu, sims, mode=mode)
    b.run([30, 24])
    b.close()
    solo[1].close()
    solo[1] = sg.Simulation(gpu, nx=64, ny=14, nz=2, omega=1.3, omegaMinus=1.0, uin=0.04,
                            rampSteps=10, flags=channel_flags(po, 64, 14, 2))
    solo[1].outflowMode = "pressure"
    solo[1].run(24)
    for a, b in zip(sims, solo):
        assert a.stepsDone == b.stepsDone
        assert a.stateDigest == b.stateDigest
        a.close()
        b.close()


def test_adjoint_refuses_the_pressure_outflow(gpu):
    from oracle import pyoracle as po

    s = sg.Simulation(gpu, nx=32, ny=14, nz=2, omega=1.3, uin=0.04, wantsForces=True,
                      flags=channel_flags(po, 32, 14, 2))
    s.outflowMode = "pressure"
    with pytest.raises(sg.StrouhalError):
        sg.Adjoint(s, 10, ((20, 30), (1, 12)))
    s.close()
