"""GPU discrete adjoint of the time-averaged dissipation (stro_adj_set_dissipation).

J = mean over the samples m = 1..K of the dissipation sum (stro_sim_dissipation:
2 nu S:S over the fluid cells) of the state after m * every steps of the
window. The GPU injects the hand-derived per-cell gradient of that sum into
its reverse sweep at every sample; the FP64 oracle differentiates its own
FP64 dissipation by dual numbers. Checked on the channel of test_gpu_adjoint
(velocity walls, Noble-Torczynski disk, LES, sponge, uniform force and a
per-cell force field): against the FP64 adjoint of the GPU's own FP32 / FP16
trajectory within 1e-3 normwise, and against FP64 central differences of the
FP64 forward within 1e-3."""
import numpy as np
import pytest

import test_gpu_adjoint as base

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,steps,every,checkpoints",
                         [("fp32", 14, 4, 3), ("fp32", 12, 4, 1), ("fp16s", 14, 4, 3),
                          ("fp16s", 12, 6, 2)])
def test_dissipation_adjoint_matches_fp64_adjoint_of_its_trajectory(gpu, oracle, precision,
                                                                     steps, every, checkpoints):
    import strouhal_gb300 as sg

    g, o, eps, _ = base._setup(sg, oracle, gpu, precision, seed=21)
    f0 = g.downloadState().astype(np.float64)
    adj = sg.Adjoint(g, steps, checkpoints=checkpoints, dissipationEvery=every)
    J = adj.forward()
    ge, gf = adj.backward()
    traj = "fp32" if precision == "fp32" else "fp16"
    Jo, geo, gfo = o.adjointDissipation(steps, every, trajectory=traj, f0=f0, threads=4)
    assert np.isfinite(J) and J > 0
    # the GPU forms each cell's term in FP32, the oracle in FP64 from the same states
    assert abs(J - Jo) <= 1e-4 * abs(Jo), (J, Jo)
    nt = eps != 0
    assert np.all(ge[~nt] == 0)
    assert base._rel(ge[nt], geo[nt]) < 1e-3, base._rel(ge[nt], geo[nt])
    assert base._rel(gf, gfo) < 1e-3, base._rel(gf, gfo)
    assert g.stepsDone == steps
    adj.close()
    g.close()


def test_dissipation_adjoint_agrees_with_fp64_central_differences(gpu, oracle):
    import strouhal_gb300 as sg

    steps, every = 14, 4
    g, o, eps, ff = base._setup(sg, oracle, gpu, "fp32", seed=23)
    f0 = g.downloadState().astype(np.float64)
    adj = sg.Adjoint(g, steps, checkpoints=3, dissipationEvery=every)
    adj.forward()
    ge, gf = adj.backward()
    adj.close()
    g.close()

    def J64(eps_v=None, ff_v=None):
        if eps_v is not None:
            o.setSolidFractions(eps_v)
        if ff_v is not None:
            o.setForceField(ff_v)
        J = o.adjointDissipation(steps, every, grads=False, f0=f0, threads=4)[0]
        o.setSolidFractions(eps)
        o.setForceField(ff)
        return J

    rng = np.random.default_rng(5)
    part = np.flatnonzero((eps > 0.05) & (eps < 0.95))
    emax, fmax = float(np.max(np.abs(ge))), float(np.max(np.abs(gf)))
    for n in rng.choice(part, 4, replace=False):
        h = 2.0 ** -12
        ep, em = eps.copy(), eps.copy()
        ep[n] += h
        em[n] -= h
        fd = (J64(eps_v=ep) - J64(eps_v=em)) / (float(ep[n]) - float(em[n]))
        assert abs(fd - ge[n]) <= 1e-3 * max(abs(fd), 1e-2 * emax), (n, fd, ge[n])
    fluid = np.flatnonzero(o.flags == 0)
    for n in rng.choice(fluid, 4, replace=False):
        h = 2.0 ** -16
        fp, fm = ff.copy(), ff.copy()
        fp[0, n] += h
        fm[0, n] -= h
        fd = (J64(ff_v=fp) - J64(ff_v=fm)) / (float(fp[0, n]) - float(fm[0, n]))
        assert abs(fd - gf[0, n]) <= 1e-3 * max(abs(fd), 1e-2 * fmax), (n, fd, gf[0, n])


def test_dissipation_adjoint_preconditions(gpu, oracle):
    import strouhal_gb300 as sg

    g, o, _, _ = base._setup(sg, oracle, gpu, "fp32", seed=2)
    for every in (3, 0, 40):  # odd, zero, beyond the window
        with pytest.raises(sg.StrouhalError):
            sg.Adjoint(g, 12, dissipationEvery=every)
    g.run(1)  # the window would start at an odd step count
    adj = sg.Adjoint(g, 12, dissipationEvery=4)
    with pytest.raises(sg.StrouhalError):
        adj.forward()
    adj.close()
    g.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_dissipation_adjoint_long_window_on_a_taylor_green_box(gpu, oracle, precision):
    """Periodic 32^3 Taylor-Green box (Re 1600 scaling, u0 0.05) with a
    nonzero per-cell force field: a 400-step window sampled every 40 steps
    with 20 checkpoints. dJ/dF against the FP64 adjoint of the GPU's own
    trajectory within 1e-3 normwise, and against FP64 central differences of
    the FP64 forward within 1e-3 (FP32 storage) or the FP16 bar 2e-2: the
    gradient about a 400-step FP16-storage trajectory is itself up to 7.5e-3
    away from the gradient about the FP64 one (FP64 adjoints of both)."""
    import strouhal_gb300 as sg

    po = oracle
    n, steps, every = 32, 400, 40
    L = n / (2 * np.pi)
    tau = 3 * 0.05 * L / 1600 + 0.5
    g = sg.Simulation(gpu, precision=precision, nx=n, ny=n, nz=n, omega=1 / tau)
    o = po.OracleSim(n, n, n, kind=po.KIND_F64, omega=1 / tau)
    rng = np.random.default_rng(8)
    ff = (rng.standard_normal((3, n ** 3)) * 2e-6).astype(np.float32)
    ff[:, rng.random(n ** 3) < 0.3] = 0.0
    g.setForceField(ff)
    o.setForceField(ff)
    g.initField(2, 0.05)
    f0 = g.downloadState().astype(np.float64)
    adj = sg.Adjoint(g, steps, checkpoints=20, dissipationEvery=every)
    J = adj.forward()
    _, gf = adj.backward()
    adj.close()
    g.close()
    traj = "fp32" if precision == "fp32" else "fp16"
    Jo, _, gfo = o.adjointDissipation(steps, every, trajectory=traj, f0=f0, checkpoint=20)
    assert abs(J - Jo) <= 1e-4 * abs(Jo), (J, Jo)
    assert np.all(np.isfinite(gf))
    assert base._rel(gf, gfo) < 1e-3, base._rel(gf, gfo)
    fmax = float(np.max(np.abs(gf)))
    for idx in rng.choice(n ** 3, 2, replace=False):
        # a small step: over 400 nearly inviscid steps a one-cell force of 2^-14
        # already moves J out of its linear range (2.9e-3 off at 2^-14, 7e-7 at 2^-20)
        h = 2.0 ** -20
        fp, fm = ff.copy(), ff.copy()
        fp[0, idx] += h
        fm[0, idx] -= h
        vals = []
        for v in (fp, fm):
            o.setForceField(v)
            vals.append(o.adjointDissipation(steps, every, grads=False, f0=f0)[0])
        o.setForceField(ff)
        fd = (vals[0] - vals[1]) / (float(fp[0, idx]) - float(fm[0, idx]))
        bar = 1e-3 if precision == "fp32" else 2e-2
        assert abs(fd - gf[0, idx]) <= bar * max(abs(fd), 1e-2 * fmax), (idx, fd, gf[0, idx])
