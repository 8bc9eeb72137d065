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
