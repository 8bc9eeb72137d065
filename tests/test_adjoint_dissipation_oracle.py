"""The FP64 oracle's adjoint of the time-averaged dissipation (CPU).

J = mean over the samples m = 1..K of the dissipation sum (2 nu S:S over the
fluid cells, the observable of Cases.swift:1254-1270 as the library sums it)
of the state after m * every steps. The oracle differentiates its FP64 step by
dual numbers and sweeps the window in reverse; here its J is checked against
the observables of a plain FP64 run and its gradients against FP64 central
differences, on a channel with velocity walls, Noble-Torczynski cells, LES, a
sponge, a uniform force and a per-cell force field."""
import numpy as np
import pytest

NX, NY, NZ = 24, 14, 3
KW = dict(omega=1.6, omegaMinus=1.25, uin=0.04, force=(1e-5, 0.0, 0.0), cSmago=0.01,
          wantsForces=True)


def _sim(po, seed=3):
    fl = np.zeros((NZ, NY, NX), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = po.INFLOW
    fl = fl.reshape(-1)
    o = po.OracleSim(NX, NY, NZ, flags=fl, kind=po.KIND_F64, **KW)
    o.sponge = (16.0, 6.0, 0.9)
    rng = np.random.default_rng(seed)
    eps = np.zeros(NX * NY * NZ, np.float32)
    xs, ys = np.meshgrid(np.arange(NX), np.arange(NY))
    disk = ((xs - 8.5) ** 2 + (ys - 6.5) ** 2 < 3.2 ** 2).reshape(-1)
    eps2 = np.where(disk, rng.uniform(0.1, 1.0, disk.size), 0.0).astype(np.float32)
    eps[:] = np.tile(eps2, NZ)
    o.setSolidFractions(eps)
    ff = (rng.standard_normal((3, NX * NY * NZ)) * 5e-6).astype(np.float32)
    ff[:, rng.random(NX * NY * NZ) < 0.3] = 0.0
    o.setForceField(ff)
    f0 = rng.standard_normal((19, NX * NY * NZ)) * 2e-3
    f0[:, fl != 0] = 0.0
    o.f[:] = f0
    return o, eps, ff, f0


def test_dissipation_objective_equals_sampled_observables(oracle):
    po = oracle
    o, _, _, f0 = _sim(po)
    steps, every = 12, 4
    J, _, _ = o.adjointDissipation(steps, every, grads=False, threads=1)
    samples = []
    for _ in range(steps // every):
        o.run(every)
        samples.append(o.observables()[1])
    assert np.isclose(J, np.mean(samples), rtol=1e-12, atol=0.0), (J, samples)


@pytest.mark.parametrize("checkpoint", [0, 5])
def test_dissipation_adjoint_matches_fp64_central_differences(oracle, checkpoint):
    po = oracle
    o, eps, ff, f0 = _sim(po)
    steps, every = 14, 4  # the final state (14) is not a sample; 4, 8, 12 are
    J, ge, gf = o.adjointDissipation(steps, every, threads=2, checkpoint=checkpoint)
    assert np.all(np.isfinite(ge)) and np.all(np.isfinite(gf))
    assert np.all(ge[eps == 0] == 0.0)

    def J_with(eps_v=None, ff_v=None):
        q, _, _, _ = _sim(po)
        if eps_v is not None:
            q.setSolidFractions(eps_v)
        if ff_v is not None:
            q.setForceField(ff_v)
        return q.adjointDissipation(steps, every, grads=False, threads=1)[0]

    rng = np.random.default_rng(11)
    part = np.flatnonzero((eps > 0.05) & (eps < 0.95))
    for n in rng.choice(part, 3, replace=False):
        h = 2.0 ** -12
        ep, em = eps.copy(), eps.copy()
        ep[n] += h
        em[n] -= h
        fd = (J_with(eps_v=ep) - J_with(eps_v=em)) / (float(ep[n]) - float(em[n]))
        assert abs(fd - ge[n]) <= 1e-5 * max(abs(fd), 1e-3 * np.max(np.abs(ge))), (n, fd, ge[n])
    fluid = np.flatnonzero(o.flags == 0)
    for n in rng.choice(fluid, 3, replace=False):
        for k in (0, 1):
            h = 2.0 ** -16
            fp, fm = ff.copy(), ff.copy()
            fp[k, n] += h
            fm[k, n] -= h
            fd = (J_with(ff_v=fp) - J_with(ff_v=fm)) / (float(fp[k, n]) - float(fm[k, n]))
            scale = max(abs(fd), 1e-3 * np.max(np.abs(gf)))
            assert abs(fd - gf[k, n]) <= 1e-5 * scale, (n, k, fd, gf[k, n])


def test_dissipation_adjoint_final_state_sample(oracle):
    """every divides steps: the final state is a sample and its gradient is
    injected before the first reverse step."""
    po = oracle
    o, eps, ff, f0 = _sim(po, seed=5)
    steps, every = 8, 4
    J, ge, gf = o.adjointDissipation(steps, every, threads=1)
    n = int(np.flatnonzero(o.flags == 0)[40])
    h = 2.0 ** -16

    def J_ff(v):
        q, _, _, _ = _sim(po, seed=5)
        q.setForceField(v)
        return q.adjointDissipation(steps, every, grads=False, threads=1)[0]

    fp, fm = ff.copy(), ff.copy()
    fp[0, n] += h
    fm[0, n] -= h
    fd = (J_ff(fp) - J_ff(fm)) / (float(fp[0, n]) - float(fm[0, n]))
    assert abs(fd - gf[0, n]) <= 1e-5 * max(abs(fd), 1e-3 * np.max(np.abs(gf))), (fd, gf[0, n])
