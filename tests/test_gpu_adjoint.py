"""GPU discrete adjoint (stro_adj_*) against the FP64 oracle.

The oracle's adjoint differentiates the restated reference arithmetic with
forward-mode dual numbers in FP64 (exact local Jacobians); the GPU adjoint is a
hand-written reverse pass in FP32. The objective is the time-averaged drag on
a Noble-Torczynski cylinder in a channel with velocity walls, LES, a uniform
Guo force, a sponge and a per-cell force field."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, NZ = 32, 18, 3
BOX = ((4, 17), (2, 15))


def _flags(po):
    fl = np.zeros((NZ, NY, NX), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = po.INFLOW
    return fl.reshape(-1)


KW = dict(omega=1.6, omegaMinus=1.25, uin=0.04, force=(1e-5, 0.0, 0.0), cSmago=0.01,
          wantsForces=True)


def _setup(sg, po, gpu, precision, seed=0):
    import strouhal_gb300 as _sg  # noqa: F401

    fl = _flags(po)
    g = sg.Simulation(gpu, precision=precision, nx=NX, ny=NY, nz=NZ, flags=fl, **KW)
    o = po.OracleSim(NX, NY, NZ, flags=fl, kind=po.KIND_F64, **KW)
    g.sponge = o.sponge = (22.0, 8.0, 0.9)
    eps = np.tile(sg.diskSolidFractions(NX, NY, 10.5, 8.5, 3.5), NZ)
    g.setSolidFractions(eps)
    o.setSolidFractions(eps)
    rng = np.random.default_rng(seed)
    # a nonzero per-cell Guo force field, some cells without a field force
    ff = (rng.standard_normal((3, NX * NY * NZ)) * 5e-6).astype(np.float32)
    ff[:, rng.random(NX * NY * NZ) < 0.3] = 0.0
    g.setForceField(ff)
    o.setForceField(ff)
    dt = np.float32 if precision == "fp32" else np.float16
    f0 = (rng.standard_normal((19, NX * NY * NZ)) * 2e-3).astype(dt)
    f0[:, fl != 0] = 0
    g.uploadState(f0)
    o.f[:] = f0.astype(np.float64)
    return g, o, eps, ff


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("steps,checkpoints", [(12, 3), (9, 2)])
def test_adjoint_matches_fp64_oracle(gpu, oracle, steps, checkpoints):
    import strouhal_gb300 as sg

    g, o, eps, _ = _setup(sg, oracle, gpu, "fp32")
    adj = sg.Adjoint(g, steps, BOX, checkpoints=checkpoints)
    J = adj.forward()
    ge, gf = adj.backward()
    Jo, geo, gfo = o.adjointForce(steps, BOX)
    assert abs(J - Jo) <= 1e-5 * abs(Jo) + 1e-12, (J, Jo)
    nt = eps != 0
    assert _rel(ge[nt], geo[nt]) < 1e-3
    assert np.all(ge[~nt] == 0)
    assert _rel(gf, gfo) < 1e-3
    assert g.stepsDone == steps
    # the forward with the field present ran the reference arithmetic
    o2 = oracle.OracleSim(NX, NY, NZ, flags=_flags(oracle), kind=oracle.KIND_F32, **KW)
    o2.sponge = (22.0, 8.0, 0.9)
    o2.setSolidFractions(eps)
    o2.setForceField(o.forceField)
    o2.f[:] = o.f.astype(np.float32)
    o2.run(steps)
    assert np.array_equal(g.downloadState(), o2.f)
    st = adj.stats()
    assert st["adjoint_steps"] == steps and st["adjoint_s"] > 0
    adj.close()


def test_adjoint_agrees_with_finite_differences(gpu, oracle):
    """Central differences of the FP64 forward, steps exactly representable in FP32."""
    import strouhal_gb300 as sg

    steps = 10
    g, o, eps, ff = _setup(sg, oracle, gpu, "fp32", seed=3)
    adj = sg.Adjoint(g, steps, BOX, checkpoints=2)
    adj.forward()
    ge, gf = adj.backward()
    scale_e = np.abs(ge).max()
    cells = np.flatnonzero((eps > 0.2) & (eps < 0.8))[:4]
    h = 2.0 ** -12
    for n in cells:
        e = eps.copy()
        e[n] += h
        o.setSolidFractions(e)
        Jp, _, _ = o.adjointForce(steps, BOX, grads=False)
        e[n] -= 2 * h
        o.setSolidFractions(e)
        Jm, _, _ = o.adjointForce(steps, BOX, grads=False)
        fd = (Jp - Jm) / (2 * h)
        assert abs(ge[n] - fd) <= 1e-3 * max(abs(fd), 1e-2 * scale_e), (n, ge[n], fd)
    o.setSolidFractions(eps)
    scale_f = np.abs(gf).max()
    for n, k in [(6 * NX + 8, 0), (9 * NX + 14 + NX * NY, 1), (4 * NX + 20, 0)]:
        f = ff.copy()
        f[k, n] = np.float32(ff[k, n] + h)
        o.setForceField(f)
        Jp, _, _ = o.adjointForce(steps, BOX, grads=False)
        f[k, n] = np.float32(ff[k, n] - h)
        o.setForceField(f)
        Jm, _, _ = o.adjointForce(steps, BOX, grads=False)
        h2 = float(np.float32(ff[k, n] + h)) - float(np.float32(ff[k, n] - h))
        fd = (Jp - Jm) / h2
        assert abs(gf[k, n] - fd) <= 1e-3 * max(abs(fd), 1e-2 * scale_f), (n, k, gf[k, n], fd)
    adj.close()


def test_adjoint_checkpoint_count_does_not_change_the_gradient(gpu, oracle):
    import strouhal_gb300 as sg

    out = []
    for ck in (1, 4, 14):
        g, _, _, _ = _setup(sg, oracle, gpu, "fp32", seed=5)
        adj = sg.Adjoint(g, 14, BOX, checkpoints=ck)
        J = adj.forward()
        ge, gf = adj.backward()
        out.append((J, ge, gf))
        adj.close()
    for J, ge, gf in out[1:]:
        assert J == out[0][0]
        assert np.array_equal(ge, out[0][1]) and np.array_equal(gf, out[0][2])


def test_adjoint_fp16_storage(gpu, oracle):
    import strouhal_gb300 as sg

    g, o, eps, _ = _setup(sg, oracle, gpu, "fp16s", seed=7)
    adj = sg.Adjoint(g, 8, BOX, checkpoints=2)
    J = adj.forward()
    ge, gf = adj.backward()
    Jo, geo, gfo = o.adjointForce(8, BOX)
    assert abs(J - Jo) <= 2e-3 * abs(Jo)
    nt = eps != 0
    assert _rel(ge[nt], geo[nt]) < 2e-2
    assert _rel(gf, gfo) < 2e-2
    adj.close()


def test_adjoint_merged_split_is_bitwise_neutral(gpu, oracle):
    """FP16 storage: the forward window and the segment recomputation (out of
    place) with the bulk and x-face blocks in one launch, one or two cells per
    thread, give the objective and gradients of the default split bit for bit."""
    import strouhal_gb300 as sg

    out = []
    for split in (True, "merged", "pair"):
        g, o, eps, _ = _setup(sg, oracle, gpu, "fp16s", seed=11)
        g.block = (8, 4)  # 8-wide blocks leave bulk blocks between the disk and the walls
        g.setBlockSplit(split)
        adj = sg.Adjoint(g, 10, BOX, checkpoints=3)
        J = adj.forward()
        ge, gf = adj.backward()
        if split != True:  # noqa: E712
            assert g.lastPath == "split-" + split, g.lastPath
            assert g.splitBlocks[0] > 0 and g.splitBlocks[1] > 0
        out.append((J, ge, gf))
        adj.close()
        g.close()
    for J, ge, gf in out[1:]:
        assert J == out[0][0]
        assert np.array_equal(ge, out[0][1]) and np.array_equal(gf, out[0][2])
