"""Conservation of the step operator, checked on the FP64 oracle (CPU).

Halfway bounce-back on resting walls returns every DDF that leaves a fluid
cell to it, the collision conserves mass per cell, and the Noble-Torczynski
term B (f_opp - f) sums to zero over the directions, so a closed box with
resting walls and solid-fraction cells keeps its total mass (the sum of the
shifted DDFs, massSum) to FP64 rounding, with any force, sponge or LES. A
periodic box also keeps its momentum up to exactly the applied force. The GPU
steps are equal in value to the FP32 oracle, which is the same operator."""
import numpy as np
import pytest


def _box(po, nx, ny, nz):
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, :, 0] = fl[:, :, -1] = po.SOLID
    fl[0, :, :] = fl[-1, :, :] = po.SOLID
    fl[3:5, 4:6, 5:7] = po.SOLID  # an obstacle
    return fl.reshape(-1)


def _mass(po, o):
    fluid = o.flags == po.FLUID
    return float(np.sum(o.f[:, fluid], dtype=np.float64))


@pytest.mark.parametrize("les,collision", [(0.0, "reference"), (0.02, "reference"), (0.0, "kbc")])
def test_closed_box_conserves_mass(oracle, les, collision):
    po = oracle
    nx, ny, nz = 12, 10, 8
    flags = _box(po, nx, ny, nz)
    o = po.OracleSim(nx, ny, nz, omega=1.5, omegaMinus=1.2, force=(3e-5, -2e-5, 1e-5),
                     cSmago=les, flags=flags, kind=po.KIND_F64)
    o.collision = collision
    if collision == "reference":  # solid-fraction cells and a sponge join the TRT run
        rng0 = np.random.default_rng(5)
        eps = np.zeros(nx * ny * nz, np.float32)
        inner = np.flatnonzero(flags == po.FLUID)
        pick = rng0.choice(inner, 40, replace=False)
        eps[pick] = rng0.uniform(0.1, 0.9, pick.size).astype(np.float32)
        o.setSolidFractions(eps)
        o.sponge = (7.0, 3.0, 0.9)
    rng = np.random.default_rng(3)
    f0 = rng.standard_normal((19, nx * ny * nz)) * 0.01
    f0[:, flags != po.FLUID] = 0.0
    o.f[:] = f0
    m0 = _mass(po, o)
    o.run(6)
    assert abs(_mass(po, o) - m0) <= 1e-12 * max(1.0, np.sum(np.abs(f0)))


def test_periodic_box_momentum_changes_by_the_force(oracle):
    """Per step the Guo forcing adds F to every cell's momentum, so a periodic
    box of N cells gains N F per step (momentum from the natural-order slots
    after an even number of steps)."""
    po = oracle
    nx, ny, nz = 8, 6, 5
    F = np.array([3e-5, -2e-5, 1e-5], np.float32).astype(np.float64)
    o = po.OracleSim(nx, ny, nz, omega=1.5, omegaMinus=1.1, force=tuple(F), kind=po.KIND_F64)
    rng = np.random.default_rng(9)
    o.f[:] = rng.standard_normal((19, nx * ny * nz)) * 0.01
    c = np.stack([po.CX, po.CY, po.CZ], axis=1).astype(np.float64)

    def momentum():
        return c.T @ np.sum(o.f, axis=1)

    p0 = momentum()
    steps = 4
    o.run(steps)
    gained = momentum() - p0
    expect = steps * nx * ny * nz * F
    assert np.allclose(gained, expect, rtol=1e-9, atol=1e-13), (gained, expect)
