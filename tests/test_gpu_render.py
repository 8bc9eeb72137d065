"""Headless |u| colormap (stro_sim_render_slice) against the oracle: the GPU
image must be bitwise equal to the oracle's colorize (pinned against the
reference's own Kernels.metal:465-500 by tests/test_colormap_oracle.py)
applied to the oracle's momentsEven of the same state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PREC = {0: "fp32", 1: "fp16s"}


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("geometry", ["periodic", "channel"])
def test_render_matches_oracle(gpu, oracle, kind, geometry):
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 48, 30, 6
    kw = dict(omega=1.6, uin=0.06, force=(2e-5, 0.0, 0.0))
    flags = eps = None
    if geometry == "channel":
        fl = np.zeros((nz, ny, nx), np.uint8)
        fl[:, 0, :] = fl[:, -1, :] = po.SOLID
        fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = po.INFLOW
        flags = fl.reshape(-1)
        rng = np.random.default_rng(kind)
        eps = np.zeros(nx * ny * nz, np.float32)
        idx = rng.choice(nx * ny * nz, 300, replace=False)
        eps[idx] = rng.choice(np.array([0.1, 0.3, 0.4999, 0.5, 0.8], np.float32), idx.size)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=nx, ny=ny, nz=nz, flags=flags, **kw)
    o = po.OracleSim(nx, ny, nz, flags=flags, kind=kind, **kw)
    if eps is not None:
        g.setSolidFractions(eps)
        o.setSolidFractions(eps)
    g.initField(2, 0.05)
    g.run(6)
    o.f[:] = g.downloadState()
    o.stepsDone = 6
    m = o.probeMoments()
    fl_all = np.zeros(nx * ny * nz, np.uint8) if flags is None else flags
    for z in (0, 3, nz - 1):
        for uref in (0.05, 0.12):
            img = g.renderSlice(z, uref)
            ref = po.colorize(m, fl_all, eps, nx, ny, z, uref)
            assert np.array_equal(img.view(np.uint16), ref.view(np.uint16)), (z, uref)
    g.close()


def test_render_preconditions(gpu):
    import strouhal_gb300 as sg

    s = sg.Simulation(gpu, precision="fp32", nx=16, ny=8, nz=4, omega=1.5)
    s.run(1)
    with pytest.raises(sg.StrouhalError):
        s.renderSlice(0, 0.1)  # odd step count
    s.run(1)
    with pytest.raises(sg.StrouhalError):
        s.renderSlice(4, 0.1)  # outside the lattice
    with pytest.raises(sg.StrouhalError):
        s.renderSlice(0, 0.0)
    img = s.renderSlice(3, 0.1)
    assert img.shape == (8, 16, 4) and np.all(img[..., 3] == 1.0)
    s.close()
