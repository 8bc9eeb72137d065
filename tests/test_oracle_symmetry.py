"""Symmetries of the step operator, checked on the FP64 oracle (CPU).

The reference checks rotation and mirror symmetry on whole cavity flows
(Cases.swift:688-765); the GPU runs of those gates are recorded. Here the
same property is asked of one step on random states: mirroring the lattice in
z (or swapping x and y), stepping and mirroring back must equal stepping, with
the walls, lid, force and LES transformed alike. The D3Q19 velocity set maps
onto itself under both maps, so the operator commutes with them up to the FP64
rounding of sums taken in another order. Two steps are taken so that the AA
slots are back in their natural order."""
import numpy as np
import pytest

TOL = 1e-12  # relative, max norm


def _perm(po, cmap):
    """Direction permutation j(i) with c_j = cmap(c_i)."""
    c = np.stack([po.CX, po.CY, po.CZ], axis=1)
    index = {tuple(v): k for k, v in enumerate(c)}
    return np.array([index[tuple(cmap(v))] for v in c])


def _mirror_z(po, f, flags, nx, ny, nz):
    p = _perm(po, lambda v: (v[0], v[1], -v[2]))
    g = np.empty_like(f)
    fr = f.reshape(19, nz, ny, nx)
    g.reshape(19, nz, ny, nx)[p] = fr[:, ::-1]
    return g, flags.reshape(nz, ny, nx)[::-1].reshape(-1).copy()


def _swap_xy(po, f, flags, nx, ny, nz):
    assert nx == ny
    p = _perm(po, lambda v: (v[1], v[0], v[2]))
    g = np.empty_like(f)
    fr = f.reshape(19, nz, ny, nx)
    g.reshape(19, nz, nx, ny)[p] = np.transpose(fr, (0, 1, 3, 2))
    return g, np.transpose(flags.reshape(nz, ny, nx), (0, 2, 1)).reshape(-1).copy()


def _close(a, b):
    scale = max(np.max(np.abs(b)), 1e-30)
    return float(np.max(np.abs(a - b)) / scale)


def _walls(po, nx, ny, nz, lid_face):
    fl = np.zeros((nz, ny, nx), np.uint8)
    if lid_face == "y":
        fl[:, 0, :] = po.SOLID
        fl[:, :, 0] = fl[:, :, -1] = po.SOLID
        fl[:, -1, :] = po.LID
    else:  # the lid is the +x face
        fl[:, :, 0] = po.SOLID
        fl[:, 0, :] = fl[:, -1, :] = po.SOLID
        fl[:, :, -1] = po.LID
    return fl.reshape(-1)


@pytest.mark.parametrize("geometry", ["periodic", "cavity"])
@pytest.mark.parametrize("les,collision", [(0.0, "reference"), (0.01, "reference"), (0.0, "kbc")])
def test_step_commutes_with_z_mirror(oracle, geometry, les, collision):
    po = oracle
    nx, ny, nz = 10, 9, 8
    flags = (np.zeros(nx * ny * nz, np.uint8) if geometry == "periodic"
             else _walls(po, nx, ny, nz, "y"))
    force = (2e-5, -1e-5, 3e-5)
    kw = dict(omega=1.6, omegaMinus=1.25, lid=(0.05, 0.0, 0.02), cSmago=les, kind=po.KIND_F64)
    rng = np.random.default_rng(7)
    f0 = rng.standard_normal((19, nx * ny * nz)) * 0.01
    a = po.OracleSim(nx, ny, nz, flags=flags, force=force, **kw)
    a.collision = collision
    a.f[:] = f0
    a.run(2)
    g0, gflags = _mirror_z(po, f0, flags, nx, ny, nz)
    kw["lid"] = (0.05, 0.0, -0.02)
    b = po.OracleSim(nx, ny, nz, flags=gflags, force=(force[0], force[1], -force[2]), **kw)
    b.collision = collision
    b.f[:] = g0
    b.run(2)
    back, _ = _mirror_z(po, b.f, gflags, nx, ny, nz)
    assert _close(back, a.f) < TOL


@pytest.mark.parametrize("geometry", ["periodic", "cavity"])
def test_step_commutes_with_xy_swap(oracle, geometry):
    po = oracle
    n, nz = 9, 4
    kw = dict(omega=1.7, omegaMinus=1.3, kind=po.KIND_F64)
    if geometry == "periodic":
        fa = fb = np.zeros(n * n * nz, np.uint8)
        la, lb = (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)
    else:  # the standard cavity against the one whose lid is the +x face
        fa, fb = _walls(po, n, n, nz, "y"), _walls(po, n, n, nz, "x")
        la, lb = (0.05, 0.0, 0.0), (0.0, 0.05, 0.0)
    rng = np.random.default_rng(11)
    f0 = rng.standard_normal((19, n * n * nz)) * 0.01
    a = po.OracleSim(n, n, nz, flags=fa, lid=la, force=(1e-5, 3e-5, 0.0), **kw)
    a.f[:] = f0
    a.run(2)
    g0, gflags = _swap_xy(po, f0, fa, n, n, nz)
    assert np.array_equal(gflags, fb)
    b = po.OracleSim(n, n, nz, flags=gflags, lid=lb, force=(3e-5, 1e-5, 0.0), **kw)
    b.f[:] = g0
    b.run(2)
    back, _ = _swap_xy(po, b.f, gflags, n, n, nz)
    assert _close(back, a.f) < TOL
