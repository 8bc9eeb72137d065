"""The |u| colormap (colorize + speedColor, Kernels.metal:465-500) of the
oracle against the reference's own kernel source compiled as C++, on the CPU:
bitwise equal RGBA half images over speeds across all three colour stops and
their boundaries, speeds above uref, walls, and solid fractions below, at and
above the 0.5 cut-off."""
import numpy as np
import pytest

from oracle import pyoracle as po


def _inputs(nx=37, ny=23, nz=3, seed=5):
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    m = np.zeros((N, 4), np.float32)
    uref = np.float32(0.08)
    s = rng.uniform(-0.1, 1.3, N).astype(np.float32)
    s[:12] = np.array([0, 0.35, 0.7, 1.0, 0.3499999, 0.3500001, 0.6999999, 0.7000001, 1.2,
                       0.999999, 1e-8, 0.5], np.float32)
    d = rng.standard_normal((N, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    m[:, :3] = d * (s * uref)[:, None]
    m[:, 3] = 1.0
    flags = np.zeros(N, np.uint8)
    flags[rng.choice(N, N // 10, replace=False)] = rng.integers(1, 5, N // 10)
    eps = np.zeros(N, np.float32)
    idx = rng.choice(N, N // 4, replace=False)
    eps[idx] = rng.choice(np.array([0.0, 1e-4, 0.25, 0.49999, 0.5, 0.7, 1.0], np.float32), idx.size)
    return m, flags, eps, nx, ny, nz, float(uref)


@pytest.mark.parametrize("use_eps", [False, True])
@pytest.mark.parametrize("z", [0, 2])
def test_colorize_matches_reference_source(use_eps, z):
    if po.ref_lib() is None:
        pytest.skip("reference tree not present")
    m, flags, eps, nx, ny, nz, uref = _inputs()
    e = eps if use_eps else None
    a = po.colorize(m, flags, e, nx, ny, z, uref)
    b = po.colorize(m, flags, e, nx, ny, z, uref, backend="ref")
    assert np.array_equal(a.view(np.uint16), b.view(np.uint16))
    assert np.all(a[..., 3] == 1.0)
