"""The KBC collision (STRO_COLLISION_KBC) in the FP64 oracle: collision
invariants, the BGK limit and the entropic stabiliser. CPU only.

KBC has no reference counterpart (the reference names a cumulant or KBC
operator as the way to the full decay of its Taylor-Green gate,
Sources/strouhal/Cases.swift:1290-1302), so these checks pin it to its
defining properties instead of to reference output."""
import numpy as np
import pytest

from oracle import pyoracle as po

C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1],
              [1, 0, -1], [-1, 0, 1], [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1]], float)
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def moments(f):
    """rho - 1 and momentum per cell of shifted DDFs (19, N)."""
    return f.sum(axis=0), C.T @ f


def feq_shifted(rho, u):
    cu = 3.0 * (C @ u)
    u2 = (u * u).sum(axis=0)
    return W[:, None] * ((rho - 1.0) + rho * (cu + 0.5 * cu * cu - 1.5 * u2))


def sim(n=6, kbc=True, omega=1.7, force=(0.0, 0.0, 0.0)):
    s = po.OracleSim(n, n, n, omega, omega, force=force, kind=po.KIND_F64)
    s.collision = "kbc" if kbc else "reference"
    return s


@pytest.mark.parametrize("force", [(0.0, 0.0, 0.0), (2e-4, -1e-4, 3e-5)])
def test_kbc_conserves_mass_and_momentum(force):
    """One collision (the even pass is purely local; it stores direction i in
    slot opp(i), which flips the sign of the momentum read from the slots):
    rho per cell unchanged, momentum per cell changed by exactly F (Guo)."""
    s = sim(force=force)
    rng = np.random.default_rng(1)
    s.f[:] = rng.standard_normal(s.f.shape) * 0.02
    r0, p0 = moments(s.f)
    s.run(1)
    r1, p1 = moments(s.f)
    assert np.abs(r1 - r0).max() < 1e-15
    F = np.array(force, np.float32).astype(np.float64)  # the step's force is FP32
    assert np.abs(-p1 - p0 - F[:, None]).max() < 1e-15


def test_kbc_is_bgk_for_pure_shear_non_equilibrium():
    """f - feq = 4.5 w_i c_i.D.c_i with D traceless: the rest dh is zero, the
    stabiliser is 2 and KBC equals BGK (the reference's SRT)."""
    n = 6
    rng = np.random.default_rng(2)
    N = n ** 3
    rho = 1.0 + 0.01 * rng.standard_normal(N)
    u = 0.05 * rng.standard_normal((3, N))
    D = 1e-3 * rng.standard_normal((3, 3, N))
    D = 0.5 * (D + D.transpose(1, 0, 2))
    tr = np.trace(D) / 3.0
    for k in range(3):
        D[k, k] -= tr
    cdc = np.einsum("ia,abn,ib->in", C, D, C)
    f = feq_shifted(rho, u) + 4.5 * W[:, None] * cdc
    a, b = sim(n, kbc=True), sim(n, kbc=False)
    a.f[:] = f
    b.f[:] = f
    a.run(1)
    b.run(1)
    assert np.abs(a.f - b.f).max() < 1e-14


def test_kbc_stabiliser_departs_from_bgk_on_higher_order_noise():
    """Non-equilibrium outside the shear part: KBC relaxes it differently from
    BGK, while both conserve the same moments."""
    a, b = sim(), sim(kbc=False)
    rng = np.random.default_rng(3)
    f = rng.standard_normal(a.f.shape) * 0.02
    a.f[:] = f
    b.f[:] = f
    a.run(1)
    b.run(1)
    assert np.abs(a.f - b.f).max() > 1e-4
    ra, pa = moments(a.f)
    rb, pb = moments(b.f)
    assert np.abs(ra - rb).max() < 1e-15 and np.abs(pa - pb).max() < 1e-15


def test_kbc_rest_is_a_fixed_point():
    s = sim(kbc=True)
    s.run(4)
    assert not s.f.any()


def test_kbc_refused_where_it_does_not_exist():
    s = sim()
    with pytest.raises(ValueError):
        s.adjointForce(2, ((0, 1), (0, 1)))
    ref = po.OracleSim(6, 6, 6, 1.7, backend="ref")
    ref.collision = "kbc"
    if po.ref_lib() is not None:
        with pytest.raises(ValueError):
            ref.run(1)
