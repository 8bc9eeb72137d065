"""The oracle's FP64 observables (orc_observables) against a numpy statement of
the same sums: kinetic energy sum |u|^2 and dissipation sum 2 nu S:S with
S = -(1.5 omega / rho) Pi_neq, over the fluid cells of a walled lattice with a
uniform force and a per-cell force field."""
import numpy as np


def _numpy_observables(po, f, flags, omega, force, ffield):
    f = f.astype(np.float64)
    fluid = flags == 0
    rho = 1.0 + f.sum(0)
    F = np.array(force, np.float64)[:, None] + ffield.astype(np.float64)
    p = np.stack([(po.CX[:, None] * f).sum(0), (po.CY[:, None] * f).sum(0),
                  (po.CZ[:, None] * f).sum(0)])
    u = (p + 0.5 * F) / rho
    u2 = (u * u).sum(0)
    W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    P = np.zeros((6, f.shape[1]))
    for i in range(1, 19):
        c = (po.CX[i], po.CY[i], po.CZ[i])
        cu = 3 * (c[0] * u[0] + c[1] * u[1] + c[2] * u[2])
        d = f[i] - W[i] * ((rho - 1) + rho * (cu + 0.5 * cu * cu - 1.5 * u2))
        for k, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
            P[k] += c[a] * c[b] * d
    pipi = P[0] ** 2 + P[1] ** 2 + P[2] ** 2 + 2 * (P[3] ** 2 + P[4] ** 2 + P[5] ** 2)
    nu = (1 / omega - 0.5) / 3
    return float(u2[fluid].sum()), float((2 * nu * (1.5 * omega / rho) ** 2 * pipi)[fluid].sum())


def test_fp64_observables_match_numpy(oracle):
    po = oracle
    nx, ny, nz = 14, 11, 6
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = po.SOLID
    fl[:, -1, :] = po.LID
    fl = fl.reshape(-1)
    rng = np.random.default_rng(3)
    force = (2e-5, -1e-5, 3e-5)
    o = po.OracleSim(nx, ny, nz, omega=1.63, force=force, flags=fl, kind=po.KIND_F64, threads=3)
    ff = (rng.standard_normal((3, o.N)) * 1e-5).astype(np.float32)
    o.setForceField(ff)
    o.f[:] = rng.standard_normal((19, o.N)) * 0.01
    ke, diss = o.observables()
    ke_n, diss_n = _numpy_observables(po, o.f, fl, o.omega, o.force, ff)
    assert np.isclose(ke, ke_n, rtol=1e-12, atol=0), (ke, ke_n)
    assert np.isclose(diss, diss_n, rtol=1e-12, atol=0), (diss, diss_n)
    # the sums do not depend on the thread count beyond FP64 rounding
    o.threads = 1
    ke1, diss1 = o.observables()
    assert np.isclose(ke1, ke, rtol=1e-13) and np.isclose(diss1, diss, rtol=1e-13)
