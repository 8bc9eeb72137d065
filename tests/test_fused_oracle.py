"""The fused-multiply-add arithmetic of the oracle (kinds 3 and 4) against
the FP64 oracle, on the CPU.

The fused arithmetic is this library's own algebraically equal form of the
reference collision, so it has no reference build to be pinned to. It is
held to the same tolerances as the reference arithmetic: DDFs within 1e-5
(FP32 storage) and 2e-3 (FP16 storage) normwise relative to the FP64 oracle
after N steps, on a periodic Taylor-Green box and on a walled lattice with
every feature switched on."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po


def _rel(a, ref):
    return float(np.linalg.norm(a.astype(np.float64) - ref) / np.linalg.norm(ref))


@pytest.mark.parametrize("kind,tol", [(po.KIND_F32, 1e-5), (po.KIND_F16, 2e-3)])
def test_fused_taylor_green_within_tolerance(kind, tol):
    n, u0 = 16, 0.05
    tau = 3 * u0 * (n / (2 * math.pi)) / 1600 + 0.5
    d = po.OracleSim(n, n, n, omega=1 / tau, kind=po.KIND_F64, threads=4)
    d.initField(2, u0)
    d.run(50)
    errs = {}
    for ar in ("reference", "fused"):
        o = po.OracleSim(n, n, n, omega=1 / tau, kind=kind, arithmetic=ar, threads=4)
        o.initField(2, u0)
        o.run(50)
        errs[ar] = _rel(o.f, d.f)
    assert errs["fused"] < tol, errs
    # as accurate as the reference arithmetic, within a quarter
    assert errs["fused"] < 1.25 * errs["reference"], errs


@pytest.mark.parametrize("kind,tol", [(po.KIND_F32, 1e-5), (po.KIND_F16, 2e-3)])
def test_fused_all_features_within_tolerance(kind, tol):
    """Solid and moving walls, ramp, TRT, uniform force and force field, LES,
    Noble-Torczynski cells, sponge."""
    nx, ny, nz = 16, 12, 4
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, 0, :] = 1
    flags[:, -1, :] = 2
    rng = np.random.default_rng(3)
    eps = np.zeros(nx * ny * nz, np.float32)
    eps[rng.choice(nx * ny * nz, 20, replace=False)] = rng.uniform(0.1, 0.9, 20)
    ff = (rng.standard_normal((3, nx * ny * nz)) * 1e-5).astype(np.float32)

    def make(k, ar):
        o = po.OracleSim(nx, ny, nz, omega=1.6, omegaMinus=1.2, lid=(0.05, 0, 0), rampSteps=10,
                         force=(1e-5, 0, 0), cSmago=0.01, flags=flags.reshape(-1), kind=k,
                         arithmetic=ar)
        o.sponge = (10.0, 5.0, 0.9)
        o.setSolidFractions(eps)
        o.setForceField(ff)
        return o

    d = make(po.KIND_F64, "reference")
    d.run(40)
    ref = make(kind, "reference")
    ref.run(40)
    fu = make(kind, "fused")
    fu.run(40)
    e_ref, e_fu = _rel(ref.f, d.f), _rel(fu.f, d.f)
    assert e_fu < tol, (e_fu, e_ref)
    assert e_fu < 1.25 * e_ref + 1e-7, (e_fu, e_ref)
    assert not np.array_equal(fu.f, ref.f)  # a different arithmetic, not an alias


def test_fused_rejected_where_it_does_not_exist():
    with pytest.raises(ValueError):
        po.OracleSim(4, 4, 4, omega=1.0, kind=po.KIND_F64, arithmetic="fused")
