"""The pressure outflow wall (STRO_OUTFLOW_PRESSURE), an extension of the
reference's dormant outflow: checked in the FP64 oracle against plane
Poiseuille flow. CPU only.

The reference leaves its outflow wall dormant: a link to an outflow cell
reflects the shifted DDF with its sign flipped (Kernels.metal:28-29,
299-300, 328-329), which is anti-bounce-back at rho_w = 1 without the
velocity terms. The pressure mode adds w_i (9 (c_i . u)^2 - 3 u^2). In a
channel with a parabolic velocity inlet and an outflow wall, Poiseuille flow
needs a uniform pressure gradient dp/dx = -8 nu rho u_max / H^2 and an
undisturbed profile up to the outlet; the pressure mode gives both, the
dormant wall distorts the profile next to the outlet."""
import numpy as np
import pytest

from oracle import pyoracle as po

NX, NY = 96, 18
H = NY - 2           # walls halfway between rows 0/1 and NY-2/NY-1
TAU, U_IN = 0.8, 0.05


def channel(mode, steps=8000, kind=po.KIND_F64):
    fl = np.zeros((1, NY, NX), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, 1:-1, 0] = po.INFLOW
    fl[:, 1:-1, -1] = po.OUTFLOW
    wp, wm = po.trt_omegas(TAU, 3.0 / 16.0)
    o = po.OracleSim(NX, NY, 1, wp, wm, uin=U_IN, rampSteps=1000, flags=fl.reshape(-1),
                     kind=kind)
    o.outflowMode = mode
    o.run(steps)
    return o, o.probeMoments().reshape(NY, NX, 4)


def parabola():
    yd = np.arange(NY) - 0.5
    p = np.maximum(4.0 * U_IN * yd * (H - yd) / H ** 2, 0.0)
    return p[1:-1]


@pytest.fixture(scope="module")
def runs():
    return {m: channel(m)[1] for m in ("dormant", "pressure")}


def test_pressure_outflow_keeps_the_poiseuille_profile(runs):
    prof = parabola()
    err = {m: np.abs(r[1:-1, NX - 2, 0] - prof).max() for m, r in runs.items()}
    # measured: 5.6e-4 (pressure) against 2.1e-2 (dormant) next to the outlet
    assert err["pressure"] < 2e-3
    assert err["pressure"] < 0.1 * err["dormant"]
    # mid-channel the flow is Poiseuille in both
    for r in runs.values():
        assert np.abs(r[1:-1, NX // 2, 0] - prof).max() < 2e-3


def test_pressure_outflow_sets_the_pressure_gradient(runs):
    """Centre-line density difference between mid-channel and the outlet row
    against 3 * dp/dx * distance of plane Poiseuille flow."""
    r = runs["pressure"]
    nu = (TAU - 0.5) / 3.0
    dpdx = 8.0 * nu * U_IN / H ** 2
    c = NY // 2
    drho = r[c, NX // 2, 3] - r[c, NX - 2, 3]
    want = 3.0 * dpdx * (NX - 2 - NX // 2)
    assert abs(drho - want) / want < 0.05, (drho, want)
    assert np.abs(r[1:-1, NX - 2, 3] - 1.0).max() < 5e-3


def test_dormant_is_the_default_and_the_reference_wall():
    o = po.OracleSim(8, 6, 1, 1.2, flags=np.zeros(48, np.uint8))
    assert o.outflowMode == "dormant"
    ref = po.OracleSim(8, 6, 1, 1.2, flags=np.zeros(48, np.uint8), backend="ref")
    ref.outflowMode = "pressure"
    if po.ref_lib() is not None:
        with pytest.raises(ValueError):
            ref.run(1)
