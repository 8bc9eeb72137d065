"""GPU discrete adjoint on crops of the cylinder (C3) and sphere-wake (C5)
lattices, against the FP64 host adjoint and FP64 central differences.

Each crop compares (tests/adjoint_crops.py):
- the GPU adjoint with the FP64 host adjoint linearised about the same forward
  trajectory (the oracle's FP32-arithmetic step is the library's, value for
  value, in FP32 and FP16 storage): normwise within 1e-3;
- the FP64 host adjoint of the FP64 trajectory with FP64 central differences:
  within 1e-3 per parameter;
- the GPU adjoint with those central differences: within 1e-3 per parameter
  for FP32 storage, and for the force-field gradient (the C5 objective) in
  FP16 storage. The solid-fraction gradient of an FP16-storage run is taken
  about a trajectory that FP16 rounding moves by about 1e-3, so it is held to
  the FP16 bar of 2e-2 against the FP64 differences (its agreement with the
  FP64 adjoint of its own trajectory is the 1e-3 check above)."""
import numpy as np
import pytest

import adjoint_crops as ac

pytestmark = pytest.mark.gpu

_cache = {}


def _sphere(gpu, oracle, precision):
    import strouhal_gb300 as sg

    if precision not in _cache:
        g, o, f0, _, box, eps, ff, _ = ac.sphere_crop(sg, oracle, gpu, precision, spinup=200,
                                                      ramp=100)
        fd = 8 if precision == "fp32" else 0
        r = ac.run_checks(sg, o, g, f0, box, eps, ff, 60, precision, fd_eps=fd, fd_force=8)
        g.close()
        _cache[precision] = r
    return _cache[precision]


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_sphere_crop_gpu_adjoint_matches_fp64_adjoint_of_its_trajectory(gpu, oracle, precision):
    r = _sphere(gpu, oracle, precision)
    assert r["finite"]
    assert r["J_rel_err"] < 1e-9, r["J_rel_err"]
    assert r["grad_force_rel_err"] < 1e-3, r["grad_force_rel_err"]
    assert r["grad_eps_rel_err"] < 1e-3, r["grad_eps_rel_err"]
    assert r["grad_eps_zero_off_nt"]


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_sphere_crop_agrees_with_fp64_central_differences(gpu, oracle, precision):
    r = _sphere(gpu, oracle, precision)
    assert len(r["fd"]) >= 8
    for d in r["fd"]:
        assert d["fp64_adjoint_rel_err"] < 1e-3, d
        bar = 1e-3 if (precision == "fp32" or d["param"].startswith("force")) else 2e-2
        assert d["gpu_adjoint_rel_err"] < bar, d


def test_cylinder_crop_adjoint(gpu, oracle):
    import strouhal_gb300 as sg

    g, o, f0, _, box, eps, ff, _ = ac.cylinder_crop(sg, oracle, gpu, "fp32", spinup=30000)
    r = ac.run_checks(sg, o, g, f0, box, eps, ff, 100, "fp32", fd_eps=8, fd_force=0)
    g.close()
    assert r["finite"]
    assert r["J_rel_err"] < 1e-9, r["J_rel_err"]
    assert r["grad_eps_rel_err"] < 1e-3, r["grad_eps_rel_err"]
    assert r["grad_eps_zero_off_nt"]
    assert len(r["fd"]) >= 8
    for d in r["fd"]:
        assert d["fp64_adjoint_rel_err"] < 1e-3, d
        assert d["gpu_adjoint_rel_err"] < 1e-3, d
