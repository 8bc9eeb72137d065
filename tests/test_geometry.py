"""Triangle meshes on the CPU: the binary STL reader and sphere generator of
the library (StlVoxels.swift:6-43, 120-143), and the oracle's voxelizer
(StlVoxels.swift:52-117) against the reference's own voxelizer gate
(Cases.swift:1074-1101): a 48x24 lat-long sphere of radius 20 at the centre of
a 64^3 lattice must match the analytic solid fractions in volume within 2%
and in the mean shell deviation within 0.10."""
import struct

import numpy as np
import pytest

import strouhal_gb300 as sg
from oracle import pyoracle as po


def _parse_py(data):
    n = struct.unpack_from("<I", data, 80)[0]
    tris = np.zeros((n, 3, 3), np.float32)
    for k in range(n):
        vals = struct.unpack_from("<9f", data, 84 + 50 * k + 12)
        tris[k] = np.array(vals, np.float32).reshape(3, 3)
    return tris


def test_sphere_stl_parses_like_the_binary_format():
    data = sg.sphereSTLData(20.0)
    assert len(data) == 84 + 50 * 48 * (2 * 24 - 2)
    mesh = sg.StlMesh(data)
    ref = _parse_py(data)
    assert mesh.triangles.shape == (48 * 46, 3, 3)
    assert np.array_equal(mesh.triangles, ref)
    assert np.array_equal(mesh.boundsMin, ref.reshape(-1, 3).min(0))
    assert np.array_equal(mesh.boundsMax, ref.reshape(-1, 3).max(0))
    # vertices lie on the sphere (FP32 sin/cos)
    r = np.linalg.norm(ref.reshape(-1, 3).astype(np.float64), axis=1)
    assert np.max(np.abs(r - 20.0)) < 1e-4


@pytest.mark.parametrize("data,msg", [
    (b"\0" * 83, "too short"),
    (b"solid name\n" + b"\0" * 80, "ASCII"),
    (b"\0" * 80 + struct.pack("<I", 3) + b"\0" * 100, "truncated"),
])
def test_stl_errors_as_the_reference(data, msg):
    with pytest.raises(sg.StrouhalError) as e:
        sg.StlMesh(data)
    assert msg in str(e.value)


def _gate(eps, ana):
    vol, vol_a = float(eps.astype(np.float64).sum()), float(ana.astype(np.float64).sum())
    d = np.abs(eps.astype(np.float64) - ana.astype(np.float64))
    shell = (ana > 0) & (ana < 1)
    return abs(vol - vol_a) / vol_a, float(d[shell].mean())


def test_oracle_voxelizer_passes_the_reference_gate():
    n, r = 64, 20.0
    mesh = sg.StlMesh(sg.sphereSTLData(r))
    c = np.full(3, n / 2, np.float32)
    eps = po.mesh_solid_fractions(mesh.triangles, n, n, n, 1.0, c)
    ana = sg.sphereSolidFractions(n, n, n, n / 2, n / 2, n / 2, r)
    vol_err, shell = _gate(eps, ana)
    assert vol_err <= 0.02 and shell <= 0.10, (vol_err, shell)
    assert eps.max() == 1.0 and eps.min() == 0.0
