"""GPU voxelizer (stro_mesh_solid_fractions) against the oracle's restatement
of meshSolidFractions (StlVoxels.swift:52-117): the fractions must be EQUAL,
on the reference's gate sphere and on meshes that exercise the corner cases
(rotation, scaling, bodies partly outside the lattice, axis-aligned faces that
are parallel to the rays, grazing crossings), and the reference's gate must
hold on the GPU result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _box(lo, hi):
    """12-triangle closed box mesh."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
         (2, 3, 7), (2, 7, 6), (1, 2, 6), (1, 6, 5), (0, 4, 7), (0, 7, 3)]
    return np.stack([v[list(t)] for t in f])


def _rotate(tris, seed):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    return (tris.reshape(-1, 3) @ q.T.astype(np.float32)).astype(np.float32).reshape(tris.shape)


def test_gate_sphere_matches_oracle_and_passes_gate(gpu, oracle):
    import strouhal_gb300 as sg

    n, r = 64, 20.0
    mesh = sg.StlMesh(sg.sphereSTLData(r))
    c = np.full(3, n / 2, np.float32)
    eps = sg.meshSolidFractions(gpu, mesh, n, n, n, 1.0, c)
    ref = oracle.mesh_solid_fractions(mesh.triangles, n, n, n, 1.0, c)
    assert np.array_equal(eps, ref)
    ana = sg.sphereSolidFractions(n, n, n, n / 2, n / 2, n / 2, r)
    vol = float(eps.astype(np.float64).sum())
    vol_a = float(ana.astype(np.float64).sum())
    shell = (ana > 0) & (ana < 1)
    assert abs(vol - vol_a) / vol_a <= 0.02
    assert float(np.abs(eps - ana)[shell].mean()) <= 0.10


@pytest.mark.parametrize("case", ["rotated_sphere", "clipped_sphere", "box", "rotated_box",
                                  "two_bodies", "empty"])
def test_meshes_match_oracle(gpu, oracle, case):
    import strouhal_gb300 as sg

    nx, ny, nz = 45, 38, 29
    scale, off = 1.0, np.array([20.3, 17.9, 13.6], np.float32)
    if case == "rotated_sphere":
        tris = _rotate(sg.StlMesh(sg.sphereSTLData(1.0, 40, 19)).triangles, 3)
        scale = 11.7
    elif case == "clipped_sphere":  # sticks out of three faces of the lattice
        tris = sg.StlMesh(sg.sphereSTLData(15.0, 32, 16)).triangles
        off = np.array([5.2, 36.1, 2.0], np.float32)
    elif case == "box":  # faces parallel to the rays and edges on sub-ray lines
        tris = _box((-8.0, -6.25, -4.75), (9.5, 6.75, 5.25))
    elif case == "rotated_box":
        tris = _rotate(_box((-8.0, -6.0, -5.0), (9.0, 7.0, 5.0)), 11)
        scale = 1.3
    elif case == "two_bodies":
        tris = np.concatenate([_box((-15.0, -5.0, -5.0), (-5.0, 5.0, 5.0)),
                               sg.StlMesh(sg.sphereSTLData(6.0, 24, 12)).triangles
                               + np.array([8.0, 0.0, 0.0], np.float32)])
    else:
        tris = np.zeros((0, 3, 3), np.float32)
    eps = sg.meshSolidFractions(gpu, tris, nx, ny, nz, scale, off)
    ref = oracle.mesh_solid_fractions(tris, nx, ny, nz, scale, off)
    assert np.array_equal(eps, ref), np.max(np.abs(eps - ref))
    assert eps.min() >= 0.0 and eps.max() <= 1.0
    if case != "empty":
        assert eps.max() == 1.0


def test_too_many_crossings_is_an_error(gpu):
    """70 thin boxes along x: one sub-ray crosses the mesh 140 times, more
    than the kernel's bound of 128. The kernel records it and returns; the
    call reports an error instead of a truncated field."""
    import strouhal_gb300 as sg

    tris = np.concatenate([_box((2.0 * k, 0.0, 0.0), (2.0 * k + 1.0, 3.0, 3.0)) for k in range(70)])
    with pytest.raises(sg.StrouhalError) as e:
        sg.meshSolidFractions(gpu, tris, 150, 6, 6, 1.0, np.array([2.0, 1.0, 1.0], np.float32))
    assert "128" in str(e.value)
    # the context stays usable
    eps = sg.meshSolidFractions(gpu, tris[:24], 150, 6, 6, 1.0, np.array([2.0, 1.0, 1.0], np.float32))
    assert eps.sum() == 19.5  # two 1x3x3 boxes, lateral edges at half-cell sub-ray spacing


def test_sphere_wake_body_full_size(gpu, oracle):
    """The sphere wake's body (D = 48 cells, 65,024 triangles) voxelized into
    the full 512x256x256 lattice: GPU equal to the oracle, with both times
    recorded (STRO_RESULTS_DIR) for the measurement notes."""
    import json
    import os
    import time

    import strouhal_gb300 as sg
    from strouhal_gb300 import cases

    r = cases.stl_voxelize(gpu)
    mesh = sg.StlMesh(sg.sphereSTLData(1.0, 256, 128))
    t0 = time.perf_counter()
    ref = oracle.mesh_solid_fractions(mesh.triangles, 512, 256, 256, 24.0,
                                      np.array([128.0, 128.0, 128.0], np.float32))
    cpu = time.perf_counter() - t0
    import hashlib
    assert hashlib.sha256(ref.tobytes()).hexdigest() == r["digest"]
    assert r["volume_rel_err"] < 0.01
    r["oracle_seconds_1core"] = cpu
    d = os.environ.get("STRO_RESULTS_DIR")
    if d:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "stl_voxelize.json"), "w") as fh:
            json.dump(r, fh)
