"""Pins the CPU oracle to the reference (CPU only).

1. Against the committed golden vectors (tests/golden/reference_cases.npz),
   produced by the reference's own Kernels.metal compiled as C++: every case is
   replayed on the oracle and must agree value-for-value.
2. Where the reference tree is present, live against that compiled source on
   seeded random cases covering each feature separately and all together.
3. The reference's own known-answer gates (Cases.swift:55-128): rest fixed
   points and the 18-direction streaming proof.
4. The FP64 instance against the FP32 instance (same algorithm, precision only).
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_cases.npz")


def _golden():
    d = np.load(GOLDEN)
    meta = json.loads(bytes(d["meta"]).decode())
    return d, meta


def _sim_for(po, case, d, backend="oracle", kind=None):
    nx, ny, nz = case["dims"]
    fl = d[case["name"] + "/flags"]
    sim = po.OracleSim(nx, ny, nz, omega=case["omega"], omegaMinus=case.get("omegaMinus"),
                       lid=case.get("lid", (0, 0, 0)), uin=case.get("uin", 0.0),
                       rampSteps=case.get("ramp", 0), force=case.get("force", (0, 0, 0)),
                       cSmago=case.get("cSmago", 0.0), wantsForces="probe" in case,
                       flags=fl if fl.size else None,
                       kind=case["kind"] if kind is None else kind, backend=backend)
    sim.inflowUniform = case.get("uniform", False)
    if "sponge" in case:
        sim.sponge = tuple(case["sponge"])
    eps = d[case["name"] + "/eps"]
    if eps.size:
        sim.setSolidFractions(eps)
    return sim


def test_oracle_matches_golden_vectors(oracle):
    po = oracle
    d, meta = _golden()
    for case in meta:
        name = case["name"]
        sim = _sim_for(po, case, d)
        sim.f[:] = d[name + "/f0"]
        sim.run(case["steps"])
        assert np.array_equal(sim.f, d[name + "/f1"]), name
        if name + "/moments" in d.files:
            assert np.array_equal(sim.probeMoments(), d[name + "/moments"]), name
        if "probe" in case:
            (x0, x1), (y0, y1) = case["probe"]
            fo = sim.probeForce((x0, x1), (y0, y1))
            assert np.array_equal(fo, d[name + "/force"]), name
            assert np.array_equal(sim.f, d[name + "/f2"]), name


def test_oracle_init_matches_golden(oracle):
    """initField: the oracle rounds double sin/cos, the reference uses sinf/cosf."""
    po = oracle
    d, _ = _golden()
    for kind in (0, 1):
        for mode in (1, 2):
            sim = po.OracleSim(10, 8, 6, omega=1.2, kind=kind)
            sim.initField(mode, 0.07)
            ref = d["init_k%d_m%d/f" % (kind, mode)]
            a = sim.f.astype(np.float64)
            b = ref.astype(np.float64)
            ulp = np.spacing(np.abs(ref).astype(ref.dtype)).astype(np.float64)
            assert np.all(np.abs(a - b) <= 4 * ulp + 1e-12), (kind, mode)


FEATURES = [(0, 0, 0, 0, 0), (1, 0, 0, 0, 0), (0, 1, 0, 0, 0), (0, 0, 1, 0, 0),
            (0, 0, 0, 1, 0), (0, 0, 0, 0, 1), (1, 1, 1, 1, 1)]


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("walls", [0, 1, 2])  # 2: the x = nx-1 wall is a (dormant) outflow
@pytest.mark.parametrize("feat", FEATURES)
def test_oracle_matches_reference_source(oracle, kind, walls, feat):
    po = oracle
    if po.ref_lib() is None:
        pytest.skip("reference tree not present")
    eps_on, les, sponge, force, ramp = feat
    nx, ny, nz = 12, 10, 5
    rng = np.random.default_rng(hash((kind, walls, feat)) & 0xFFFF)

    def fl(x, y, z):
        if y == ny - 1:
            return po.LID
        if y == 0:
            return po.SOLID
        if x == nx - 1 and walls == 2:
            return po.OUTFLOW
        if x == 0 or x == nx - 1:
            return po.INFLOW
        if (x, y) == (5, 4):
            return po.SOLID
        return po.FLUID

    def mk(backend):
        s = po.OracleSim(nx, ny, nz, omega=1.3, omegaMinus=1.1, lid=(0.08, 0.01, -0.02), uin=0.05,
                         rampSteps=4 if ramp else 0,
                         force=(1e-4, -2e-5, 3e-5) if force else (0, 0, 0),
                         cSmago=0.01 if les else 0.0, wantsForces=True,
                         flags=fl if walls else None, kind=kind, backend=backend)
        if sponge:
            s.sponge = (6.0, 4.0, 0.9)
        return s

    a, b = mk("oracle"), mk("ref")
    if eps_on:
        e = np.zeros(a.N, np.float32)
        e[rng.integers(0, a.N, 40)] = rng.random(40).astype(np.float32)
        a.setSolidFractions(e)
        b.setSolidFractions(e)
    init = (rng.standard_normal((19, a.N)) * 0.01).astype(a.f.dtype)
    a.f[:] = init
    b.f[:] = init
    a.run(6)
    b.run(6)
    assert np.array_equal(a.f, b.f)
    assert np.array_equal(a.probeForce((2, 9), (1, 8)), b.probeForce((2, 9), (1, 8)))
    assert np.array_equal(a.forceBuf, b.forceBuf)
    assert np.array_equal(a.probeMoments(), b.probeMoments())


def test_rest_fixed_points(oracle):
    """Cases.swift:58-83: rest is a bitwise fixed point, periodic and with walls."""
    po = oracle
    s = po.OracleSim(12, 12, 12, omega=1.7)
    d0 = s.stateDigest
    s.run(20)
    assert s.stateDigest == d0
    n = 18

    def cav(x, y, z):
        if y == n - 1:
            return po.LID
        if x == 0 or x == n - 1 or y == 0:
            return po.SOLID
        return po.FLUID

    s = po.OracleSim(n, n, 1, omega=1.7, flags=cav)
    d0 = s.stateDigest
    s.run(40)
    assert s.stateDigest == d0


def test_streaming_proof(oracle):
    """Cases.swift:85-125: with omega=0 a lone DDF moves exactly T*c_i, bit-identical."""
    po = oracle
    n, T = 16, 4
    s = po.OracleSim(n, n, n, omega=0.0)
    idx = lambda x, y, z: (z * n + y) * n + x  # noqa: E731
    inj = np.zeros(19, np.float32)
    for i in range(1, 19):
        inj[i] = np.float32(i) * np.float32(0.001)
        s.f[i, idx(8, 8, 8)] = inj[i]
    s.run(T)
    for i in range(1, 19):
        dest = idx((8 + T * po.CX[i]) % n, (8 + T * po.CY[i]) % n, (8 + T * po.CZ[i]) % n)
        assert s.f[i, dest] == inj[i]
    assert np.count_nonzero(s.f) == 18


def test_fp64_oracle_tracks_fp32(oracle):
    po = oracle
    kw = dict(nx=16, ny=12, nz=8, omega=1.8, omegaMinus=1.4)
    a = po.OracleSim(kind=po.KIND_F32, **kw)
    b = po.OracleSim(kind=po.KIND_F64, **kw)
    a.initField(2, 0.05)
    b.f[:] = a.f.astype(np.float64)
    a.run(20)
    b.run(20)
    err = np.linalg.norm(a.f.astype(np.float64) - b.f) / np.linalg.norm(b.f)
    assert err < 1e-5, err
