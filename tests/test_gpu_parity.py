"""GPU parity of the D3Q19 step through the C ABI.

The CUDA kernels keep the reference's FP32 operation order (compiled with
-fmad=false), so against the FP32-arithmetic oracle — and the golden vectors
of the reference's own kernel source — the DDFs must be EQUAL in value after
any number of steps, in FP32 and FP16 storage. Against the FP64 oracle the
tolerance is the stated one: normwise relative 1e-5 (FP32 storage) and 2e-3
(FP16 storage) on the DDFs after N steps.
"""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_cases.npz")
PREC = {0: "fp32", 1: "fp16s"}


def _mk_pair(sg, po, gpu, kind, nx, ny, nz, flags=None, eps=None, sponge=None, uniform=False,
             **kw):
    g = sg.Simulation(gpu, precision=PREC[kind], nx=nx, ny=ny, nz=nz, flags=flags, **kw)
    o = po.OracleSim(nx, ny, nz, flags=flags, kind=kind, **kw)
    if sponge is not None:
        g.sponge = sponge
        o.sponge = sponge
    if uniform:
        g.inflowUniform = True
        o.inflowUniform = True
    if eps is not None:
        g.setSolidFractions(eps)
        o.setSolidFractions(eps)
    return g, o


def test_golden_vectors_on_gpu(gpu, oracle):
    import strouhal_gb300 as sg

    d = np.load(GOLDEN)
    meta = json.loads(bytes(d["meta"]).decode())
    for case in meta:
        name = case["name"]
        nx, ny, nz = case["dims"]
        fl = d[name + "/flags"]
        g = sg.Simulation(gpu, precision=PREC[case["kind"]], nx=nx, ny=ny, nz=nz,
                          omega=case["omega"], omegaMinus=case.get("omegaMinus"),
                          lid=case.get("lid", (0, 0, 0)), uin=case.get("uin", 0.0),
                          rampSteps=case.get("ramp", 0), force=case.get("force", (0, 0, 0)),
                          cSmago=case.get("cSmago", 0.0), wantsForces="probe" in case,
                          flags=fl if fl.size else None)
        g.inflowUniform = case.get("uniform", False)
        if "sponge" in case:
            g.sponge = tuple(case["sponge"])
        eps = d[name + "/eps"]
        if eps.size:
            g.setSolidFractions(eps)
        g.uploadState(d[name + "/f0"])
        g.run(case["steps"])
        assert np.array_equal(g.downloadState(), d[name + "/f1"]), name
        if name + "/moments" in d.files:
            assert np.array_equal(g.probeMoments(), d[name + "/moments"]), name
        if "probe" in case:
            (x0, x1), (y0, y1) = case["probe"]
            fo = g.probeForce((x0, x1), (y0, y1))
            ref = d[name + "/force"]
            assert np.allclose(fo, ref, rtol=1e-12, atol=1e-13), (name, fo, ref)
            assert np.array_equal(g.downloadState(), d[name + "/f2"]), name
        g.close()


FEATURES = {
    "plain": {},
    "force": dict(force=(3e-5, -1e-5, 2e-5)),
    "les": dict(cSmago=0.01),
    "sponge": dict(sponge=(14.0, 8.0, 0.85)),
    "eps": dict(eps=True),
    "all": dict(force=(3e-5, -1e-5, 2e-5), cSmago=0.01, sponge=(14.0, 8.0, 0.85), eps=True),
    # per-cell Guo force field (the library's extension), some cells without a field force
    "ffield": dict(ffield=True),
    "ffield_all": dict(force=(3e-5, -1e-5, 2e-5), cSmago=0.01, sponge=(14.0, 8.0, 0.85),
                       eps=True, ffield=True),
}


def random_force_field(rng, N, scale=2e-5, zero_frac=0.3):
    """A nonzero per-cell force field (3, N) with a fraction of all-zero cells."""
    ff = (rng.standard_normal((3, N)) * scale).astype(np.float32)
    ff[:, rng.random(N) < zero_frac] = 0.0
    return ff


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("geometry", ["periodic", "cavity", "channel", "xfaces", "xfaces_uniform"])
@pytest.mark.parametrize("feature", list(FEATURES))
def test_step_matches_oracle(gpu, oracle, kind, geometry, feature):
    """xfaces: inflow columns at both x ends over every row (periodic y and z),
    so the blocks along them run the x-face kernels of the block split; a solid
    box and the NT cells keep some blocks on the wall-aware kernels."""
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 37, 21, 9  # odd sizes: partial blocks, wrap at every face
    rng = np.random.default_rng(hash((kind, geometry, feature)) & 0xFFFFFF)
    flags = None
    if geometry == "cavity":
        flags = np.zeros((nz, ny, nx), np.uint8)
        flags[:, :, 0] = flags[:, :, -1] = flags[:, 0, :] = po.SOLID
        flags[:, -1, :] = po.LID
    elif geometry == "channel":
        flags = np.zeros((nz, ny, nx), np.uint8)
        flags[:, 0, :] = flags[:, -1, :] = po.SOLID
        flags[:, 1:-1, 0] = flags[:, 1:-1, -1] = po.INFLOW
        flags[:, 8:11, 12:15] = po.SOLID
    elif geometry.startswith("xfaces"):
        flags = np.zeros((nz, ny, nx), np.uint8)
        flags[:, :, 0] = flags[:, :, -1] = po.INFLOW
        flags[:, 8:11, 12:15] = po.SOLID
    opts = dict(FEATURES[feature])
    eps = None
    if opts.pop("eps", False):
        eps = np.zeros(nx * ny * nz, np.float32)
        if geometry.startswith("xfaces"):  # NT cells in x = 10..25 only
            cand = np.flatnonzero((np.arange(nx * ny * nz) % nx >= 10) &
                                  (np.arange(nx * ny * nz) % nx <= 25))
            idx = rng.choice(cand, 120, replace=False)
        else:
            idx = rng.choice(nx * ny * nz, 120, replace=False)
        eps[idx] = rng.uniform(0.02, 0.98, idx.size).astype(np.float32)
    ffield = opts.pop("ffield", False)
    g, o = _mk_pair(sg, po, gpu, kind, nx, ny, nz,
                    flags=None if flags is None else flags.reshape(-1), eps=eps,
                    omega=1.55, omegaMinus=1.2, lid=(0.07, 0.0, 0.01), uin=0.05, rampSteps=7,
                    wantsForces=True, uniform=geometry == "xfaces_uniform", **opts)
    if ffield:
        ff = random_force_field(rng, nx * ny * nz)
        g.setForceField(ff)
        o.setForceField(ff)
    f0 = (rng.standard_normal((19, nx * ny * nz)) * 0.01).astype(o.f.dtype)
    o.f[:] = f0
    g.uploadState(f0)
    for chunk in (1, 4, 3):  # odd chunks cross the AA parity between calls
        g.run(chunk)
        o.run(chunk)
        assert np.array_equal(g.downloadState(), o.f), (chunk, g.stepsDone)
    if geometry.startswith("xfaces"):
        assert g.splitBlocks[1] > 0  # the x-face kernels ran
    assert np.array_equal(g.probeMoments(), o.probeMoments())
    box = ((3, 30), (1, 18))
    fg, fo = g.probeForce(*box), o.probeForce(*box)
    assert np.allclose(fg, fo, rtol=1e-12, atol=1e-12), (fg, fo)
    assert np.array_equal(g.downloadState(), o.f)
    g.close()


@pytest.mark.parametrize("split,kind", [("pair", 1), ("merged", 1), ("merged", 0)])
@pytest.mark.parametrize("arith", ["reference", "fused"])
@pytest.mark.parametrize("geometry", ["channel", "xfaces", "ywalls"])
@pytest.mark.parametrize("feature", ["plain", "les", "ffield_all"])
@pytest.mark.parametrize("block", [(16, 4), (64, 1), (8, 8), (32, 3)])
def test_merged_split_matches_oracle(gpu, oracle, split, kind, arith, geometry, feature, block):
    """Block splits "merged" and "pair": the bulk and x-face blocks of a walled
    lattice run in one launch from one list, beside the wall-aware blocks;
    "pair" takes the bulk blocks of FP16 storage two x-adjacent cells per
    thread (4-byte words) and the x-face blocks two cells per thread one after
    the other. ywalls: walls at y = 0 and y = ny - 1 only, so bulk blocks reach
    x = 0 and x = nx - 1 and the pair gather wraps in x. Odd ny and nz leave
    partial blocks."""
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 134, 21, 7
    rng = np.random.default_rng(hash((split, kind, arith, geometry, feature, block)) & 0xFFFFFF)
    flags = np.zeros((nz, ny, nx), np.uint8)
    if geometry == "channel":
        flags[:, 0, :] = flags[:, -1, :] = po.SOLID
        flags[:, 1:-1, 0] = flags[:, 1:-1, -1] = po.INFLOW
        flags[:, 8:11, 70:74] = po.SOLID
    elif geometry == "xfaces":
        flags[:, :, 0] = flags[:, :, -1] = po.INFLOW
        flags[:, 8:11, 70:74] = po.SOLID
    else:
        flags[:, 0, :] = po.SOLID
        flags[:, -1, :] = po.LID
    opts = dict(FEATURES[feature])
    eps = None
    if opts.pop("eps", False):  # NT cells in x = 40..60 only
        eps = np.zeros(nx * ny * nz, np.float32)
        cand = np.flatnonzero((np.arange(nx * ny * nz) % nx >= 40) &
                              (np.arange(nx * ny * nz) % nx <= 60))
        idx = rng.choice(cand, 150, replace=False)
        eps[idx] = rng.uniform(0.02, 0.98, idx.size).astype(np.float32)
    ffield = opts.pop("ffield", False)
    g, o = _mk_pair(sg, po, gpu, kind, nx, ny, nz, flags=flags.reshape(-1), eps=eps,
                    omega=1.55, omegaMinus=1.2, lid=(0.07, 0.0, 0.01), uin=0.05, rampSteps=7,
                    wantsForces=True, arithmetic=arith, **opts)
    if ffield:
        ff = random_force_field(rng, nx * ny * nz)
        g.setForceField(ff)
        o.setForceField(ff)
    g.setBlockSplit(split)
    g.block = block
    f0 = (rng.standard_normal((19, nx * ny * nz)) * 0.01).astype(o.f.dtype)
    o.f[:] = f0
    g.uploadState(f0)
    for chunk in (1, 4, 3):
        g.run(chunk)
        o.run(chunk)
        assert g.lastPath == "split-" + split, g.lastPath
        assert np.array_equal(g.downloadState(), o.f), (chunk, g.stepsDone)
    assert g.splitBlocks[0] > 0  # the merged launch ran bulk blocks
    if geometry == "xfaces":
        assert g.splitBlocks[1] > 0  # and x-face blocks
    box = ((3, 100), (1, 18))
    fg, fo = g.probeForce(*box), o.probeForce(*box)
    assert np.allclose(fg, fo, rtol=1e-12, atol=1e-12), (fg, fo)
    g.run(2)
    o.run(2)
    assert np.array_equal(g.downloadState(), o.f)
    g.close()


@pytest.mark.parametrize("kind,tol", [(0, 1e-5), (1, 2e-3)])
def test_fp64_oracle_tolerance(gpu, oracle, kind, tol):
    """DDFs after N = 50 steps vs the FP64 oracle: normwise relative error <= tol.

    FP16 storage rounds every DDF at every step (relative 2^-11), so its error
    grows like sqrt(N): on this nearly inviscid 24^3 TGV (tau = 0.50036) the
    FP16-storage oracle reads 1.6e-3 at N = 50, 2.2e-3 at 100, 3.2e-3 at 200;
    FP32 storage reads 1.8e-6 at 50 and 5.2e-6 at 200."""
    import strouhal_gb300 as sg

    po = oracle
    n = 24
    u0 = 0.05
    L = n / (2 * np.pi)
    tau = 3 * u0 * L / 1600 + 0.5
    wp, wm = sg.trtOmegas(tau, 3.0 / 16.0) if kind == 0 else sg.trtOmegas(tau)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm)
    o = po.OracleSim(n, n, n, omega=wp, omegaMinus=wm, kind=po.KIND_F64, threads=8)
    o.initField(2, u0)
    g.uploadState(o.f.astype(np.float32 if kind == 0 else np.float16))
    steps = 50
    g.run(steps)
    o.run(steps)
    a = g.downloadState().astype(np.float64)
    err = np.linalg.norm(a - o.f) / np.linalg.norm(o.f)
    assert err <= tol, err
    # observables vs FP64
    m_o = o.probeMoments()
    ke_o = float(np.sum(m_o[:, 0] ** 2 + m_o[:, 1] ** 2 + m_o[:, 2] ** 2))
    ke_g = g.kineticEnergySum()
    assert abs(ke_g - ke_o) / ke_o <= (1e-5 if kind == 0 else 5e-3), (ke_g, ke_o)
    g.close()


def test_init_field_matches_oracle(gpu, oracle):
    import strouhal_gb300 as sg

    po = oracle
    for kind in (0, 1):
        for mode in (0, 1, 2):
            g = sg.Simulation(gpu, precision=PREC[kind], nx=20, ny=18, nz=12, omega=1.3)
            o = po.OracleSim(20, 18, 12, omega=1.3, kind=kind)
            g.initField(mode, 0.06)
            o.initField(mode, 0.06)
            a = g.downloadState()
            ulp = np.spacing(np.abs(o.f)).astype(np.float64)
            assert np.all(np.abs(a.astype(np.float64) - o.f.astype(np.float64)) <= ulp), (kind, mode)
            g.close()


def test_selftest_rest_and_streaming(gpu):
    """Cases.swift:55-128 on the GPU."""
    import strouhal_gb300 as sg

    s = sg.Simulation(gpu, nx=32, ny=32, nz=32, omega=1.7)
    d0 = s.stateDigest
    s.run(100)
    assert s.stateDigest == d0
    n = 34

    def cav(x, y, z):
        if y == n - 1:
            return sg.Cell.lid
        if x == 0 or x == n - 1 or y == 0:
            return sg.Cell.solid
        return sg.Cell.fluid

    s = sg.Simulation(gpu, nx=n, ny=n, nz=1, omega=1.7, flags=cav)
    d0 = s.stateDigest
    s.run(100)
    assert s.stateDigest == d0
    n, T = 16, 4
    s = sg.Simulation(gpu, nx=n, ny=n, nz=n, omega=0.0)
    f = np.zeros((19, n ** 3), np.float32)
    c = (8 * n + 8) * n + 8
    cx = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
    cy = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1]
    cz = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1]
    for i in range(1, 19):
        f[i, c] = np.float32(i) * np.float32(0.001)
    s.uploadState(f)
    s.run(T)
    g = s.downloadState()
    for i in range(1, 19):
        dest = (((8 + T * cz[i]) % n) * n + (8 + T * cy[i]) % n) * n + (8 + T * cx[i]) % n
        assert g[i, dest] == np.float32(i) * np.float32(0.001)
    assert np.count_nonzero(g) == 18


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_determinism_and_digest(gpu, precision):
    """Cases.swift:374-399: run twice, identical digests; digest = SHA-256 of the bytes."""
    import strouhal_gb300 as sg

    digests = []
    for _ in range(2):
        s = sg.Simulation(gpu, precision=precision, nx=64, ny=64, nz=64, omega=1.9)
        s.initField(1, 0.05)
        s.run(100)
        dg = s.stateDigest
        assert dg == hashlib.sha256(s.downloadState().tobytes()).hexdigest()
        digests.append((dg, s.massSum(), s.kineticEnergySum(), s.dissipationSum()))
        s.close()
    assert digests[0] == digests[1]


def test_mass_energy_dissipation_vs_oracle(gpu, oracle):
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 30, 26, 10
    wp = 1.6

    def cav(x, y, z):
        if y == ny - 1:
            return po.LID
        if x == 0 or x == nx - 1 or y == 0:
            return po.SOLID
        return po.FLUID

    g, o = _mk_pair(sg, po, gpu, 0, nx, ny, nz, flags=cav, omega=wp, lid=(0.1, 0, 0))
    o.initField(2, 0.04)
    g.uploadState(o.f)
    g.run(10)
    o.run(10)
    assert np.isclose(g.massSum(), o.massSum(), rtol=1e-12, atol=1e-9)
    assert np.isclose(g.kineticEnergySum(), o.kineticEnergySum(), rtol=1e-12, atol=0)
    # both sums from one reduction, as the separate calls return them
    assert g.observables() == (g.kineticEnergySum(), g.dissipationSum())
    # dissipation: 2 nu S:S from Pi_neq, recomputed in float64 from the same state
    f = o.f.astype(np.float64)
    m = o.probeMoments().astype(np.float64)
    fluid = o.flags == 0
    rho = 1.0 + f.sum(0)
    ux, uy, uz = m[:, 0], m[:, 1], m[:, 2]
    u2 = ux * ux + uy * uy + uz * uz
    W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    P = np.zeros((6, f.shape[1]))
    for i in range(1, 19):
        cu = 3 * (po.CX[i] * ux + po.CY[i] * uy + po.CZ[i] * uz)
        d = f[i] - W[i] * ((rho - 1) + rho * (cu + 0.5 * cu * cu - 1.5 * u2))
        c = (po.CX[i], po.CY[i], po.CZ[i])
        for k, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
            P[k] += c[a] * c[b] * d
    pipi = P[0] ** 2 + P[1] ** 2 + P[2] ** 2 + 2 * (P[3] ** 2 + P[4] ** 2 + P[5] ** 2)
    nu = (1 / np.float32(wp) - 0.5) / 3
    diss = np.sum((2 * nu * (1.5 * np.float32(wp) / rho) ** 2 * pipi)[fluid])
    assert np.isclose(g.dissipationSum(), diss, rtol=1e-4), (g.dissipationSum(), diss)


def test_probe_preconditions(gpu):
    import strouhal_gb300 as sg

    s = sg.Simulation(gpu, nx=8, ny=8, nz=8, omega=1.5)
    s.run(1)
    with pytest.raises(sg.StrouhalError) as ei:
        s.probeMoments()
    assert ei.value.code == 5
    with pytest.raises(sg.StrouhalError) as ei:
        s.probeForce((0, 3), (0, 3))
    assert ei.value.code == 5
    with pytest.raises(ValueError):
        s.uploadState(np.zeros(10, np.float32))
    small = np.zeros(10, np.float32)  # the C ABI checks the size too
    assert sg.lib().stro_sim_upload_state(s._h, small.ctypes.data, small.nbytes) == 1
    assert s.checkFinite()
    bad = np.zeros((19, 512), np.float32)
    bad[3, 17] = np.nan
    s.uploadState(bad)
    assert not s.checkFinite()
