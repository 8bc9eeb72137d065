"""GPU parity of the fused-multiply-add arithmetic (stro_sim_set_arithmetic).

The fused arithmetic is a fixed operation sequence that the oracle evaluates
identically (oracle kinds 3 and 4), so the GPU's DDFs must be EQUAL in value
to the fused oracle's after any number of steps, for every kernel variant,
the bulk / boundary block split and the force-probe steps. Against the FP64
oracle the stated tolerances hold (1e-5 FP32 storage, 2e-3 FP16 storage,
normwise relative after N = 50 steps)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PREC = {0: "fp32", 1: "fp16s"}


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("geometry", ["periodic", "channel", "xfaces"])
@pytest.mark.parametrize("split", [True, False, "columns", "noface"])
@pytest.mark.parametrize("collision", ["trt", "srt"])
@pytest.mark.parametrize("ffield", [False, True])
def test_fused_step_matches_fused_oracle(gpu, oracle, kind, geometry, split, collision, ffield):
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 37, 21, 9
    rng = np.random.default_rng(17 + kind + 2 * (geometry == "channel") + 4 * bool(split))
    flags = None
    eps = None
    kw = dict(omega=1.55, omegaMinus=1.2 if collision == "trt" else 1.55, uin=0.05, rampSteps=7,
              force=(3e-5, -1e-5, 2e-5), cSmago=0.01, wantsForces=True)
    if geometry == "channel":
        fl = np.zeros((nz, ny, nx), np.uint8)
        fl[:, 0, :] = fl[:, -1, :] = po.SOLID
        fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = po.INFLOW
        fl[:, 8:11, 12:15] = po.SOLID
        flags = fl.reshape(-1)
        eps = np.zeros(nx * ny * nz, np.float32)
        idx = rng.choice(nx * ny * nz, 120, replace=False)
        eps[idx] = rng.uniform(0.02, 0.98, idx.size).astype(np.float32)
    elif geometry == "xfaces":  # inflow columns over every row: x-face blocks
        fl = np.zeros((nz, ny, nx), np.uint8)
        fl[:, :, 0] = fl[:, :, -1] = po.INFLOW
        fl[:, 8:11, 12:15] = po.SOLID
        flags = fl.reshape(-1)
        eps = np.zeros(nx * ny * nz, np.float32)
        cand = np.flatnonzero((np.arange(nx * ny * nz) % nx >= 18) &
                              (np.arange(nx * ny * nz) % nx <= 28))
        idx = rng.choice(cand, 120, replace=False)
        eps[idx] = rng.uniform(0.02, 0.98, idx.size).astype(np.float32)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=nx, ny=ny, nz=nz, flags=flags,
                      arithmetic="fused", **kw)
    o = po.OracleSim(nx, ny, nz, flags=flags, kind=kind, arithmetic="fused", **kw)
    assert g.arithmetic == "fused"
    g.sponge = o.sponge = (14.0, 8.0, 0.85)
    if eps is not None:
        g.setSolidFractions(eps)
        o.setSolidFractions(eps)
    if ffield:  # per-cell Guo force field, some cells without a field force
        ff = (rng.standard_normal((3, nx * ny * nz)) * 2e-5).astype(np.float32)
        ff[:, rng.random(nx * ny * nz) < 0.3] = 0.0
        g.setForceField(ff)
        o.setForceField(ff)
    g.setBlockSplit(split)
    # 16-wide blocks on xfaces: the NT cells (x = 18..28) fill the middle
    # column of blocks only, both x faces get blocks of their own
    g.block = (16, 4) if geometry == "xfaces" else (32, 4)
    f0 = (rng.standard_normal((19, nx * ny * nz)) * 0.01).astype(o.f.dtype)
    o.f[:] = f0
    g.uploadState(f0)
    for chunk in (1, 4, 3):
        g.run(chunk)
        o.run(chunk)
        assert np.array_equal(g.downloadState(), o.f), (chunk, g.stepsDone)
    if geometry == "xfaces" and split in (True, "columns"):
        assert g.splitBlocks[1] > 0  # the x-face kernels ran
    if split == "noface":
        assert g.splitBlocks[1] == 0
    if geometry != "periodic":
        box = ((3, 30), (1, 18))
        fg, fo = g.probeForce(*box), o.probeForce(*box)
        assert np.allclose(fg, fo, rtol=1e-12, atol=1e-12), (fg, fo)
        assert np.array_equal(g.downloadState(), o.f)
    g.close()


@pytest.mark.parametrize("variant,shape", [(0, (64, 2)), (2, (128, 1)), (2, (256, 2)),
                                           (3, (32, 4)), (1, None), (4, (32, 2)), (5, (32, 1))])
@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("feature", ["plain", "force_les_sponge", "ffield"])
@pytest.mark.parametrize("srt", [False, True])
def test_fused_variants_match_fused_oracle(gpu, oracle, variant, shape, kind, feature, srt):
    """Periodic lattice: every variant in the fused arithmetic (variants 1, 4
    and 5 exist for FP16 storage; with FP32 storage they run variant 0)."""
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = (256 if variant in (4, 5) else 64), 6, 5
    kw = dict(omega=1.7, omegaMinus=1.7 if srt else 1.3)
    if feature == "force_les_sponge":
        kw.update(force=(2e-5, -3e-5, 1e-5), cSmago=0.01)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=nx, ny=ny, nz=nz, arithmetic="fused", **kw)
    o = po.OracleSim(nx, ny, nz, kind=kind, arithmetic="fused", **kw)
    if feature == "force_les_sponge":
        g.sponge = o.sponge = (nx * 0.6, nx * 0.3, 0.9)
    g.variant = variant
    if variant == 2:
        g.rowsTile = shape
    elif shape is not None:
        g.block = shape
    rng = np.random.default_rng(nx + variant + 10 * kind)
    if feature == "ffield":  # per-cell Guo force field, some cells without a field force
        ff = (rng.standard_normal((3, nx * ny * nz)) * 2e-5).astype(np.float32)
        ff[:, rng.random(nx * ny * nz) < 0.3] = 0.0
        g.setForceField(ff)
        o.setForceField(ff)
    f0 = (rng.standard_normal((19, nx * ny * nz)) * 0.01).astype(o.f.dtype)
    g.uploadState(f0)
    o.f[:] = f0
    for chunk in (1, 2, 3):
        g.run(chunk)
        o.run(chunk)
        assert np.array_equal(g.downloadState(), o.f), chunk
    expect = {0: "cell", 1: "pair" if kind == 1 else "cell", 2: "rows", 3: "capped",
              4: "wide4" if kind == 1 else "cell", 5: "wide8" if kind == 1 else "cell"}[variant]
    assert g.lastPath == expect, g.lastPath
    g.close()


@pytest.mark.parametrize("kind,tol", [(0, 1e-5), (1, 2e-3)])
def test_fused_fp64_tolerance(gpu, oracle, kind, tol):
    import strouhal_gb300 as sg

    po = oracle
    n, u0 = 24, 0.05
    tau = 3 * u0 * (n / (2 * np.pi)) / 1600 + 0.5
    wp, wm = sg.trtOmegas(tau, 3.0 / 16.0) if kind == 0 else sg.trtOmegas(tau)
    g = sg.Simulation(gpu, precision=PREC[kind], nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm,
                      arithmetic="fused")
    o = po.OracleSim(n, n, n, omega=wp, omegaMinus=wm, kind=po.KIND_F64, threads=8)
    o.initField(2, u0)
    g.uploadState(o.f.astype(np.float32 if kind == 0 else np.float16))
    g.run(50)
    o.run(50)
    err = np.linalg.norm(g.downloadState().astype(np.float64) - o.f) / np.linalg.norm(o.f)
    assert err <= tol, err
    g.close()


def test_fused_is_deterministic_and_differs_from_reference(gpu):
    import strouhal_gb300 as sg

    digests = {}
    for ar in ("fused", "fused", "reference"):
        s = sg.Simulation(gpu, precision="fp16s", nx=64, ny=32, nz=16, omega=1.9, arithmetic=ar)
        s.initField(2, 0.05)
        s.run(20)
        digests.setdefault(ar, []).append(s.stateDigest)
        s.close()
    assert digests["fused"][0] == digests["fused"][1]
    assert digests["fused"][0] != digests["reference"][0]


def test_batch_and_adjoint_refuse_the_fused_arithmetic(gpu):
    import strouhal_gb300 as sg

    s = sg.Simulation(gpu, precision="fp32", nx=16, ny=8, nz=4, omega=1.5, arithmetic="fused",
                      wantsForces=True)
    with pytest.raises(sg.StrouhalError):
        sg.Batch(gpu, [s])
    with pytest.raises(sg.StrouhalError):
        sg.Adjoint(s, 4, ((1, 3), (1, 3)))
    s.arithmetic = "reference"
    a = sg.Adjoint(s, 4, ((1, 3), (1, 3)))
    a.close()
    s.close()
