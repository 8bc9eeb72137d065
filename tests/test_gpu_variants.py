"""GPU tests of the FP16 pair variant, the batched engine and the autotuners.

All of them must leave the lattice arithmetic untouched: DDFs are compared
value-for-value with the oracle or bitwise with plain stro_sim_run runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


VARIANT_CASES = [
    # (variant, precision, nx, ny, nz, launch shape: block of variants 0/1/3,
    #  (threads, rows per tile) of variant 2)
    (1, "fp16s", 64, 7, 5, (32, 1)), (1, "fp16s", 128, 6, 4, (64, 1)),
    (1, "fp16s", 192, 3, 3, (96, 1)), (1, "fp16s", 256, 3, 2, (128, 1)),
    (1, "fp16s", 512, 2, 2, (256, 1)), (1, "fp16s", 128, 5, 3, None),
    (2, "fp16s", 64, 7, 5, (256, 1)), (2, "fp16s", 40, 6, 4, (128, 2)),
    (2, "fp16s", 256, 3, 2, (256, 1)), (2, "fp16s", 256, 4, 2, (224, 2)),
    (2, "fp16s", 256, 4, 3, (256, 4)), (2, "fp16s", 256, 2, 3, (64, 1)),
    (2, "fp16s", 8, 9, 4, (32, 3)), (2, "fp16s", 24, 1, 3, (64, 1)),
    (2, "fp32", 36, 7, 5, (64, 1)), (2, "fp32", 128, 6, 3, (96, 2)), (2, "fp32", 4, 6, 5, (32, 6)),
    (2, "fp32", 256, 4, 2, (256, 2)),
    (3, "fp16s", 37, 7, 5, (32, 4)), (3, "fp32", 64, 6, 4, (32, 4)),
    # wide FP16 kernels: 4 / 8 cells per thread, one warp per row segment
    (4, "fp16s", 128, 6, 4, (32, 2)), (4, "fp16s", 256, 3, 3, (64, 1)),
    (4, "fp16s", 512, 2, 2, (32, 1)), (5, "fp16s", 256, 4, 3, (32, 4)),
    (5, "fp16s", 512, 3, 2, (64, 1)), (5, "fp16s", 256, 2, 2, (32, 2)),
]


PATHS = {0: "cell", 1: "pair", 2: "rows", 3: "capped", 4: "wide4", 5: "wide8"}


@pytest.mark.parametrize("variant,precision,nx,ny,nz,shape", VARIANT_CASES)
@pytest.mark.parametrize("feature", ["plain", "force", "les", "sponge", "ffield"])
def test_variant_matches_oracle(gpu, oracle, variant, precision, nx, ny, nz, shape, feature):
    import strouhal_gb300 as sg

    po = oracle
    kw = dict(omega=1.7, omegaMinus=1.3)
    if feature == "force":
        kw["force"] = (2e-5, -3e-5, 1e-5)
    if feature == "les":
        kw["cSmago"] = 0.01
    g = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, **kw)
    kind = po.KIND_F16 if precision == "fp16s" else po.KIND_F32
    o = po.OracleSim(nx, ny, nz, kind=kind, **kw)
    if feature == "sponge":
        g.sponge = (nx * 0.6, nx * 0.3, 0.9)
        o.sponge = (nx * 0.6, nx * 0.3, 0.9)
    g.variant = variant
    if variant == 2:
        g.rowsTile = shape
    elif variant == 1 and shape is not None:
        g.pairBlock = shape
    elif shape is not None:
        g.block = shape
    rng = np.random.default_rng(nx * 31 + ny + variant)
    if feature == "ffield":  # per-cell Guo force field with zero-force cells, on top of a uniform one
        ff = (rng.standard_normal((3, nx * ny * nz)) * 2e-5).astype(np.float32)
        ff[:, rng.random(nx * ny * nz) < 0.3] = 0.0
        g.force = o.force = (1e-5, 0.0, -1e-5)
        g.setForceField(ff)
        o.setForceField(ff)
    f0 = (rng.standard_normal((19, nx * ny * nz)) * 0.01).astype(o.f.dtype)
    g.uploadState(f0)
    o.f[:] = f0
    for chunk in (1, 2, 3):
        g.run(chunk)
        o.run(chunk)
        assert np.array_equal(g.downloadState(), o.f), chunk
    assert g.lastPath == PATHS[variant], g.lastPath  # the variant's own kernel ran
    g.close()


@pytest.mark.parametrize("precision", ["fp16s", "fp32"])
def test_variants_agree_bitwise(gpu, precision):
    import strouhal_gb300 as sg

    digests = []
    for variant, shape in ([(0, None), (1, None), (2, (256, 1)), (2, (256, 2)), (3, (64, 2)),
                            (4, (32, 4)), (4, (64, 1)), (5, (32, 2)), (5, (32, 1))]
                           if precision == "fp16s" else
                           [(0, None), (2, (128, 1)), (2, (256, 4)), (3, (64, 2))]):
        s = sg.Simulation(gpu, precision=precision, nx=256, ny=40, nz=24, omega=1.95)
        s.variant = variant
        if variant == 2:
            s.rowsTile = shape
        elif shape is not None:
            s.block = shape
        s.initField(2, 0.05)
        s.run(11)
        assert s.lastPath == PATHS[variant], (variant, s.lastPath)
        digests.append(s.stateDigest)
        s.close()
    assert len(set(digests)) == 1


@pytest.mark.parametrize("precision", ["fp16s", "fp32"])
def test_block_split_is_bitwise_neutral(gpu, precision):
    """Walled lattice with a Noble-Torczynski body, LES and a sponge: the
    bulk/boundary split and the single wall-aware kernel give identical states."""
    import strouhal_gb300 as sg

    nx, ny, nz = 96, 40, 24
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = sg.Cell.inflow
    flags[:, 0, :] = sg.Cell.solid
    eps = sg.sphereSolidFractions(nx, ny, nz, 30.5, 20.0, 12.0, 6.0, 4)
    digests = []
    for split in (True, False, "columns", "noface", "merged", "pair"):
        s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=1.8, uin=0.05,
                          rampSteps=10, cSmago=0.01, flags=flags.reshape(-1))
        s.inflowUniform = True
        s.setSolidFractions(eps)
        s.sponge = (70.0, 20.0, 1.0)
        s.setBlockSplit(split)
        s.initField(2, 0.02)
        s.run(13)
        digests.append(s.stateDigest)
        s.close()
    assert len(set(digests)) == 1


def _field(n_cells, seed):
    """A per-cell Guo force field with some zero-force cells."""
    rng = np.random.default_rng(seed)
    ff = (rng.standard_normal((3, n_cells)) * 2e-6).astype(np.float32)
    ff[:, rng.random(n_cells) < 0.3] = 0.0
    return ff


def _ladder(sg, gpu, precision="fp32"):
    """Uneven periodic TGV boxes (one with a per-cell force field) plus a ramped
    cavity and a channel with NT cells and a force field."""
    sims, steps, logs = [], [], []
    for n, u0, nsteps, le in [(32, 0.05, 40, 10), (48, 0.025, 62, 0), (16, 0.05, 12, 4),
                              (64, 0.05, 26, 2)]:
        L = n / (2 * np.pi)
        tau = 3 * u0 * L / 1600 + 0.5
        s = sg.Simulation(gpu, precision=precision, nx=n, ny=n, nz=n, omega=1 / tau)
        s.initField(2, u0)
        if n == 32:
            s.setForceField(_field(n ** 3, 3))
        sims.append(s)
        steps.append(nsteps)
        logs.append(le)
    n = 40

    def cav(x, y, z):
        if y == n - 1:
            return sg.Cell.lid
        if x == 0 or x == n - 1 or y == 0:
            return sg.Cell.solid
        return sg.Cell.fluid

    c = sg.Simulation(gpu, precision=precision, nx=n, ny=n, nz=3, omega=1.2, omegaMinus=1.0,
                      lid=(0.1, 0, 0), rampSteps=30, flags=cav)
    sims.append(c)
    steps.append(50)
    logs.append(10)
    ch = np.zeros((4, 20, 50), np.uint8)
    ch[:, 0, :] = ch[:, -1, :] = sg.Cell.solid
    ch[:, 1:-1, 0] = ch[:, 1:-1, -1] = sg.Cell.inflow
    d = sg.Simulation(gpu, precision=precision, nx=50, ny=20, nz=4, omega=1.5, omegaMinus=1.2,
                      uin=0.05, rampSteps=20, force=(1e-5, 0, 0), cSmago=0.01,
                      flags=ch.reshape(-1))
    eps = sg.diskSolidFractions(50, 20, 15.5, 9.5, 4.0)
    d.setSolidFractions(np.tile(eps, 4))
    d.setForceField(_field(50 * 20 * 4, 4))
    d.sponge = (35.0, 10.0, 0.9)
    sims.append(d)
    steps.append(33)
    logs.append(0)
    return sims, steps, logs


@pytest.mark.parametrize("mode", ["persistent", "rounds", "sequential", "streams"])
@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_batch_matches_independent_runs(gpu, mode, precision):
    import strouhal_gb300 as sg

    ref, steps, logs = _ladder(sg, gpu, precision)
    ref_traces = []
    for s, k, le in zip(ref, steps, logs):
        tr = []
        if le:
            tr.append(s.kineticEnergySum())
            for _ in range(k // le):
                s.run(le)
                tr.append(s.kineticEnergySum())
            s.run(k - (k // le) * le)
        else:
            s.run(k)
        ref_traces.append(np.array(tr))
    sims, _, _ = _ladder(sg, gpu, precision)
    b = sg.Batch(gpu, sims, mode=mode)
    traces = b.run(steps, logs)
    assert b.lastPath.startswith({"persistent": "persistent", "rounds": "rounds",
                                  "sequential": "sequential", "streams": "streams"}[mode])
    if mode == "rounds":  # the walled channel's bulk tiles ran on the wall-free kernels
        assert min(b.splitTiles) > 0, b.splitTiles
    for s, r, k, tr, rtr in zip(sims, ref, steps, traces, ref_traces):
        assert s.stepsDone == r.stepsDone == k
        assert np.array_equal(s.downloadState(), r.downloadState())
        assert len(tr) == len(rtr)
        assert np.allclose(tr, rtr, rtol=1e-12, atol=0)
    # a second run replays the cached graph from the new state
    steps2 = [6] * len(sims)
    b.run(steps2)
    for s, r in zip(sims, ref):
        r.run(6)
        assert np.array_equal(s.downloadState(), r.downloadState())
    b.close()


def test_batch_barrier_timeout_is_an_error_status(gpu):
    """A persistent batch whose barrier waits may poll only once gives up with
    STRO_ERR_TIMEOUT instead of waiting; the context stays usable."""
    import strouhal_gb300 as sg

    sims = [sg.Simulation(gpu, nx=96, ny=96, nz=96, omega=1.8) for _ in range(2)]
    b = sg.Batch(gpu, sims, mode="persistent")
    b.setSpinLimit(1)
    with pytest.raises(sg.StrouhalError) as ei:
        b.run([20, 20])
    assert ei.value.code == 6
    b.close()
    s = sg.Simulation(gpu, nx=16, ny=16, nz=16, omega=1.5)
    s.initField(2, 0.05)
    s.run(4)
    assert s.checkFinite()


@pytest.mark.parametrize("precision", ["fp16s", "fp32"])
def test_rows_wait_timeout_is_an_error_status(gpu, oracle, precision):
    """Variant 2 with a zero poll limit: its first bulk-copy wait gives up, the
    block drains its copies in flight and returns, the run fails with
    STRO_ERR_TIMEOUT, and the context and the lattice stay usable."""
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 256, 8, 6
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=1.7)
    s.variant = 2
    s.rowsTile = (256, 1)
    s.initField(2, 0.05)
    f0 = s.downloadState()
    s.setSpinLimit(0)
    with pytest.raises(sg.StrouhalError) as ei:
        s.run(2)
    assert ei.value.code == 6
    assert s.lastPath == "rows"
    # back to the default limit: the same lattice steps correctly again
    s.setSpinLimit(1 << 22)
    s.uploadState(f0)
    s.stepsDone = 0
    s.run(3)
    o = po.OracleSim(nx, ny, nz, omega=1.7, kind=po.KIND_F16 if precision == "fp16s" else po.KIND_F32)
    o.f[:] = f0
    o.run(3)
    assert np.array_equal(s.downloadState(), o.f)
    s.close()
    with pytest.raises(sg.StrouhalError):
        s2 = sg.Simulation(gpu, nx=8, ny=8, nz=8, omega=1.5)
        try:
            s2.setSpinLimit(-1)
        finally:
            s2.close()


def test_autotune_restores_state(gpu):
    import strouhal_gb300 as sg

    for precision in ("fp32", "fp16s"):
        s = sg.Simulation(gpu, precision=precision, nx=128, ny=64, nz=32, omega=1.9)
        s.initField(2, 0.05)
        s.run(3)
        d0, t0 = s.stateDigest, s.stepsDone
        bx, by, glups = s.autotune(steps=8)
        assert bx * by % 32 == 0 and glups > 0
        assert s.stateDigest == d0 and s.stepsDone == t0
        ref = sg.Simulation(gpu, precision=precision, nx=128, ny=64, nz=32, omega=1.9)
        ref.initField(2, 0.05)
        ref.run(3)
        s.run(5)
        ref.run(5)
        assert s.stateDigest == ref.stateDigest


def test_batch_autotune_restores_state(gpu):
    import strouhal_gb300 as sg

    sims, steps, _ = _ladder(sg, gpu)
    before = [s.stateDigest for s in sims]
    b = sg.Batch(gpu, sims)
    mode, bx, by, sec = b.autotune(rounds=6)
    assert mode in ("persistent", "rounds") and sec > 0
    assert [s.stateDigest for s in sims] == before
    assert all(s.stepsDone == 0 for s in sims)
    b.close()
