"""The credibility ladder on the GPU: stro_sim_run_sampled against the host
loop of Ladder.measure (Ladder.swift:54-66) and against the oracle, and a
short DFG 2D-2 ladder whose budget is re-derived with the oracle's
statistics (oracle/uq_oracle.py)."""
import math

import numpy as np
import pytest

import strouhal_gb300 as sg
from strouhal_gb300 import credibility as cr
from oracle import uq_oracle as uo

pytestmark = pytest.mark.gpu


def same(a, b):
    return (math.isnan(a) and math.isnan(b)) or a == b


def host_loop(sim, transient, sample, stride, box):
    """Ladder.measure's own loop: run(chunk), then the two-step probe."""
    sim.run(transient & ~1)
    chunk = max(2, stride - 2) & ~1
    forces, at, taken = [], [], 0
    while taken < sample:
        sim.run(chunk)
        forces.append(sim.probeForce(*box))
        taken += chunk + 2
        at.append(sim.stepsDone)
    return np.array(forces).reshape(-1, 3), np.array(at, np.int64)


@pytest.mark.parametrize("D,transient,sample,stride", [(10, 301, 600, 26), (12, 0, 97, 8),
                                                       (8, 40, 40, 3), (10, 20, 0, 26)])
def test_run_sampled_equals_host_loop(gpu, D, transient, sample, stride):
    case = cr.StreetLadder()
    a = case.variant(gpu, D, 1.0)
    b = case.variant(gpu, D, 1.0)
    fa, ata = a.sim.runSampled(transient, sample, stride, *a.box)
    fb, atb = host_loop(b.sim, transient, sample, stride, b.box)
    assert np.array_equal(fa, fb) and np.array_equal(ata, atb)
    assert list(ata) == uo.sample_schedule(0, transient, sample, stride)
    assert a.sim.stepsDone == b.sim.stepsDone and a.sim.stateDigest == b.sim.stateDigest
    if sample:
        assert np.all(np.isfinite(fa)) and np.any(fa[:, 0] != 0.0)
    a.sim.close()
    b.sim.close()


def test_run_sampled_matches_oracle(gpu, oracle):
    """Forces within 1e-12 of the oracle (FP64 box sums in different orders),
    final DDFs bitwise equal."""
    po = oracle
    D = 8
    v = cr.StreetLadder().variant(gpu, D, 1.0)
    s = v.sim
    o = po.OracleSim(s.nx, s.ny, 1, s.omega, s.omegaMinus, uin=s.uinTarget,
                     rampSteps=s.rampSteps, wantsForces=True, flags=s._flags, kind=po.KIND_F32)
    o.setSolidFractions(sg.diskSolidFractions(s.nx, s.ny, 0.5 + 2.0 * D, 0.5 + 2.0 * D, D / 2.0))
    o.sponge = s.sponge
    fg, at = s.runSampled(60, 120, 10, *v.box)
    fo, ato = host_loop(o, 60, 120, 10, v.box)
    assert np.array_equal(at, ato)
    assert np.allclose(fg, fo, rtol=1e-12, atol=1e-15), np.abs(fg - fo).max()
    assert np.array_equal(s.downloadState(), o.f)
    s.close()


@pytest.mark.parametrize("mode", ["persistent", "rounds", "rounds-unsplit", "sequential",
                                  "streams"])
def test_batch_run_sampled_equals_single_runs(gpu, mode):
    """Three variants of different sizes and schedules in one batched sampled
    run: DDFs and step counts bitwise those of Simulation.runSampled, forces
    within FP64 rounding (box sums folded per tile). Rounds mode runs the bulk
    tiles on the wall-free kernels unless the split is switched off."""
    unsplit = mode == "rounds-unsplit"
    mode = "rounds" if unsplit else mode
    case = cr.StreetLadder()
    plan = [(8, 1.0, 101, 300, 10), (10, 1.0, 40, 120, 26), (12, 0.5, 0, 64, 4)]
    solo, group = [], []
    for D, ms, tr, sa, sd in plan:
        a, b = case.variant(gpu, D, ms), case.variant(gpu, D, ms)
        solo.append((a, a.sim.runSampled(tr, sa, sd, *a.box)))
        group.append(b)
    batch = sg.Batch(gpu, [v.sim for v in group], mode=mode)
    if unsplit:
        batch.setSplit(False)
    out = batch.runSampled([p[2] for p in plan], [p[3] for p in plan], [p[4] for p in plan],
                           [v.box for v in group])
    assert batch.lastPath in ({"persistent": "persistent-graph", "rounds": "rounds-graph",
                               "sequential": "sequential", "streams": "streams"}[mode],)
    bulk, edge = batch.splitTiles
    if mode == "rounds" and not unsplit:
        assert bulk > 0 and edge > 0, (bulk, edge)
    else:
        assert (bulk, edge) == (0, 0)
    for (a, (fa, ata)), b, (fb, atb) in zip(solo, group, out):
        assert np.array_equal(ata, atb)
        assert b.sim.stepsDone == a.sim.stepsDone and b.sim.stateDigest == a.sim.stateDigest
        assert fa.shape == fb.shape and np.allclose(fb, fa, rtol=1e-12, atol=1e-16)
        if mode in ("sequential", "streams"):
            assert np.array_equal(fa, fb)
    batch.close()
    for (a, _), b in zip(solo, group):
        a.sim.close()
        b.sim.close()


def test_batch_run_sampled_long_rounds_stream(gpu):
    """A rounds-mode sampled run longer than one graph holds is launched round
    by round on the stream, with the same result. (Re 20 keeps the 6-cell
    cylinder stable over 33000 steps.)"""
    case = cr.StreetLadder(re=20.0)
    a, b = case.variant(gpu, 6, 1.0), case.variant(gpu, 6, 1.0)
    fa, _ = a.sim.runSampled(32000, 1000, 40, *a.box)
    assert np.all(np.isfinite(fa)) and np.all(fa[:, 0] > 0)
    batch = sg.Batch(gpu, [b.sim], mode="rounds")
    (fb, _), = batch.runSampled([32000], [1000], [40], [b.box])
    assert batch.lastPath == "rounds-stream" and min(batch.splitTiles) > 0
    assert b.sim.stateDigest == a.sim.stateDigest
    assert np.allclose(fb, fa, rtol=1e-12, atol=1e-16)
    batch.close()
    a.sim.close()
    b.sim.close()


def test_batch_run_sampled_errors(gpu):
    case = cr.StreetLadder()
    v = case.variant(gpu, 8, 1.0)
    batch = sg.Batch(gpu, [v.sim])
    with pytest.raises(sg.StrouhalError):
        batch.runSampled([10], [10], [0], [v.box])                 # stride < 1
    with pytest.raises(sg.StrouhalError):
        batch.runSampled([10], [10], [10], [((0, v.sim.nx), (0, 2))])  # box outside
    v.sim.run(1)
    with pytest.raises(sg.StrouhalError):
        batch.runSampled([10], [10], [10], [v.box])                # odd step count
    assert v.sim.stepsDone == 1
    batch.close()
    v.sim.close()


def test_run_sampled_errors(gpu):
    v = cr.StreetLadder().variant(gpu, 8, 1.0)
    s = v.sim
    L = sg.lib()
    f = np.zeros((2, 3))
    n = sg.ctypes.c_int64()
    # the capacity is checked before any step: state and step count unchanged
    rc = L.stro_sim_run_sampled(s._h, 10, 100, 10, *v.box[0], *v.box[1], f.ctypes.data, 2,
                                sg.ctypes.byref(n), None)
    assert rc != 0
    assert n.value == 10 and s.stepsDone == 0
    with pytest.raises(sg.StrouhalError):
        s.runSampled(10, 10, 10, (0, s.nx), (0, 3))    # box outside the lattice
    with pytest.raises(sg.StrouhalError):
        s.runSampled(10, 10, 0, *v.box)               # stride < 1
    s.run(1)
    with pytest.raises(sg.StrouhalError):
        s.runSampled(10, 10, 10, *v.box)              # odd step count
    s.close()
    plain = sg.Simulation(gpu, nx=16, ny=8, nz=1, omega=1.2)
    with pytest.raises(sg.StrouhalError):
        plain.runSampled(2, 10, 10, (1, 4), (1, 4))   # wantsForces off
    plain.close()


def _budget_from_oracle(run, finest):
    """The budget re-derived from the run's sampled tails with the oracle."""
    rungs = []
    for r in run.rungs:
        tail = run.series["%d" % r.cellsPerFeature]
        st = uo.stat_uncertainty(tail)
        assert same(r.value, uo.qoi_mean(tail)) and same(r.stat, st.half_width95)
        rungs.append((r.cellsPerFeature, r.value, r.stat))
    num = uo.num_uncertainty(rungs)
    half = uo.qoi_mean(run.series["%d half-Mach" % finest])
    u_ma = uo.mach_uncertainty(rungs[-1][1], half)
    fine = uo.stat_uncertainty(run.series["%d" % finest])
    v = uo.street_variant(finest, 1.0)
    verdict = uo.classify(100.0, v["mach"], finest, "bluff body in channel")
    return num, fine, u_ma, verdict, uo.combined(num.u_num, fine.half_width95, u_ma, verdict)


def test_short_ladder_budget_matches_oracle_and_modes_agree(gpu):
    case = cr.StreetLadder(stepsFactor=0.01)
    res = [24, 32, 40]
    seq = cr.Ladder.credibility(gpu, case, "mean C_D", res)
    con = cr.Ladder.credibility(gpu, case, "mean C_D", res, mode="concurrent")
    bat = cr.Ladder.credibility(gpu, case, "mean C_D", res, mode="batched")
    stm = cr.Ladder.credibility(gpu, case, "mean C_D", res, mode="streams")
    for r in (seq, con, bat, stm):
        assert [x.cellsPerFeature for x in r.rungs] == res
        assert r.digest == seq.digest
    # concurrent streams give the same bits as one variant after another
    assert [(x.value, x.stat) for x in seq.rungs] == [(x.value, x.stat) for x in con.rungs]
    assert seq.series == con.series == stm.series
    assert stm.path == "streams"
    # the batch folds box sums per tile: same QoIs to FP64 rounding
    for key, vals in seq.series.items():
        assert np.allclose(bat.series[key], vals, rtol=1e-12, atol=0), key
    assert bat.path in ("persistent-graph", "rounds-graph", "rounds-stream", "sequential")
    num, fine, u_ma, verdict, comb = _budget_from_oracle(seq, 40)
    b = seq.budget
    assert same(b.uNum, num.u_num) and same(b.uStat, fine.half_width95) and b.uMa == u_ma
    assert b.verdict.kind == verdict.verdict == uo.INSIDE
    assert same(b.combined, comb) and math.isfinite(b.combined)
    # the finest rung keeps the second half of its samples (transient 600, sample 1200)
    n = len(uo.sample_schedule(0, 600, 1200, uo.street_variant(40, 1.0)["stride"]))
    assert len(seq.series["40"]) == n - int(n * 0.5)
    md = cr.report_markdown(seq)
    assert "Inside" in md and "| 40 |" in md
