"""Uncertainty budget: the oracle pinned to the reference's gate arithmetic and
hand-worked cases, and the library's stro_uq_* entry points (through
strouhal_gb300.credibility) equal to the oracle bit for bit. CPU only."""
import math
import os
import re

import numpy as np
import pytest

import strouhal_gb300 as sg
from strouhal_gb300 import credibility as cr
from oracle import uq_oracle as uo


def same(a, b):
    """Equal doubles, NaN equal to NaN."""
    return (math.isnan(a) and math.isnan(b)) or a == b


def ar1(n, rho, seed, mean=3.2, sd=0.01):
    rng = np.random.default_rng(seed)
    e = rng.standard_normal(n)
    x = np.empty(n)
    x[0] = e[0]
    for k in range(1, n):
        x[k] = rho * x[k - 1] + e[k]
    return mean + sd * x


# ------------------------------------------------------------ oracle pins
def test_oracle_out_of_domain_refusal():
    # Sources/strouhal/Cases.swift:1143-1153: Re 250000, Ma 0.09, 48 cells,
    # "bluff body in channel" must be OUTSIDE and withhold the bar.
    v = uo.classify(250000.0, 0.09, 48, "bluff body in channel")
    assert v.verdict == uo.OUTSIDE
    assert v.reasons == uo.OUT_RE
    assert math.isnan(uo.combined(0.01, 0.01, 0.01, v))


def test_oracle_street_ladder_in_domain():
    # The DFG 2D-2 ladder the reference's M4 gate runs ([32, 48, 64] cells,
    # base Mach 0.075): finest rung 64 at Ma = 0.075 * 2/3 * sqrt(3) = 0.0866.
    v64 = uo.street_variant(64, 1.0)
    assert abs(v64["mach"] - 0.0866) < 1e-4
    verdict = uo.classify(100.0, v64["mach"], 64, "bluff body in channel")
    assert verdict.verdict == uo.INSIDE and verdict.anchor == 2 and verdict.factor == 1.0
    # 32 cells lies (40 - 32) / 40 = 0.2 below DFG 2D-2's 40-80; DFG 2D-1 (Re 20) is
    # (100 - 20) / max(0, 10) = 8 away in Re, so 2D-2 is the nearest anchor
    near = uo.classify(100.0, v64["mach"], 32, "bluff body in channel")
    assert near.verdict == uo.NEAR_EDGE and near.anchor == 2
    assert near.distance == 8.0 / 40.0 and near.factor == 1.0 + 2.0 * (8.0 / 40.0)


def test_oracle_distance_and_geometry():
    assert uo.classify(50.0, 0.1, 64, "a wing").verdict == uo.OUTSIDE
    assert uo.classify(50.0, 0.1, 64, "a wing").reasons == uo.OUT_GEOMETRY
    # Poiseuille/TG anchor, Re 0-100: Re 120 is 20 / max(100, 50) = 0.2 outside
    v = uo.classify(120.0, 0.1, 64, "periodic / channel")
    assert v.verdict == uo.NEAR_EDGE and v.distance == 0.2
    # Ma 0.5 vs 0-0.35: (0.5 - 0.35) / 0.35 = 0.43 -> near edge; Ma 0.6 -> outside
    assert uo.classify(50.0, 0.5, 64, "periodic / channel").verdict == uo.NEAR_EDGE
    out = uo.classify(50.0, 0.6, 300, "periodic / channel")
    assert out.verdict == uo.OUTSIDE and out.reasons == uo.OUT_MACH | uo.OUT_RESOLUTION


def test_oracle_num_uncertainty_hand_worked():
    # monotone, converging: d1 = 0.08, d2 = 0.02, r = 64/48 -> order log(4)/log(4/3)
    n = uo.num_uncertainty([(64, 3.20, 0.001), (32, 3.10, 0.002), (48, 3.18, 0.002)])
    assert n.u_num == abs(3.20 - 3.18)
    assert n.observed_order == math.log(abs((3.18 - 3.10) / (3.20 - 3.18))) / math.log(64 / 48)
    assert n.note == uo.NOTE_SPREAD
    # finest pair within noise: u_num is the finest rung's stat
    n = uo.num_uncertainty([(48, 3.200, 0.01), (64, 3.205, 0.01)])
    assert n.u_num == 0.01 and n.note == uo.NOTE_INSENSITIVE and n.observed_order is None
    # non-monotone: no order
    assert uo.num_uncertainty([(32, 3.1, 0.0), (48, 3.3, 0.0), (64, 3.2, 0.0)]).observed_order is None
    one = uo.num_uncertainty([(64, 3.2, 0.01)])
    assert math.isnan(one.u_num) and one.note == uo.NOTE_SINGLE


def test_oracle_stat_hand_worked():
    # 24 samples of period-2 alternation: every batch (of an even length) has the
    # same mean, so the batch-means variance is zero and lag-1 is NaN -> no batch
    # count qualifies, the min-batch attempt is returned, untrustworthy.
    v = [1.0, 3.0] * 12
    s = uo.stat_uncertainty(v)
    assert s.batches == 6 and s.mean == 2.0 and s.half_width95 == 0.0 and math.isnan(s.lag1)
    assert not s.trustworthy
    short = uo.stat_uncertainty([1.0] * 23)
    assert short.batches == 0 and math.isnan(short.half_width95) and short.mean == 1.0
    # independent samples: the first (largest) batch count qualifies
    w = ar1(4000, 0.0, 7)
    s = uo.stat_uncertainty(w)
    assert s.batches == 16 and s.trustworthy


def test_oracle_schedule_matches_ladder_measure():
    # Ladder.swift:55-66 for the finest M4 rung: transient 96000, sample 192000,
    # stride max(8, int(26 * 1.6)) & ~1 = 40, chunk 38 -> 40 steps per sample
    v = uo.street_variant(64, 1.0)
    assert (v["transient"], v["sample"], v["stride"]) == (96000, 192000, 40)
    at = uo.sample_schedule(0, v["transient"], v["sample"], v["stride"])
    assert len(at) == 4800 and at[0] == 96040 and at[-1] == 96000 + 192000
    assert uo.sample_schedule(0, 11, 5, 8) == [10 + 8]
    assert uo.sample_schedule(0, 10, 0, 8) == []


# ------------------------------------------------------ library == oracle
@pytest.mark.parametrize("rho,n,seed", [(0.0, 4000, 1), (0.5, 4000, 2), (0.9, 4000, 3),
                                        (0.98, 2400, 4), (0.0, 24, 5), (0.3, 23, 6),
                                        (0.7, 97, 7), (-0.6, 500, 8)])
def test_stat_matches_oracle(rho, n, seed):
    v = ar1(n, rho, seed)
    got = cr.StatUncertainty.of(v)
    want = uo.stat_uncertainty(v)
    assert got.batches == want.batches
    assert same(got.mean, want.mean) and same(got.halfWidth95, want.half_width95)
    assert same(got.lag1, want.lag1) and got.trustworthy == want.trustworthy


def test_stat_batch_bounds_and_errors():
    v = ar1(1000, 0.4, 9)
    for mx, mn in [(16, 6), (20, 4), (8, 8), (7, 3)]:
        got = cr.StatUncertainty.of(v, mx, mn)
        want = uo.stat_uncertainty(v, mx, mn)
        assert (got.batches, got.mean, got.halfWidth95) == (want.batches, want.mean,
                                                            want.half_width95)
    with pytest.raises(sg.StrouhalError):
        cr.StatUncertainty.of(v, 4, 6)
    with pytest.raises(sg.StrouhalError):
        cr.StatUncertainty.of(v, 6, 1)


@pytest.mark.parametrize("rungs", [
    [(32, 3.10, 0.002), (48, 3.18, 0.002), (64, 3.20, 0.001)],
    [(64, 3.20, 0.001), (32, 3.10, 0.002), (48, 3.18, 0.002)],
    [(48, 3.200, 0.01), (64, 3.205, 0.01)],
    [(32, 3.1, 0.0), (48, 3.3, 0.0), (64, 3.2, 0.0)],
    [(64, 3.2, float("nan"))],
    [(40, 3.2, float("nan")), (42, 3.19, float("nan")), (41, 3.0, 0.1)],
    [(32, 3.0, 0.01), (48, 3.1, 0.01), (64, 3.1, 0.01)],
    [(16, 2.5, 0.05), (24, 2.9, 0.04), (32, 3.05, 0.03), (48, 3.15, 0.02)],
])
def test_num_matches_oracle(rungs):
    got = cr.NumUncertainty.of([cr.LadderRung(*r) for r in rungs])
    want = uo.num_uncertainty(rungs)
    assert same(got.uNum, want.u_num) and got.noteCode == want.note
    assert (got.observedOrder is None) == (want.observed_order is None)
    if want.observed_order is not None:
        assert got.observedOrder == want.observed_order


def test_mach_matches_oracle():
    for a, b in [(3.21, 3.19), (3.19, 3.21), (1.0, 1.0), (0.1, 0.3)]:
        assert cr.MachUncertainty.of(a, b).uMa == uo.mach_uncertainty(a, b)


def test_anchors_match_oracle():
    got = cr.ValidationDomain.anchors()
    assert len(got) == len(uo.ANCHORS)
    for a, (name, re, ma, n, geo) in zip(got, uo.ANCHORS):
        assert (a.name, a.re, a.mach, a.cellsPerFeature, a.geometry) == (name, re, ma, n, geo)


CLASSIFY_CASES = [
    (100.0, 0.0866, 64, "bluff body in channel"), (100.0, 0.0866, 32, "bluff body in channel"),
    (250000.0, 0.09, 48, "bluff body in channel"), (20.0, 0.1, 50, "bluff body in channel"),
    (60.0, 0.1, 50, "bluff body in channel"), (100.0, 0.2, 90, "bluff body in channel"),
    (500.0, 0.1, 192, "enclosed"), (2000.0, 0.1, 192, "enclosed"), (90.0, 0.1, 192, "enclosed"),
    (50.0, 0.5, 64, "periodic / channel"), (50.0, 0.6, 300, "periodic / channel"),
    (120.0, 0.1, 64, "periodic / channel"), (50.0, 0.1, 64, "a wing"),
    (float("nan"), 0.1, 64, "enclosed"), (100.0, float("nan"), 64, "bluff body in channel"),
]


@pytest.mark.parametrize("re,ma,n,geo", CLASSIFY_CASES)
def test_classify_and_combined_match_oracle(re, ma, n, geo):
    got = cr.ValidationDomain.classify(re, ma, n, geo)
    want = uo.classify(re, ma, n, geo)
    assert got.kind == want.verdict and got._c.anchor == want.anchor
    assert got._c.reasons == want.reasons
    assert same(got.distance, want.distance) and same(got.factor, want.factor)
    for parts in [(0.01, 0.02, 0.03), (float("nan"), 0.02, 0.03), (0.5, float("nan"), 0.0)]:
        b = cr.UncertaintyBudget("C_D", 3.2, *parts, verdict=got)
        assert same(b.combined, uo.combined(*parts, want))
    if want.verdict == uo.OUTSIDE:
        assert "OUTSIDE" in cr.UncertaintyBudget("C_D", 1.0, 0.01, 0.01, 0.01, got).headline
        assert got.reasons


def test_series_tail_and_mean_match_oracle():
    v = list(ar1(101, 0.5, 11))
    s = cr.QoISeries("C_D")
    for k, x in enumerate(v):
        s.append(k, x)
    t = s.stationaryTail(0.5)
    assert t.values == uo.stationary_tail(v, 0.5)
    assert t.mean == uo.qoi_mean(uo.stationary_tail(v, 0.5))
    assert math.isnan(cr.QoISeries("x").mean)


def test_street_variant_constants_match_oracle():
    """StreetLadder's lattice and schedule without building a simulation."""
    for n, ms in [(32, 1.0), (48, 1.0), (64, 1.0), (64, 0.5), (24, 1.0)]:
        o = uo.street_variant(n, ms)
        D = n
        scale = float(D) / 40.0 / ms
        assert o["transient"] == int(60000 * scale) & ~1
        assert o["nx"] == 22 * D + 2 and o["ny"] == int(4.1 * D) + 2
        # the half-Mach variant runs twice the steps of the base one
    assert uo.street_variant(64, 0.5)["sample"] == 2 * uo.street_variant(64, 1.0)["sample"]


def test_report_renders_outside_and_inside():
    inside = cr.ValidationDomain.classify(100.0, 0.0866, 64, "bluff body in channel")
    far = cr.ValidationDomain.classify(250000.0, 0.09, 48, "bluff body in channel")
    rungs = [cr.LadderRung(32, 3.10, 0.002), cr.LadderRung(48, 3.18, 0.002),
             cr.LadderRung(64, 3.20, 0.001)]
    num = cr.NumUncertainty.of(rungs)
    stat = cr.StatUncertainty.of(ar1(2400, 0.0, 12))
    mach = cr.MachUncertainty.of(3.20, 3.19)
    for verdict, word in [(inside, "Inside"), (far, "Outside")]:
        b = cr.UncertaintyBudget("mean C_D", 3.20, num.uNum, stat.halfWidth95, mach.uMa, verdict,
                                 [num.note])
        run = cr.CredibilityRun("mean C_D", b, rungs, num, stat, mach, 1.0, 0.5, 10, "ab" * 32,
                                "setup", "sequential")
        md = cr.report_markdown(run, ["a gate"])
        assert word in md and "| 64 | 3.2000 | 0.0010 |" in md and "a gate" in md
        if verdict is far:
            assert "withheld" in md and "Re 250000" in md


# ---------------------------------------------- pins read from the reference text
REF = os.environ.get("STRO_REFERENCE_ROOT", "/root/reference")


def ref_text(*parts):
    path = os.path.join(REF, "Sources", *parts)
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    with open(path, encoding="utf-8") as fh:
        return fh.read()


def test_oracle_anchors_equal_the_reference_table():
    """The anchors as written in Uncertainty.swift's `anchors` table."""
    src = ref_text("StrouhalCore", "Uncertainty.swift")
    body = re.search(r"static let anchors: \[Anchor\] = \[(.*?)\n    \]", src, re.S).group(1)
    pat = re.compile(r'\.init\(name: "(.*?)",\s*re: ([\d.]+)\.\.\.([\d.]+), mach: ([\d.]+)'
                     r'\.\.\.([\d.]+), cellsPerFeature: (\d+)\.\.\.(\d+),\s*geometry: "(.*?)"\)', re.S)
    ref = [(m[0], (float(m[1]), float(m[2])), (float(m[3]), float(m[4])), (int(m[5]), int(m[6])),
            m[7]) for m in pat.findall(body)]
    assert len(ref) == 4 and ref == uo.ANCHORS


def test_oracle_refusal_inputs_equal_the_reference_gate():
    """The M4 gate's out-of-domain inputs and reference mean (Cases.swift)."""
    src = ref_text("strouhal", "Cases.swift")
    m = re.search(r"classify\(re: ([\d_]+), mach: ([\d.]+),\s*cellsPerFeature: (\d+), "
                  r'geometry: "(.*?)"\)', src)
    re_, ma, n, geo = float(m[1].replace("_", "")), float(m[2]), int(m[3]), m[4]
    assert (re_, ma, n, geo) == (250000.0, 0.09, 48, "bluff body in channel")
    v = uo.classify(re_, ma, n, geo)
    assert v.verdict == uo.OUTSIDE and math.isnan(uo.combined(0.01, 0.01, 0.01, v))
    assert "let refMean = 3.18" in src and "resolutions: [Int] = [32, 48, 64]" in src


def test_oracle_street_schedule_equals_the_reference_source():
    """StreetLadder.variant's schedule constants as written in CaseSetups.swift."""
    src = ref_text("StrouhalCore", "CaseSetups.swift")
    for needle in ("let scale = Double(cellsPerFeature) / 40.0 / machScale",
                   "let transient = Int(60_000 * scale) & ~1",
                   "let sample = Int(120_000 * scale) & ~1",
                   "let stride = max(8, Int(26 * scale)) & ~1",
                   "mach: Double(u) * 2.0 / 3.0 * 3.0.squareRoot()",
                   "return 2.0 * f.x / (uMean * uMean * Double(cellsPerFeature))",
                   "let nx = lengthD * D + 2", "let ny = Int(4.1 * Double(D)) + 2",
                   "rampSteps: 24_000", "lambda: 3.0 / 16.0"):
        assert needle in src, needle
    lad = ref_text("StrouhalCore", "Ladder.swift")
    for needle in ("try v.sim.run(steps: v.transientSteps & ~1)",
                   "let chunk = max(2, v.stride - 2) & ~1", "taken += chunk + 2",
                   "series.stationaryTail(discarding: 0.5)"):
        assert needle in lad, needle
