"""Oracle (test infrastructure only): the uncertainty-budget statistics of the
reference, restated in pure Python doubles, one function per reference type.

Only the tests import this module. It is the checker for the library's
`stro_uq_*` entry points and for `strouhal_gb300.credibility`, never part of
the product path.

Every expression keeps the reference's operation order, so the results are
the same IEEE doubles (Python floats are binary64; `math.sqrt` is correctly
rounded; `math.log` is the host's libm, the same one the library links):

- `qoi_mean`, `stationary_tail`: Sources/StrouhalCore/Uncertainty.swift:33-44
- `stat_uncertainty`:            Uncertainty.swift:66-100 (batch means)
- `num_uncertainty`:             Uncertainty.swift:129-162 (ladder spread)
- `mach_uncertainty`:            Uncertainty.swift:172-178 (half-Mach shift)
- `ANCHORS`, `classify`:         Uncertainty.swift:200-259 (validation domain)
- `combined`, `headline`:        Uncertainty.swift:272-297
- `sample_schedule`:             Sources/StrouhalCore/Ladder.swift:54-72 (Ladder.measure)
- `street_variant`:              Sources/StrouhalCore/CaseSetups.swift:29-64, 164-203

Parity pin: the reference ships no golden vectors for these statistics; the
tests pin this restatement to the reference's own gate arithmetic
(Sources/strouhal/Cases.swift:1103-1160: the out-of-domain refusal at
Re 250000, the in-domain classification of the DFG 2D-2 ladder) and to
hand-worked cases.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

NAN = float("nan")


def smax(x: float, y: float) -> float:
    """The reference language's max for doubles: y if y >= x else x."""
    return y if y >= x else x


# --- QoISeries (Uncertainty.swift:33-44) ----------------------------------------------
def qoi_mean(values) -> float:
    if len(values) == 0:
        return NAN
    s = 0.0
    for v in values:
        s += float(v)
    return s / float(len(values))


def stationary_tail(values, fraction: float = 0.5):
    cut = int(float(len(values)) * fraction)
    return list(values)[cut:]


# --- StatUncertainty (Uncertainty.swift:66-100) ---------------------------------------
@dataclass
class Stat:
    mean: float
    half_width95: float
    batches: int
    lag1: float

    @property
    def trustworthy(self) -> bool:
        return self.batches >= 6 and abs(self.lag1) <= 0.3


def _batch_stats(v, M):
    per = len(v) // M
    means = []
    for b in range(M):
        s = 0.0
        for x in v[b * per:(b + 1) * per]:
            s += x
        means.append(s / float(per))
    m = 0.0
    for x in means:
        m += x
    m = m / float(M)
    var_sum = 0.0
    for x in means:
        var_sum = var_sum + (x - m) * (x - m)
    sd = math.sqrt(var_sum / float(M - 1))
    num = den = 0.0
    for i in range(len(means)):
        den += (means[i] - m) * (means[i] - m)
        if i > 0:
            num += (means[i] - m) * (means[i - 1] - m)
    return m, 1.96 * sd / math.sqrt(float(M)), (num / den if den > 0 else NAN)


def stat_uncertainty(values, max_batches: int = 16, min_batches: int = 6) -> Stat:
    v = [float(x) for x in values]
    if len(v) < min_batches * 4:
        return Stat(qoi_mean(v), NAN, 0, NAN)
    for M in range(max_batches, min_batches - 1, -2):
        m, half, rho = _batch_stats(v, M)
        if abs(rho) <= 0.3:
            return Stat(m, half, M, rho)
    m, half, rho = _batch_stats(v, min_batches)
    return Stat(m, half, min_batches, rho)


# --- NumUncertainty (Uncertainty.swift:129-162) ---------------------------------------
NOTE_SINGLE = 0
NOTE_INSENSITIVE = 1
NOTE_SPREAD = 2


@dataclass
class Num:
    u_num: float
    observed_order: float | None
    note: int


def num_uncertainty(rungs) -> Num:
    """rungs: (cells_per_feature, value, stat) triples in any order."""
    r = sorted(rungs, key=lambda t: t[0])
    if len(r) < 2:
        return Num(NAN, None, NOTE_SINGLE)
    fine, mid = r[-1], r[-2]
    delta = abs(fine[1] - mid[1])
    fine_stat = 0.0 if math.isnan(fine[2]) else fine[2]
    u = smax(delta, fine_stat)
    order = None
    if len(r) >= 3:
        c = r[-3]
        d1 = mid[1] - c[1]
        d2 = fine[1] - mid[1]
        if d1 * d2 > 0 and abs(d2) < abs(d1) and abs(d2) > 0:
            ratio = float(fine[0]) / float(mid[0])
            if ratio > 1.05:
                order = math.log(abs(d1 / d2)) / math.log(ratio)
    return Num(u, order, NOTE_INSENSITIVE if delta <= fine_stat else NOTE_SPREAD)


# --- MachUncertainty (Uncertainty.swift:172-178) --------------------------------------
def mach_uncertainty(baseline: float, half_mach: float) -> float:
    return abs(baseline - half_mach) * 4.0 / 3.0


# --- ValidationDomain (Uncertainty.swift:200-259) -------------------------------------
# (name, (re_lo, re_hi), (ma_lo, ma_hi), (n_lo, n_hi), geometry): the reference's
# anchors, which are the gates its CLI runs on every build.
ANCHORS = [
    ("Ghia lid-driven cavity (RMS 0.004 vs published)", (100.0, 1000.0), (0.0, 0.18),
     (128, 256), "enclosed"),
    ("Schäfer–Turek DFG 2D-1 (C_D within 0.16%)", (20.0, 20.0), (0.0, 0.14),
     (40, 64), "bluff body in channel"),
    ("Schäfer–Turek DFG 2D-2 (St 0.2996, max C_L 0.9998)", (100.0, 100.0),
     (0.0, 0.14), (40, 80), "bluff body in channel"),
    ("Poiseuille (exact) / Taylor–Green (order 1.96)", (0.0, 100.0), (0.0, 0.35),
     (32, 128), "periodic / channel"),
]

INSIDE, NEAR_EDGE, OUTSIDE = 0, 1, 2
OUT_RE, OUT_MACH, OUT_RESOLUTION, OUT_GEOMETRY = 1, 2, 4, 8


def _distance(x, lo, hi):
    if lo <= x <= hi:
        return 0.0
    span = smax(smax(hi - lo, abs(hi) * 0.5), 1e-9)
    return (lo - x) / span if x < lo else (x - hi) / span


@dataclass
class Verdict:
    verdict: int
    anchor: int
    distance: float
    factor: float
    reasons: int


def classify(re: float, mach: float, cells_per_feature: int, geometry: str) -> Verdict:
    best, best_d = -1, 0.0
    for k, (_, (rl, rh), (ml, mh), (nl, nh), geo) in enumerate(ANCHORS):
        if geo != geometry:
            continue
        d = smax(_distance(re, rl, rh),
                 smax(_distance(mach, ml, mh), _distance(float(cells_per_feature), float(nl), float(nh))))
        if best < 0 or d < best_d:
            best, best_d = k, d
    if best < 0:
        return Verdict(OUTSIDE, -1, NAN, NAN, OUT_GEOMETRY)
    if best_d == 0:
        return Verdict(INSIDE, best, best_d, 1.0, 0)
    if best_d <= 0.5:
        return Verdict(NEAR_EDGE, best, best_d, 1.0 + 2.0 * best_d, 0)
    _, (rl, rh), (ml, mh), (nl, nh), _ = ANCHORS[best]
    reasons = 0
    if _distance(re, rl, rh) > 0:
        reasons |= OUT_RE
    if _distance(mach, ml, mh) > 0:
        reasons |= OUT_MACH
    if _distance(float(cells_per_feature), float(nl), float(nh)) > 0:
        reasons |= OUT_RESOLUTION
    return Verdict(OUTSIDE, best, best_d, NAN, reasons)


# --- UncertaintyBudget (Uncertainty.swift:272-297) ------------------------------------
def combined(u_num: float, u_stat: float, u_ma: float, v: Verdict) -> float:
    rss2 = 0.0
    for p in (u_num, u_stat, u_ma):
        if not math.isnan(p):
            rss2 = rss2 + p * p
    rss = math.sqrt(rss2)
    if v.verdict == INSIDE:
        return 2.0 * rss
    if v.verdict == NEAR_EDGE:
        return 2.0 * rss * v.factor
    return NAN


# --- Ladder.measure schedule (Ladder.swift:54-72) -------------------------------------
def sample_schedule(steps_done: int, transient: int, sample_steps: int, stride: int):
    """Step counts after each probe, in the order Ladder.measure takes them."""
    t = steps_done + (transient & ~1)
    chunk = max(2, stride - 2) & ~1
    taken, at = 0, []
    while taken < sample_steps:
        t += chunk + 2
        taken += chunk + 2
        at.append(t)
    return at


# --- StreetLadder.variant (CaseSetups.swift:29-64, 164-203) ---------------------------
def street_variant(cells_per_feature: int, mach_scale: float, base_mach: float = 0.075,
                   re: float = 100.0):
    """The lattice, schedule and probe constants of one ladder variant."""
    D = cells_per_feature
    u = float(np.float32(base_mach * mach_scale))        # Float(baseMach * machScale)
    nx = 22 * D + 2
    ny = int(4.1 * float(D)) + 2
    u_mean = u * 2.0 / 3.0
    nu = u_mean * float(D) / re
    tau = 3.0 * nu + 0.5
    cx = cy = 0.5 + 2.0 * float(D)
    scale = float(D) / 40.0 / mach_scale
    return {
        "nx": nx, "ny": ny, "uin": u, "u_mean": u_mean, "tau": tau,
        "cx": cx, "cy": cy, "r": float(D) / 2.0,
        "box_x": (int(cx) - D // 2 - 3, int(cx) + D // 2 + 3),
        "box_y": (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3),
        "sponge": (float(np.float32(nx - 1 - 3 * D)), float(np.float32(3 * D)), 1.0),
        "transient": int(60000 * scale) & ~1,
        "sample": int(120000 * scale) & ~1,
        "stride": max(8, int(26 * scale)) & ~1,
        "mach": u * 2.0 / 3.0 * math.sqrt(3.0),
    }
