"""The credibility layer: a resolution ladder plus a half-Mach anchor around
a time-averaged quantity of interest, and the uncertainty budget built from
them (Sources/StrouhalCore/Uncertainty.swift, Ladder.swift and the
`StreetLadder` case of CaseSetups.swift:161-203).

    U(phi) = k sqrt(u_num^2 + u_stat^2 + u_Ma^2),  k = 2,

published only when the run lies inside (or near the edge of) the validated
domain. The statistics are the library's `stro_uq_*` entry points (host
doubles, the reference's operation order). Each variant's stepping is one
`stro_sim_run_sampled` submission: the transient, then chunk + force-probe
pairs whose FP64 box forces are reduced on the GPU into a device buffer and
read back once, instead of one host round trip per sample. The variants are
independent lattices, and `Ladder.credibility(mode=...)` runs them
  "sequential"  one after another (the reference's order),
  "concurrent"  each on its own context (its own CUDA stream) from its own
                host thread,
  "batched"     all in one batched submission (`stro_batch_run_sampled`: one
                persistent kernel or one launch per round over every
                variant's tiles, force probes fused into the odd pass),
  "streams"     one `stro_batch_run_sampled` submission in the batch's
                streams mode: every variant's own schedule on its own stream
                of one context, enqueued from one host thread.
The lattices end bitwise the same in every mode; the batched box-force sums
are folded per tile instead of per block, so its samples agree to FP64
rounding (the other modes' samples are equal).
"""
from __future__ import annotations

import ctypes
import math
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import (Batch, Cell, DomainVerdict, GPU, LadderRungC, NumUQ, Simulation, StatUQ,
               _check, diskSolidFractions, lib, trtOmegas)

MODES = ("sequential", "concurrent", "batched", "streams")

NAN = float("nan")


# --------------------------------------------------------------------- series
@dataclass
class QoISeries:
    """A scalar QoI sampled at step counts (Uncertainty.swift:21-45)."""
    name: str
    steps: list = field(default_factory=list)
    values: list = field(default_factory=list)

    def append(self, step, value):
        self.steps.append(float(step))
        self.values.append(float(value))

    @property
    def mean(self):
        if not self.values:
            return NAN
        s = 0.0
        for v in self.values:
            s += v
        return s / float(len(self.values))

    def stationaryTail(self, discarding=0.5):
        """Drop the first `discarding` fraction of the record."""
        cut = int(float(len(self.values)) * discarding)
        return QoISeries(self.name, self.steps[cut:], self.values[cut:])


@dataclass
class StatUncertainty:
    """Batch-means u_stat (Uncertainty.swift:47-101)."""
    mean: float
    halfWidth95: float
    batches: int
    lag1: float
    trustworthy: bool

    @classmethod
    def of(cls, series, maxBatches=16, minBatches=6):
        v = np.ascontiguousarray(series.values if isinstance(series, QoISeries) else series,
                                 np.float64)
        out = StatUQ()
        _check(lib().stro_uq_stat(v.ctypes.data, v.size, maxBatches, minBatches,
                                  ctypes.byref(out)))
        return cls(out.mean, out.half_width95, out.batches, out.lag1, bool(out.trustworthy))


@dataclass
class LadderRung:
    cellsPerFeature: int
    value: float
    stat: float


_NUM_NOTES = (
    "one resolution only: u_num is not estimated without a ladder",
    "the two finest rungs agree within their statistical noise: the QoI does not move "
    "with resolution over the tested range",
    "u_num is the spread between the two finest rungs (no Richardson extrapolation, "
    "no GCI)",
)


@dataclass
class NumUncertainty:
    """Ladder spread u_num (Uncertainty.swift:115-163)."""
    rungs: list
    uNum: float
    observedOrder: float | None
    noteCode: int

    @property
    def note(self):
        return _NUM_NOTES[self.noteCode]

    @classmethod
    def of(cls, rungs):
        arr = (LadderRungC * max(len(rungs), 1))()
        for i, r in enumerate(rungs):
            arr[i] = LadderRungC(int(r.cellsPerFeature), float(r.value), float(r.stat))
        out = NumUQ()
        _check(lib().stro_uq_num(arr, len(rungs), ctypes.byref(out)))
        return cls(sorted(rungs, key=lambda r: r.cellsPerFeature), out.u_num,
                   out.observed_order if out.has_order else None, out.note)


@dataclass
class MachUncertainty:
    """u_Ma from the half-Mach shift, error ~ Ma^2 (Uncertainty.swift:165-179)."""
    baseline: float
    halfMach: float
    uMa: float

    @classmethod
    def of(cls, baseline, halfMach):
        u = ctypes.c_double()
        _check(lib().stro_uq_mach(float(baseline), float(halfMach), ctypes.byref(u)))
        return cls(float(baseline), float(halfMach), u.value)


# --------------------------------------------------------- validation domain
INSIDE, NEAR_EDGE, OUTSIDE = 0, 1, 2


@dataclass
class Anchor:
    name: str
    re: tuple
    mach: tuple
    cellsPerFeature: tuple
    geometry: str


@dataclass
class Verdict:
    kind: int                  # INSIDE, NEAR_EDGE or OUTSIDE
    anchor: str | None
    factor: float
    distance: float
    reasons: list
    _c: DomainVerdict = None

    @property
    def isOutside(self):
        return self.kind == OUTSIDE


class ValidationDomain:
    """The validated domain: the reference's anchors (Uncertainty.swift:181-259)."""
    _anchors = None

    @classmethod
    def anchors(cls):
        if cls._anchors is None:
            out = []
            for k in range(64):
                name = ctypes.create_string_buffer(256)
                geo = ctypes.create_string_buffer(64)
                rng = np.zeros(4, np.float64)
                cells = np.zeros(2, np.int32)
                if lib().stro_uq_anchor(k, name, 256, rng.ctypes.data, cells.ctypes.data,
                                        geo, 64) != 0:
                    break
                out.append(Anchor(name.value.decode(), (rng[0], rng[1]), (rng[2], rng[3]),
                                  (int(cells[0]), int(cells[1])), geo.value.decode()))
            cls._anchors = out
        return cls._anchors

    @classmethod
    def classify(cls, re, mach, cellsPerFeature, geometry):
        v = DomainVerdict()
        _check(lib().stro_uq_classify(float(re), float(mach), int(cellsPerFeature),
                                      geometry.encode(), ctypes.byref(v)))
        anchors = cls.anchors()
        a = anchors[v.anchor] if v.anchor >= 0 else None
        reasons = []
        if v.verdict == OUTSIDE:
            if a is None:
                reasons.append("no validated case has the geometry class “%s”" % geometry)
            else:
                if v.reasons & 1:
                    reasons.append("Re %.0f is outside the validated %.0f–%.0f"
                                   % (re, a.re[0], a.re[1]))
                if v.reasons & 2:
                    reasons.append("Ma %.3f is outside the validated ≤%.2f" % (mach, a.mach[1]))
                if v.reasons & 4:
                    reasons.append("%d cells per feature is outside the validated %d–%d"
                                   % (cellsPerFeature, a.cellsPerFeature[0], a.cellsPerFeature[1]))
                if not reasons:
                    reasons.append("outside the validated domain")
        return Verdict(v.verdict, a.name if a else None, v.factor, v.distance, reasons, v)


# -------------------------------------------------------------------- budget
@dataclass
class UncertaintyBudget:
    """The assembled answer for one QoI (Uncertainty.swift:262-297)."""
    qoi: str
    value: float
    uNum: float
    uStat: float
    uMa: float
    verdict: Verdict
    notes: list = field(default_factory=list)

    @property
    def combined(self):
        c = ctypes.c_double()
        _check(lib().stro_uq_combined(float(self.uNum), float(self.uStat), float(self.uMa),
                                      ctypes.byref(self.verdict._c), ctypes.byref(c)))
        return c.value

    @property
    def headline(self):
        if self.verdict.isOutside:
            return "%s = %.4f, OUTSIDE the validated domain: no calibrated uncertainty" % (
                self.qoi, self.value)
        return "%s = %.4f ± %.4f (k=2)" % (self.qoi, self.value, self.combined)


# ---------------------------------------------------------------- the ladder
@dataclass
class LadderVariant:
    """One rebuilt case: the simulation, its Mach number, the force box whose
    samples make the QoI, the map from box forces (n, 3) to QoI values, and
    the schedule (Ladder.swift:37-51)."""
    sim: Simulation
    mach: float
    box: tuple
    qoi: object
    transientSteps: int
    sampleSteps: int
    stride: int


class StreetLadder:
    """The DFG 2D-2 vortex street rebuilt at any resolution and Mach scale,
    QoI mean C_D (CaseSetups.swift:29-64, 161-203): a channel 22 D long and
    4.1 D + 2 high, velocity-wall inlet and outlet, NT disk of diameter D at
    (2 D, 2 D), TRT Lambda = 3/16, cosine ramp over 24000 steps, outlet sponge
    3 D wide with tau 1. The schedule scales with D / 40 / machScale so every
    variant covers the same number of shedding cycles. `stepsFactor` < 1
    shortens the transient and the sampled record together (for tests; the
    reference schedule is 1)."""
    geometryClass = "bluff body in channel"

    def __init__(self, re=100.0, baseMach=0.075, precision="fp32", stepsFactor=1.0):
        self.re = float(re)
        self.baseMach = float(baseMach)
        self.precision = precision
        self.stepsFactor = float(stepsFactor)

    @property
    def setupDescription(self):
        return ("DFG 2D-2 cylinder in a channel, Re %.0f, velocity-wall inlet and outlet, "
                "NT curved body, outlet sponge, cosine ramp" % self.re)

    def variant(self, gpu, cellsPerFeature, machScale):
        D = int(cellsPerFeature)
        u = float(np.float32(self.baseMach * machScale))
        nx, ny = 22 * D + 2, int(4.1 * float(D)) + 2
        u_mean = u * 2.0 / 3.0
        wp, wm = trtOmegas(3.0 * (u_mean * float(D) / self.re) + 0.5, 3.0 / 16.0)
        cx = cy = 0.5 + 2.0 * float(D)
        flags = np.full((ny, nx), int(Cell.fluid), np.uint8)
        flags[:, 0] = flags[:, -1] = int(Cell.inflow)
        flags[0, :] = flags[-1, :] = int(Cell.solid)
        sim = Simulation(gpu, precision=self.precision, nx=nx, ny=ny, nz=1, omega=wp,
                         omegaMinus=wm, uin=u, rampSteps=24000, wantsForces=True,
                         flags=flags.reshape(-1))
        sim.setSolidFractions(diskSolidFractions(nx, ny, cx, cy, float(D) / 2.0))
        sim.sponge = (float(nx - 1 - 3 * D), float(3 * D), 1.0)
        scale = float(D) / 40.0 / machScale
        box = ((int(cx) - D // 2 - 3, int(cx) + D // 2 + 3),
               (int(cy) - D // 2 - 3, int(cy) + D // 2 + 3))

        def cd(forces, u_mean=u_mean, D=D):
            return 2.0 * forces[:, 0] / (u_mean * u_mean * float(D))

        f = self.stepsFactor
        return LadderVariant(sim=sim, mach=u * 2.0 / 3.0 * math.sqrt(3.0), box=box, qoi=cd,
                             transientSteps=int(60000 * scale * f) & ~1,
                             sampleSteps=int(120000 * scale * f) & ~1,
                             stride=max(8, int(26 * scale)) & ~1)


@dataclass
class Measurement:
    series: QoISeries
    stat: StatUncertainty
    digest: str
    gpuSeconds: float
    steps: int
    cells: int


@dataclass
class CredibilityRun:
    qoi: str
    budget: UncertaintyBudget
    rungs: list
    num: NumUncertainty
    stat: StatUncertainty
    mach: MachUncertainty
    wallSeconds: float
    gpuSeconds: float
    cellUpdates: int
    digest: str
    setup: str
    mode: str
    series: dict = field(default_factory=dict)  # label -> sampled tail values
    path: str = ""                               # kernel path (batched: the batch's)


class Ladder:
    @staticmethod
    def _measurement(v, qoi, forces, at, gpu_seconds, steps):
        series = QoISeries(qoi)
        for step, value in zip(at, v.qoi(forces)):
            series.append(step, value)
        tail = series.stationaryTail(0.5)
        return Measurement(tail, StatUncertainty.of(tail), v.sim.stateDigest, gpu_seconds, steps,
                           v.sim.cells)

    @staticmethod
    def measure(v, qoi):
        """One variant's time-averaged QoI (Ladder.swift:54-72): the second
        half of the sampled record, batch-means statistics."""
        sim = v.sim
        g0, s0 = sim.gpuSeconds, sim.stepsDone
        forces, at = sim.runSampled(v.transientSteps, v.sampleSteps, v.stride, *v.box)
        return Ladder._measurement(v, qoi, forces, at, sim.gpuSeconds - g0, sim.stepsDone - s0)

    @staticmethod
    def credibility(gpu, case, qoi, resolutions, progress=None, mode="sequential",
                    autotune=True):
        """Every resolution at the base Mach number plus the finest at half
        Mach, then the budget (Ladder.swift:74-121). `autotune` picks each
        variant's kernel and launch shape (or the batch's mode and tile) with
        a short timed trial on a copy of the state; results do not depend on
        it."""
        if mode not in MODES:
            raise ValueError("mode must be one of %s" % (MODES,))
        t0 = time.perf_counter()
        res = sorted(int(n) for n in resolutions)
        finest = res[-1]
        jobs = [(n, 1.0) for n in res] + [(finest, 0.5)]
        results = [None] * len(jobs)
        paths = []

        def one(k, g):
            n, ms = jobs[k]
            if progress:
                progress("%d cells per feature, Mach scale %.1f" % (n, ms))
            v = case.variant(g, n, ms)
            try:
                if autotune:
                    v.sim.autotune(200)
                results[k] = (v.mach, Ladder.measure(v, qoi))
                paths.append(v.sim.lastPath)
            finally:
                v.sim.close()

        if mode in ("batched", "streams"):
            variants = [case.variant(gpu, n, ms) for n, ms in jobs]
            batch = None
            try:
                if mode == "streams" and autotune:
                    for v in variants:  # each variant keeps its own kernel and shape
                        v.sim.autotune(200)
                batch = Batch(gpu, [v.sim for v in variants],
                              mode="persistent" if mode == "batched" else "streams")
                if autotune and mode == "batched":
                    batch.autotune(rounds=200)
                g0 = batch.gpuSeconds
                s0 = [v.sim.stepsDone for v in variants]
                out = batch.runSampled([v.transientSteps for v in variants],
                                       [v.sampleSteps for v in variants],
                                       [v.stride for v in variants], [v.box for v in variants])
                g = batch.gpuSeconds - g0
                paths.append(batch.lastPath)
                cells = sum(v.sim.cells * (v.sim.stepsDone - s) for v, s in zip(variants, s0))
                for k, (v, (forces, at)) in enumerate(zip(variants, out)):
                    steps = v.sim.stepsDone - s0[k]
                    # the batch's GPU time, shared out by cell updates
                    share = g * v.sim.cells * steps / cells if cells else 0.0
                    results[k] = (v.mach, Ladder._measurement(v, qoi, forces, at, share, steps))
            finally:
                if batch is not None:
                    batch.close()
                for v in variants:
                    v.sim.close()
        elif mode == "concurrent":
            errors = []
            ctxs = [GPU(gpu.device) for _ in jobs]

            def guarded(k):
                try:
                    one(k, ctxs[k])
                except BaseException as e:  # re-raised on the calling thread
                    errors.append(e)

            threads = [threading.Thread(target=guarded, args=(k,)) for k in range(len(jobs))]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            for c in ctxs:
                c.close()
            if errors:
                raise errors[0]
        else:
            for k in range(len(jobs)):
                one(k, gpu)

        rungs = [LadderRung(n, m.series.mean, m.stat.halfWidth95)
                 for (n, _), (_, m) in zip(jobs[:-1], results[:-1])]
        fine_mach, fine = results[len(res) - 1]
        half = results[-1][1]
        num = NumUncertainty.of(rungs)
        mach = MachUncertainty.of(rungs[-1].value, half.series.mean)
        verdict = ValidationDomain.classify(case.re, fine_mach, finest, case.geometryClass)
        notes = [num.note]
        if not fine.stat.trustworthy:
            notes.append("weak statistics: %d batches, lag-1 rho = %.2f; average over more "
                         "shedding cycles" % (fine.stat.batches, fine.stat.lag1))
        budget = UncertaintyBudget(qoi, rungs[-1].value, num.uNum, fine.stat.halfWidth95,
                                   mach.uMa, verdict, notes)
        return CredibilityRun(
            qoi=qoi, budget=budget, rungs=rungs, num=num, stat=fine.stat, mach=mach,
            wallSeconds=time.perf_counter() - t0,
            gpuSeconds=sum(m.gpuSeconds for _, m in results),
            cellUpdates=sum(m.steps * m.cells for _, m in results),
            digest=fine.digest, setup=case.setupDescription, mode=mode,
            series={("%d" % n if ms == 1.0 else "%d half-Mach" % n): m.series.values
                    for (n, ms), (_, m) in zip(jobs, results)},
            path=",".join(sorted(set(paths))))


def report_markdown(run, buildGates=()):
    """A markdown credibility report: the result, the budget by component,
    the ladder, the validation-domain verdict and what the bar leaves out
    (the sections of CredibilityReport.markdown, Ladder.swift:125-200)."""
    b = run.budget
    out = ["# Credibility report: %s" % run.qoi, "", "## Result", "",
           "**%s**" % b.headline, "", run.setup, "",
           "## Uncertainty budget", "",
           "U(phi) = k sqrt(u_num^2 + u_stat^2 + u_Ma^2) with k = 2 (about 95%).", "",
           "| component | value | how it was estimated |", "|---|---|---|",
           "| u_num (resolution) | %.4f | %s |" % (b.uNum, run.num.note),
           "| u_stat (time average) | %.4f | batch means of the second half of the record: "
           "%d batches, lag-1 rho %.2f |" % (b.uStat, run.stat.batches, run.stat.lag1),
           "| u_Ma (compressibility) | %.4f | rerun at half the lattice velocity: %.4f to %.4f, "
           "scaled by 4/3 for an O(Ma^2) error |" % (b.uMa, run.mach.baseline, run.mach.halfMach)]
    if b.verdict.kind == INSIDE:
        out.append("| **U(phi), k=2** | **%.4f** | inside the domain validated by %s |"
                   % (b.combined, b.verdict.anchor))
    elif b.verdict.kind == NEAR_EDGE:
        out.append("| **U(phi), k=2** | **%.4f** | near the edge of the domain validated by %s; "
                   "widened by a factor %.2f |" % (b.combined, b.verdict.anchor, b.verdict.factor))
    else:
        out.append("| **U(phi)** | **withheld** | outside the validated domain |")
    out += ["", "## Resolution ladder", "", "| cells per feature | value | u_stat |",
            "|---|---|---|"]
    out += ["| %d | %.4f | %.4f |" % (r.cellsPerFeature, r.value, r.stat) for r in run.rungs]
    out.append("")
    if run.num.observedOrder is not None:
        out.append("Observed order of convergence %.2f. It is a diagnostic: the bar does not "
                   "use it, because a fitted order assumes monotone convergence that "
                   "scale-resolving runs do not promise." % run.num.observedOrder)
    else:
        out.append("No observed order: the three finest rungs do not converge monotonically.")
    out += ["", "## Validation domain", ""]
    if b.verdict.kind == INSIDE:
        out.append("Inside the domain validated by %s." % b.verdict.anchor)
    elif b.verdict.kind == NEAR_EDGE:
        out.append("Near the edge of the domain validated by %s; the bar is widened by a "
                   "factor %.2f for the extrapolation distance." % (b.verdict.anchor,
                                                                    b.verdict.factor))
    else:
        out.append("**Outside the validated domain.** No calibrated bar is given:")
        out += ["- " + r for r in b.verdict.reasons]
    notes = [n for n in b.notes if n]
    if notes:
        out += ["", "## Notes", ""] + ["- " + n for n in notes]
    if buildGates:
        out += ["", "## Solver checks of this build", ""] + ["- " + g for g in buildGates]
    out += ["", "## Reproducibility", "",
            "- SHA-256 of the finest rung's final state: `%s`" % run.digest,
            "- %.1f s wall time, %.1f s on the GPU, %.3g cell updates, variants run %s" % (
                run.wallSeconds, run.gpuSeconds, float(run.cellUpdates),
                {"sequential": "one after another", "concurrent": "on concurrent streams",
                 "batched": "in one batched submission",
                 "streams": "on one stream each from one host thread"}[run.mode]),
            "", "## Not covered by the bar", "",
            "- Model-form error of the collision closure.",
            "- A grid convergence index: not defined for scale-resolving runs.",
            "- Agreement with experiment: a small u_num says the solver converged, not that "
            "the model is right; the validation-domain verdict is the only claim about that.",
            ""]
    return "\n".join(out)
