"""The reference's physics gates applied to recorded GPU runs (CPU only).

tests/records/*.json hold the measurements of full-size runs of
`python -m strouhal_gb300.cases <name>` (and the GPU gate tests with
STRO_RESULTS_DIR set) on a GB300. The published reference values these gates
compare against (Ghia centreline tables, DFG 2D-2 intervals, the TGV Re=1600
dissipation peak, the sphere drag correlation) are read from the reference's
own sources at test time and are not stored in this repository; those checks
skip where the reference tree is absent."""
import json
import math
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REC = os.path.join(HERE, "records")
REF = os.environ.get("STRO_REFERENCE_ROOT", "/root/reference")
CASES_SWIFT = os.path.join(REF, "Sources", "strouhal", "Cases.swift")
SETUPS_SWIFT = os.path.join(REF, "Sources", "StrouhalCore", "CaseSetups.swift")


def rec(name):
    path = os.path.join(REC, name + ".json")
    if not os.path.exists(path):
        pytest.skip("no record " + name)
    with open(path) as fh:
        return json.load(fh)


def ref_source(path):
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    with open(path) as fh:
        return fh.read()


def ref_table(src, name):
    m = re.search(r"let %s:[^=]*=\s*\[(.*?)\n\]" % name, src, re.S)
    rows = re.findall(r"\(\s*([-\d.]+)\s*,\s*([-\d.]+)(?:\s*,\s*([-\d.]+)\s*,\s*([-\d.]+))?\s*\)",
                      m.group(1))
    return [tuple(float(v) for v in r if v != "") for r in rows]


def ref_interval(src, var):
    m = re.search(r"%s >= ([\d.]+) && %s <= ([\d.]+)" % (re.escape(var), re.escape(var)), src)
    return float(m.group(1)), float(m.group(2))


def test_taylor_green_order_record():
    r = rec("tg_order")
    assert r["min_order"] >= 1.9  # Cases.swift:365


def test_poiseuille_record():
    """Wall error at the reference's level; the interior sits at the FP32
    floor of the uncontracted reference arithmetic (the oracle built from the
    reference's own kernel source reproduces this value bit for bit)."""
    r = rec("poiseuille")
    assert r["wall_err"] <= 3e-5
    assert r["max_err"] < 1e-4


def test_cavity_ghia_rms():
    src = ref_source(CASES_SWIFT)
    r = rec("cavity")
    from strouhal_gb300.cases import ghia_rms

    col = {100.0: 1, 400.0: 2, 1000.0: 3}[r["re"]]
    tu = [(row[0], row[col]) for row in ref_table(src, "ghiaU")]
    tv = [(row[0], row[col]) for row in ref_table(src, "ghiaV")]
    assert len(tu) >= 10 and len(tv) >= 10
    rms, _ = ghia_rms(r, tu, tv)
    assert rms <= 0.02, rms  # Cases.swift:270


def test_dfg2_windows():
    src = ref_source(CASES_SWIFT)
    r = rec("dfg2")
    lo, hi = ref_interval(src, "r.strouhal")
    assert lo <= r["strouhal"] <= hi, r["strouhal"]
    lo, hi = ref_interval(src, "r.maxCl")
    assert lo <= r["max_cl"] <= hi, r["max_cl"]
    assert r["cycles"] >= 15  # Cases.swift:964


def test_tgv_dissipation_peak():
    src = ref_source(CASES_SWIFT)
    m = re.search(r"let tgvRefPeak = \(t: ([\d.]+), eps: ([\d.]+)\)", src)
    t_ref, e_ref = float(m.group(1)), float(m.group(2))
    r = rec("tgv")
    assert r["nonfinite_at"] is None
    assert abs(r["peak_t"] - t_ref) <= 0.5  # Cases.swift:1312
    assert abs(r["peak_eps"] - e_ref) / e_ref <= 0.10  # Cases.swift:1322


def test_tgv_fp32_trt_is_reported():
    """TRT at u0 = 0.05 can go non-finite at transition (Cases.swift:1219-1221);
    the run must report where it stopped rather than hide it."""
    r = rec("tgv_fp32_trt")
    assert r["nonfinite_at"] is None or r["nonfinite_at"] > 1.0


@pytest.mark.parametrize("record", ["sphere", "sphere_fused"])
def test_sphere_drag_against_the_reference_correlation(record):
    src = ref_source(SETUPS_SWIFT)
    m = re.search(r"cdRef = ([\d.]+) / re \* \(1\.0 \+ ([\d.]+) \* pow\(re, ([\d.]+)\)\)", src)
    a, b, c = (float(m.group(k)) for k in (1, 2, 3))
    r = rec(record)
    assert r["finite"]
    cd = sum(r["cd"][-20:]) / 20
    ref = a / r["re"] * (1.0 + b * r["re"] ** c)
    assert abs(cd - ref) / ref < 0.10, (cd, ref)


def test_batched_ladder_reproduces_sequential():
    r = rec("ladder")
    for mode in ("persistent", "rounds", "streams"):
        if mode in r and "identical_states" in r[mode]:
            assert r[mode]["identical_states"]
            assert r[mode]["max_trace_rel_diff"] < 1e-12


def test_batched_small_rungs_beat_sequential():
    """Rungs too small to fill the GPU alone (edges 16-32): one batched launch
    per round against per-rung launches; identical states and traces."""
    r = rec("ladder_small")
    assert max(i["n"] for i in r["instances"]) <= 32
    for mode in ("persistent", "rounds", "streams"):
        assert r[mode]["identical_states"]
        assert r[mode]["max_trace_rel_diff"] < 1e-12
    assert max(r["persistent"]["speedup_vs_sequential"],
               r["rounds"]["speedup_vs_sequential"]) >= 3.0


def test_voxelizer_record_equals_oracle():
    """The GPU voxelization of the sphere wake's body at full size (512x256x256,
    65,024 triangles) hashed to the same SHA-256 as the oracle's restatement,
    recomputed here on the CPU."""
    import hashlib

    import numpy as np

    import strouhal_gb300 as sg
    from oracle import pyoracle as po

    r = rec("stl_voxelize")
    mesh = sg.StlMesh(sg.sphereSTLData(1.0, 256, 128))
    eps = po.mesh_solid_fractions(mesh.triangles, 512, 256, 256, 24.0,
                                  np.array([128.0, 128.0, 128.0], np.float32))
    assert hashlib.sha256(eps.tobytes()).hexdigest() == r["digest"]
    assert r["volume_rel_err"] < 0.01


def test_adjoint_cost_and_gradients():
    """Cost of the full-size adjoint windows: the whole backward sweep,
    recomputation included, within 3x the forward window (C3 cylinder, C5
    sphere wake). The gradients' 1e-3 check is test_adjoint_crop_records: an
    FP32 forward cannot resolve 1e-3 by finite differences (its own central
    differences at two step sizes disagree by more than that; the record keeps
    them as an indication only)."""
    r = rec("sphere_adjoint")
    assert r["grad_finite"]
    assert r["adjoint_step_over_forward_step"] <= 3.0
    assert r["backward_over_forward"] <= 3.0
    a = rec("dfg2_adjoint")
    assert a["backward_over_forward"] <= 3.0


def test_adjoint_crop_records():
    """Long windows (2,000 steps, sqrt(N) checkpoints) on crops of the C3
    cylinder and C5 sphere-wake lattices (tests/adjoint_crops.py): the GPU
    adjoint against the FP64 host adjoint of its own trajectory, and the GPU
    and FP64 adjoints against FP64 central differences, all within 1e-3
    (the FP16-storage solid-fraction gradient against differences of the FP64
    trajectory: the FP16 bar, 2e-2)."""
    for name in ("adjoint_crop_cylinder", "adjoint_crop_sphere"):
        r = rec(name)
        assert r["runs"]
        for run in r["runs"]:
            assert run["window"] >= 2000 and run["finite"], (name, run["precision"])
            assert run["J_rel_err"] < 1e-9
            assert run["grad_eps_rel_err"] < 1e-3, (name, run["precision"])
            assert run["grad_eps_zero_off_nt"]
            if name == "adjoint_crop_sphere":
                assert run["grad_force_rel_err"] < 1e-3, (name, run["precision"])
            for d in run["fd"]:
                assert d["fp64_adjoint_rel_err"] < 1e-3, (name, d)
                fp16_eps = run["precision"] == "fp16s" and d["param"].startswith("eps")
                assert d["gpu_adjoint_rel_err"] < (2e-2 if fp16_eps else 1e-3), (name, d)
        assert sum(len(run["fd"]) for run in r["runs"]) >= 8


# Error of each observable against the FP64 oracle (tests/precision_observables.py),
# FP32-arithmetic GPU runs over FP32 / FP16 storage: the bars the records are held to.
PRECISION_BARS = {
    "fp32": {"kinetic_energy": 1e-6, "dissipation_sum": 1e-6, "eps_dEdt": 1e-3,
             "drag_coefficient": 1e-5, "lift_coefficient_over_max_cd": 1e-4, "ddf_final": 1e-4},
    "fp16s": {"kinetic_energy": 1e-4, "dissipation_sum": 1e-2, "eps_dEdt": 5e-2,
              "drag_coefficient": 2e-2, "lift_coefficient_over_max_cd": 2e-2, "ddf_final": 3e-2},
}


def test_precision_records():
    """Per observable, per storage: the 48^3 and 256^3 (C2 lattice, 200 steps)
    Taylor-Green boxes and the D = 10 and D = 20 cylinder channels (20,000 steps,
    shedding: max |C_L| 0.73)."""
    seen = set()
    for name in ("precision_tgv48", "precision_tgv256", "precision_cylinder_d10",
                 "precision_cylinder_d20"):
        r = rec(name)
        for run in r["runs"]:
            for k, v in run["err"].items():
                bar = PRECISION_BARS[run["precision"]].get(k)
                if bar is None:
                    continue
                assert v < bar, (name, run["precision"], k, v)
                seen.add(k)
    assert {"kinetic_energy", "dissipation_sum", "eps_dEdt", "drag_coefficient",
            "lift_coefficient_over_max_cd"} <= seen
    assert rec("precision_tgv256")["lattice"] == [256, 256, 256]


def test_credibility_gates_and_budget_from_the_oracle():
    """The reference's credibility gate (Cases.swift:1103-1160) on the recorded
    DFG 2D-2 ladder ([32, 48, 64] cells and a half-Mach anchor at 64): a finite
    calibrated bar inside the validated domain, a bar within 0.05 of covering
    the published mean C_D 3.18, every rung recorded, and a refusal out of the
    domain. The budget is re-derived from the recorded sample tails with the
    oracle's statistics and must be the same doubles."""
    from oracle import uq_oracle as uo

    r = rec("credibility")
    assert r["resolutions"] == [32, 48, 64] and r["steps_factor"] == 1.0
    # every mode ends on the same lattice; QoIs equal (batched: to FP64 rounding)
    for mode in ("sequential", "concurrent", "batched", "streams"):
        assert r[mode + "_digest_equal"], mode
    assert r["concurrent_max_rel_diff"] == 0.0 and r["batched_max_rel_diff"] <= 1e-12
    assert r["streams_max_rel_diff"] == 0.0
    rungs = []
    for n, value, stat in r["rungs"]:
        tail = r["series"][str(n)]
        st = uo.stat_uncertainty(tail)
        assert value == uo.qoi_mean(tail) and stat == st.half_width95
        rungs.append((n, value, stat))
    num = uo.num_uncertainty(rungs)
    fine = uo.stat_uncertainty(r["series"]["64"])
    u_ma = uo.mach_uncertainty(rungs[-1][1], uo.qoi_mean(r["series"]["64 half-Mach"]))
    verdict = uo.classify(100.0, uo.street_variant(64, 1.0)["mach"], 64, "bluff body in channel")
    combined = uo.combined(num.u_num, fine.half_width95, u_ma, verdict)
    assert (r["u_num"], r["u_stat"], r["u_ma"], r["combined"]) == (
        num.u_num, fine.half_width95, u_ma, combined)
    assert (r["stat_batches"], r["stat_lag1"]) == (fine.batches, fine.lag1)
    # the four gates
    assert verdict.verdict == uo.INSIDE and math.isfinite(combined) and combined > 0
    assert abs(r["value"] - 3.18) <= combined + 0.05
    assert len(r["rungs"]) == 3
    far = uo.classify(250000.0, 0.09, 48, "bluff body in channel")
    assert far.verdict == uo.OUTSIDE and math.isnan(uo.combined(0.01, 0.01, 0.01, far))
    assert all(r["gates"].values())


def test_tgv_kbc_dissipation_peak_and_curve():
    """The KBC collision on the 256^3 FP16 TGV: the reference's peak gates
    (Cases.swift:1311-1327) and a dissipation curve at least as close to the
    DNS table as the SRT run's."""
    src = ref_source(CASES_SWIFT)
    m = re.search(r"let tgvRefPeak = \(t: ([\d.]+), eps: ([\d.]+)\)", src)
    t_ref, e_ref = float(m.group(1)), float(m.group(2))
    table = ref_table(src, "tgvReference")
    r, srt = rec("tgv_kbc"), rec("tgv")
    assert r["collision"] == "KBC" and r["nonfinite_at"] is None
    assert abs(r["peak_t"] - t_ref) <= 0.5
    assert abs(r["peak_eps"] - e_ref) / e_ref <= 0.10

    def rms(rr):
        t, e = rr["t_fd"], rr["eps_fd"]
        d = [min(range(len(t)), key=lambda k: abs(t[k] - tr)) for tr, _ in table
             if 1.0 <= tr <= 10.5]
        ref = [er for tr, er in table if 1.0 <= tr <= 10.5]
        return math.sqrt(sum((e[j] - v) ** 2 for j, v in zip(d, ref)) / len(ref))

    assert rms(r) <= rms(srt)


def test_kbc_carries_the_transitional_tgv_through_the_decay():
    """128^3, u0 = 0.1 (tau 0.5038): TRT Lambda = 1/4 goes non-finite in the
    transition (the reference measured t* = 5.4, Cases.swift:1290-1293); KBC
    runs the whole decay to t* = 14."""
    trt, kbc = rec("tgv_trt128_u01"), rec("tgv_kbc128_u01")
    assert trt["nonfinite_at"] is not None and trt["nonfinite_at"] < 6.0
    assert kbc["nonfinite_at"] is None and kbc["t"][-1] >= 13.9  # last sample before t* = 14
    assert all(b <= a for a, b in zip(kbc["E"], kbc["E"][1:]))


def test_tgv_m5_configuration_trt_reproduces_and_kbc_passes():
    """The reference's own TGV gate configuration (runTGV1600,
    Cases.swift:1217-1327: 288^3 and 320^3, u0 = 0.1, FP32, t* <= 10.5).
    With its TRT Lambda = 1/4 the library reproduces the peak the reference
    reports for Ma 0.173 (0.011887, 7.5% below the DNS); with KBC the three
    gates pass and the peak comes within 1% of the DNS."""
    src = ref_source(CASES_SWIFT)
    m = re.search(r"peak ([\d.]+) vs ([\d.]+) at Ma 0\.173", src)
    ref_trt_peak = float(m.group(2))
    m = re.search(r"let tgvRefPeak = \(t: ([\d.]+), eps: ([\d.]+)\)", src)
    t_ref, e_ref = float(m.group(1)), float(m.group(2))
    trt = {n: rec("tgv_m5_trt%d" % n) for n in (288, 320)}
    kbc = {n: rec("tgv_m5_kbc%d" % n) for n in (288, 320)}
    for r in list(trt.values()) + list(kbc.values()):
        assert r["u0"] == 0.1 and r["precision"] == "fp32" and r["nonfinite_at"] is None
    assert abs(trt[320]["peak_eps"] - ref_trt_peak) / ref_trt_peak < 1e-3
    f = kbc[320]
    assert abs(f["peak_t"] - t_ref) <= 0.5                                 # Cases.swift:1312
    assert abs(kbc[320]["peak_eps"] - kbc[288]["peak_eps"]) / e_ref <= 0.01  # Cases.swift:1316
    assert abs(f["peak_eps"] - e_ref) / e_ref <= 0.01                      # gate 10%, 1% here


def test_cavity_zperiodic_record():
    """3-D lattice, 2-D physics (Cases.swift:642-686): the z-periodic cavity's
    Re 400 centreline u against Ghia (the reference's interpolation) within an
    RMS of 0.02, and every z slice equal to z = 0 within 1e-5."""
    src = ref_source(CASES_SWIFT)
    r = rec("cavity_zperiodic")
    n, u = r["n"], r["u_centerline"]
    rows = ref_table(src, "ghiaU")
    ssq = 0.0
    for row in rows:
        pos = row[0] * n + 0.5
        k0 = min(max(int(math.floor(pos)), 1), n - 1)
        frac = pos - k0
        ours = u[k0 - 1] * (1.0 - frac) + u[k0] * frac
        ssq += (ours - row[2]) ** 2
    rms = math.sqrt(ssq / len(rows))
    assert rms <= 0.02, rms
    assert r["max_z_dev"] <= 1e-5, r["max_z_dev"]


def test_cavity_cubic_record():
    """Cubic cavity (Cases.swift:688-728): stable and mirror symmetric about
    the mid-z plane within 5e-4 u_lid RMS."""
    r = rec("cavity_cubic")
    assert r["finite"] and math.isfinite(r["centerline_umin"])
    assert r["asym_rms"] <= 5e-4, r["asym_rms"]


def test_rotation_record():
    """Rotation / anisotropy (Cases.swift:730-765): the +x-face lid cavity
    equals the standard one transposed within 5e-4 u_lid RMS."""
    r = rec("rotation")
    assert r["finite"]
    assert r["transposed_rms"] <= 5e-4, r["transposed_rms"]


def test_mass_drift_record():
    """Lid mass drift (Cases.swift:787-799): |sum(rho - 1)| <= 1e-2 after
    50,000 steps."""
    r = rec("mass_drift")
    assert r["steps"] == 50000
    assert abs(r["mass_drift"]) <= 1e-2, r["mass_drift"]


def test_dfg1_record():
    """Schaefer-Turek 2D-1 (Cases.swift:440-536): C_D within 1% of the
    spectral 5.57953523384."""
    r = rec("dfg1")
    assert r["cd_err"] <= 0.01, (r["cd"], r["cd_err"])


def test_cpu_baseline_port_against_the_reference_source():
    """The CPU baseline times the oracle port; the reference's own kernel
    source (compiled as C++) cannot run on the GPU machine. On the build host
    both run one thread on the same 96^3 Taylor-Green state
    (tests/cpu_reference_timing.py): they end on the same state bit for bit
    and the port's speed is within a factor of two of the reference code's, so
    the port's figure stands for the reference's CPU speed."""
    r = rec("cpu_reference_vs_port")
    assert {run["precision"] for run in r["runs"]} == {"fp16s", "fp32"}
    for run in r["runs"]:
        assert run["identical_states"], run["precision"]
        assert 0.5 <= run["port_over_reference_1_thread"] <= 2.0, run
