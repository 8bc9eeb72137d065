"""The CPU baseline's speed against the reference's own kernel source.

bench.py's CPU baseline (and its reference arm) time the oracle port (the
scalar restatement of Kernels.metal in oracle/lbm_oracle.cpp, OpenMP over
cells). The reference's own kernel source, compiled as C++ through the Metal
shim (oracle/_ref), only exists where the reference tree is present, which the
GPU machine is not. This script times both on the same host, one thread each, on
the same lattice (the 3-D Taylor-Green box, FP16 and FP32 storage, SRT), and
the port with every host thread, so the port's figure on the box can be read
against the reference's code:

    python tests/cpu_reference_timing.py --n 96 --out tests/records/cpu_reference_vs_port.json
"""
import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def time_pairs(sim, pairs):
    sim.run(2)  # warm-up pair
    t0 = time.perf_counter()
    sim.run(2 * pairs)
    return time.perf_counter() - t0


def main(argv=None):
    from oracle import build_oracle
    from oracle import pyoracle as po

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=96)
    ap.add_argument("--pairs", type=int, default=2)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    build_oracle.build_oracle()
    if build_oracle.build_ref() is None or po.ref_lib() is None:
        print("the reference tree is absent: nothing to time")
        return 1
    n = a.n
    L = n / (2 * np.pi)
    tau = 3 * 0.05 * L / 1600 + 0.5
    cells = n ** 3
    threads = os.cpu_count() or 1
    out = {"lattice": [n, n, n], "case": "TGV Re=1600, u0 0.05, SRT", "pairs": a.pairs,
           "host": platform.machine(), "host_threads": threads, "runs": []}
    for kind, name in ((po.KIND_F16, "fp16s"), (po.KIND_F32, "fp32")):
        row = {"precision": name}
        init = po.OracleSim(n, n, n, omega=1 / tau, kind=kind)
        init.initField(2, 0.05)  # one start state for all three (the initialisers may differ by an ulp)
        for label, backend, th in (("reference_source_1_thread", "ref", 1),
                                   ("port_1_thread", "oracle", 1),
                                   ("port_all_threads", "oracle", threads)):
            s = po.OracleSim(n, n, n, omega=1 / tau, kind=kind, backend=backend, threads=th)
            s.f[:] = init.f
            dt = time_pairs(s, a.pairs)
            row[label] = {"seconds": dt, "glups": cells * 2 * a.pairs / dt / 1e9, "threads": th}
            row.setdefault("states", []).append(s.stateDigest)
        row["identical_states"] = len(set(row.pop("states"))) == 1
        row["port_over_reference_1_thread"] = (row["port_1_thread"]["glups"] /
                                               row["reference_source_1_thread"]["glups"])
        out["runs"].append(row)
    out["command"] = "python tests/cpu_reference_timing.py --n %d --pairs %d" % (n, a.pairs)
    text = json.dumps(out, indent=1)
    print(text)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(text + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
