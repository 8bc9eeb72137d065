"""Time the D3Q19 step for one kernel variant on a periodic Taylor-Green box,
or (--street D) on the DFG 2D-2 street of the credibility ladder at D cells
per diameter (FP32 TRT, walls, NT disk, sponge; 22 D + 2 by 4.1 D + 2).

    python -m strouhal_gb300.stepbench --n 256 --precision fp16s --variant 2 --steps 20
    python -m strouhal_gb300.stepbench --street 64 --variant 0 --block 32 4 --split 0

Prints one line: lattice, precision, variant, launch shape, ms per step and
GLUPS (CUDA-event device time of the step launches). Useful for comparing the
variants on a given lattice and as a fixed command for profilers.
"""
import argparse
import math

import strouhal_gb300 as sg


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256, help="edge of the cubic lattice")
    ap.add_argument("--precision", default="fp16s", choices=["fp32", "fp16s"])
    ap.add_argument("--variant", type=int, default=-1, help="0, 1, 2, 3 or -1 = autotune")
    ap.add_argument("--block", type=int, nargs=2, default=None, metavar=("BX", "BY"),
                    help="launch shape of variants 0, 1 and 3; threads and rows per tile of variant 2")
    ap.add_argument("--trt", action="store_true", help="TRT Lambda=3/16 instead of SRT")
    ap.add_argument("--arith", default="reference", choices=["reference", "fused"],
                    help="step arithmetic (stro_sim_set_arithmetic)")
    ap.add_argument("--street", type=int, default=0, metavar="D",
                    help="the DFG 2D-2 street at D cells per diameter instead of the TGV box")
    ap.add_argument("--sphere", action="store_true",
                    help="the 512x256x256 sphere wake (FP16 storage, LES, NT sphere, sponge)")
    ap.add_argument("--split", type=int, default=-1, choices=[-1, 0, 1, 2, 3, 4, 5],
                    help="bulk / boundary split of walled lattices (-1 = library default, "
                         "2 = split with column-major boundary blocks in the odd pass, "
                         "3 = split without the x-face blocks, 4 = bulk and x-face blocks "
                         "in one launch, 5 = as 4 with FP16 bulk blocks two cells per thread)")
    ap.add_argument("--collision", default="reference", choices=["reference", "kbc"],
                    help="collision operator (stro_sim_set_collision)")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=4)
    a = ap.parse_args(argv)
    n = a.n
    L = n / (2 * math.pi)
    tau = 3 * 0.05 * L / 1600 + 0.5
    wp, wm = sg.trtOmegas(tau, 3.0 / 16.0 if a.trt else None)
    gpu = sg.GPU(0)
    if a.sphere:
        from . import cases
        s = cases.sphere_sim(gpu, precision=a.precision, arithmetic=a.arith)
        what = "sphere 512x256x256 LES"
    elif a.street:
        from . import credibility as cr
        s = cr.StreetLadder(precision=a.precision).variant(gpu, a.street, 1.0).sim
        if a.arith != "reference":
            s.arithmetic = a.arith
        what = "street D=%d %dx%d" % (a.street, s.nx, s.ny)
    else:
        s = sg.Simulation(gpu, precision=a.precision, nx=n, ny=n, nz=n, omega=wp, omegaMinus=wm,
                          arithmetic=a.arith)
        s.initField(2, 0.05)
        what = "lattice %d^3" % n
    if a.collision != "reference":
        s.collision = a.collision
    if a.split >= 0:
        s.setBlockSplit({2: "columns", 3: "noface", 4: "merged", 5: "pair"}.get(
            a.split, bool(a.split)))
    if a.variant < 0:
        s.autotune(steps=10)
    else:
        s.variant = a.variant
        if a.block and a.variant == 2:
            s.rowsTile = tuple(a.block)
        elif a.block and a.variant == 1:
            s.pairBlock = tuple(a.block)
        elif a.block:
            s.block = tuple(a.block)
    s.run(a.warmup)
    t0 = s.gpuSeconds
    s.run(a.steps)
    dt = s.gpuSeconds - t0
    bx, by = {1: s.pairBlock, 2: s.rowsTile}.get(s.variant, s.block)
    print("%s %s %s %s variant %d (%s) block %dx%d split %s: %.4f ms/step, %.2f GLUPS"
          % (what, a.precision, "KBC" if a.collision == "kbc" else
             ("TRT" if a.trt or a.street else "SRT"), a.arith, s.variant,
             s.lastPath, bx, by, a.split if a.split >= 0 else "default",
             1e3 * dt / a.steps, s.cells * a.steps / dt / 1e9))
    s.close()
    gpu.close()


if __name__ == "__main__":
    main()
