"""Per-stage cycle shares of the intra lattice tiles on a 1080p I-frame.

    python -m uavs3e_gb300.lattice_stages

Builds the profiling variant libuavs3e_cuda_stageclk.so (the library with
UAVS3E_LAT_STAGE_CLOCKS: thread 0 of each CTA reads clock64 at every CTA barrier of a tile),
runs the lattice of the benchmark's frame (1920x1080 intra_frame(seed 11), neighbours = org
+ uniform noise in [-5, 5] from seed 12, every CU of the 23 shapes, 33 modes, QP 27/32/37/42,
tuned layouts) three times and prints, for the last run, each stage's share of the summed CTA
cycles overall and per shape class.  The cycles are CTA residency between barriers (4 CTAs
share an SM), so the shares say where a tile spends its time, not SM issue counts.
"""
import ctypes as C
import importlib

import numpy as np

STAGES = ["tables/setup", "org+nbrs", "org rows", "predict", "satd+fwd row", "fwd col", "quant", "inv col",
          "inv row+ssd", "records"]


def main():
    import uavs3e_gb300 as u
    from uavs3e_gb300.synth import intra_frame
    path = importlib.import_module("uavs3e_gb300.build").build(stage_clocks=True)
    L = C.CDLL(path)
    u._declare(L)
    L.uavs3e_cuda_lattice_stage_clocks.argtypes = [C.c_void_p, C.c_int]
    u._lib = L
    u.init(0)
    W, H = 1920, 1080
    org = intra_frame(W, H, seed=11)
    rec = np.clip(org.astype(int) + np.random.default_rng(12).integers(-5, 6, org.shape), 0, 255).astype(np.uint8)
    cus = u.lattice_cus(W, H)
    clk = np.zeros((25, len(STAGES)), np.uint64)
    for _ in range(3):
        u.intra_lattice(org, rec, cus)
        u.check(L.uavs3e_cuda_lattice_stage_clocks(clk.ctypes.data, 1), "lattice_stage_clocks")
    tot = float(clk.sum())
    print("library:", path)
    print("summed CTA cycles of the frame: %.4g" % tot)
    print("stage shares:", "  ".join("%s %.3f" % (n, clk[:, k].sum() / tot) for k, n in enumerate(STAGES)))
    for c in range(25):
        ct = float(clk[c].sum())
        if ct:
            print("%2dx%-2d %.3f |" % (4 << (c // 5), 4 << (c % 5), ct / tot),
                  " ".join("%.2f" % (clk[c, k] / ct) for k in range(len(STAGES))))


if __name__ == "__main__":
    main()
