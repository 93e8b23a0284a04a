#!/usr/bin/env python3
"""Benchmark of the batched motion search on 1080p frames (the hot path's headline workload).

One step = one 1080p frame through the GPU path: the newest reconstructed picture becomes a
reference (device padding + 15-plane quarter-sample interpolation), then the integer full
search (+-64, 129^2 candidates) and the half/quarter-sample SATD refinement of every block of
the ten shapes 8x8..64x64 against 2 references.  Inputs are seeded synthetic 1080p frames
(the external sequence is unavailable).

  python bench.py [--gpus N --steps K --warmup W]         GPU path (one JSON line on rank 0)
  python bench.py --impl reference [...]                  the CPU restatement of the same path

Under torchrun each rank runs an independent replica on its own GPU (the path has no exchange
step); value is the sum of frames over all ranks / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, N_REFS, RANGE, QP, PAD = 1920, 1080, 2, 64, 32, 144
RING = 8                      # distinct frames cycled through (working set > L2)
CPU_SAMPLE_ROWS = 2           # CTU rows of one frame timed for the CPU baseline
METRIC = ("1080p full-search ME frames/s (batched motion-search kernel: +-64 integer full search + quarter-sample "
          "SATD refinement of every 8x8..64x64 block, 2 refs, bit-exact per-candidate costs)")
REF_SAMPLE_CTUS = 8           # CTUs of a frame searched per step by the reference arm
REF_CTU_STRIDE = 67           # CTU k of step s: (s * REF_SAMPLE_CTUS + k) * 67 mod 510 (67 is prime to 510)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--legs", default="me,lattice,pruning,lookahead,tz,rdoq,affme",
                    help="comma list of legs: me (the headline line), lattice, pruning, lookahead, tz, rdoq, affme")
    ap.add_argument("--pruning-steps", type=int, default=3000, help="training steps of the pruning leg")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(value, world, device):
    """the largest of every rank's value (replicas: the job's time is its slowest rank's)"""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank):
    """each replica searches its own synthetic sequence"""
    return 1000 * rank


def workload_config():
    """the workload of both arms (identical dicts: the GPU arm and the reference arm)"""
    from uavs3e_gb300.synth import lambda_mv_for_qp
    ctus = ((W + 63) // 64) * ((H + 63) // 64)
    return {
        "workload": "batched motion search of one 1920x1080 8-bit luma frame (the hot path's frame-level ME kernel, "
                    "not a full encode): integer full search +-64 and quarter-sample SATD refinement of every block "
                    "8x8..64x64 incl. 2:1 on the 64x64 CTU grid, against 2 references",
        "search_rule": "full search of the +-64 window (candidate costs bit-exact with cost_sad / com_had / the "
                       "me.c cost formula; the TZ search order of me_search_tz is the separate per-call kernel)",
        "width": W, "height": H, "refs": N_REFS, "search_range": RANGE, "qp": QP,
        "lambda_mv": lambda_mv_for_qp(QP), "ctus": ctus, "blocks_per_ctu": 169,
        "int_candidates_per_block": (2 * RANGE + 1) ** 2, "subpel_candidates_per_block": 17,
        "parallelism": "replicas",
        "l2": "GPU arm: flushed (256 MiB write) before every timed step; per-step CUDA events",
        "reference_arm_sample": f"each step searches {REF_SAMPLE_CTUS} CTUs spread over the frame (CTU "
                                f"(step*{REF_SAMPLE_CTUS}+k)*{REF_CTU_STRIDE} mod {ctus}); frames/s = CTUs searched / "
                                f"{ctus} / time",
    }


def frames_ring(seed=0):
    from uavs3e_gb300.synth import motion_sequence
    return motion_sequence(W, H, RING, seed=seed)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region"""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.p = None
        self.index = index
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sms, mx, reasons = [], 0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sms)}


class CpuSearch:
    """The oracle (C restatement, OpenMP over blocks) on the bench workload: reference planes are
    interpolated once; time_rows() times the search of `rows` CTU rows of one frame."""

    def __init__(self, frames, lam, threads=None):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import numpy as np
        import pyoracle
        from gpu_util import padded
        import uavs3e_gb300 as u
        self.np, self.pyoracle = np, pyoracle
        self.oracle = pyoracle.Oracle()
        self.threads = threads or os.cpu_count() or 1
        self.lam = lam
        self.stride = ((W + 2 * PAD) + 15) & ~15
        self.keep, self.ptrs = [], []
        for f in (frames[1], frames[0]):
            p0 = padded(f, PAD, self.stride)
            planes = [np.zeros_like(p0) for _ in range(15)]
            base = PAD * self.stride + PAD
            self.oracle.if_luma_frame(p0.ctypes.data + base, [p.ctypes.data + base for p in planes], W, H, PAD, self.stride)
            self.keep += [p0] + planes
            self.ptrs += [p0.ctypes.data + base] + [p.ctypes.data + base for p in planes]
        self.bl = u.me_blocks(W, H)
        self.org = np.ascontiguousarray(frames[2])

    def time_ctus(self, ctus):
        """search every block of the listed CTUs (indices in raster order); returns (seconds, blocks)"""
        np, bl = self.np, self.bl
        sel = np.isin(bl[:, 4], np.asarray(ctus)) & (bl[:, 0] + bl[:, 2] <= W) & (bl[:, 1] + bl[:, 3] <= H)
        blocks = np.zeros(int(sel.sum()), dtype=self.pyoracle.ME_BLOCK)
        blocks["x"], blocks["y"], blocks["w"], blocks["h"] = bl[sel, 0], bl[sel, 1], bl[sel, 2], bl[sel, 3]
        t0 = time.perf_counter()
        self.oracle.me_frame(self.org.ctypes.data, W, self.ptrs, self.stride, W, H, N_REFS, blocks, RANGE, self.lam,
                             threads=self.threads)
        return time.perf_counter() - t0, len(blocks)

    def time_rows(self, rows, first_row=4):
        cw = (W + 63) // 64
        return self.time_ctus(list(range(first_row * cw, (first_row + rows) * cw)))


def sample_ctus(step, n_ctu):
    return [((step * REF_SAMPLE_CTUS + k) * REF_CTU_STRIDE) % n_ctu for k in range(REF_SAMPLE_CTUS)]


def cpu_baseline(frames, lam, rows=CPU_SAMPLE_ROWS):
    cs = CpuSearch(frames, lam)
    dt, nb = cs.time_rows(rows)
    ctu_rows = (H + 63) // 64
    return {"value": (rows / ctu_rows) / dt, "unit": "frames/s", "cores": cs.threads, "kind": "port",
            "sample": f"{rows} of {ctu_rows} CTU rows of one 1080p frame ({nb} blocks x {N_REFS} refs, integer search "
                      f"+ refinement; reference interpolation not timed), {dt:.2f} s.  The oracle restatement is timed: "
                      f"the reference's own sources are not present on this host"}


def run_reference(args):
    """The CPU arm: the oracle restatement of the path (C, OpenMP over blocks, all host cores) on
    the GPU arm's workload, a bounded sample of CTUs per step.  Loads only the oracle's library:
    the block table and the frames are plain Python / numpy."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from uavs3e_gb300.synth import lambda_mv_for_qp
    frames = frames_ring()
    lam = lambda_mv_for_qp(QP)
    cs = CpuSearch(frames, lam)
    n_ctu = ((H + 63) // 64) * ((W + 63) // 64)
    for k in range(args.warmup):
        cs.time_ctus(sample_ctus(k, n_ctu)[:1])
    tot, blocks = 0.0, 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        dt, nb = cs.time_ctus(sample_ctus(k, n_ctu))
        tot += dt
        blocks += nb
    wall = time.perf_counter() - t0
    v = args.steps * (REF_SAMPLE_CTUS / n_ctu) / tot
    cb = {"value": v, "unit": "frames/s", "cores": cs.threads, "kind": "port",
          "sample": f"each step: every block of {REF_SAMPLE_CTUS} of the {n_ctu} CTUs of a 1080p frame, spread over "
                    f"the frame (interior and edge CTUs), 2 refs, integer + refinement ({blocks} blocks in "
                    f"{args.steps} steps); oracle restatement (the reference's own sources are not on the GPU host) "
                    f"on all host cores; frames/s = CTUs searched / {n_ctu} / time"}
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / max(1, args.steps),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
           "config": workload_config(), "cpu_baseline": cb,
           "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


LAT_QPS = (27, 32, 37, 42)
LAT_STRIP = (256, 320)        # rows of the CPU baseline's lattice sample


def lattice_frame():
    """config of the intra lattice leg: a 1080p I-frame, its reconstructed neighbours, all CUs"""
    import numpy as np
    from uavs3e_gb300.synth import intra_frame
    org = intra_frame(W, H, seed=11)
    rec = np.clip(org.astype(int) + np.random.default_rng(12).integers(-5, 6, org.shape), 0, 255).astype(np.uint8)
    return org, rec


def lattice_macs(cus):
    """transform multiply-adds of the lattice in matrix form: forward row + column pass, then per
    QP the inverse column + row pass (64-point transforms keep 32 coefficient lines)"""
    tot = 0
    for w, h in zip(cus["w"].astype(int), cus["h"].astype(int)):
        kw, kh = min(w, 32), min(h, 32)
        tot += kw * h * w + kh * kw * h + len(LAT_QPS) * (kh * kw * h + w * h * kw)
    return int(33 * tot)


def lattice_cpu_baseline(org, rec, cus):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import pyoracle
    sel = (cus["y"] >= LAT_STRIP[0]) & (cus["y"].astype(int) + cus["h"] <= LAT_STRIP[1])
    c = np.zeros(int(sel.sum()), dtype=pyoracle.CU)
    for f in ("x", "y", "w", "h"):
        c[f] = cus[f][sel]
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle()
    t0 = time.perf_counter()
    o.intra_lattice(org.ctypes.data, W, rec.ctypes.data, W, W, H, c, 0, list(LAT_QPS), is_intra=1, threads=threads)
    dt = time.perf_counter() - t0
    frac = (c["w"].astype(int) * c["h"]).sum() / float((cus["w"].astype(int) * cus["h"]).sum())
    return {"value": float(frac / dt), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"the CUs of rows {LAT_STRIP[0]}..{LAT_STRIP[1] - 1} ({len(c)} CUs, {100 * frac:.1f} % of the "
                      f"lattice's samples), oracle restatement, {dt:.2f} s"}


def lattice_leg(u, torch, stream, flush, peaks, sm_count, sm_mhz, with_cpu, reps=5):
    """intra/transform lattice of a 1080p I-frame: every CU of the 23 shapes, 33 modes, 4 QPs"""
    import numpy as np
    org, rec = lattice_frame()
    cus = u.lattice_cus(W, H)
    n = len(cus)
    lib = u.lib()
    d_org = torch.from_numpy(org).cuda()
    d_rec = torch.from_numpy(rec).cuda()
    d_cus = torch.from_numpy(cus.view(np.uint8).copy()).cuda()
    d_satd = torch.empty(n * 33, dtype=torch.int32, device="cuda")
    d_q = torch.empty(n * 33 * len(LAT_QPS) * 16, dtype=torch.uint8, device="cuda")
    qps = np.array(LAT_QPS, np.int32)
    sp = stream.cuda_stream

    def run():
        u.check(lib.uavs3e_cuda_intra_lattice_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(),
                                                     n, 0, qps.ctypes.data, len(qps), 1, d_satd.data_ptr(),
                                                     d_q.data_ptr(), sp), "intra_lattice")

    for _ in range(2):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    samples = 33 * int((cus["w"].astype(int) * cus["h"]).sum())
    macs = lattice_macs(cus)
    _, dp_clk = u.measure_dp2a_rate()
    peak = 2.0 * max(dp_clk, 64.0) * sm_count * sm_mhz * 1e6 / 1e9     # G multiply-adds/s at max clock
    out = {"workload": "intra lattice of a 1080p I-frame: all 468,750 CUs of the 23 shapes 4x4..64x64 (aspect <= 8), "
                       "33 modes, SATD + DCT2 + quant/dequant/inverse/recon/SSD at QP 27/32/37/42",
           "ms_per_frame": ms, "frames_per_s": 1000.0 / ms, "cus": n,
           "tuned_budgets_kb": {f"{4 << (c // 5)}x{4 << (c % 5)}": b // 1024
                                for c, b in enumerate(u.lattice_budgets(33)) if b},
           "predicted_samples_per_s": samples / (ms / 1000.0),
           "roofline": {"bound": "int", "kernel": "k_intra_lattice (all shape instances of a frame)",
                        "achieved": macs / (ms / 1000.0) / 1e9, "peak": peak, "unit": "GMAC/s",
                        "frac": macs / (ms / 1000.0) / 1e9 / peak, "traffic": None,
                        "macs_per_frame": macs,
                        "peak_source": f"2 x dp2a issue rate max(measured {dp_clk:.1f}, 64) per clk per SM x "
                                       f"{sm_count} SMs x {sm_mhz:.0f} MHz; matrix-form transform multiply-adds only "
                                       f"(prediction, SATD, quantisation not counted)"}}
    # end to end through the host-buffer entry uavs3e_cuda_intra_lattice: pinned picture, CUs and
    # records, the copies inside each call
    pin_org, pin_rec = (torch.from_numpy(a).pin_memory() for a in (org, rec))
    pin_cus = torch.from_numpy(cus.view(np.uint8).copy()).pin_memory()
    pin_satd = torch.empty(n * 33, dtype=torch.int32).pin_memory()
    pin_q = torch.empty(n * 33 * len(LAT_QPS) * 16, dtype=torch.uint8).pin_memory()

    def e2e():
        u.check(lib.uavs3e_cuda_intra_lattice(pin_org.data_ptr(), W, pin_rec.data_ptr(), W, W, H, pin_cus.data_ptr(),
                                              n, 0, qps.ctypes.data, len(qps), 1, pin_satd.data_ptr(),
                                              pin_q.data_ptr()), "intra_lattice (host)")

    e2e()
    t0 = time.perf_counter()
    for _ in range(reps):
        e2e()
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / reps
    out["e2e"] = {"ms_per_frame": e2e_ms, "frames_per_s": 1000.0 / e2e_ms,
                  "h2d_bytes_per_step": int(2 * W * H + n * 8),
                  "d2h_bytes_per_step": int(n * 33 * 4 + n * 33 * len(LAT_QPS) * 16),
                  "path": "uavs3e_cuda_intra_lattice (pinned host picture, CUs and records; copies inside the call)"}
    out["rmd"] = rmd_part(u, torch, stream, flush, d_satd, cus, with_cpu)
    out["intra_decision"] = intra_decision_part(u, torch, stream, flush, d_org, d_rec, d_cus, cus, qps)
    if with_cpu:
        out["cpu_baseline"] = lattice_cpu_baseline(org, rec, cus)
    return out


def intra_decision_part(u, torch, stream, flush, d_org, d_rec, d_cus, cus, qps, reps=5):
    """the encoder's order on the lattice: SATD of every mode (no transforms), make_ipred_list per
    CU (I-slice: no inter cut), then the transform / quantisation records of each CU's listed
    modes only"""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import cases
    n = len(cus)
    lib = u.lib()
    sp = stream.cuda_stream
    reqs, _, _, _, _ = cases.rmd_inputs(np.random.default_rng(37), 1)
    reqs = np.repeat(reqs, n)
    rng = np.random.default_rng(38)
    reqs["satd_row"] = np.arange(n)
    reqs["pb_w"], reqs["pb_h"] = cus["w"], cus["h"]
    reqs["mpm"] = np.sort(rng.integers(0, 33, (n, 2)), axis=1)
    reqs["skip_ipd"] = 0
    reqs["fast"] = 1
    reqs["range"] = rng.integers(256, 512, n)
    reqs["ctx"] = cases.rmd_ctx(rng, 7 * n).reshape(n, 7)
    reqs["sqrt_lambda"] = 30.0
    reqs["inter_satd"] = np.iinfo(np.uint64).max
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_satd = torch.empty(n * 33, dtype=torch.int32, device="cuda")
    d_lists = torch.empty(n * u.RMD_OUT.itemsize, dtype=torch.uint8, device="cuda")
    d_satd5 = torch.empty(n * 33, dtype=torch.int32, device="cuda")
    d_q5 = torch.empty(n * 33 * len(qps) * 16, dtype=torch.uint8, device="cuda")
    fn = lib.uavs3e_cuda_intra_lattice_modes_device

    def run(sp=sp):
        u.check(fn(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(), n, None, 33, 1, None, 0, 1,
                   d_satd.data_ptr(), None, sp), "intra_lattice (SATD)")
        u.intra_rmd_device(d_satd.data_ptr(), n, d_req.data_ptr(), n, d_lists.data_ptr(), sp)
        lists = d_lists.view(torch.int8).view(n, u.RMD_OUT.itemsize)[:, :5].to(torch.int16)
        modes = torch.where(lists < 0, lists[:, :1], lists).to(torch.uint8).contiguous()
        u.check(fn(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(), n, modes.data_ptr(), 5, 1,
                   qps.ctypes.data, len(qps), 1, d_satd5.data_ptr(), d_q5.data_ptr(), sp), "intra_lattice (lists)")

    with torch.cuda.stream(stream):
        for _ in range(2):
            run()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            run()
            e1.record(stream)
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    counts = d_lists.view(n, u.RMD_OUT.itemsize)[:, 5].cpu().numpy()
    # the same frame as one captured CUDA graph (SATD lattice, candidate lists, mode gather,
    # listed-mode lattice), replayed per frame
    want = d_q5.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        run(torch.cuda.current_stream().cuda_stream)
    with torch.cuda.stream(stream):
        d_q5.zero_()
        g.replay()
        torch.cuda.synchronize()
        graph_equal = bool(torch.equal(d_q5, want))
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            g.replay()
            e1.record(stream)
        torch.cuda.synchronize()
    graph_ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    return {"workload": "1080p intra decision in the encoder's order: SATD of the 33 modes of every lattice CU, "
                        "make_ipred_list (fast RMD), then transform + 4-QP quantisation records of the listed modes",
            "ms_per_frame": ms, "frames_per_s": 1000.0 / ms, "mean_candidates": float(counts.mean()),
            "graph": {"ms_per_frame": graph_ms, "records_equal_plain": graph_equal,
                      "note": "the frame's launches captured once into a CUDA graph and replayed"}}


def rmd_part(u, torch, stream, flush, d_satd, cus, with_cpu, reps=10):
    """make_ipred_list of every CU of the lattice from the lattice's own SATD records (random MPM
    pairs, coder states, fast / full searches, inter-SATD cuts)"""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cases
    n = len(cus)
    reqs, _, _, _, _ = cases.rmd_inputs(np.random.default_rng(29), 1)
    reqs = np.repeat(reqs, n)
    base = np.random.default_rng(31)
    reqs["satd_row"] = np.arange(n)
    reqs["pb_w"], reqs["pb_h"] = cus["w"], cus["h"]
    m = np.sort(base.integers(0, 34, (n, 2)), axis=1)
    reqs["mpm"] = m
    reqs["skip_ipd"] = base.random(n) < 0.3
    reqs["fast"] = base.random(n) < 0.7
    reqs["range"] = base.integers(256, 512, n)
    reqs["ctx"] = cases.rmd_ctx(base, 7 * n).reshape(n, 7)
    reqs["sqrt_lambda"] = base.uniform(4.0, 60.0, n)
    cut = base.random(n) < 0.5
    reqs["inter_satd"] = np.where(cut, (base.integers(1, 40, n) * cus["w"].astype(np.int64) * cus["h"]).astype(np.uint64),
                                  np.uint64(np.iinfo(np.uint64).max))
    reqs["satd_threshold"] = base.uniform(0.9, 1.6, n)
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_out = torch.empty(n * u.RMD_OUT.itemsize, dtype=torch.uint8, device="cuda")
    sp = stream.cuda_stream

    def run():
        u.intra_rmd_device(d_satd.data_ptr(), n, d_req.data_ptr(), n, d_out.data_ptr(), sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    satd = d_satd.cpu().numpy().view(np.uint32).reshape(n, 33)
    t0 = time.perf_counter()
    for _ in range(reps):
        got = u.intra_rmd(satd, reqs)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / reps
    out = {"workload": f"make_ipred_list of the {n} lattice CUs from its SATD records (70 % fast search, 30 % "
                       "DC/planar/bilinear skipped, MPM pairs, LBAC states for the mode bits, 50 % inter-SATD cuts)",
           "blocks": n, "ms_per_batch": ms, "blocks_per_s": n / (ms / 1000.0),
           "mean_candidates": float(got["count"].mean()),
           "e2e": {"ms_per_batch": e2e_ms, "blocks_per_s": n / (e2e_ms / 1000.0),
                   "h2d_bytes": int(satd.nbytes + reqs.nbytes), "d2h_bytes": int(got.nbytes),
                   "path": "uavs3e_cuda_intra_rmd (host SATD records and requests)"}}
    if with_cpu:
        import pyoracle
        t0 = time.perf_counter()
        pyoracle.Oracle().intra_rmd(satd, reqs)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "blocks/s", "cores": 1, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement (one core), {dt:.2f} s"}
    return out


LOKA_PAD = 144


def loka_pictures(seed=21):
    """the lookahead leg's pictures: POC 0, 7, 8, 16 of the 1080p motion sequence (pan
    (+3.25, -1.5) per frame), chroma = 2x-downsampled luma offset by +16 / -16"""
    import numpy as np
    from uavs3e_gb300.synth import motion_sequence
    seq = motion_sequence(W, H, 17, seed=seed)
    pics = {}
    for t in (0, 7, 8, 16):
        y = seq[t]
        c = y.reshape(H // 2, 2, W // 2, 2).astype(np.int32).mean((1, 3)).astype(np.int32)
        pics[t] = (y, np.clip(c + 16, 0, 255).astype(np.uint8), np.clip(c - 16, 0, 255).astype(np.uint8))
    return pics


def loka_padded(y):
    import numpy as np
    s = W + 2 * LOKA_PAD
    return np.pad(y, LOKA_PAD, mode="edge").reshape(H + 2 * LOKA_PAD, s)


def lookahead_leg(u, torch, stream, flush, sm_count, sm_mhz, with_cpu, reps=20):
    """loka_estimate_coding_cost of a 1080p picture: the encoder's picture-level estimate of
    POC 8 in a random-access GOP of 16 (references POC 0 in list 0 and POC 16 in list 1, padded,
    search range 384) and the lookahead's scene-cut estimate of POC 8 against POC 7 (no padding,
    search range 64).  Device path timed with CUDA events (L2 flushed before each call), the
    host-buffer entry point end to end."""
    import numpy as np
    pics = loka_pictures()
    lib = u.lib()
    n_units = (W // 16) * (H // 16)
    sp = stream.cuda_stream
    confs = {
        "encoder_ra_bi": (u.loka_cfg(W, H, 1, 384, 16, 8, [0], [16]), [0], [16]),
        "scenecut": (u.loka_cfg(W, H, 0, 64, 16, 8, [7], []), [7], []),
    }
    y, cu, cv = pics[8]
    d_y, d_u, d_v = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (y, cu, cv))
    d_units = torch.empty(n_units * u.LOKA_UNIT.itemsize, dtype=torch.uint8, device="cuda")
    d_energy = torch.empty(n_units, dtype=torch.int64, device="cuda")
    d_tot = torch.empty(5, dtype=torch.int64, device="cuda")
    _, sad_clk = u.measure_sad4_rate()
    int_peak = max(sad_clk, 64.0) * sm_count * sm_mhz * 1e6 / 1e9
    out = {"workload": "lookahead cost estimation (loka_estimate_coding_cost) of a 1080p 4:2:0 picture: "
                       f"{n_units} 16x16 units, integer TZ search per reference + uni/bi SATD + 11 intra modes + "
                       "chroma SATD + dQP energy", "units": n_units}
    for name, (cfg, l0, l1) in confs.items():
        padded = {t: loka_padded(pics[t][0]) for t in l0 + l1}
        d_ref = {t: torch.from_numpy(padded[t]).cuda() for t in padded}
        off = LOKA_PAD * (W + 2 * LOKA_PAD) + LOKA_PAD
        i_ref = W + 2 * LOKA_PAD

        def run():
            u.loka_units_device(cfg, d_y.data_ptr(), W, d_u.data_ptr(), d_v.data_ptr(), W // 2,
                                [d_ref[t].data_ptr() + off for t in l0], [d_ref[t].data_ptr() + off for t in l1],
                                i_ref, LOKA_PAD, d_units.data_ptr(), d_energy.data_ptr(), d_tot.data_ptr(), sp)

        for _ in range(3):
            run()
        torch.cuda.synchronize()
        l0c = u.launch_count()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            run()
            e1.record(stream)
        torch.cuda.synchronize()
        launches = (u.launch_count() - l0c) / reps
        ms = sum(a.elapsed_time(b) for a, b in evs) / reps
        sads = int(d_tot.cpu().numpy().view(np.uint64)[4])
        # end to end: host planes (pinned) in, the reference's outputs back
        pin_y, pin_u, pin_v = (torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (y, cu, cv))
        pin_r = {t: torch.from_numpy(padded[t]).pin_memory() for t in padded}
        cfg_c = np.ascontiguousarray(cfg)
        import ctypes as C
        a0 = (C.c_void_p * 4)(*([pin_r[t].data_ptr() + off for t in l0] + [None] * (4 - len(l0))))
        a1 = (C.c_void_p * 4)(*([pin_r[t].data_ptr() + off for t in l1] + [None] * (4 - len(l1))))
        cost, icost = C.c_double(), C.c_double()
        uv = (C.c_double * 2)()
        dqp = np.zeros(n_units, np.float32)

        def e2e():
            u.check(lib.uavs3e_cuda_loka_estimate(cfg_c.ctypes.data, pin_y.data_ptr(), W, pin_u.data_ptr(),
                                                  pin_v.data_ptr(), W // 2, a0, a1, i_ref, LOKA_PAD, C.byref(cost),
                                                  C.byref(icost), uv, dqp.ctypes.data, None), "loka_estimate")

        for _ in range(3):
            e2e()
        t0 = time.perf_counter()
        for _ in range(reps):
            e2e()
        e2e_ms = (time.perf_counter() - t0) * 1000.0 / reps
        ops = sads * 64.0                     # 16x16 SAD = 64 four-sample vabsdiff4 operations
        # the padded search copies each reference with its padding, the other one the picture only
        ref_bytes = (W + 2 * LOKA_PAD) * (H + 2 * LOKA_PAD) if cfg["is_padding"][0] else W * H
        r = {"ms_per_picture": ms, "pictures_per_s": 1000.0 / ms, "units_per_s": n_units / (ms / 1000.0),
             "gpu_launches_per_picture": launches, "sad16_evaluations": sads,
             "e2e": {"ms_per_picture": e2e_ms, "pictures_per_s": 1000.0 / e2e_ms,
                     "h2d_bytes": int(W * H * 3 // 2 + len(padded) * ref_bytes),
                     "d2h_bytes": int(5 * 8 + n_units * 8),
                     "path": "uavs3e_cuda_loka_estimate on pinned host planes (cost, icost, icost_uv, map_dqp)"},
             "picture_cost": cost.value, "icost": icost.value,
             "roofline": {"bound": "int", "kernel": "k_loka_search + k_loka_unit (SAD work of the searches only)",
                          "achieved": ops / (ms / 1000.0) / 1e9, "peak": int_peak, "unit": "Gop/s",
                          "frac": ops / (ms / 1000.0) / 1e9 / int_peak,
                          "peak_source": f"vabsdiff4.add rate max(measured {sad_clk:.1f}, 64)/clk/SM x {sm_count} "
                                         f"SMs x {sm_mhz:.0f} MHz"}}
        if with_cpu:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import pyoracle
            o = pyoracle.Oracle()
            threads = os.cpu_count() or 1
            refs_addr = [[padded[t].ctypes.data + off for t in lst] for lst in (l0, l1)]
            t0 = time.perf_counter()
            o.loka_units(cfg, y, W, cu, cv, W // 2, refs_addr[0], refs_addr[1], i_ref, threads)
            dt = time.perf_counter() - t0
            r["cpu_baseline"] = {"value": 1.0 / dt, "unit": "pictures/s", "cores": threads, "kind": "port",
                                 "sample": f"the whole picture through the oracle restatement, {dt:.2f} s"}
        out[name] = r
    return out


def loka_chroma(y):
    """chroma planes of a synthetic luma picture: 2x-downsampled luma offset by +16 / -16"""
    import numpy as np
    c = y.reshape(y.shape[0] // 2, 2, y.shape[1] // 2, 2).astype(np.int32).mean((1, 3)).astype(np.int32)
    return np.clip(c + 16, 0, 255).astype(np.uint8), np.clip(c - 16, 0, 255).astype(np.uint8)


def tz_leg(u, torch, stream, flush, with_cpu, hbm_peak, reps=10):
    """per-call TZ motion searches (me_search_tz) of a 1080p frame: every block of the ten shapes
    on the CTU grid against 2 references, each at a random AMVR resolution with a random
    predictor, 30 % of them bi calls against the other reference's prediction"""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cases
    from uavs3e_gb300.synth import motion_sequence
    seq = motion_sequence(W, H, 3, seed=31)
    ms = u.MotionSearch(W, H, n_refs=2, search_range=RANGE, pad=PAD)
    sp = stream.cuda_stream
    d_seq = [torch.from_numpy(f).cuda() for f in seq]
    ms.set_ref_device(0, d_seq[1].data_ptr(), W, sp)
    ms.set_ref_device(1, d_seq[0].data_ptr(), W, sp)
    rng = np.random.default_rng(17)
    b = u.me_blocks(W, H)
    blocks = b[(b[:, 0] + b[:, 2] <= W) & (b[:, 1] + b[:, 3] <= H)]
    reqs = cases.tz_requests(rng, W, H, 2 * len(blocks), [1, 2])
    for i, f in enumerate(("x", "y", "w", "h")):
        reqs[f] = np.repeat(blocks[:, i], 2)
    reqs["ref_slot"] = np.tile([0, 1], len(blocks))
    reqs["other_slot"] = 1 - reqs["ref_slot"]
    reqs["dist"] = reqs["ref_slot"] + 1
    n = len(reqs)
    planes = [ms.plane_ptr(s, ph) for s in range(2) for ph in range(16)]
    pic = (W, H, 1, 384, 16)
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_out = torch.empty(n * u.TZ_OUT.itemsize, dtype=torch.uint8, device="cuda")

    def run():
        u.me_tz_device(pic, d_seq[2].data_ptr(), W, planes, ms.stride, PAD, d_req.data_ptr(), n, d_out.data_ptr(), sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms_gpu = sum(a.elapsed_time(b) for a, b in evs) / reps
    # CU motion compensation of the same blocks at the MVs found: luma + chroma, one list, or
    # both lists for the bi calls (the other list at its own MV)
    tz_out = d_out.cpu().numpy().view(u.TZ_OUT)
    mreq = np.zeros(n, dtype=u.MC_REQ)
    for f in ("x", "y", "w", "h"):
        mreq[f] = reqs[f]
    mreq["slot"][:, 0] = reqs["ref_slot"]
    mreq["slot"][:, 1] = np.where(reqs["bi"] == 1, reqs["other_slot"].astype(np.int8), np.int8(-1))
    mreq["mv"][:, 0] = tz_out["mv"]
    mreq["mv"][:, 1] = reqs["other_mv"]
    sizes = mreq["w"].astype(np.int64) * mreq["h"] * 3 // 2
    mreq["out_offset"] = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    mc_bytes = int(sizes.sum())
    ms.set_ref_chroma(0, *[np.ascontiguousarray(c) for c in loka_chroma(seq[1])])
    ms.set_ref_chroma(1, *[np.ascontiguousarray(c) for c in loka_chroma(seq[0])])
    d_mreq = torch.from_numpy(mreq.view(np.uint8).copy()).cuda()
    d_pred = torch.empty(mc_bytes, dtype=torch.uint8, device="cuda")
    chroma_ptrs = [ms.chroma_plane_ptr(s, c) for s in range(2) for c in range(2)]

    def mc_run():
        u.mc_cu_device(W, H, planes, ms.stride, PAD, chroma_ptrs, ms.chroma_stride(), 72, d_mreq.data_ptr(), n,
                       d_pred.data_ptr(), mc_bytes, sp)

    for _ in range(3):
        mc_run()
    torch.cuda.synchronize()
    mevs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in mevs:
        flush.zero_()
        e0.record(stream)
        mc_run()
        e1.record(stream)
    torch.cuda.synchronize()
    mc_ms = sum(a.elapsed_time(b) for a, b in mevs) / reps
    # bytes: every prediction written once, each used list's reference block read once (chroma
    # filter halo not counted)
    mc_traffic = mc_bytes + int((sizes * ((mreq["slot"][:, 1] >= 0) + 1)).sum())
    # affine predictions of every block of 16x16 and larger (random 2/3 control-point MVs)
    big = blocks[(blocks[:, 2] >= 16) & (blocks[:, 3] >= 16)]
    areq, a_bytes = cases.affine_requests(np.random.default_rng(23), W, H, len(big))
    for i, f in enumerate(("x", "y", "w", "h")):
        areq[f] = big[:, i]
    asz = areq["w"].astype(np.int64) * areq["h"] * 3 // 2
    areq["out_offset"] = np.concatenate([[0], np.cumsum(asz)[:-1]])
    a_bytes = int(asz.sum())
    d_areq = torch.from_numpy(areq.view(np.uint8).copy()).cuda()
    d_apred = torch.empty(a_bytes, dtype=torch.uint8, device="cuda")

    def aff_run():
        u.mc_affine_device(W, H, planes, ms.stride, PAD, chroma_ptrs, ms.chroma_stride(), 72, d_areq.data_ptr(),
                           len(areq), d_apred.data_ptr(), a_bytes, sp)

    for _ in range(3):
        aff_run()
    torch.cuda.synchronize()
    aevs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in aevs:
        flush.zero_()
        e0.record(stream)
        aff_run()
        e1.record(stream)
    torch.cuda.synchronize()
    aff_ms = sum(a.elapsed_time(b) for a, b in aevs) / reps
    # end to end: host org + requests in, results out, through the session entry
    org_pin = torch.from_numpy(seq[2]).pin_memory()
    t0 = time.perf_counter()
    for _ in range(reps):
        got = ms.tz(pic, org_pin.numpy(), reqs)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / reps
    out = {"workload": f"me_search_tz calls of a 1080p frame: {len(blocks)} blocks (10 shapes 8x8..64x64 on the CTU "
                       "grid) x 2 references, AMVR resolutions 0..4, 30 % bi, SATD/SAD refinement mixed",
           "calls": n, "ms_per_batch": ms_gpu, "calls_per_s": n / (ms_gpu / 1000.0),
           "bi_calls": int(reqs["bi"].sum()),
           "mc": {"workload": "com_mc_cu of the same blocks at the MVs found (luma + 4-tap chroma, bi calls "
                              "averaged with the other list)", "ms_per_batch": mc_ms,
                  "bytes": mc_traffic, "gb_per_s": mc_traffic / (mc_ms / 1000.0) / 1e9,
                  "roofline": {"bound": "hbm", "achieved": mc_traffic / (mc_ms / 1000.0) / 1e9, "peak": hbm_peak,
                               "unit": "GB/s", "frac": mc_traffic / (mc_ms / 1000.0) / 1e9 / hbm_peak,
                               "peak_source": "hbm_gbs of MEASURED_PEAKS.json"}},
           "affine": {"workload": f"com_mc_cu_affine of the {len(areq)} blocks of 16x16 and larger (2 or 3 "
                                  "control points, one or two lists, luma 16-phase + chroma 32-phase filters)",
                      "ms_per_batch": aff_ms, "cus_per_s": len(areq) / (aff_ms / 1000.0),
                      "samples_per_s": a_bytes / (aff_ms / 1000.0)},
           "e2e": {"ms_per_batch": e2e_ms, "calls_per_s": n / (e2e_ms / 1000.0),
                   "h2d_bytes": int(W * H + reqs.nbytes), "d2h_bytes": int(got.nbytes),
                   "path": "uavs3e_cuda_me_tz (host org and requests, session references)"}}
    if with_cpu:
        import pyoracle
        o = pyoracle.Oracle()
        keep, addrs, stride = cases.tz_planes(o, {t: (seq[t],) for t in range(3)}, [1, 0], W, H)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        o.me_tz(pic, seq[2], W, addrs, stride, reqs, threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "calls/s", "cores": threads, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement, {dt:.2f} s"}
    ms.close()
    return out


def affmvp_part(u, torch, stream, flush, with_cpu, reps=10):
    """com_get_affine_mvp_scaling for every 8x8..128x128 CU position of a 1080p motion field, both
    lists (uavs3e_cuda_affine_mvp_device, one thread per CU)"""
    import cases
    import numpy as np
    p = dict(w=480, h=270, nref=4, n=0, big=1)
    ptr_cur, ref_ptr, mv, refi, i_scu, _ = cases.affmvp_inputs(p, 91)
    rng = np.random.default_rng(92)
    n = 1 << 20
    reqs = np.zeros(n, dtype=u.AFFMVP_REQ)
    cw = rng.choice([8, 16, 32, 64, 128], n)
    x = (rng.random(n) * (481 - cw // 4)).astype(np.int64)
    y = rng.integers(0, 270, n)
    reqs["scup"] = y * i_scu + x
    reqs["cu_width"] = cw
    reqs["lidx"] = rng.integers(0, 2, n)
    reqs["cur_refi"] = rng.integers(0, 4, n)
    reqs["mvr"] = rng.integers(0, 3, n)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()  # noqa: E731
    d_ref, d_mv, d_refi, d_req = d(ref_ptr), d(mv), d(refi), d(reqs)
    d_out = torch.zeros(n * 16, dtype=torch.uint8, device="cuda")
    rows = len(refi) // i_scu
    sp = stream.cuda_stream

    def run():
        u.affine_mvp_device(ptr_cur, d_ref.data_ptr(), len(ref_ptr), d_mv.data_ptr(), d_refi.data_ptr(), i_scu, rows,
                            d_req.data_ptr(), n, d_out.data_ptr(), None, sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms_gpu = sum(a.elapsed_time(b) for a, b in evs) / reps
    moved = n * (12 + 16)
    out = {"workload": "affine control-point MVP of 1,048,576 CUs (8x8..128x128, both lists, 4 references, AMVR "
                       "0..2) on a 1080p motion field (480 x 270 SCUs)", "cus": n, "ms_per_batch": ms_gpu,
           "cus_per_s": n / (ms_gpu / 1000.0),
           "request_result_gb_s": moved / (ms_gpu / 1000.0) / 1e9}
    if with_cpu:
        import pyoracle
        o = pyoracle.Oracle()
        t0 = time.perf_counter()
        o.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "CUs/s", "cores": 1, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement, {dt:.2f} s"}
    return out


def affmrg_part(u, torch, stream, flush, with_cpu, reps=10):
    """com_get_affine_merge_candidate for 262,144 CUs (16x16..64x64, B slice) of a 1080p picture's
    coded-CU maps (uavs3e_cuda_affine_merge_device, one thread per CU)"""
    import cases
    import numpy as np
    n = 1 << 18
    args = cases.affmrg_inputs(dict(w=480, h=270, nref=3, slice="B", n=n), 93)
    pic, reqs = args[0], args[7]
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()  # noqa: E731
    dm = [d(a) for a in args[1:8]]
    d_out = torch.zeros(n * u.AFFMRG_OUT.itemsize, dtype=torch.uint8, device="cuda")
    sp = stream.cuda_stream

    def run():
        u.affine_merge_device(pic, *[a.data_ptr() for a in dm], n, d_out.data_ptr(), None, sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms_gpu = sum(a.elapsed_time(b) for a, b in evs) / reps
    moved = n * (8 + u.AFFMRG_OUT.itemsize)
    out = {"workload": "affine merge candidates of 262,144 CUs (16x16..64x64, B slice, colocated scaling) on a "
                       "1080p picture's coded-CU maps (480 x 270 SCUs)", "cus": n, "ms_per_batch": ms_gpu,
           "cus_per_s": n / (ms_gpu / 1000.0), "request_result_gb_s": moved / (ms_gpu / 1000.0) / 1e9}
    if with_cpu:
        import pyoracle
        o = pyoracle.Oracle()
        t0 = time.perf_counter()
        o.affine_merge(*args)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "CUs/s", "cores": 1, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement, {dt:.2f} s"}
    return out


def affme_leg(u, torch, stream, flush, with_cpu, reps=10):
    """affine motion searches (affine_me_gradient) of a 1080p frame: every block of 16x16 and
    larger on the CTU grid against 2 references, AMVR indices 0..2, 70 % uni calls (60 % of them
    with analyze_affine_uni's start selection), 30 % bi calls against the other list's prediction"""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cases
    from uavs3e_gb300.synth import motion_sequence
    seq = motion_sequence(W, H, 3, seed=33)
    ms = u.MotionSearch(W, H, n_refs=2, search_range=RANGE, pad=PAD)
    sp = stream.cuda_stream
    d_seq = [torch.from_numpy(f).cuda() for f in seq]
    ms.set_ref_device(0, d_seq[1].data_ptr(), W, sp)
    ms.set_ref_device(1, d_seq[0].data_ptr(), W, sp)
    b = u.me_blocks(W, H)
    blocks = b[(b[:, 0] + b[:, 2] <= W) & (b[:, 1] + b[:, 3] <= H) & (b[:, 2] >= 16) & (b[:, 3] >= 16)]
    reqs = cases.affme_requests(np.random.default_rng(19), W, H, 2 * len(blocks), 2)
    for i, f in enumerate(("x", "y", "w", "h")):
        reqs[f] = np.repeat(blocks[:, i], 2)
    reqs["ref_slot"] = np.tile([0, 1], len(blocks))
    reqs["other_slot"] = 1 - reqs["ref_slot"]
    n = len(reqs)
    planes = [ms.plane_ptr(s, ph) for s in range(2) for ph in range(16)]
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_out = torch.empty(n * u.AFFME_OUT.itemsize, dtype=torch.uint8, device="cuda")

    def run():
        u.me_affine_device(W, H, d_seq[2].data_ptr(), W, planes, ms.stride, PAD, d_req.data_ptr(), n,
                           d_out.data_ptr(), sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms_gpu = sum(a.elapsed_time(b) for a, b in evs) / reps
    org_pin = torch.from_numpy(seq[2]).pin_memory()
    t0 = time.perf_counter()
    for _ in range(reps):
        got = ms.affine(org_pin.numpy(), reqs)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / reps
    moved = int((got["mv"] != reqs["mv"]).any(axis=(1, 2)).sum())
    out = {"workload": f"affine_me_gradient calls of a 1080p frame: {len(blocks)} blocks of 16x16..64x64 on the CTU "
                       "grid x 2 references, AMVR indices 0..2, 30 % bi, uni calls with and without the "
                       "analyze_affine_uni start selection, 4x4 / 8x8 sub-blocks",
           "calls": n, "ms_per_batch": ms_gpu, "calls_per_s": n / (ms_gpu / 1000.0),
           "bi_calls": int((reqs["flags"] & u.AFFME_BI != 0).sum()), "calls_that_moved": moved,
           "predicted_samples": int((reqs["w"].astype(np.int64) * reqs["h"]).sum()),
           "e2e": {"ms_per_batch": e2e_ms, "calls_per_s": n / (e2e_ms / 1000.0),
                   "h2d_bytes": int(W * H + reqs.nbytes), "d2h_bytes": int(got.nbytes),
                   "path": "uavs3e_cuda_me_affine (host org and requests, session references)"}}
    if with_cpu:
        import pyoracle
        o = pyoracle.Oracle()
        keep, addrs, stride = cases.tz_planes(o, {t: (seq[t],) for t in range(3)}, [1, 0], W, H)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        o.me_affine(W, H, seq[2], W, addrs, stride, reqs, threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "calls/s", "cores": threads, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement, {dt:.2f} s"}
    ms.close()
    out["mvp"] = affmvp_part(u, torch, stream, flush, with_cpu, reps)
    out["merge"] = affmrg_part(u, torch, stream, flush, with_cpu, reps)
    return out


def coef_rate_part(u, torch, stream, flush, rreqs, nz, d_levels, levels, with_cpu, reps=10):
    """the coefficient rate (lbac_enc_run_length_cc_rdo) of every block RDOQ coded, each from a
    random coder state, on the GPU's RDOQ output"""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import cases
    rng = np.random.default_rng(41)
    sel = np.nonzero(nz > 0)[0]
    r = np.zeros(len(sel), dtype=u.COEF_RATE_REQ)
    r["coef_offset"] = rreqs["coef_offset"][sel]
    r["log2w"], r["log2h"] = rreqs["log2w"][sel], rreqs["log2h"][sel]
    r["ch_type"] = (rreqs["ch_type"][sel] != 0).astype(np.uint8)
    r["num_sig"] = nz[sel]
    r["range"] = rng.integers(256, 512, len(r))
    for f, k in (("run", 12), ("run_rdoq", 12), ("level", 12), ("last1", 6), ("last2", 12)):
        r[f] = cases.coef_models(rng, k * len(r)).reshape(len(r), k)
    d_req = torch.from_numpy(r.view(np.uint8).copy()).cuda()
    d_out = torch.empty(len(r) * u.COEF_RATE_OUT.itemsize, dtype=torch.uint8, device="cuda")
    sp = stream.cuda_stream

    def run():
        u.coef_rate_device(d_req.data_ptr(), len(r), d_levels.data_ptr(), levels.size, d_out.data_ptr(), sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    got = d_out.cpu().numpy().view(u.COEF_RATE_OUT)
    out = {"workload": f"lbac_enc_run_length_cc_rdo of the {len(r)} blocks RDOQ coded (their levels, random coder "
                       "states)", "blocks": len(r), "levels": int(r["num_sig"].sum()), "ms_per_batch": ms,
           "blocks_per_s": len(r) / (ms / 1000.0), "mean_bits": float(got["bits"].mean())}
    if with_cpu:
        import pyoracle
        t0 = time.perf_counter()
        pyoracle.Oracle().coef_rate(levels, r)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(r) / dt, "unit": "blocks/s", "cores": 1, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement (one core), {dt:.2f} s"}
    return out


def rdoq_leg(u, torch, stream, flush, with_cpu, reps=10):
    """RDOQ (quant_non_zero -> rdoq_quant_block) of 60,000 transform blocks of every shape
    4x4..64x64 (DCT2 coefficients of Laplacian residuals, steps 10..60, intra / inter, luma /
    chroma, 8 estimate sets)"""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cases
    import pyoracle
    o = pyoracle.Oracle()
    reqs, ests, coefs = cases.rdoq_inputs(o, dict(n=60000, k=8), 77)
    sp = stream.cuda_stream
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_est = torch.from_numpy(ests.view(np.uint8).copy()).cuda()
    d_src = torch.from_numpy(coefs.copy()).cuda()
    d_coef = torch.empty_like(d_src)
    d_nz = torch.empty(len(reqs), dtype=torch.int32, device="cuda")

    def run():
        d_coef.copy_(d_src)
        u.rdoq_device(d_req.data_ptr(), len(reqs), d_est.data_ptr(), len(ests), d_coef.data_ptr(), coefs.size,
                      d_nz.data_ptr(), sp)

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        run()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    nz = d_nz.cpu().numpy()
    c = coefs.copy()
    t0 = time.perf_counter()
    for _ in range(3):
        c[:] = coefs
        u.rdoq(reqs, ests, c)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / 3
    out = {"workload": "RDOQ of 60,000 transform blocks 4x4..64x64 (21 shapes), steps 10..60, intra/inter, "
                       "luma/chroma, 8 bin-cost estimate sets", "blocks": len(reqs), "coefficients": int(coefs.size),
           "ms_per_batch": ms, "blocks_per_s": len(reqs) / (ms / 1000.0),
           "coded_blocks": int((nz > 0).sum()),
           "note": "the device time includes a device copy of the input coefficients before each call",
           "e2e": {"ms_per_batch": e2e_ms, "blocks_per_s": len(reqs) / (e2e_ms / 1000.0),
                   "h2d_bytes": int(coefs.nbytes + reqs.nbytes + ests.nbytes), "d2h_bytes": int(coefs.nbytes + 4 * len(reqs)),
                   "path": "uavs3e_cuda_rdoq (host coefficients in, levels out)"}}
    if with_cpu:
        c[:] = coefs
        t0 = time.perf_counter()
        o.rdoq(reqs, ests, c)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(reqs) / dt, "unit": "blocks/s", "cores": 1, "kind": "port",
                               "sample": f"the whole batch through the oracle restatement (one core), {dt:.2f} s"}
    out["rate"] = coef_rate_part(u, torch, stream, flush, reqs, nz, d_coef, c, with_cpu)
    return out


def pruning_leg(steps=3000):
    """the learned CU pruning beside the lattice: trained on the plain path's decisions over 16
    synthetic 1080p I-frames, evaluated on a held-out frame (RD-cost increase of the pruned
    search, share of the lattice's work it searches, GPU time of the pruned lattice)"""
    from uavs3e_gb300 import cnn
    r = cnn.experiment(steps=steps)
    # the same network trained on the reference encoder's own CU decisions (committed fixture)
    r["encoder_labels"] = cnn.encoder_label_experiment(os.path.join(ROOT, "tests", "golden", "encoder_labels.npz"))
    r["workload"] = ("CNN 2 -> 16/32/32/64 ch (3x3, stride 2) + 1x1 head, bf16 tcgen05 tensor cores with FP32 "
                     "accumulation in TMEM; labels: quad-tree + mode decisions from the lattice's RD costs at QP 32")
    # one training step at a batch of 1,024 CTUs against the measured bf16 tensor peak
    ms, flops = cnn.step_time(1024)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("bf16_tflops", 1900.0))
    tf = flops / (ms / 1000.0) / 1e12
    r["train_step_b1024"] = {"ms": ms, "ctus_per_s": 1024 / (ms / 1000.0), "tflops": tf,
                             "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s",
                                          "frac": tf / peak,
                                          "peak_source": "bf16_tflops of MEASURED_PEAKS.json" if "bf16_tflops" in peaks
                                          else "fallback 1.9 PFLOP/s"},
                             "note": "forward + loss + backward + Adam of 1,024 CTUs; FLOPs = the convolutions' GEMMs "
                                     "(real K); the layers' K (18..288) and N (16..64) are small, so the step is bound "
                                     "by the operand gathers, not the tensor pipe"}
    return r


def run_ours(args):
    import numpy as np
    import torch
    import uavs3e_gb300 as u
    from uavs3e_gb300.synth import lambda_mv_for_qp

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    u.build()
    u.init(local)
    lam = lambda_mv_for_qp(QP)
    frames = frames_ring(seed=replica_seed(rank))
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    d_frames = [torch.from_numpy(f).cuda() for f in frames]
    ms = u.MotionSearch(W, H, n_refs=N_REFS, search_range=RANGE, pad=PAD)
    d_out = torch.empty(ms.n_results * 32, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ms.set_ref_device(0, d_frames[0].data_ptr(), W, sp)

    def step(t):
        # one captured CUDA graph per frame: the newest reference's planes, then the search
        ms.frame_graph((t - 1) % N_REFS, d_frames[(t - 1) % RING].data_ptr(), W, d_frames[t % RING].data_ptr(), W,
                       lam, d_out.data_ptr(), sp)

    t = 2
    for _ in range(max(3, args.warmup)):
        step(t)
        t += 1
    torch.cuda.synchronize()

    # ---- kernel path: inputs resident in HBM, L2 flushed (256 MiB write) before every step
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    launches0 = u.launch_count()
    for k in range(args.steps):
        flush.zero_()
        evs[k][0].record(stream)
        step(t)
        evs[k][1].record(stream)
        t += 1
    torch.cuda.synchronize()
    launches = u.launch_count() - launches0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    # per-kernel times for the roofline: the same frames with plain launches, each kernel
    # bracketed by CUDA events on its stream (a captured graph records no events)
    prof_steps = max(10, args.steps // 4)
    u.profile_collect()
    u.profile_enable(True)
    for _ in range(prof_steps):
        flush.zero_()
        ms.set_ref_device((t - 1) % N_REFS, d_frames[(t - 1) % RING].data_ptr(), W, sp)
        ms.run_device(d_frames[t % RING].data_ptr(), W, lam, d_out.data_ptr(), sp)
        t += 1
    torch.cuda.synchronize()
    u.profile_enable(False)
    prof = u.profile_collect()
    total_s = sum(step_ms) / 1000.0
    total_s = max_over_ranks(total_s, world, "cuda")
    if world > 1:
        torch.distributed.barrier()
    value = world * args.steps / total_s

    # ---- end to end through the C ABI with host buffers (pinned), copies inside the region
    pin = [torch.from_numpy(f).pin_memory() for f in frames]
    h_out = torch.empty(ms.n_results * 32, dtype=torch.uint8).pin_memory()
    torch.cuda.synchronize()
    e2e_steps = max(5, args.steps // 2)

    def e2e_step(t):
        # one call: the new reference and the frame up, the captured frame graph, the results down
        ms.frame_ptr((t - 1) % N_REFS, pin[(t - 1) % RING].data_ptr(), W, pin[t % RING].data_ptr(), W, lam,
                     h_out.data_ptr())

    for k in range(2):
        e2e_step(2 + k)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_step(4 + k)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    cfg = workload_config()
    n_cand = cfg["int_candidates_per_block"]
    gcand = N_REFS * cfg["ctus"] * 169 * n_cand  # per frame, integer candidates over all blocks
    # roofline of the dominant kernel (integer search): SAD on the integer pipe, 4 samples per
    # vabsdiff4; algorithmic ops = refs * picture samples * candidates / 4 per frame
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    # denominator: the measured issue rate of vabsdiff4.add on this GPU (the instruction that
    # carries the SAD work), scaled to the maximum SM clock; MEASURED_PEAKS.json has no
    # integer peak
    rate, per_clk_sm = u.measure_sad4_rate()
    per_clk = max(per_clk_sm, 64.0)        # never below 16 lanes/clk per SM sub-partition
    int_peak = per_clk * sm_count * sm_mhz * 1e6 / 1e9          # Gop/s at max clock
    ms_int, n_int = prof["me_int"]
    avg_int_ms = ms_int / max(1, prof_steps)                   # both integer-search launches of a step
    alg_ops = N_REFS * W * H * n_cand / 4.0
    achieved = alg_ops / (avg_int_ms / 1000.0) / 1e9
    # DRAM traffic of the two integer-search launches of one frame: the ncu capture of the interior
    # launch (3,480 CTAs) read 21.9 MB and wrote nothing; the edge launch (600 CTAs of the same
    # window size) is counted in proportion to its CTAs
    traffic = 21.9e6 * 4080.0 / 3480.0
    roofline = {"bound": "int", "kernel": "k_me_int (integer full search, both launches of a frame)",
                "achieved": achieved, "peak": int_peak, "unit": "Gop/s", "frac": achieved / int_peak,
                "traffic": traffic,
                "traffic_note": "DRAM bytes per frame (both launches): the interior launch's ncu capture scaled "
                                "by CTAs to both; algorithmic ops, not bytes, bind",
                "peak_source": f"vabsdiff4.add issue rate max(measured {per_clk_sm:.1f}, 64) ops/clk/SM x {sm_count} "
                               f"SMs x {sm_mhz:.0f} MHz max SM clock (MEASURED_PEAKS.json has no integer peak)",
                "ops_per_launch": alg_ops, "avg_launch_ms": avg_int_ms,
                "kernel_ms_per_step": {k: v[0] / max(1, prof_steps) for k, v in prof.items()},
                "kernel_times": f"CUDA events around each kernel over {prof_steps} plain-launch frames"}
    # the HBM-side kernel of the frame: 15 quarter-sample planes of the newest reference written,
    # its padded integer plane read (16 padded planes of stride x rows bytes)
    stride = ((W + 2 * PAD) + 15) & ~15
    sub_bytes = 16.0 * stride * (H + 2 * PAD)
    sub_ms = prof["subpel_planes"][0] / max(1, prof_steps)
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    roofline_hbm = {"bound": "hbm", "kernel": "k_subpel_planes (15 quarter-sample planes of one reference)",
                    "achieved": sub_bytes / (sub_ms / 1000.0) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                    "frac": sub_bytes / (sub_ms / 1000.0) / 1e9 / hbm_peak, "traffic": 2.26e6 + 0.20e6,
                    "bytes_per_launch": sub_bytes,
                    "peak_source": "hbm_gbs of MEASURED_PEAKS.json" if "hbm_gbs" in peaks else "fallback 6.8 TB/s",
                    "traffic_note": "ncu DRAM bytes per launch: the written planes stay in the 129 MB L2"}
    legs = set(args.legs.split(","))
    lattice = lattice_leg(u, torch, stream, flush, peaks, sm_count, sm_mhz, not args.no_cpu) if "lattice" in legs else None
    pruning = pruning_leg(args.pruning_steps) if "pruning" in legs else None
    lookahead = (lookahead_leg(u, torch, stream, flush, sm_count, sm_mhz, not args.no_cpu)
                 if "lookahead" in legs else None)
    tz = tz_leg(u, torch, stream, flush, not args.no_cpu, hbm_peak) if "tz" in legs else None
    rdoq = rdoq_leg(u, torch, stream, flush, not args.no_cpu) if "rdoq" in legs else None
    affme = affme_leg(u, torch, stream, flush, not args.no_cpu) if "affme" in legs else None
    h2d = 2 * W * H
    d2h = ms.n_results * 32
    out = {
        "metric": METRIC,
        "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": cfg,
        "launch": "each frame replayed as a captured CUDA graph (uavs3e_cuda_me_frame_graph)",
        "gcandidates_per_s": gcand * value / 1e9,
        "e2e": {"value": world * e2e_steps / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "uavs3e_cuda_me_frame (reference and frame up, graph replay, results down) with pinned host buffers"},
        "gpu_launches": launches,
        "gpu_launches_per_step": launches / args.steps,
        "roofline": roofline,
        "roofline_hbm": roofline_hbm,
        "lattice": lattice,
        "pruning": pruning,
        "lookahead": lookahead,
        "tz": tz,
        "rdoq": rdoq,
        "affme": affme,
        "clocks": clk,
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(frames, lam)
    print(json.dumps(out))
    ms.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_legs(args):
    """the lattice and / or pruning legs alone (profiling runs of those kernels)"""
    import torch
    import uavs3e_gb300 as u
    legs = set(args.legs.split(","))
    u.build()
    u.init(0)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    sm_count = torch.cuda.get_device_properties(0).multi_processor_count
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = {}
    if "lattice" in legs:
        out["lattice"] = lattice_leg(u, torch, torch.cuda.current_stream(), flush, peaks, sm_count, sm_mhz,
                                     not args.no_cpu)
    if "pruning" in legs:
        out["pruning"] = pruning_leg(args.pruning_steps)
    if "lookahead" in legs:
        out["lookahead"] = lookahead_leg(u, torch, torch.cuda.current_stream(), flush, sm_count, sm_mhz,
                                         not args.no_cpu)
    if "tz" in legs:
        out["tz"] = tz_leg(u, torch, torch.cuda.current_stream(), flush, not args.no_cpu,
                           float(peaks.get("hbm_gbs", 6800.0)))
    if "rdoq" in legs:
        out["rdoq"] = rdoq_leg(u, torch, torch.cuda.current_stream(), flush, not args.no_cpu)
    if "affme" in legs:
        out["affme"] = affme_leg(u, torch, torch.cuda.current_stream(), flush, not args.no_cpu)
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif "me" not in args.legs.split(","):
        run_legs(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
