"""Generate tests/golden/encoder_labels.npz: the reference encoder's own CU decisions on seeded
synthetic I-frames, as labels for the pruning network.

The reference encoder (oracle/_ref/uavs3enc, built by `make -C oracle ref REF=<uavs3e tree>`)
codes each frame alone (intra, 64x64 CTUs, one thread) at QP 27, 32, 37 and 42; its library is
linked so that every final CU it writes to the bitstream (lbac_enc_unit) is logged as
"x y w h intra ipm" (oracle/ref_glue.c); when it writes a picture more than once, the last pass
(the one in the bitstream) is kept.  Per 64x64 CTU the labels have the layout of the
network's training labels: [0] the CTU is not one CU, [1..4] each 32x32 quadrant is not one CU,
[5..20] each 16x16 cell is not one CU, [21..36] the intra mode of the CU at each cell's top-left
sample.  Frames: uavs3e_gb300.synth.intra_frame(512, 256, seed) for seeds 300..317 (the first 16
for training, the last 2 held out); chroma = 2x2-averaged luma + 16 (U) / - 16 (V).

    python tests/golden/make_encoder_labels.py
"""
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
ENC = os.path.join(ROOT, "oracle", "_ref", "uavs3enc")
W, H = 512, 256
QPS = (27, 32, 37, 42)
SEEDS = tuple(range(300, 318))


def encode_cus(args):
    """the final CUs of one frame at one QP: int array [n][6] (x, y, w, h, intra, ipm)"""
    seed, qp = args
    from uavs3e_gb300.synth import intra_frame
    y = intra_frame(W, H, seed=seed)
    t = y.astype(np.int32)
    d = (t[0::2, 0::2] + t[1::2, 0::2] + t[0::2, 1::2] + t[1::2, 1::2] + 2) >> 2
    with tempfile.TemporaryDirectory() as tmp:
        src, log = os.path.join(tmp, "in.yuv"), os.path.join(tmp, "cu.log")
        with open(src, "wb") as f:
            f.write(y.tobytes())
            f.write(np.clip(d + 16, 0, 255).astype(np.uint8).tobytes())
            f.write(np.clip(d - 16, 0, 255).astype(np.uint8).tobytes())
        env = dict(os.environ, UAVS3E_CU_LOG=log)
        cmd = [ENC, "-i", src, "-w", str(W), "-h", str(H), "-d", "8", "-f", "1", "-q", str(qp), "-p", "1", "-g", "0",
               "--ctu_size", "64", "--wpp_threads", "1", "--frm_threads", "1", "--fps_num", "30", "--fps_den", "1",
               "-v", "0", "-o", os.path.join(tmp, "o.bin"), "-r", os.path.join(tmp, "r.yuv")]
        r = subprocess.run(cmd, env=env, capture_output=True, cwd=tmp)
        if r.returncode:
            raise RuntimeError(r.stderr.decode()[-2000:])
        cus = np.loadtxt(log, dtype=np.int64, ndmin=2)
    # the encoder may write a picture more than once (a pass restarts at CU (0, 0)); the last
    # pass is the one in the bitstream
    starts = np.nonzero((cus[:, 0] == 0) & (cus[:, 1] == 0))[0]
    cus = cus[starts[-1]:]
    area = int((cus[:, 2] * cus[:, 3]).sum())
    assert area == W * H, (seed, qp, area)
    return cus


def ctu_labels(cus, w=W, h=H):
    """labels [n_ctu][40] (u8) and CTU origins [n_ctu][2] from a frame's final CUs"""
    sw, sh = w // 4, h // 4
    cid = np.full((sh, sw), -1, np.int64)
    for i, (x, y, cw, ch, _, _) in enumerate(cus):
        cid[y // 4:(y + ch) // 4, x // 4:(x + cw) // 4] = i
    assert (cid >= 0).all()
    one = lambda x, y, s: len(np.unique(cid[y // 4:(y + s) // 4, x // 4:(x + s) // 4])) == 1  # noqa: E731
    xy, lab = [], []
    for cy in range(0, h // 64 * 64, 64):
        for cx in range(0, w // 64 * 64, 64):
            v = np.zeros(40, np.uint8)
            v[0] = not one(cx, cy, 64)
            for q in range(4):
                v[1 + q] = not one(cx + 32 * (q & 1), cy + 32 * (q >> 1), 32)
            for c in range(16):
                x, y = cx + 16 * (c % 4), cy + 16 * (c // 4)
                v[5 + c] = not one(x, y, 16)
                v[21 + c] = cus[cid[y // 4, x // 4], 5]
            xy.append((cx, cy))
            lab.append(v)
    return np.array(lab, np.uint8), np.array(xy, np.int32)


def main():
    if not os.path.exists(ENC):
        sys.exit("reference encoder not built: make -C oracle ref REF=<uavs3e source tree>")
    jobs = [(s, q) for s in SEEDS for q in QPS]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        res = pool.map(encode_cus, jobs)
    labels = np.zeros((len(SEEDS), len(QPS), (W // 64) * (H // 64), 40), np.uint8)
    for (s, q), cus in zip(jobs, res):
        lab, xy = ctu_labels(cus)
        labels[SEEDS.index(s), QPS.index(q)] = lab
    out = os.path.join(HERE, "encoder_labels.npz")
    np.savez_compressed(out, seeds=np.array(SEEDS), qps=np.array(QPS), labels=labels, xy=xy, width=W, height=H,
                        n_train=16)
    print(f"{len(jobs)} encodes -> {out}: split64 {labels[..., 0].mean():.2f}, split32 {labels[..., 1:5].mean():.2f}, "
          f"split16 {labels[..., 5:21].mean():.2f}")


if __name__ == "__main__":
    main()
