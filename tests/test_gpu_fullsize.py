"""Parity at the benchmarked sizes: the 1080p motion-search frame and the 1080p intra lattice
that bench.py times, checked against the oracle on sampled parts of the picture.

The GPU runs the whole picture exactly as the bench does; the oracle recomputes a subset that
covers every kind of CTA the GPU splits the picture into: for the motion search, the top CTU row,
an interior row and the partial bottom row (56 of 64 lines), each across all 30 columns (the
interior and right/bottom-edge launches of the integer search both appear); for the lattice, a
seeded sample of CUs of all 23 shapes plus every CU touching the right or bottom picture edge, at
the four QPs of the bench.
"""
import os

import numpy as np
import pytest

import pyoracle
from test_gpu_me import oracle_planes
from uavs3e_gb300.synth import intra_frame, lambda_mv_for_qp, motion_sequence

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
THREADS = os.cpu_count() or 8


def test_me_frame_1080p_rows_match_oracle(gpu, oracle):
    # the bench's frame: seeded 1080p motion sequence, references = the two previous frames,
    # range +-64, lambda of QP 32, padding 144
    frames = motion_sequence(W, H, 3, seed=0)
    lam = lambda_mv_for_qp(32)
    rng, pad = 64, 144
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=rng, pad=pad)
    ms.set_ref(0, frames[1])
    ms.set_ref(1, frames[0])
    got = ms.run(frames[2], lam).reshape(-1, 2)
    ms.close()

    stride = ((W + 2 * pad) + 15) & ~15
    keep, ptrs = [], []
    for f in (frames[1], frames[0]):
        p0, planes = oracle_planes(oracle, f, pad, stride)
        keep += [p0] + planes
        base = pad * stride + pad
        ptrs += [p0.ctypes.data + base] + [p.ctypes.data + base for p in planes]
    bl = gpu.me_blocks(W, H)
    rows = (0, 8, (H + 63) // 64 - 1)
    sel = np.isin(bl[:, 1] // 64, rows) & (bl[:, 0] + bl[:, 2] <= W) & (bl[:, 1] + bl[:, 3] <= H)
    blocks = np.zeros(int(sel.sum()), dtype=pyoracle.ME_BLOCK)
    blocks["x"], blocks["y"], blocks["w"], blocks["h"] = bl[sel, 0], bl[sel, 1], bl[sel, 2], bl[sel, 3]
    org = np.ascontiguousarray(frames[2])
    want = oracle.me_frame(org.ctypes.data, W, ptrs, stride, W, H, 2, blocks, rng, lam,
                           threads=THREADS).reshape(len(blocks), 2)
    g = got[sel]
    assert len(g) > 3 * 30 * 100
    for f in ("mv_int", "mv_sub", "sad_int", "satd_sub", "cost_int", "cost_sub"):
        bad = np.argwhere((g[f] != want[f]).reshape(len(g), -1).any(axis=1)).ravel()
        assert bad.size == 0, (f"{f} differs in {bad.size} blocks, e.g. {bl[sel][bad[:4]]}: "
                               f"got {g[bad[:2]]} want {want[bad[:2]]}")
    # blocks of the bottom row that leave the picture carry no result
    out = (bl[:, 1] + bl[:, 3] > H)
    assert out.any() and np.all(got[out]["cost_int"] == np.iinfo(np.uint64).max)


def lattice_sample(cus, n_sample, seed):
    rng = np.random.default_rng(seed)
    idx = set(rng.choice(len(cus), n_sample, replace=False).tolist())
    edge = np.nonzero((cus["x"].astype(int) + cus["w"] == W) | (cus["y"].astype(int) + cus["h"] == H))[0]
    idx |= set(edge.tolist())
    for w in (4, 8, 16, 32, 64):                       # the first CU of every shape as well
        for h in (4, 8, 16, 32, 64):
            k = np.nonzero((cus["w"] == w) & (cus["h"] == h))[0]
            if k.size:
                idx.add(int(k[0]))
    return np.array(sorted(idx))


@pytest.mark.parametrize("ipf,n_sample", [(0, 12000), (1, 3000)])
def test_intra_lattice_1080p_sample_matches_oracle(gpu, oracle, ipf, n_sample):
    # the bench's lattice: seeded 1080p I-frame, reconstruction = org + noise, all CUs of the 23
    # shapes, QP 27/32/37/42
    org = intra_frame(W, H, seed=11)
    rec = np.clip(org.astype(int) + np.random.default_rng(12).integers(-5, 6, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    assert len(cus) == 468750
    qps = [27, 32, 37, 42]
    satd, q = gpu.intra_lattice(org, rec, cus, qps, ipf=ipf)
    pick = lattice_sample(cus, n_sample, seed=40 + ipf)
    shapes = {(int(w), int(h)) for w, h in zip(cus["w"][pick], cus["h"][pick])}
    assert len(shapes) == 23
    c = np.zeros(len(pick), dtype=pyoracle.CU)
    for f in ("x", "y", "w", "h"):
        c[f] = cus[f][pick]
    satd_o, q_o = oracle.intra_lattice(org.ctypes.data, W, rec.ctypes.data, W, W, H, c, ipf, qps, is_intra=1,
                                       threads=THREADS)
    rows = (pick[:, None] * 33 + np.arange(33)[None, :]).ravel()
    g_satd = satd[rows]
    bad = np.nonzero(g_satd != satd_o)[0]
    assert bad.size == 0, f"SATD differs at (cu, mode) {[(pick[b // 33], b % 33) for b in bad[:6]]}"
    qrows = (rows[:, None] * len(qps) + np.arange(len(qps))[None, :]).ravel()
    g_q = q[qrows]
    for f in ("ssd", "coef_hash", "num_nz", "last_nz", "sum_abs"):
        bad = np.nonzero(g_q[f] != q_o[f])[0]
        assert bad.size == 0, f"{f} differs at {bad[:6]}: got {g_q[f][bad[:3]]} want {q_o[f][bad[:3]]}"


def test_intra_lattice_host_entry_matches_device_entry(gpu):
    # uavs3e_cuda_intra_lattice (host buffers, copies inside the call) writes the device entry's
    # records, on a strided host picture and twice in a row with different CU counts
    Wp, Hp = 256, 136
    org = intra_frame(Wp, Hp, seed=3)
    rec = np.clip(org.astype(int) + np.random.default_rng(4).integers(-5, 6, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(Wp, Hp)
    for sub, qps in ((cus, [22, 37]), (cus[::3], [30, 31, 45, 51])):
        want_satd, want_q = gpu.intra_lattice(org, rec, sub, qps, ipf=1)
        big_org = np.zeros((Hp, Wp + 40), np.uint8)
        big_org[:, 8:8 + Wp] = org
        got_satd, got_q = gpu.intra_lattice_host(big_org[:, 8:8 + Wp], rec, sub, qps, ipf=1)
        assert np.array_equal(got_satd, want_satd)
        assert np.array_equal(got_q, want_q)


def test_intra_lattice_host_entry_in_ranges_at_1080p(gpu):
    # a 1080p call (468,750 CUs) runs as four CU ranges whose record downloads overlap the next
    # range's lattice; the records equal one device-entry launch over all CUs
    org = intra_frame(W, H, seed=21)
    rec = np.clip(org.astype(int) + np.random.default_rng(22).integers(-5, 6, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    assert len(cus) >= 4 * 65536
    qps = [27, 32, 37, 42]
    want_satd, want_q = gpu.intra_lattice(org, rec, cus, qps)
    got_satd, got_q = gpu.intra_lattice_host(org, rec, cus, qps)
    assert np.array_equal(got_satd, want_satd)
    assert np.array_equal(got_q.view(np.uint8), want_q.view(np.uint8))
