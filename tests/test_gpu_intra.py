"""Batched intra lattice on the GPU against the oracle (bit-exact SATD, levels, reconstruction)."""
import numpy as np
import pytest

import pyoracle
from uavs3e_gb300.synth import intra_frame

pytestmark = pytest.mark.gpu


def oracle_lattice(oracle, org, rec, cus, ipf, qps, is_intra=1):
    H, W = org.shape
    c = np.zeros(len(cus), dtype=pyoracle.CU)
    for f in ("x", "y", "w", "h"):
        c[f] = cus[f]
    return oracle.intra_lattice(np.ascontiguousarray(org).ctypes.data, W, np.ascontiguousarray(rec).ctypes.data, W,
                                W, H, c, ipf, qps, is_intra=is_intra, threads=8)


@pytest.mark.parametrize("W,H,ipf,seed", [(128, 96, 0, 1), (136, 88, 1, 2), (64, 64, 1, 3)])
def test_intra_lattice_matches_oracle(gpu, oracle, W, H, ipf, seed):
    org = intra_frame(W, H, seed=seed)
    rng = np.random.default_rng(seed)
    rec = np.clip(org.astype(int) + rng.integers(-6, 7, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    qps = [27, 32, 37, 42]
    satd, q = gpu.intra_lattice(org, rec, cus, qps, ipf=ipf)
    satd_o, q_o = oracle_lattice(oracle, org, rec, cus, ipf, qps)
    bad = np.nonzero(satd != satd_o)[0]
    assert bad.size == 0, f"SATD differs at {bad[:8]} (cu, mode) = {[(b // 33, b % 33) for b in bad[:8]]}"
    for f in ("ssd", "coef_hash", "num_nz", "last_nz", "sum_abs"):
        bad = np.nonzero(q[f] != q_o[f])[0]
        assert bad.size == 0, f"{f} differs at {bad[:8]}: got {q[f][bad[:4]]} want {q_o[f][bad[:4]]}"


def test_intra_lattice_edge_cases(gpu, oracle):
    # flat and extreme content, inter-slice rounding offset, a single QP
    W, H = 64, 48
    org = np.zeros((H, W), np.uint8)
    org[:, W // 2:] = 255
    rec = 255 - org
    cus = gpu.lattice_cus(W, H)
    for is_intra in (0, 1):
        satd, q = gpu.intra_lattice(org, rec, cus, [5], ipf=1, is_intra=is_intra)
        satd_o, q_o = oracle_lattice(oracle, org, rec, cus, 1, [5], is_intra)
        assert np.array_equal(satd, satd_o)
        assert np.array_equal(q, q_o)


def test_intra_lattice_unsorted_and_invalid_cus(gpu, oracle):
    # CUs in random order with unsupported entries mixed in: outputs go by CU index, the
    # unsupported ones (outside the picture, sides not a power of two) come back zeroed
    W, H = 96, 64
    org = intra_frame(W, H, seed=5)
    rec = np.clip(org.astype(int) + np.random.default_rng(5).integers(-4, 5, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    rng = np.random.default_rng(7)
    cus = cus[rng.permutation(len(cus))]
    bad = np.zeros(3, dtype=cus.dtype)
    bad[0] = (80, 48, 32, 32, 0)      # crosses the right and bottom edges
    bad[1] = (0, 0, 12, 16, 0)        # width not a power of two
    bad[2] = (0, 0, 128, 8, 0)        # side above 64
    allc = np.concatenate([cus[:40], bad[:1], cus[40:90], bad[1:], cus[90:]])
    qps = [22, 37]
    satd, q = gpu.intra_lattice(org, rec, allc, qps, ipf=0)
    valid = np.ones(len(allc), bool)
    valid[[40, 91, 92]] = False
    satd = satd.reshape(len(allc), 33)
    q = q.reshape(len(allc), 33, len(qps))
    assert not satd[~valid].any() and not q[~valid].view(np.uint8).any()
    satd_o, q_o = oracle_lattice(oracle, org, rec, allc[valid], 0, qps)
    assert np.array_equal(satd[valid].ravel(), satd_o)
    assert np.array_equal(q[valid].ravel(), q_o)


def test_intra_lattice_odd_pitch_and_unaligned_cus(gpu, oracle):
    # the org blocks are read by words only where the picture and its pitch are word-aligned: an
    # odd row pitch takes the byte path with the same records; CUs off the 4x4 grid are outside
    # the supported set and come back zeroed
    import torch
    W, H = 96, 64
    org = intra_frame(W, H, seed=9)
    rec = np.clip(org.astype(int) + np.random.default_rng(9).integers(-4, 5, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)[::5]
    odd = np.zeros(3, dtype=cus.dtype)
    odd[0] = (1, 4, 8, 8, 0)
    odd[1] = (8, 18, 16, 4, 0)
    odd[2] = (30, 2, 4, 16, 0)
    allc = np.concatenate([cus, odd])
    qps = [27, 42]
    satd_o, q_o = oracle_lattice(oracle, org, rec, cus, 1, qps)
    n, nv = len(allc), len(cus)
    for pitch in (W, W + 1):
        po = np.zeros((H, pitch), np.uint8)
        po[:, :W] = org
        d_org = torch.from_numpy(po).cuda()
        d_rec = torch.from_numpy(rec).cuda()
        d_cus = torch.from_numpy(np.ascontiguousarray(allc).view(np.uint8)).cuda()
        q = np.array(qps, np.int32)
        d_satd = torch.full((n * 33,), -1, dtype=torch.int32, device="cuda")
        d_q = torch.full((n * 33 * len(q) * gpu.LAT_Q.itemsize,), 255, dtype=torch.uint8, device="cuda")
        gpu.check(gpu.lib().uavs3e_cuda_intra_lattice_device(d_org.data_ptr(), pitch, d_rec.data_ptr(), W, W, H,
                                                             d_cus.data_ptr(), n, 1, q.ctypes.data, len(q), 1,
                                                             d_satd.data_ptr(), d_q.data_ptr(),
                                                             torch.cuda.current_stream().cuda_stream), "intra_lattice")
        torch.cuda.synchronize()
        satd = d_satd.cpu().numpy().view(np.uint32)
        rq = d_q.cpu().numpy().view(gpu.LAT_Q)
        assert np.array_equal(satd[:nv * 33], satd_o), pitch
        assert np.array_equal(rq[:nv * 33 * len(q)], q_o), pitch
        assert not satd[nv * 33:].any() and not rq[nv * 33 * len(q):].view(np.uint8).any(), pitch


def test_intra_lattice_mode_subset(gpu):
    # a shortlist of modes per CU writes exactly those records, equal to the full lattice's
    import ctypes as C
    import torch
    W, H = 96, 64
    org = intra_frame(W, H, seed=8)
    rec = np.clip(org.astype(int) + np.random.default_rng(8).integers(-4, 5, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    qps = [27, 37]
    satd_all, q_all = gpu.intra_lattice(org, rec, cus, qps, ipf=1)
    rng = np.random.default_rng(9)
    K = 8
    modes = np.stack([rng.permutation(33)[:K] for _ in range(len(cus))]).astype(np.uint8)
    L = gpu.lib()
    P, I = C.c_void_p, C.c_int
    L.uavs3e_cuda_intra_lattice_modes_device.argtypes = [P, I, P, I, I, I, P, I, P, I, I, P, I, I, P, P, P]
    d_org = torch.from_numpy(org).cuda()
    d_rec = torch.from_numpy(rec).cuda()
    d_cus = torch.from_numpy(cus.view(np.uint8).copy()).cuda()
    d_modes = torch.from_numpy(modes).cuda()
    n = len(cus)
    d_satd = torch.full((n * 33,), -1, dtype=torch.int32, device="cuda")
    d_q = torch.full((n * 33 * len(qps) * 16,), 0xAB, dtype=torch.uint8, device="cuda")
    q = np.array(qps, np.int32)
    rc = L.uavs3e_cuda_intra_lattice_modes_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(), n,
                                                  d_modes.data_ptr(), K, 1, q.ctypes.data, len(qps), 1,
                                                  d_satd.data_ptr(), d_q.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    satd = d_satd.cpu().numpy().view(np.uint32).reshape(n, 33)
    qq = d_q.cpu().numpy().view(gpu.LAT_Q).reshape(n, 33, len(qps))
    sel = np.zeros((n, 33), bool)
    np.put_along_axis(sel, modes.astype(int), True, 1)
    assert np.array_equal(satd[sel], satd_all.reshape(n, 33)[sel])
    assert np.array_equal(qq[sel], q_all.reshape(n, 33, len(qps))[sel])
    assert (satd[~sel] == 0xFFFFFFFF).all()
    assert (qq[~sel].view(np.uint8) == 0xAB).all()


def test_lattice_autotuned_layouts_give_the_same_records(gpu):
    """records do not depend on the CTA layout the autotuner picks"""
    from uavs3e_gb300.synth import intra_frame
    W, H = 384, 256
    org = intra_frame(W, H, seed=41)
    rec = np.clip(org.astype(int) + np.random.default_rng(42).integers(-4, 5, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    gpu.lattice_autotune(False)
    want_s, want_q = gpu.intra_lattice(org, rec, cus)
    gpu.lattice_autotune(True)
    got_s, got_q = gpu.intra_lattice(org, rec, cus)       # tunes the shapes with >= 512 CUs
    again_s, again_q = gpu.intra_lattice(org, rec, cus)   # runs the tuned layouts
    assert np.array_equal(want_s, got_s) and np.array_equal(want_q.view(np.uint8), got_q.view(np.uint8))
    assert np.array_equal(want_s, again_s) and np.array_equal(want_q.view(np.uint8), again_q.view(np.uint8))
    tuned = gpu.lattice_budgets(33)
    assert any(tuned)


def test_intra_lattice_is_one_graph(gpu):
    # after a first plain call (which tunes the layouts), the whole lattice of a frame -- classify,
    # plan, scatter and the persistent tile kernel -- is captured into one CUDA graph; replays give
    # the plain launches' records, also for new frame content copied into the same buffers
    import torch
    W, H = 256, 192
    lib = gpu.lib()
    cus = gpu.lattice_cus(W, H)
    n = len(cus)
    qps = np.array([22, 37], np.int32)
    d_org = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    d_rec = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    d_cus = torch.from_numpy(cus.view(np.uint8).copy()).cuda()
    d_satd = torch.zeros(n * 33, dtype=torch.int32, device="cuda")
    d_q = torch.zeros(n * 33 * len(qps) * 16, dtype=torch.uint8, device="cuda")

    def frame(seed):
        org = intra_frame(W, H, seed=seed)
        rec = np.clip(org.astype(int) + np.random.default_rng(seed).integers(-5, 6, org.shape), 0, 255)
        d_org.copy_(torch.from_numpy(org))
        d_rec.copy_(torch.from_numpy(rec.astype(np.uint8)))

    def run():
        gpu.check(lib.uavs3e_cuda_intra_lattice_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H,
                                                       d_cus.data_ptr(), n, 1, qps.ctypes.data, len(qps), 1,
                                                       d_satd.data_ptr(), d_q.data_ptr(),
                                                       torch.cuda.current_stream().cuda_stream), "intra_lattice")

    want = {}
    for seed in (21, 22):
        frame(seed)
        run()
        torch.cuda.synchronize()
        want[seed] = (d_satd.clone(), d_q.clone())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        run()
    for seed in (21, 22, 21):
        frame(seed)
        d_satd.zero_()
        d_q.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(d_satd, want[seed][0]) and torch.equal(d_q, want[seed][1]), seed
