"""Batched motion search and frame interpolation on the GPU against the oracle (bit-exact)."""
import numpy as np
import pytest

import pyoracle
from gpu_util import download, padded
from uavs3e_gb300.synth import lambda_mv_for_qp, motion_sequence

pytestmark = pytest.mark.gpu


def oracle_planes(oracle, frame, pad, stride):
    H, W = frame.shape
    p0 = padded(frame, pad, stride)
    planes = [np.zeros_like(p0) for _ in range(15)]
    base = pad * stride + pad
    oracle.if_luma_frame(p0.ctypes.data + base, [p.ctypes.data + base for p in planes], W, H, pad, stride)
    return p0, planes


@pytest.mark.parametrize("W,H", [(200, 136), (256, 192)])
def test_subpel_planes_match_oracle(gpu, oracle, W, H):
    frames = motion_sequence(W, H, 1, seed=3)
    ms = gpu.MotionSearch(W, H, n_refs=1, search_range=16, pad=144)
    ms.set_ref(0, frames[0])
    stride, pad = ms.stride, 144
    p0, planes = oracle_planes(oracle, frames[0], pad, stride)
    nbytes = (H + 2 * pad) * stride
    for ph in range(16):
        got = download(ms.plane_ptr(0, ph) - (pad * stride + pad), nbytes)
        want = p0 if ph == 0 else planes[ph - 1]
        assert np.array_equal(got, want), f"phase {ph} differs at {np.argwhere(got != want)[:5]}"
    ms.close()


def run_oracle_me(oracle, org, refs, W, H, rng, lam, pad=144, threads=8):
    stride = ((W + 2 * pad) + 15) & ~15
    keep, ptrs = [], []
    for f in refs:
        p0, planes = oracle_planes(oracle, f, pad, stride)
        keep += [p0] + planes
        base = pad * stride + pad
        ptrs += [p0.ctypes.data + base] + [p.ctypes.data + base for p in planes]
    import uavs3e_gb300 as u
    bl = u.me_blocks(W, H)
    blocks = np.zeros(len(bl), dtype=pyoracle.ME_BLOCK)
    blocks["x"], blocks["y"], blocks["w"], blocks["h"] = bl[:, 0], bl[:, 1], bl[:, 2], bl[:, 3]
    valid = (bl[:, 0] + bl[:, 2] <= W) & (bl[:, 1] + bl[:, 3] <= H)
    vb = blocks[valid]
    org = np.ascontiguousarray(org)
    res = oracle.me_frame(org.ctypes.data, W, ptrs, stride, W, H, len(refs), vb, rng, lam, threads=threads)
    return valid, res.reshape(len(vb), len(refs))


# search ranges cover every split of the dy range into 8-row items plus leftover rows:
# 2r+1 = 129, 49, 33, 17 (one row left), 13 (five), 21 (five), 7 and 5 (no full item)
@pytest.mark.parametrize("W,H,rng,qp", [(192, 128, 64, 32), (200, 136, 24, 27), (128, 64, 16, 45), (320, 200, 8, 37),
                                        (256, 128, 6, 32), (136, 72, 10, 40), (192, 128, 3, 30), (160, 96, 2, 22)])
def test_me_frame_matches_oracle(gpu, oracle, W, H, rng, qp):
    frames = motion_sequence(W, H, 3, seed=W + H, n_rects=3)
    lam = lambda_mv_for_qp(qp)
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=rng, pad=144)
    ms.set_ref(0, frames[1])
    ms.set_ref(1, frames[0])
    got = ms.run(frames[2], lam).reshape(-1, 2)
    valid, want = run_oracle_me(oracle, frames[2], [frames[1], frames[0]], W, H, rng, lam)
    g = got[valid]
    for f in ("mv_int", "mv_sub", "sad_int", "satd_sub", "cost_int", "cost_sub"):
        ok = np.array_equal(g[f], want[f])
        if not ok:
            bad = np.argwhere((g[f] != want[f]).reshape(g.shape[0], -1).any(axis=1))[:5].ravel()
            raise AssertionError(f"{f} differs in {len(np.unique(bad))}+ blocks, e.g. {bad}: got {g[bad]} want {want[bad]}")
    assert np.all(got[~valid]["cost_int"] == np.iinfo(np.uint64).max)
    ms.close()


def test_me_frame_repeatable_and_device_path(gpu):
    import torch
    W, H = 256, 128
    frames = motion_sequence(W, H, 3, seed=11)
    lam = lambda_mv_for_qp(32)
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=32)
    ms.set_ref(0, frames[1])
    ms.set_ref(1, frames[0])
    a = ms.run(frames[2], lam)
    d_org = torch.from_numpy(frames[2]).cuda()
    d_out = torch.zeros(ms.n_results * 32, dtype=torch.uint8, device="cuda")
    ms.run_device(d_org.data_ptr(), W, lam, d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    b = d_out.cpu().numpy().view(gpu.ME_RESULT)
    assert np.array_equal(a, b)
    c = ms.run(frames[2], lam)
    assert np.array_equal(a, c)


def test_me_frame_graph_matches_plain_launches(gpu):
    """the frame replayed as a captured CUDA graph gives the plain launches' results, across cached
    graphs, new argument sets and a lambda change"""
    import torch
    W, H = 256, 192
    frames = motion_sequence(W, H, 6, seed=21)
    d_frames = [torch.from_numpy(f).cuda() for f in frames]
    n = gpu.MotionSearch(W, H, n_refs=2, search_range=32, pad=144).n_results
    plain = gpu.MotionSearch(W, H, n_refs=2, search_range=32, pad=144)
    graph = gpu.MotionSearch(W, H, n_refs=2, search_range=32, pad=144)
    sp = torch.cuda.current_stream().cuda_stream
    d_a = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
    d_b = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
    schedule = [(1, 32), (2, 32), (3, 32), (1, 32), (2, 27), (4, 27), (5, 27), (2, 27)]
    for t, qp in schedule:
        lam = lambda_mv_for_qp(qp)
        slot = (t - 1) % 2
        for ms in (plain, graph):                # the other slot: the same picture in both sessions
            ms.set_ref_device(1 - slot, d_frames[max(0, t - 2)].data_ptr(), W, sp)
        plain.set_ref_device(slot, d_frames[t - 1].data_ptr(), W, sp)
        plain.run_device(d_frames[t].data_ptr(), W, lam, d_a.data_ptr(), sp)
        graph.frame_graph(slot, d_frames[t - 1].data_ptr(), W, d_frames[t].data_ptr(), W, lam, d_b.data_ptr(), sp)
        torch.cuda.synchronize()
        assert torch.equal(d_a, d_b), f"frame {t} (qp {qp}) differs"
    plain.close()
    graph.close()


def test_me_frame_host_matches_set_ref_run(gpu):
    """uavs3e_cuda_me_frame (host reference + host frame, one graph replay) gives what
    uavs3e_cuda_me_set_ref followed by uavs3e_cuda_me_run gives, over alternating slots, reused
    cached graphs and a lambda change"""
    W, H = 200, 136
    frames = motion_sequence(W, H, 6, seed=23)
    plain = gpu.MotionSearch(W, H, n_refs=2, search_range=32, pad=144)
    onecall = gpu.MotionSearch(W, H, n_refs=2, search_range=32, pad=144)
    out = np.zeros(onecall.n_results, dtype=gpu.ME_RESULT)
    schedule = [(1, 32), (2, 32), (3, 32), (4, 32), (5, 27), (2, 27)]
    for t, qp in schedule:
        lam = lambda_mv_for_qp(qp)
        slot = (t - 1) % 2
        for ms in (plain, onecall):
            ms.set_ref(1 - slot, frames[max(0, t - 2)])
        plain.set_ref(slot, frames[t - 1])
        want = plain.run(frames[t], lam)
        ref = np.ascontiguousarray(frames[t - 1])
        org = np.ascontiguousarray(frames[t])
        onecall.frame_ptr(slot, ref.ctypes.data, W, org.ctypes.data, W, lam, out.ctypes.data)
        assert np.array_equal(want, out), f"frame {t} (qp {qp}) differs"
    plain.close()
    onecall.close()
