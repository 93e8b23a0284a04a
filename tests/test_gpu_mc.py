"""GPU: CU motion compensation (uavs3e_cuda_mc_cu*, com_mc_cu src/com_mc.c:140) and affine CU
motion compensation (uavs3e_cuda_mc_affine*, com_mc_cu_affine :361) bit-exact against the
reference's golden digests and the oracle: luma and 4-tap chroma, one or two lists, identical
motion, MVs reaching past the picture edges, every channel selection, 2 / 3 control points, 4x4 /
8x8 sub-blocks, the session entries."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

_ALL = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
GOLDEN = [c for c in _ALL if c["kernel"] == "mc"]
GOLDEN_AFFINE = [c for c in _ALL if c["kernel"] == "affine"]


def _gpu_mc(gpu, p, luma, chroma, reqs, nbytes):
    import torch
    keep, addrs, stride = luma
    cplanes, caddrs, sc = chroma
    d_l = [torch.from_numpy(a).cuda() for a in keep]
    d_c = [torch.from_numpy(a).cuda() for a in cplanes]
    base = cases.TZ_PAD * stride + cases.TZ_PAD
    cbase = cases.MC_PAD_C * sc + cases.MC_PAD_C
    d_req = torch.from_numpy(np.ascontiguousarray(reqs).view(np.uint8).copy()).cuda()
    d_out = torch.zeros(max(1, nbytes), dtype=torch.uint8, device="cuda")
    gpu.mc_cu_device(p["w"], p["h"], [t.data_ptr() + base for t in d_l], stride, cases.TZ_PAD,
                     [t.data_ptr() + cbase for t in d_c], sc, cases.MC_PAD_C, d_req.data_ptr(), len(reqs),
                     d_out.data_ptr(), nbytes)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()[:nbytes]


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[f"{c['params']['w']}x{c['params']['h']}" for c in GOLDEN])
def test_mc_matches_reference_golden(gpu, oracle, case):
    luma, chroma, reqs, nbytes = cases.mc_inputs(oracle, case["params"], case["seed"])
    assert cases.digest(_gpu_mc(gpu, case["params"], luma, chroma, reqs, nbytes)) == case["md5"]


@pytest.mark.gpu
@pytest.mark.parametrize("p", cases.MC_CASES, ids=[f"{p['w']}x{p['h']}" for p in cases.MC_CASES])
def test_mc_matches_oracle_many_seeds(gpu, oracle, p):
    for seed in range(500, 516):
        luma, chroma, reqs, nbytes = cases.mc_inputs(oracle, dict(p, n=400), seed)
        want = oracle.mc_cu(p["w"], p["h"], luma[1], luma[2], chroma[1], chroma[2], reqs, nbytes)
        got = _gpu_mc(gpu, p, luma, chroma, reqs, nbytes)
        bad = np.nonzero(want != got)[0]
        assert len(bad) == 0, f"seed {seed}: {len(bad)} bytes differ, first at {bad[:5]}"


@pytest.mark.gpu
def test_mc_session_entry(gpu, oracle):
    p = cases.MC_CASES[0]
    W, H = p["w"], p["h"]
    rng = np.random.default_rng(99)
    frames = cases.loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    luma = cases.tz_planes(oracle, frames, [4, 0], W, H)
    sc = W // 2 + 2 * cases.MC_PAD_C
    cpl = [cases.padded_plane(frames[t][c], cases.MC_PAD_C, sc).reshape(-1) for t in (4, 0) for c in (1, 2)]
    caddrs = [a.ctypes.data + cases.MC_PAD_C * sc + cases.MC_PAD_C for a in cpl]
    reqs, nbytes = cases.mc_requests(rng, W, H, 500)
    want = oracle.mc_cu(W, H, luma[1], luma[2], caddrs, sc, reqs, nbytes)
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=64, pad=144)
    for slot, t in enumerate((4, 0)):
        ms.set_ref(slot, frames[t][0])
        ms.set_ref_chroma(slot, frames[t][1], frames[t][2])
    got = ms.mc_cu(reqs, nbytes)
    ms.close()
    assert np.array_equal(want, got)


@pytest.mark.gpu
def test_mc_skips_requests_outside_the_domain(gpu, oracle):
    """a CU past the picture, an unknown slot, or an output past the buffer is skipped"""
    p = cases.MC_CASES[1]
    luma, chroma, reqs, nbytes = cases.mc_inputs(oracle, dict(p, n=8), 3)
    bad = reqs.copy()
    bad[0]["x"] = p["w"]                 # outside the picture
    bad[1]["slot"] = [5, -1]             # unknown slot
    bad[2]["out_offset"] = nbytes        # output past the buffer
    got = _gpu_mc(gpu, p, luma, chroma, bad, nbytes)
    want = oracle.mc_cu(p["w"], p["h"], luma[1], luma[2], chroma[1], chroma[2], reqs[3:], nbytes)
    # the valid CUs keep their bytes; the skipped ones leave zeros
    for i in range(3, 8):
        o, w, h, ch = (int(reqs[i][f]) for f in ("out_offset", "w", "h", "channel"))
        size = (w * h if ch != 2 else 0) + (w * h // 2 if ch != 1 else 0)
        assert np.array_equal(got[o:o + size], want[o:o + size])
    o0 = int(reqs[0]["out_offset"])
    assert not got[o0:o0 + 8].any()
    assert gpu.lib().uavs3e_cuda_status() == 0


@pytest.mark.gpu
def test_mc_rejects_bad_padding(gpu):
    import torch
    d = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
    with pytest.raises(gpu.CudaError):
        gpu.mc_cu_device(64, 64, [d.data_ptr()] * 16, 512, 144, [d.data_ptr()] * 2, 256, 32, d.data_ptr(), 1,
                         d.data_ptr(), 16)
    assert gpu.lib().uavs3e_cuda_status() == 0


def _gpu_affine(gpu, p, luma, chroma, reqs, nbytes):
    import torch
    keep, addrs, stride = luma
    cplanes, caddrs, sc = chroma
    d_l = [torch.from_numpy(a).cuda() for a in keep]
    d_c = [torch.from_numpy(a).cuda() for a in cplanes]
    base = cases.TZ_PAD * stride + cases.TZ_PAD
    cbase = cases.MC_PAD_C * sc + cases.MC_PAD_C
    d_req = torch.from_numpy(np.ascontiguousarray(reqs).view(np.uint8).copy()).cuda()
    d_out = torch.zeros(max(1, nbytes), dtype=torch.uint8, device="cuda")
    gpu.mc_affine_device(p["w"], p["h"], [t.data_ptr() + base for t in d_l], stride, cases.TZ_PAD,
                         [t.data_ptr() + cbase for t in d_c], sc, cases.MC_PAD_C, d_req.data_ptr(), len(reqs),
                         d_out.data_ptr(), nbytes)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()[:nbytes]


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN_AFFINE, ids=[f"{c['params']['w']}x{c['params']['h']}" for c in GOLDEN_AFFINE])
def test_affine_matches_reference_golden(gpu, oracle, case):
    p = case["params"]
    luma, chroma, _, _ = cases.mc_inputs(oracle, dict(p, n=1), case["seed"])
    reqs, nbytes = cases.affine_requests(np.random.default_rng(case["seed"] + 1), p["w"], p["h"], p["n"])
    assert cases.digest(_gpu_affine(gpu, p, luma, chroma, reqs, nbytes)) == case["md5"]


@pytest.mark.gpu
@pytest.mark.parametrize("p", cases.MC_CASES, ids=[f"{p['w']}x{p['h']}" for p in cases.MC_CASES])
def test_affine_matches_oracle_many_seeds(gpu, oracle, p):
    for seed in range(700, 712):
        luma, chroma, _, _ = cases.mc_inputs(oracle, dict(p, n=1), seed)
        reqs, nbytes = cases.affine_requests(np.random.default_rng(seed), p["w"], p["h"], 300)
        want = oracle.mc_affine(p["w"], p["h"], luma[1], luma[2], chroma[1], chroma[2], reqs, nbytes)
        got = _gpu_affine(gpu, p, luma, chroma, reqs, nbytes)
        bad = np.nonzero(want != got)[0]
        assert len(bad) == 0, f"seed {seed}: {len(bad)} bytes differ, first at {bad[:5]}"


@pytest.mark.gpu
def test_affine_session_entry(gpu, oracle):
    p = cases.MC_CASES[0]
    W, H = p["w"], p["h"]
    rng = np.random.default_rng(5)
    frames = cases.loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    luma = cases.tz_planes(oracle, frames, [4, 0], W, H)
    sc = W // 2 + 2 * cases.MC_PAD_C
    cpl = [cases.padded_plane(frames[t][c], cases.MC_PAD_C, sc).reshape(-1) for t in (4, 0) for c in (1, 2)]
    caddrs = [a.ctypes.data + cases.MC_PAD_C * sc + cases.MC_PAD_C for a in cpl]
    reqs, nbytes = cases.affine_requests(rng, W, H, 200)
    want = oracle.mc_affine(W, H, luma[1], luma[2], caddrs, sc, reqs, nbytes)
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=64, pad=144)
    for slot, t in enumerate((4, 0)):
        ms.set_ref(slot, frames[t][0])
        ms.set_ref_chroma(slot, frames[t][1], frames[t][2])
    got = ms.mc_affine(reqs, nbytes)
    ms.close()
    assert np.array_equal(want, got)
