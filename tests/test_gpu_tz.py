"""GPU: per-call TZ motion search (uavs3e_cuda_me_tz*, me_search_tz src/me.c:529) bit-exact against
the reference's golden digests and the oracle restatement: every MV resolution, bi-prediction,
SAD/SATD refinement, adaptive raster ranges, padded and unpadded searches, and a 1080p batch."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"] if c["kernel"] == "tz"]
THREADS = os.cpu_count() or 4


def _id(p):
    return f"{p['w']}x{p['h']}-pad{p['pad']}-sr{p['range']}"


def _gpu_tz(gpu, pic, org, keep, stride, reqs):
    import torch
    d_planes = [torch.from_numpy(a).cuda() for a in keep]
    base = cases.TZ_PAD * stride + cases.TZ_PAD
    d_org = torch.from_numpy(np.ascontiguousarray(org)).cuda()
    d_req = torch.from_numpy(np.ascontiguousarray(reqs).view(np.uint8).copy()).cuda()
    d_out = torch.zeros(max(1, len(reqs)) * gpu.TZ_OUT.itemsize, dtype=torch.uint8, device="cuda")
    gpu.me_tz_device(pic, d_org.data_ptr(), org.shape[1], [t.data_ptr() + base for t in d_planes], stride,
                     cases.TZ_PAD, d_req.data_ptr(), len(reqs), d_out.data_ptr())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(gpu.TZ_OUT)[:len(reqs)]


def _assert_same(reqs, want, got):
    bad = [i for i in range(len(want)) if want[i].tobytes() != got[i].tobytes()]
    assert not bad, f"{len(bad)} of {len(want)} differ; first: req {reqs[bad[0]]} want {want[bad[0]]} got {got[bad[0]]}"


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[_id(c["params"]) for c in GOLDEN])
def test_tz_matches_reference_golden(gpu, oracle, case):
    pic, org, keep, addrs, stride, reqs = cases.tz_inputs(oracle, case["params"], case["seed"])
    got = _gpu_tz(gpu, pic, org, keep, stride, reqs)
    assert cases.digest(got.view(np.uint8)) == case["md5"]


@pytest.mark.gpu
@pytest.mark.parametrize("p", cases.TZ_CASES, ids=[_id(p) for p in cases.TZ_CASES])
def test_tz_matches_oracle_many_seeds(gpu, oracle, p):
    for seed in range(300, 312):
        q = dict(p, n=256)
        pic, org, keep, addrs, stride, reqs = cases.tz_inputs(oracle, q, seed)
        want = oracle.me_tz(pic, org, q["w"], addrs, stride, reqs)
        _assert_same(reqs, want, _gpu_tz(gpu, pic, org, keep, stride, reqs))


@pytest.mark.gpu
def test_tz_session_entry(gpu, oracle):
    """the host-buffer entry on a motion-search session's interpolated references"""
    p = cases.TZ_CASES[0]
    rng = np.random.default_rng(77)
    W, H = p["w"], p["h"]
    frames = cases.loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    keep, addrs, stride = cases.tz_planes(oracle, frames, [4, 0], W, H)
    reqs = cases.tz_requests(rng, W, H, 300, [4, 8])
    pic = (W, H, 1, p["range"], p["gop"])
    want = oracle.me_tz(pic, frames[8][0], W, addrs, stride, reqs)
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=64, pad=144)
    ms.set_ref(0, frames[4][0])
    ms.set_ref(1, frames[0][0])
    got = ms.tz(pic, frames[8][0], reqs)
    ms.close()
    _assert_same(reqs, want, got)


@pytest.mark.gpu
def test_tz_1080p_batch(gpu, oracle):
    """a frame's worth of calls: every block of the ten shapes on the CTU grid, 2 references, AMVR
    resolutions and bi calls mixed"""
    from uavs3e_gb300.synth import motion_sequence
    W, H = 1920, 1080
    seq = motion_sequence(W, H, 3, seed=9)
    frames = {t: (seq[t],) for t in range(3)}
    keep, addrs, stride = cases.tz_planes(oracle, frames, [1, 0], W, H)
    rng = np.random.default_rng(1080)
    reqs = cases.tz_requests(rng, W, H, 6000, [1, 2])
    pic = (W, H, 1, 384, 16)
    want = oracle.me_tz(pic, seq[2], W, addrs, stride, reqs, THREADS)
    _assert_same(reqs, want, _gpu_tz(gpu, pic, seq[2], keep, stride, reqs))


@pytest.mark.gpu
def test_tz_repeatable(gpu, oracle):
    """the same calls three times give byte-identical results (each warp's search depends only on
    its request: no cross-warp state, integer atomics only)"""
    p = cases.TZ_CASES[0]
    q = dict(p, n=512)
    pic, org, keep, addrs, stride, reqs = cases.tz_inputs(oracle, q, 321)
    runs = [_gpu_tz(gpu, pic, org, keep, stride, reqs).tobytes() for _ in range(3)]
    assert runs[0] == runs[1] == runs[2]


@pytest.mark.gpu
def test_tz_rejects_bad_arguments(gpu):
    import torch
    d = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
    base = d.data_ptr() + 144 * 512 + 144
    with pytest.raises(gpu.CudaError):     # padding below 144
        gpu.me_tz_device((64, 64, 1, 384, 16), base, 64, [base] * 16, 512, 64, d.data_ptr(), 1, d.data_ptr())
    with pytest.raises(gpu.CudaError):     # search range above 1024
        gpu.me_tz_device((64, 64, 1, 4096, 16), base, 64, [base] * 16, 512, 144, d.data_ptr(), 1, d.data_ptr())
    assert gpu.lib().uavs3e_cuda_status() == 0
