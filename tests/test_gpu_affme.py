"""GPU: batched affine motion search (uavs3e_cuda_me_affine*, affine_me_gradient src/inter.c:1339)
bit-exact against the reference's golden digests and the oracle restatement: AMVR indices 0..2,
uni calls with analyze_affine_uni's start selection, bi calls with analyze_affine_bi's org, 4x4 and
8x8 sub-blocks, singular normal equations, 18-bit CPMV limits, the session entry and a 1080p
frame's batch."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"] if c["kernel"] == "affme"]
THREADS = os.cpu_count() or 4


def _id(p):
    return f"{p['w']}x{p['h']}-paint{p.get('paint', 0)}"


def _gpu_affme(gpu, W, H, org, keep, stride, reqs):
    import torch
    d_planes = [torch.from_numpy(a).cuda() for a in keep]
    base = cases.TZ_PAD * stride + cases.TZ_PAD
    d_org = torch.from_numpy(np.ascontiguousarray(org)).cuda()
    d_req = torch.from_numpy(np.ascontiguousarray(reqs).view(np.uint8).copy()).cuda()
    d_out = torch.zeros(max(1, len(reqs)) * gpu.AFFME_OUT.itemsize, dtype=torch.uint8, device="cuda")
    gpu.me_affine_device(W, H, d_org.data_ptr(), org.shape[1], [t.data_ptr() + base for t in d_planes], stride,
                         cases.TZ_PAD, d_req.data_ptr(), len(reqs), d_out.data_ptr())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(gpu.AFFME_OUT)[:len(reqs)]


def _assert_same(reqs, want, got):
    bad = [i for i in range(len(want)) if want[i].tobytes() != got[i].tobytes()]
    assert not bad, f"{len(bad)} of {len(want)} differ; first: req {reqs[bad[0]]} want {want[bad[0]]} got {got[bad[0]]}"


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[_id(c["params"]) for c in GOLDEN])
def test_affme_matches_reference_golden(gpu, oracle, case):
    p = case["params"]
    org, keep, addrs, stride, reqs = cases.affme_inputs(oracle, p, case["seed"])
    got = _gpu_affme(gpu, p["w"], p["h"], org, keep, stride, reqs)
    assert cases.digest(got.view(np.uint8)) == case["md5"]


@pytest.mark.gpu
@pytest.mark.parametrize("p", cases.AFFME_CASES, ids=[_id(p) for p in cases.AFFME_CASES])
def test_affme_matches_oracle_many_seeds(gpu, oracle, p):
    for seed in range(700, 712):
        q = dict(p, n=256)
        org, keep, addrs, stride, reqs = cases.affme_inputs(oracle, q, seed)
        want = oracle.me_affine(q["w"], q["h"], org, q["w"], addrs, stride, reqs, THREADS)
        _assert_same(reqs, want, _gpu_affme(gpu, q["w"], q["h"], org, keep, stride, reqs))


@pytest.mark.gpu
def test_affme_out_of_domain_requests(gpu, oracle):
    """requests outside the supported domain return cost UINT64_MAX and their start CPMVs, and
    do not disturb the others"""
    p = cases.AFFME_CASES[0]
    org, keep, addrs, stride, reqs = cases.affme_inputs(oracle, dict(p, n=40), 6300)
    reqs[0]["w"] = 8
    reqs[1]["x"] = p["w"] - 8
    reqs[2]["mvr"] = 3
    reqs[3]["refi"] = reqs[3]["num_refp"]
    reqs[4]["mvp"][0][0] = 1 << 17
    reqs[5]["flags"] = 0
    reqs[5]["mv"][1][1] = -(1 << 17) - 1
    want = oracle.me_affine(p["w"], p["h"], org, p["w"], addrs, stride, reqs)
    got = _gpu_affme(gpu, p["w"], p["h"], org, keep, stride, reqs)
    assert (got["cost"][:6] == np.iinfo(np.uint64).max).all()
    _assert_same(reqs, want, got)


@pytest.mark.gpu
def test_affme_session_entry(gpu, oracle):
    """the host-buffer entry on a motion-search session's references"""
    p = cases.AFFME_CASES[1]
    rng = np.random.default_rng(78)
    W, H = p["w"], p["h"]
    frames = cases.loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    cases.affme_paint(rng, frames, W, H)
    keep, addrs, stride = cases.tz_planes(oracle, frames, [4, 0], W, H)
    reqs = cases.affme_requests(rng, W, H, 300, 2)
    want = oracle.me_affine(W, H, frames[8][0], W, addrs, stride, reqs, THREADS)
    ms = gpu.MotionSearch(W, H, n_refs=2, search_range=64, pad=144)
    ms.set_ref(0, frames[4][0])
    ms.set_ref(1, frames[0][0])
    got = ms.affine(frames[8][0], reqs)
    ms.close()
    _assert_same(reqs, want, got)


@pytest.mark.gpu
def test_affme_1080p_batch(gpu, oracle):
    """a frame's worth of calls on the synthetic 1080p sequence"""
    from uavs3e_gb300.synth import motion_sequence
    W, H = 1920, 1080
    seq = motion_sequence(W, H, 3, seed=10)
    frames = {t: (seq[t],) for t in range(3)}
    keep, addrs, stride = cases.tz_planes(oracle, frames, [1, 0], W, H)
    reqs = cases.affme_requests(np.random.default_rng(1081), W, H, 3000, 2)
    want = oracle.me_affine(W, H, seq[2], W, addrs, stride, reqs, THREADS)
    _assert_same(reqs, want, _gpu_affme(gpu, W, H, seq[2], keep, stride, reqs))


@pytest.mark.gpu
def test_affme_rejects_bad_arguments(gpu):
    import torch
    d = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
    base = d.data_ptr() + 144 * 512 + 144
    with pytest.raises(gpu.CudaError):     # padding below 144
        gpu.me_affine_device(64, 64, base, 64, [base] * 16, 512, 64, d.data_ptr(), 1, d.data_ptr())
    with pytest.raises(gpu.CudaError):     # more than 8 reference slots
        gpu.me_affine_device(64, 64, base, 64, [base] * 16 * 9, 512, 144, d.data_ptr(), 1, d.data_ptr())
    assert gpu.lib().uavs3e_cuda_status() == 0
