"""GPU: coefficient rate (uavs3e_cuda_coef_rate*, lbac_enc_run_length_cc_rdo src/entropy.c:1688)
bit-exact against the reference's golden digests and the oracle restatement, alone and on the
levels the GPU RDOQ leaves."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
          if c["kernel"] == "coef_rate"]


def _gpu_rate_device(gpu, levels, reqs):
    import torch
    d_lev = torch.from_numpy(np.ascontiguousarray(levels, dtype=np.int16).copy()).cuda()
    d_req = torch.from_numpy(np.ascontiguousarray(reqs).view(np.uint8).copy()).cuda()
    d_out = torch.zeros(max(1, len(reqs)) * gpu.COEF_RATE_OUT.itemsize, dtype=torch.uint8, device="cuda")
    gpu.coef_rate_device(d_req.data_ptr(), len(reqs), d_lev.data_ptr(), levels.size, d_out.data_ptr())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(gpu.COEF_RATE_OUT)[:len(reqs)]


def _assert_same(reqs, want, got):
    bad = [i for i in range(len(want)) if want[i].tobytes() != got[i].tobytes()]
    assert not bad, f"{len(bad)} of {len(want)} differ; first: req {reqs[bad[0]]} want {want[bad[0]]} got {got[bad[0]]}"


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[str(c["params"]["n"]) for c in GOLDEN])
def test_coef_rate_matches_reference_golden(gpu, case):
    levels, reqs = cases.coef_rate_inputs(np.random.default_rng(case["seed"]), case["params"]["n"])
    assert cases.digest(_gpu_rate_device(gpu, levels, reqs).view(np.uint8)) == case["md5"]
    assert cases.digest(gpu.coef_rate(levels, reqs).view(np.uint8)) == case["md5"]     # host entry


@pytest.mark.gpu
def test_coef_rate_matches_oracle_many_seeds(gpu, oracle):
    for seed in range(500, 506):
        levels, reqs = cases.coef_rate_inputs(np.random.default_rng(seed), 1500)
        _assert_same(reqs, oracle.coef_rate(levels, reqs), _gpu_rate_device(gpu, levels, reqs))


@pytest.mark.gpu
def test_coef_rate_of_gpu_rdoq_levels(gpu, oracle):
    """RDOQ then rate on the GPU, as an RDO pipeline would chain them"""
    reqs, ests, coefs = cases.rdoq_inputs(oracle, dict(n=2000, k=3), 7500)
    levels = coefs.copy()
    nz = gpu.rdoq(reqs, ests, levels)
    rng = np.random.default_rng(7501)
    sel = np.nonzero(nz > 0)[0]
    r = np.zeros(len(sel), dtype=gpu.COEF_RATE_REQ)
    r["coef_offset"] = reqs["coef_offset"][sel]
    r["log2w"], r["log2h"] = reqs["log2w"][sel], reqs["log2h"][sel]
    r["ch_type"] = (reqs["ch_type"][sel] != 0).astype(np.uint8)
    r["num_sig"] = nz[sel]
    r["range"] = rng.integers(256, 512, len(r))
    for f, k in (("run", 12), ("run_rdoq", 12), ("level", 12), ("last1", 6), ("last2", 12)):
        r[f] = cases.coef_models(rng, k * len(r)).reshape(len(r), k)
    _assert_same(r, oracle.coef_rate(levels, r), _gpu_rate_device(gpu, levels, r))


@pytest.mark.gpu
def test_coef_rate_out_of_domain_requests(gpu, oracle):
    levels, reqs = cases.coef_rate_inputs(np.random.default_rng(92), 12)
    want = oracle.coef_rate(levels, reqs)
    bad = reqs.copy()
    bad[0]["num_sig"] = bad[0]["num_sig"] + 1          # more levels than the block holds
    bad[1]["coef_offset"] = levels.size               # past the array
    bad[2]["log2w"] = 7
    bad[3]["range"] = 100
    bad[4]["level"][3] = 2                             # zero LPS range
    bad[5]["ch_type"] = 1
    bad[5]["log2w"] = 6                                # chroma block of 64 columns
    got = _gpu_rate_device(gpu, levels, bad)
    assert (got["bits"][:6] == np.iinfo(np.uint32).max).all()
    assert np.array_equal(got["run"][:6], bad["run"][:6]) and np.array_equal(got["range"][:6], bad["range"][:6])
    _assert_same(reqs[6:], want[6:], got[6:])
