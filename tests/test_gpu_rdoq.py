"""GPU: RDOQ of transform blocks (uavs3e_cuda_rdoq*, quant_non_zero / rdoq_quant_block
src/quant.c:196-383) bit-exact against the reference's golden digests and the oracle: every TB
shape 4x4..64x64, steps 10..60, intra / inter, luma / chroma, several estimate sets."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"] if c["kernel"] == "rdoq"]
WQ_GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"] if c["kernel"] == "quant_wq"]


class GpuRdoq:
    def __init__(self, u):
        self.u = u

    def trans_dct2(self, lw, lh, src, dst, bd=8):
        raise NotImplementedError

    def rdoq(self, reqs, ests, coefs):
        return self.u.rdoq(reqs, ests, coefs)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[f"n{c['params']['n']}-k{c['params']['k']}" for c in GOLDEN])
def test_rdoq_matches_reference_golden(gpu, oracle, case):
    reqs, ests, coefs = cases.rdoq_inputs(oracle, case["params"], case["seed"])
    nz = gpu.rdoq(reqs, ests, coefs)
    assert cases.digest(coefs, nz) == case["md5"]


@pytest.mark.gpu
def test_rdoq_matches_oracle_many_seeds(gpu, oracle):
    for seed in range(900, 930):
        reqs, ests, coefs = cases.rdoq_inputs(oracle, dict(n=300, k=3), seed)
        want_c, got_c = coefs.copy(), coefs.copy()
        want = oracle.rdoq(reqs, ests, want_c)
        got = gpu.rdoq(reqs, ests, got_c)
        bad = np.nonzero(want != got)[0]
        assert len(bad) == 0, f"seed {seed}: num_nz differs for blocks {bad[:5]}"
        assert np.array_equal(want_c, got_c), f"seed {seed}: levels differ"


@pytest.mark.gpu
def test_rdoq_device_entry(gpu, oracle):
    import torch
    reqs, ests, coefs = cases.rdoq_inputs(oracle, dict(n=400, k=2), 31)
    want_c = coefs.copy()
    want = oracle.rdoq(reqs, ests, want_c)
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_est = torch.from_numpy(ests.view(np.uint8).copy()).cuda()
    d_coef = torch.from_numpy(coefs.copy()).cuda()
    d_nz = torch.zeros(len(reqs), dtype=torch.int32, device="cuda")
    gpu.rdoq_device(d_req.data_ptr(), len(reqs), d_est.data_ptr(), len(ests), d_coef.data_ptr(), coefs.size,
                    d_nz.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d_nz.cpu().numpy(), want)
    assert np.array_equal(d_coef.cpu().numpy(), want_c)


@pytest.mark.gpu
def test_rdoq_skips_requests_outside_the_domain(gpu, oracle):
    reqs, ests, coefs = cases.rdoq_inputs(oracle, dict(n=6, k=1), 3)
    bad = reqs.copy()
    bad[0]["log2w"] = 7                         # block size
    bad[1]["est"] = 5                           # unknown estimate set
    bad[2]["coef_offset"] = coefs.size          # past the buffer
    got_c = coefs.copy()
    nz = gpu.rdoq(bad, ests, got_c)
    assert list(nz[:3]) == [-1, -1, -1]
    want_c = coefs.copy()
    want = oracle.rdoq(reqs[3:], ests, want_c)
    assert np.array_equal(nz[3:], want)
    for i in range(3):                          # skipped blocks keep their coefficients
        o, n = int(reqs[i]["coef_offset"]), (1 << int(reqs[i]["log2w"])) * (1 << int(reqs[i]["log2h"]))
        assert np.array_equal(got_c[o:o + n], coefs[o:o + n])
    assert gpu.lib().uavs3e_cuda_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("case", WQ_GOLDEN, ids=[str(c["params"]["n"]) for c in WQ_GOLDEN])
def test_quant_wq_matches_reference_golden(gpu, oracle, case):
    """quant_non_zero's weighted branch (pic_wq_enable) against the reference's digests"""
    reqs, _, coefs = cases.rdoq_inputs(oracle, dict(case["params"], k=1), case["seed"])
    wq4, wq8 = cases.wq_matrices(np.random.default_rng(case["seed"] + 1))
    nz = gpu.quant_wq(reqs, wq4, wq8, coefs)
    assert cases.digest(nz, coefs) == case["md5"]


@pytest.mark.gpu
def test_quant_wq_matches_oracle_many_blocks(gpu, oracle):
    reqs, _, coefs = cases.rdoq_inputs(oracle, dict(n=4000, k=1), 8400)
    wq4, wq8 = cases.wq_matrices(np.random.default_rng(8401))
    a, b = coefs.copy(), coefs.copy()
    assert np.array_equal(gpu.quant_wq(reqs, wq4, wq8, a), oracle.quant_wq(reqs, wq4, wq8, b))
    assert np.array_equal(a, b)
