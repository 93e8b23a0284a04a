"""GPU: the affine control-point MVP (uavs3e_cuda_affine_mvp*, com_get_affine_mvp_scaling
src/com_util.c:1983-2058) bit-exact against the reference's golden digests and the oracle."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
          if c["kernel"] == "affmvp"]


class GpuAffMvp:
    def __init__(self, u):
        self.u = u

    def affine_mvp(self, ptr_cur, ref_ptr, map_mv, map_refi, i_scu, reqs):
        return self.u.affine_mvp(ptr_cur, ref_ptr, map_mv, map_refi, i_scu, reqs)


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"seed{c['seed']}")
def test_affmvp_golden_gpu(gpu, case):
    assert cases.run_case(GpuAffMvp(gpu), case) == case["md5"]


@pytest.mark.parametrize("seed", [11, 12, 13, 14])
def test_affmvp_matches_oracle_gpu(gpu, oracle, seed):
    p = dict(w=120, h=68, nref=2 + seed % 3, n=20000, big=seed % 2)
    ptr_cur, ref_ptr, mv, refi, i_scu, reqs = cases.affmvp_inputs(p, seed)
    want, bad = oracle.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    assert bad == 0
    got = gpu.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    assert np.array_equal(got, want)


def test_affmvp_device_entry_and_domain(gpu, oracle):
    """the device entry gives the host entry's results; requests outside the domain are counted in
    d_err with zero predictors and make the host entry fail"""
    import torch
    p = dict(w=64, h=40, nref=3, n=3000, big=1)
    ptr_cur, ref_ptr, mv, refi, i_scu, reqs = cases.affmvp_inputs(p, 31)
    reqs[5]["cur_refi"] = 3
    reqs[9]["mvr"] = 3
    reqs[17]["scup"] = -3 * i_scu
    want, bad = oracle.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    assert bad == 3
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()  # noqa: E731
    d_ref, d_mv, d_refi, d_req = d(ref_ptr), d(mv), d(refi), d(reqs)
    d_out = torch.zeros(len(reqs) * 16, dtype=torch.uint8, device="cuda")
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.affine_mvp_device(ptr_cur, d_ref.data_ptr(), len(ref_ptr), d_mv.data_ptr(), d_refi.data_ptr(), i_scu,
                          len(refi) // i_scu, d_req.data_ptr(), len(reqs), d_out.data_ptr(), d_err.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy().view(gpu.AFFMVP_OUT)
    assert int(d_err.item()) == 3
    assert np.array_equal(got, want)
    with pytest.raises(RuntimeError):
        gpu.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
