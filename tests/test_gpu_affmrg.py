"""GPU: the affine merge candidates (uavs3e_cuda_affine_merge*, com_get_affine_merge_candidate
src/com_util.c:1761-1981) bit-exact against the reference's golden digests and the oracle."""
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
          if c["kernel"] == "affmrg"]


class GpuAffMrg:
    def __init__(self, u):
        self.u = u

    def affine_merge(self, *args):
        return self.u.affine_merge(*args)


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['params']['slice']}-seed{c['seed']}")
def test_affmrg_golden_gpu(gpu, case):
    assert cases.run_case(GpuAffMrg(gpu), case) == case["md5"]


@pytest.mark.parametrize("slice_type,seed", [("B", 11), ("P", 12)])
def test_affmrg_1080p_matches_oracle_gpu(gpu, oracle, slice_type, seed):
    # a 1920x1080 picture's maps (480 x 270 SCUs) and 30,000 requests of all affine CU sizes
    p = dict(w=480, h=270, nref=3, slice=slice_type, n=30000)
    args = cases.affmrg_inputs(p, seed)
    want, bad = oracle.affine_merge(*args)
    assert bad == 0
    got = gpu.affine_merge(*args)
    assert got.tobytes() == want.tobytes()


def test_affmrg_device_entry_and_domain(gpu, oracle):
    """the device entry gives the oracle's results; requests outside the domain are counted in
    d_err with zero results and make the host entry fail"""
    import torch
    p = dict(w=64, h=40, nref=2, slice="B", n=2000)
    pic, mv, refi, scu, pos, cmv, crefi, reqs = cases.affmrg_inputs(p, 31)
    i_scu = int(pic["i_scu"][0])
    reqs[5]["cu_width"] = 8
    reqs[9]["scup"] = -3 * i_scu
    want, bad = oracle.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, reqs)
    assert bad == 2
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()  # noqa: E731
    dm = [d(a) for a in (mv, refi, scu, pos, cmv, crefi, reqs)]
    d_out = torch.full((len(reqs) * gpu.AFFMRG_OUT.itemsize,), 255, dtype=torch.uint8, device="cuda")
    d_err = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.affine_merge_device(pic, *[a.data_ptr() for a in dm], len(reqs), d_out.data_ptr(), d_err.data_ptr(),
                            torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(d_err.item()) == 2
    assert d_out.cpu().numpy().tobytes() == want.tobytes()
    with pytest.raises(gpu.CudaError):
        gpu.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, reqs)
