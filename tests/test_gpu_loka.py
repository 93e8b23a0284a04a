"""GPU: the lookahead cost estimation (uavs3e_cuda_loka_*, loka_estimate_coding_cost
src/lookahead.c:82) bit-exact against the reference's golden digests and, record by record,
against the oracle restatement -- on the seeded small cases, at 1920x1080, and on the edges
(no reference, 4 + 4 references, the smallest picture, sizes that are not multiples of 16)."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import json  # noqa: E402

import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"] if c["kernel"] == "loka"]
THREADS = os.cpu_count() or 4


class GpuLoka:
    """cases.run_loka backend over uavs3e_cuda_loka_estimate (host buffers)"""

    def __init__(self, u):
        self.u = u

    def loka_estimate(self, cfg, org_y, i_org, org_u, org_v, i_org_c, ref_l0, ref_l1, i_ref, want_uv=True,
                      want_dqp=True):
        cfg = np.ascontiguousarray(cfg, dtype=self.u.LOKA_CFG).reshape(1)
        n = (int(cfg["width"][0]) // 16) * (int(cfg["height"][0]) // 16)
        a0 = (C.c_void_p * 4)(*(list(ref_l0) + [None] * (4 - len(ref_l0))))
        a1 = (C.c_void_p * 4)(*(list(ref_l1) + [None] * (4 - len(ref_l1))))
        cost, icost = C.c_double(), C.c_double()
        uv = (C.c_double * 2)()
        dqp = np.zeros(n, dtype=np.float32)
        self.u.check(self.u.lib().uavs3e_cuda_loka_estimate(
            cfg.ctypes.data, org_y.ctypes.data, i_org, org_u.ctypes.data, org_v.ctypes.data, i_org_c, a0, a1, i_ref,
            cases.LOKA_PAD, C.byref(cost), C.byref(icost), uv if want_uv else None,
            dqp.ctypes.data if want_dqp else None, None), "loka_estimate")
        return cost.value, icost.value, (uv[0], uv[1]) if want_uv else None, dqp if want_dqp else None


def _case_id(p):
    return f"{p['w']}x{p['h']}-pad{p['pad']}-sr{p['range']}-l0{len(p['l0'])}-l1{len(p['l1'])}"


def _run_both(gpu, oracle, p, seed, threads=1):
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, seed)
    a0, a1 = cases.loka_ref_addrs(refs, stride)
    W = p["w"]
    want = oracle.loka_units(cfg, y, W, u, v, W // 2, a0, a1, stride, threads)
    got = gpu.loka_estimate(cfg, y, u, v, refs[0], refs[1], cases.LOKA_PAD, units=True)
    return cfg, want, got


def _assert_records(want, got):
    for f in ("mv", "satd", "bi_satd", "zero_satd", "min_cost", "min_icost", "icost_u", "icost_v", "energy",
              "best_mode"):
        bad = np.nonzero(np.any((want[f] != got[f]).reshape(len(want), -1), axis=1))[0]
        assert len(bad) == 0, f"{f}: {len(bad)} units differ, first {bad[:5]}"
    assert want.view(np.uint8).tobytes() == got.view(np.uint8).tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[_case_id(c["params"]) for c in GOLDEN])
def test_loka_matches_reference_golden(gpu, case):
    assert cases.run_case(GpuLoka(gpu), case) == case["md5"]


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [11, 12])
@pytest.mark.parametrize("p", cases.LOKA_CASES, ids=[_case_id(p) for p in cases.LOKA_CASES])
def test_loka_records_match_oracle(gpu, oracle, p, seed):
    cfg, want, got = _run_both(gpu, oracle, p, seed)
    _assert_records(want, got["units"])
    cost, icost, uv, dqp = oracle.loka_finish(cfg, want)
    assert got["cost"] == cost and got["icost"] == icost and got["icost_uv"] == uv
    assert np.array_equal(got["map_dqp"], dqp)


@pytest.mark.gpu
@pytest.mark.parametrize("p", [
    dict(w=1920, h=1080, pad=1, range=384, gop=16, l0=[0, 4], l1=[16, 12], vel=(1.25, -0.5)),
    dict(w=1920, h=1080, pad=0, range=64, gop=4, l0=[7], l1=[], vel=(3.25, -1.5)),
], ids=["1080p-ra-bi-2+2", "1080p-scenecut"])
def test_loka_1080p_matches_oracle(gpu, oracle, p):
    cfg, want, got = _run_both(gpu, oracle, p, 2024, threads=THREADS)
    _assert_records(want, got["units"])
    cost, icost, uv, dqp = oracle.loka_finish(cfg, want)
    assert (got["cost"], got["icost"], got["icost_uv"]) == (cost, icost, uv)
    assert np.array_equal(got["map_dqp"], dqp)


@pytest.mark.gpu
def test_loka_device_entry_and_finish(gpu, oracle):
    import torch
    p = cases.LOKA_CASES[0]
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, 31)
    W, H = p["w"], p["h"]
    n = (W // 16) * (H // 16)
    a0, a1 = cases.loka_ref_addrs(refs, stride)
    want = oracle.loka_units(cfg, y, W, u, v, W // 2, a0, a1, stride)
    d_y, d_u, d_v = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (y, u, v))
    d_refs = [[torch.from_numpy(r).cuda() for r in lst] for lst in refs]
    off = cases.LOKA_PAD * stride + cases.LOKA_PAD
    d_units = torch.zeros(n * gpu.LOKA_UNIT.itemsize, dtype=torch.uint8, device="cuda")
    d_energy = torch.zeros(n, dtype=torch.int64, device="cuda")
    d_tot = torch.zeros(5, dtype=torch.int64, device="cuda")
    gpu.loka_units_device(cfg, d_y.data_ptr(), W, d_u.data_ptr(), d_v.data_ptr(), W // 2,
                          [t.data_ptr() + off for t in d_refs[0]], [t.data_ptr() + off for t in d_refs[1]], stride,
                          cases.LOKA_PAD, d_units.data_ptr(), d_energy.data_ptr(), d_tot.data_ptr())
    torch.cuda.synchronize()
    got = d_units.cpu().numpy().view(gpu.LOKA_UNIT)
    _assert_records(want, got)
    tot = d_tot.cpu().numpy().view(np.uint64)
    assert list(tot[:4]) == [int(want[f].astype(np.uint64).sum()) for f in ("min_cost", "min_icost", "icost_u",
                                                                            "icost_v")]
    assert tot[4] >= n * 4 * 50          # every search costs the first diamond at least
    energy = d_energy.cpu().numpy().view(np.uint64)
    assert np.array_equal(energy, want["energy"])
    assert gpu.loka_finish(cfg, tot, energy)[:3] == oracle.loka_finish(cfg, want)[:3]
    assert np.array_equal(gpu.loka_finish(cfg, tot, energy)[3], oracle.loka_finish(cfg, want)[3])


@pytest.mark.gpu
def test_loka_sc_ratio_matches_oracle(gpu, oracle):
    p = dict(w=320, h=192, pad=0, range=64, gop=4, l0=[7], l1=[], vel=(4.0, -2.5))
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, 8)
    a0, _ = cases.loka_ref_addrs(refs, stride)
    cost, icost, _, _ = oracle.loka_estimate(cfg, y, p["w"], u, v, p["w"] // 2, a0, [], stride)
    r = gpu.loka_sc_ratio(p["w"], p["h"], 0, 64, 4, 8, y, u, v, refs[0][0], 7, cases.LOKA_PAD)
    assert r == cost / icost


@pytest.mark.gpu
@pytest.mark.parametrize("p", [
    dict(w=128, h=96, pad=1, range=384, gop=16, l0=[], l1=[], vel=(1.0, 1.0)),
    dict(w=96, h=64, pad=1, range=384, gop=16, l0=[0, 2, 4, 6], l1=[16, 14, 12, 10], vel=(2.0, -1.0)),
    dict(w=18, h=18, pad=0, range=64, gop=4, l0=[7], l1=[], vel=(1.0, 0.0)),
    dict(w=18, h=34, pad=1, range=384, gop=16, l0=[0], l1=[16], vel=(0.5, 0.5)),
    dict(w=200, h=46, pad=1, range=64, gop=4, l0=[4, 5], l1=[], vel=(-7.0, 2.0)),
], ids=["intra-only", "4+4-refs", "18x18-scenecut", "18x34-bi", "200x46-ld"])
def test_loka_edges_match_oracle(gpu, oracle, p):
    for seed in (3, 4):
        cfg, want, got = _run_both(gpu, oracle, p, seed)
        _assert_records(want, got["units"])
        cost, icost, uv, dqp = oracle.loka_finish(cfg, want)
        assert (got["cost"], got["icost"], got["icost_uv"]) == (cost, icost, uv)


@pytest.mark.gpu
def test_loka_rejects_bad_arguments(gpu):
    p = cases.LOKA_CASES[0]
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, 1)
    bad = cfg.copy()
    bad["num_ref"][0, 0] = 5
    with pytest.raises(gpu.CudaError):
        gpu.loka_estimate(bad, y, u, v, refs[0], refs[1], cases.LOKA_PAD)
    with pytest.raises(gpu.CudaError):       # padded search with less than 144 samples of padding
        gpu.loka_estimate(cfg, y, u, v, refs[0], refs[1], 64)
    small = cfg.copy()
    small["width"] = 16
    with pytest.raises(gpu.CudaError):
        gpu.loka_estimate(small, y, u, v, refs[0], refs[1], cases.LOKA_PAD)
    assert gpu.lib().uavs3e_cuda_status() == 0
