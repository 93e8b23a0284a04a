"""GPU: intra mode candidates (uavs3e_cuda_intra_rmd*, make_ipred_list src/intra.c:226) bit-exact
against the reference's golden digests and the oracle restatement, alone and on the intra
lattice's own SATD records."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"] if c["kernel"] == "rmd"]


def _gpu_rmd_device(gpu, satd, reqs):
    import torch
    d_satd = torch.from_numpy(np.ascontiguousarray(satd, dtype=np.uint32).view(np.int32).reshape(-1).copy()).cuda()
    d_req = torch.from_numpy(np.ascontiguousarray(reqs).view(np.uint8).copy()).cuda()
    d_out = torch.zeros(max(1, len(reqs)) * gpu.RMD_OUT.itemsize, dtype=torch.uint8, device="cuda")
    gpu.intra_rmd_device(d_satd.data_ptr(), satd.size // 33, d_req.data_ptr(), len(reqs), d_out.data_ptr())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(gpu.RMD_OUT)[:len(reqs)]


def _assert_same(reqs, want, got):
    bad = [i for i in range(len(want)) if want[i].tobytes() != got[i].tobytes()]
    assert not bad, f"{len(bad)} of {len(want)} differ; first: req {reqs[bad[0]]} want {want[bad[0]]} got {got[bad[0]]}"


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[str(c["params"]["n"]) for c in GOLDEN])
def test_rmd_matches_reference_golden(gpu, oracle, case):
    reqs, nbs, orgs, avails, ipfs = cases.rmd_inputs(np.random.default_rng(case["seed"]), case["params"]["n"])
    satd = cases.rmd_satd(oracle, reqs, nbs, orgs, avails, ipfs)
    assert cases.digest(_gpu_rmd_device(gpu, satd, reqs).view(np.uint8)) == case["md5"]
    assert cases.digest(gpu.intra_rmd(satd, reqs).view(np.uint8)) == case["md5"]     # host entry


@pytest.mark.gpu
def test_rmd_matches_oracle_many_requests(gpu, oracle):
    """random SATD rows (ties included) and requests, 40,000 blocks"""
    rng = np.random.default_rng(88)
    n = 40000
    reqs, _, _, _, _ = cases.rmd_inputs(rng, 1)
    reqs = np.repeat(reqs, n)
    base, _, _, _, _ = cases.rmd_inputs(np.random.default_rng(89), n)
    for f in ("pb_w", "pb_h", "mpm", "skip_ipd", "fast", "range", "ctx", "sqrt_lambda", "inter_satd", "satd_threshold"):
        reqs[f] = base[f]
    reqs["satd_row"] = rng.integers(0, 5000, n)
    satd = rng.integers(0, 3000, (5000, 33)).astype(np.uint32)
    satd[::7] //= 64                      # coarse values: equal costs
    want = oracle.intra_rmd(satd, reqs)
    _assert_same(reqs, want, _gpu_rmd_device(gpu, satd, reqs))


@pytest.mark.gpu
def test_rmd_on_lattice_records(gpu, oracle):
    """the lattice's SATD records of a picture feed the candidate search directly"""
    from uavs3e_gb300.synth import intra_frame
    W, H = 256, 128
    org = intra_frame(W, H, seed=5)
    rec = intra_frame(W, H, seed=6)
    cus = gpu.lattice_cus(W, H)
    satd, _ = gpu.intra_lattice(org, rec, cus, [32], ipf=1)
    satd = np.asarray(satd, dtype=np.uint32).reshape(-1, 33)
    reqs, _, _, _, _ = cases.rmd_inputs(np.random.default_rng(90), len(cus))
    reqs["satd_row"] = np.arange(len(cus))
    reqs["pb_w"], reqs["pb_h"] = cus["w"], cus["h"]
    want = oracle.intra_rmd(satd, reqs)
    _assert_same(reqs, want, _gpu_rmd_device(gpu, satd, reqs))


@pytest.mark.gpu
def test_rmd_out_of_domain_requests(gpu, oracle):
    reqs, nbs, orgs, avails, ipfs = cases.rmd_inputs(np.random.default_rng(91), 12)
    satd = cases.rmd_satd(oracle, reqs, nbs, orgs, avails, ipfs)
    want = oracle.intra_rmd(satd, reqs)
    bad = reqs.copy()
    bad[0]["satd_row"] = 12               # past the array
    bad[1]["pb_w"] = 12                   # not a power of two
    bad[2]["mpm"][0] = 40                 # no such mode
    bad[3]["range"] = 200                 # not a coder range
    bad[4]["ctx"][2] = 3                  # zero LPS range
    bad[5]["sqrt_lambda"] = -1.0
    got = _gpu_rmd_device(gpu, satd, bad)
    assert (got["count"][:6] == 255).all() and (got["list"][:6] == -1).all()
    _assert_same(reqs[6:], want[6:], got[6:])


@pytest.mark.gpu
def test_intra_decision_pipeline(gpu, oracle):
    """SATD-only lattice -> candidate lists -> lattice over each CU's list: the SATD records equal
    the full lattice's, the lists the oracle's, and the list modes' records the full lattice's"""
    import ctypes as C

    import torch
    from uavs3e_gb300.synth import intra_frame
    W, H = 160, 96
    org = intra_frame(W, H, seed=11)
    rec = np.clip(org.astype(int) + np.random.default_rng(11).integers(-4, 5, org.shape), 0, 255).astype(np.uint8)
    cus = gpu.lattice_cus(W, H)
    n = len(cus)
    qps = [27, 37]
    satd_all, q_all = gpu.intra_lattice(org, rec, cus, qps, ipf=1)
    L = gpu.lib()
    P, I = C.c_void_p, C.c_int
    L.uavs3e_cuda_intra_lattice_modes_device.argtypes = [P, I, P, I, I, I, P, I, P, I, I, P, I, I, P, P, P]
    d_org = torch.from_numpy(org).cuda()
    d_rec = torch.from_numpy(rec).cuda()
    d_cus = torch.from_numpy(cus.view(np.uint8).copy()).cuda()
    d_satd = torch.zeros(n * 33, dtype=torch.int32, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    assert L.uavs3e_cuda_intra_lattice_modes_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(),
                                                    n, None, 33, 1, None, 0, 1, d_satd.data_ptr(), None, sp) == 0
    torch.cuda.synchronize()
    satd0 = d_satd.cpu().numpy().view(np.uint32).reshape(n, 33)
    assert np.array_equal(satd0, satd_all.reshape(n, 33).view(np.uint32))
    reqs, _, _, _, _ = cases.rmd_inputs(np.random.default_rng(12), n)
    reqs["satd_row"] = np.arange(n)
    reqs["pb_w"], reqs["pb_h"] = cus["w"], cus["h"]
    reqs["inter_satd"] = np.iinfo(np.uint64).max
    lists = gpu.intra_rmd(satd0, reqs)
    assert lists.tobytes() == oracle.intra_rmd(satd0, reqs).tobytes()
    modes = lists["list"].astype(np.int16).copy()
    for k in range(1, 5):
        modes[:, k] = np.where(modes[:, k] < 0, modes[:, 0], modes[:, k])
    modes = modes.astype(np.uint8)
    d_modes = torch.from_numpy(modes.copy()).cuda()
    d_satd5 = torch.full((n * 33,), -1, dtype=torch.int32, device="cuda")
    d_q5 = torch.zeros(n * 33 * len(qps) * gpu.LAT_Q.itemsize, dtype=torch.uint8, device="cuda")
    q = np.array(qps, np.int32)
    assert L.uavs3e_cuda_intra_lattice_modes_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(),
                                                    n, d_modes.data_ptr(), 5, 1, q.ctypes.data, len(qps), 1,
                                                    d_satd5.data_ptr(), d_q5.data_ptr(), sp) == 0
    torch.cuda.synchronize()
    q5 = d_q5.cpu().numpy().view(gpu.LAT_Q).reshape(n, 33, len(qps))
    sel = np.zeros((n, 33), bool)
    np.put_along_axis(sel, modes.astype(int), True, 1)
    assert np.array_equal(q5[sel], q_all.reshape(n, 33, len(qps))[sel])


@pytest.mark.gpu
def test_intra_decision_frame_is_one_graph(gpu):
    """the intra decision of a frame in the encoder's order -- SATD lattice, candidate lists,
    gather of each CU's listed modes, lattice over the lists -- captured once into a CUDA graph:
    replays on new frame content give the plain launches' records"""
    import ctypes as C

    import torch
    from uavs3e_gb300.synth import intra_frame
    W, H = 192, 128
    cus = gpu.lattice_cus(W, H)
    n = len(cus)
    L = gpu.lib()
    P, I = C.c_void_p, C.c_int
    L.uavs3e_cuda_intra_lattice_modes_device.argtypes = [P, I, P, I, I, I, P, I, P, I, I, P, I, I, P, P, P]
    reqs, _, _, _, _ = cases.rmd_inputs(np.random.default_rng(13), n)
    reqs["satd_row"] = np.arange(n)
    reqs["pb_w"], reqs["pb_h"] = cus["w"], cus["h"]
    reqs["inter_satd"] = np.iinfo(np.uint64).max
    d_req = torch.from_numpy(reqs.view(np.uint8).copy()).cuda()
    d_org = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    d_rec = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    d_cus = torch.from_numpy(cus.view(np.uint8).copy()).cuda()
    d_satd = torch.zeros(n * 33, dtype=torch.int32, device="cuda")
    d_lists = torch.zeros(n * gpu.RMD_OUT.itemsize, dtype=torch.uint8, device="cuda")
    d_satd5 = torch.zeros(n * 33, dtype=torch.int32, device="cuda")
    qps = np.array([27, 37], np.int32)
    d_q5 = torch.zeros(n * 33 * len(qps) * gpu.LAT_Q.itemsize, dtype=torch.uint8, device="cuda")

    def frame(seed):
        org = intra_frame(W, H, seed=seed)
        rec = np.clip(org.astype(int) + np.random.default_rng(seed).integers(-4, 5, org.shape), 0, 255)
        d_org.copy_(torch.from_numpy(org))
        d_rec.copy_(torch.from_numpy(rec.astype(np.uint8)))

    def run():
        sp = torch.cuda.current_stream().cuda_stream
        assert L.uavs3e_cuda_intra_lattice_modes_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H,
                                                        d_cus.data_ptr(), n, None, 33, 1, None, 0, 1,
                                                        d_satd.data_ptr(), None, sp) == 0
        gpu.intra_rmd_device(d_satd.data_ptr(), n, d_req.data_ptr(), n, d_lists.data_ptr(), sp)
        lists = d_lists.view(torch.int8).view(n, gpu.RMD_OUT.itemsize)[:, :5].to(torch.int16)
        modes = torch.where(lists < 0, lists[:, :1], lists).to(torch.uint8).contiguous()
        assert L.uavs3e_cuda_intra_lattice_modes_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H,
                                                        d_cus.data_ptr(), n, modes.data_ptr(), 5, 1, qps.ctypes.data,
                                                        len(qps), 1, d_satd5.data_ptr(), d_q5.data_ptr(), sp) == 0

    want = {}
    for seed in (41, 42):
        frame(seed)
        d_lists.zero_()
        d_q5.zero_()  # records of modes off a CU's list are left untouched
        run()
        torch.cuda.synchronize()
        want[seed] = (d_lists.clone(), d_q5.clone())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        run()
    for seed in (41, 42, 41):
        frame(seed)
        d_lists.zero_()
        d_q5.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(d_lists, want[seed][0]) and torch.equal(d_q5, want[seed][1]), seed
