"""CPU: the intra mode candidate restatement (orc_intra_rmd) against the reference's own
make_ipred_list (src/intra.c:226, reached by compiling src/intra.c into the checker library): fast
and full searches, skipped DC / planar / bilinear, MPM pairs (equal, IPCM, unsorted), 4:1 blocks,
LBAC states for the mode bits and inter-SATD cuts; the SATDs the restatement takes are the
reference's own com_intra_pred + calc_satd_intra."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402


def test_rmd_oracle_matches_reference(oracle, ref):
    import pyoracle
    for seed in range(5):
        reqs, nbs, orgs, avails, ipfs = cases.rmd_inputs(np.random.default_rng(7100 + seed), 200)
        want = np.zeros(len(reqs), dtype=pyoracle.RMD_OUT)
        satd = np.zeros((len(reqs), 33), np.uint32)
        for i in range(len(reqs)):
            want[i], satd[i] = ref.make_ipred_list(nbs[i], orgs[i].ctypes.data, int(reqs[i]["pb_w"]), avails[i],
                                                   ipfs[i], reqs[i])
        assert np.array_equal(cases.rmd_satd(oracle, reqs, nbs, orgs, avails, ipfs), satd)
        got = oracle.intra_rmd(satd, reqs)
        bad = [i for i in range(len(reqs)) if got[i].tobytes() != want[i].tobytes()]
        assert not bad, f"{len(bad)} differ; first {reqs[bad[0]]}: reference {want[bad[0]]} oracle {got[bad[0]]}"


def test_intra_dir_bits_follow_the_coder_state(oracle):
    """an MPM costs 2 bins, another mode 6; a state whose flag context strongly predicts 'MPM'
    makes the MPM cheaper than any other mode"""
    import ctypes as C
    ctx = np.array([(8 << 1) | 1] + [(512 << 1)] * 5 + [(8 << 1) | 1], dtype=np.int16)   # MPS 1, LPS tiny
    mpm = np.array([3, 20], dtype=np.uint8)
    f = oracle.L.orc_intra_dir_bits
    bits = [f(511, C.c_void_p(ctx.ctypes.data), m, C.c_void_p(mpm.ctypes.data)) for m in range(33)]
    assert bits[3] < min(b for m, b in enumerate(bits) if m not in (3, 20))
