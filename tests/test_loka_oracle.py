"""CPU: the lookahead estimate's restatement (oracle/oracle.c, orc_loka_*) unit by unit against
the reference's own me_search_tz (src/me.c:529) run with the estimate's settings, and its
picture-level outputs against loka_estimate_coding_cost itself (both through oracle/_ref)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402


def _case_id(p):
    return f"{p['w']}x{p['h']}-pad{p['pad']}-sr{p['range']}-l0{len(p['l0'])}-l1{len(p['l1'])}"


@pytest.mark.parametrize("p", cases.LOKA_CASES, ids=[_case_id(p) for p in cases.LOKA_CASES])
def test_loka_search_mv_per_unit_matches_reference(oracle, ref, p):
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, 4242)
    a0, a1 = cases.loka_ref_addrs(refs, stride)
    W = p["w"]
    units = oracle.loka_units(cfg, y, W, u, v, W // 2, a0, a1, stride)
    nux = W // 16
    moved = 0
    for li, (lst, addrs) in enumerate(((p["l0"], a0), (p["l1"], a1))):
        for r, (t, a) in enumerate(zip(lst, addrs)):
            for i in range(len(units)):
                mx, my, _ = ref.loka_search(cfg, y, W, a, stride, t, r, len(lst), (i % nux) * 16, (i // nux) * 16)
                assert (mx, my) == tuple(units[i]["mv"][li, r]), (li, r, i)
                moved += max(abs(mx), abs(my)) > 8
    # the cases move far enough for the raster stage to run on most searches
    assert moved > 0


def test_loka_intra_only_picture(oracle, ref):
    """no reference in either list: the picture cost is the intra cost"""
    p = dict(cases.LOKA_CASES[0], l0=[], l1=[], uv=True, dqp=True)
    got = cases.run_loka(oracle, p, 5151)
    assert got == cases.run_loka(ref, p, 5151)
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, 5151)
    units = oracle.loka_units(cfg, y, p["w"], u, v, p["w"] // 2, [], [], stride)
    assert np.array_equal(units["min_cost"], units["min_icost"])


def test_loka_planted_mistake_is_seen(oracle, ref):
    """a one-unit change of the records changes the digest the reference is compared on"""
    p = cases.LOKA_CASES[1]
    cfg, (y, u, v), refs, stride = cases.loka_inputs(p, 99)
    a0, a1 = cases.loka_ref_addrs(refs, stride)
    W = p["w"]
    units = oracle.loka_units(cfg, y, W, u, v, W // 2, a0, a1, stride)
    good = oracle.loka_finish(cfg, units)
    want = ref.loka_estimate(cfg, y, W, u, v, W // 2, a0, a1, stride)
    assert good[0] == want[0] and good[1] == want[1] and good[2] == want[2]
    assert np.array_equal(good[3], want[3])
    units["min_cost"][3] += 1
    bad = oracle.loka_finish(cfg, units)
    assert bad[0] != want[0]
