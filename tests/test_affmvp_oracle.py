"""Oracle: the affine control-point MVP (com_get_affine_mvp_scaling, src/com_util.c:1983-2058)
against the reference's own function on seeded motion fields, and the oracle's domain checks."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
          if c["kernel"] == "affmvp"]


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"seed{c['seed']}")
def test_affmvp_golden(oracle, case):
    assert cases.run_case(oracle, case) == case["md5"]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_affmvp_matches_reference(oracle, ref, seed):
    p = dict(w=40, h=24, nref=3 + seed % 2, n=400, big=seed % 2)
    ptr_cur, ref_ptr, mv, refi, i_scu, reqs = cases.affmvp_inputs(p, 500 + seed)
    got, bad = oracle.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    assert bad == 0
    want = ref.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    assert np.array_equal(got, want)


def test_affmvp_domain(oracle):
    """requests outside the domain are counted and get zero predictors; the others are unchanged"""
    p = dict(w=16, h=8, nref=2, n=40)
    ptr_cur, ref_ptr, mv, refi, i_scu, reqs = cases.affmvp_inputs(p, 77)
    good, bad = oracle.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    assert bad == 0
    r = reqs.copy()
    r[0]["cur_refi"] = 2                      # >= n_ref
    r[1]["mvr"] = 3
    r[2]["lidx"] = 2
    r[3]["scup"] = -2 * i_scu                 # neighbours above the field
    out, bad = oracle.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, r)
    assert bad == 4
    assert not out["mvp"][:4].any()
    assert np.array_equal(out[4:], good[4:])
    rp = ref_ptr.copy()
    rp[:, :] = ptr_cur                        # zero POC distance
    out, bad = oracle.affine_mvp(ptr_cur, rp, mv, refi, i_scu, reqs)
    assert bad == len(reqs)
