"""Oracle: the affine merge candidates (com_get_affine_merge_candidate, src/com_util.c:1761-1981)
against the reference's own function on seeded coded-CU maps, and the oracle's domain checks."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = [c for c in json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
          if c["kernel"] == "affmrg"]


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['params']['slice']}-seed{c['seed']}")
def test_affmrg_golden(oracle, case):
    assert cases.run_case(oracle, case) == case["md5"]


@pytest.mark.parametrize("slice_type,seed", [("B", 1), ("B", 2), ("P", 3), ("P", 4)])
def test_affmrg_matches_reference(oracle, ref, slice_type, seed):
    p = dict(w=56, h=40, nref=3, slice=slice_type, n=500)
    args = cases.affmrg_inputs(p, 600 + seed)
    got, bad = oracle.affine_merge(*args)
    assert bad == 0
    want = ref.affine_merge(*args)
    assert got.tobytes() == want.tobytes()
    # the cases reach every list length and both control-point counts
    assert set(np.unique(got["num"])) >= {0, 1, 2, 3}
    assert (got["cp_num"] == 3).any() and (got["cp_num"] == 2).any()


def test_affmrg_ctu_row_boundary(oracle, ref):
    """CUs on a CTU row boundary whose affine neighbours above end there take the 4-parameter
    model from the neighbours' bottom corners"""
    p = dict(w=48, h=48, nref=2, slice="B", n=300)
    pic, mv, refi, scu, pos, cmv, crefi, reqs = cases.affmrg_inputs(p, 41)
    i_scu = int(pic["i_scu"][0])
    xs = np.random.default_rng(5).integers(0, 40, len(reqs))
    reqs["scup"] = 16 * i_scu + (xs & ~3)      # y = 64 luma samples: the second CTU row
    got, bad = oracle.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, reqs)
    assert bad == 0
    assert got.tobytes() == ref.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, reqs).tobytes()


def test_affmrg_domain(oracle):
    """requests outside the domain are counted and get zero results; the others are unchanged"""
    p = dict(w=32, h=24, nref=2, slice="B", n=60)
    pic, mv, refi, scu, pos, cmv, crefi, reqs = cases.affmrg_inputs(p, 77)
    good, bad = oracle.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, reqs)
    assert bad == 0
    i_scu = int(pic["i_scu"][0])
    r = reqs.copy()
    r[0]["cu_width"] = 24                      # not a power of two
    r[1]["cu_height"] = 8                      # below 16
    r[2]["scup"] = -3 * i_scu                  # neighbours above the field
    out, bad = oracle.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, r)
    assert bad == 3
    assert not out[:3].view(np.uint8).any()
    assert out[3:].tobytes() == good[3:].tobytes()
    c2 = crefi.copy()
    c2[c2 >= 0] = 20                           # colocated reference index past the list
    out, bad = oracle.affine_merge(pic, mv, refi, scu, pos, cmv, c2, reqs)
    zero = ~out.view(np.uint8).reshape(len(out), -1).any(1)
    assert 0 < bad == int(zero.sum())          # those whose colocated SCU has a reference
