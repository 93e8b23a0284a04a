"""CPU: the affine motion search restatement (orc_me_affine) against the reference's own
affine_me_gradient (src/inter.c:1339, reached by compiling src/inter.c into the checker library),
with analyze_affine_uni's start selection and analyze_affine_bi's org: every AMVR index, uni and
bi calls, 4x4 and 8x8 sub-blocks, CPMVs at the 18-bit limits, and blocks over flat and stripe
patches whose normal equations are singular (the solve's NaN path)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402


def _same(reqs, a, b):
    bad = [i for i in range(len(a)) if a[i].tobytes() != b[i].tobytes()]
    assert not bad, f"{len(bad)} of {len(a)} differ; first: {reqs[bad[0]]} oracle {a[bad[0]]} reference {b[bad[0]]}"


def test_affme_oracle_matches_reference(oracle, ref):
    for k in range(6):
        p = dict(w=(192, 160, 256)[k % 3], h=(128, 96, 128)[k % 3], vel=((2.5, -1.25), (-3, 2), (6, 4))[k % 3],
                 n=200, paint=k % 2)
        org, keep, addrs, stride, reqs = cases.affme_inputs(oracle, p, 6100 + k)
        _same(reqs, oracle.me_affine(p["w"], p["h"], org, p["w"], addrs, stride, reqs, threads=4),
              ref.me_affine(p["w"], p["h"], org, p["w"], addrs, stride, reqs))


def test_affme_oracle_rejects_out_of_domain(oracle):
    """requests outside the supported domain keep their start CPMVs and report cost UINT64_MAX"""
    p = cases.AFFME_CASES[0]
    org, keep, addrs, stride, reqs = cases.affme_inputs(oracle, p, 6200)
    reqs = reqs[:6].copy()
    reqs[0]["w"] = 8                          # below the affine CU size
    reqs[1]["x"] = p["w"] - 8                 # CU leaves the picture
    reqs[2]["mvr"] = 3                        # no such affine AMVR index
    reqs[3]["refi"] = reqs[3]["num_refp"]     # reference index past the list
    reqs[4]["mvp"][0][0] = 1 << 17            # CPMV beyond 18 bits
    reqs[5]["flags"] = 0
    reqs[5]["mv"][1][1] = -(1 << 17) - 1
    out = oracle.me_affine(p["w"], p["h"], org, p["w"], addrs, stride, reqs)
    assert (out["cost"] == np.iinfo(np.uint64).max).all()
    assert np.array_equal(out["mv"], reqs["mv"])
