"""CPU: the coefficient rate restatement (orc_coef_rate) against the reference's own
lbac_enc_run_length_cc_rdo (src/entropy.c:1688), and the computed context-model update against
every entry of the reference's transition table (tbl_plps / tbl_plps_ext)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402


def test_model_update_rule_equals_the_reference_table(oracle, ref):
    bad = [(m, b) for m in range(8192) for b in (0, 1) if oracle.lbac_next(m, b) != ref.lbac_next(m, b)]
    assert not bad, bad[:4]


def test_coef_rate_oracle_matches_reference(oracle, ref):
    for seed in range(4):
        levels, reqs = cases.coef_rate_inputs(np.random.default_rng(7300 + seed), 250)
        a, b = oracle.coef_rate(levels, reqs), ref.coef_rate(levels, reqs)
        bad = [i for i in range(len(a)) if a[i].tobytes() != b[i].tobytes()]
        assert not bad, f"{len(bad)} differ; first {reqs[bad[0]]}: oracle {a[bad[0]]} reference {b[bad[0]]}"


def test_coef_rate_follows_rdoq_levels(oracle, ref):
    """the levels RDOQ leaves (the reference's quant_non_zero) coded from fresh coder states"""
    import pyoracle
    reqs, ests, coefs = cases.rdoq_inputs(oracle, dict(n=150, k=2), 7400)
    nz = ref.rdoq(reqs, ests, coefs)
    rng = np.random.default_rng(7401)
    sel = np.nonzero(nz > 0)[0]
    r = np.zeros(len(sel), dtype=pyoracle.COEF_RATE_REQ)
    r["coef_offset"] = reqs["coef_offset"][sel]
    r["log2w"], r["log2h"] = reqs["log2w"][sel], reqs["log2h"][sel]
    r["ch_type"] = (reqs["ch_type"][sel] != 0).astype(np.uint8)
    keep = (r["ch_type"] == 0) | ((r["log2w"] <= 5) & (r["log2h"] <= 5))
    r, sel = r[keep], sel[keep]
    r["num_sig"] = nz[sel]
    r["range"] = rng.integers(256, 512, len(r))
    for f, k in (("run", 12), ("run_rdoq", 12), ("level", 12), ("last1", 6), ("last2", 12)):
        r[f] = cases.coef_models(rng, k * len(r)).reshape(len(r), k)
    a, b = oracle.coef_rate(coefs, r), ref.coef_rate(coefs, r)
    assert len(r) > 50 and a.tobytes() == b.tobytes()
