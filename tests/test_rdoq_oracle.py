"""CPU: the RDOQ restatement (orc_rdoq) against the reference's quant_non_zero on blocks whose bin-cost
estimates come from the reference's own rdoq_init_cu_est_bits over random entropy-coder contexts."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402


def test_rdoq_with_estimates_from_contexts(oracle, ref):
    rng = np.random.default_rng(12)
    for seed in range(8):
        reqs, _, coefs = cases.rdoq_inputs(oracle, dict(n=150, k=3), 4000 + seed)
        # context models: 10-bit LPS probability << 1 | MPS
        ests = np.stack([ref.rdoq_est_from_ctx((rng.integers(8, 1016, 86) << 1) | rng.integers(0, 2, 86))
                         for _ in range(3)])
        a, b = coefs.copy(), coefs.copy()
        assert np.array_equal(oracle.rdoq(reqs, ests, a), ref.rdoq(reqs, ests, b))
        assert np.array_equal(a, b)


def test_weighted_quant_oracle_matches_reference(oracle, ref):
    """quant_non_zero with pic_wq_enable: the restatement equals the reference on every shape"""
    for seed in range(3):
        reqs, _, coefs = cases.rdoq_inputs(oracle, dict(n=200, k=1), 8200 + seed)
        wq4, wq8 = cases.wq_matrices(np.random.default_rng(8300 + seed))
        a, b = coefs.copy(), coefs.copy()
        assert np.array_equal(oracle.quant_wq(reqs, wq4, wq8, a), ref.quant_wq(reqs, wq4, wq8, b))
        assert np.array_equal(a, b)
