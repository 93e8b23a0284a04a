"""CPU: the fixed-point form of com_had's 2:1 tile normalisation (uavs3e_gb300/csrc/common.cuh,
had_scale) equals (int)((double)s / sqrt(n) * 2.0) (src/com_cost.c:344-710) for every s < 2^23
wherever it does not fall back to the double expression."""
import math

import numpy as np


def test_fixed_point_scale_matches_the_double_expression():
    for n in (32, 128):
        sq = math.sqrt(float(n))
        k = int(2199023255552.0 / sq + 0.5)          # had_scale_k: round(2^41 / sq) in double arithmetic
        s = np.arange(0, 1 << 23, dtype=np.uint64)
        want = np.floor(s.astype(np.float64) / sq * 2.0).astype(np.int64)
        prod = s * np.uint64(k)                       # < 2^63: no wrap
        assert int(prod.max()) < (1 << 63)
        frac = prod & np.uint64((1 << 40) - 1)
        fast = (frac >= np.uint64(1 << 24)) & (frac <= np.uint64((1 << 40) - (1 << 24)))
        got = (prod >> np.uint64(40)).astype(np.int64)
        assert np.array_equal(got[fast], want[fast])
        # the double expression is the rare case
        assert np.count_nonzero(~fast) < 1000
