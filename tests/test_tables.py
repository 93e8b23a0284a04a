"""CPU: the frozen integer DCT2 / DCT8 / DST7 matrices the library compiles in
(uavs3e_gb300/csrc/dct_matrices.inc) equal the oracle's tables and, where the reference checker
is built, the reference's own com_tbl_tm2 .. com_tbl_tm64 after com_dct_coef_create."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def frozen():
    txt = open(os.path.join(ROOT, "uavs3e_gb300", "csrc", "dct_matrices.inc")).read()
    out = {}
    for n, body in re.findall(r"kDctMat(\d+)\[[^\]]*\] = \{([^}]*)\}", txt):
        out[int(n)] = np.array([int(v) for v in body.replace("\n", " ").split(",") if v.strip()], np.int8)
    return out


def test_frozen_matrices_match_oracle(oracle):
    f = frozen()
    assert sorted(f) == [2, 4, 8, 16, 32, 64]
    for ln in range(1, 7):
        n = 1 << ln
        assert f[n].size == 3 * n * n
        assert np.array_equal(f[n], np.asarray(oracle.dct_table(ln), np.int8).ravel()[:3 * n * n])


def test_frozen_matrices_match_reference(ref):
    f = frozen()
    for ln in range(1, 7):
        n = 1 << ln
        assert np.array_equal(f[n], np.asarray(ref.dct_table(ln), np.int8).ravel()[:3 * n * n]), n
