"""Writes dct_matrices.inc: the integer DCT2 / DCT8 / DST7 matrices (N = 2..64) as constant data.

The encoder builds these at start-up in floating point (com_dct_coef_create,
src/com_tables.c:222-278: sqrt(N) * 32 times the orthonormal basis, rounded half away from
zero).  The library does not recompute them: a cos() that differs between host C libraries in
the last bit could move an entry across a .5 rounding boundary.  This script evaluated the closed
forms once; tests/test_tables.py checks the frozen entries against the oracle's tables and, where
the reference checker is built, against the reference's own com_tbl_tm* arrays.

    python uavs3e_gb300/csrc/gen_dct_matrices.py
"""
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def matrices(L):
    c = 1 << L
    s = math.sqrt(c) * 32
    rnd = lambda v: int(s * v + (0.5 if v > 0 else -0.5))   # C's (s8) truncation toward zero
    out = [[0] * (c * c) for _ in range(3)]
    for k in range(c):
        for n in range(c):
            w0 = math.sqrt(0.5) if k == 0 else 1.0
            out[0][k * c + n] = rnd(math.cos(math.pi * (n + 0.5) * k / c) * w0 * math.sqrt(2.0 / c))
            out[1][k * c + n] = rnd(math.cos(math.pi * (k + 0.5) * (n + 0.5) / (c + 0.5)) * math.sqrt(2.0 / (c + 0.5)))
            out[2][k * c + n] = rnd(math.sin(math.pi * (k + 0.5) * (n + 1) / (c + 0.5)) * math.sqrt(2.0 / (c + 0.5)))
    return out


def main():
    lines = ["// Generated by gen_dct_matrices.py: integer DCT2 / DCT8 / DST7 matrices, [type][k][n] per size.",
             "// clang-format off"]
    for L in range(1, 7):
        c = 1 << L
        lines.append(f"static const s8 kDctMat{c}[3 * {c} * {c}] = {{")
        flat = sum(matrices(L), [])
        for i in range(0, len(flat), 32):
            lines.append("    " + ", ".join(str(v) for v in flat[i:i + 32]) + ",")
        lines.append("};")
    lines.append("static const s8 *const kDctMat[7] = { nullptr, kDctMat2, kDctMat4, kDctMat8, kDctMat16, kDctMat32, "
                 "kDctMat64 };")
    lines.append("// clang-format on")
    with open(os.path.join(HERE, "dct_matrices.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
