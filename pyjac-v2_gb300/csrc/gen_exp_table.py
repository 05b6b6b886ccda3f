"""Write pjg_exp_table.h: the tables and polynomial coefficients of fexp
(pjg_math.cuh), Tang's table-driven exponential.

For B table bits the kernels read 2^(j/2^B), j = 0 .. 2^B - 1, each the double
nearest the exact value (computed here in 200-bit arithmetic).  The residual
r of the argument reduction lies in |r| <= h = ln 2 / 2^(B+1), where exp(r) is
a polynomial:

* B = 8: the degree-4 Taylor polynomial (truncation below 4e-17 relative);
* B = 10, 11: a degree-3 polynomial 1 + r + c2 r^2 + c3 r^3 whose c2, c3
  minimise the largest relative error |p(r) / e^r - 1| over [-h, h] (a
  linear program over 4,001 Chebyshev points of the interval, the discrete
  form of the Remez minimax problem), 9.4e-17 for B = 10 and 5.9e-18 for
  B = 11.

Run: python gen_exp_table.py  (needs mpmath and scipy; the output is committed)
"""
import os

import mpmath as mp
from scipy.optimize import linprog

mp.mp.prec = 200
BITS = (8, 10, 11)


def minimax_deg3(B):
    h = mp.log(2) / 2 ** (B + 1)
    scale = float(h ** 4)
    A, b = [], []
    for k in range(4001):
        r = h * mp.cos(mp.pi * k / 4000)
        er = mp.e ** r
        a2, a3 = r ** 2 / er, r ** 3 / er
        b0 = (1 + r) / er - 1 + a2 / 2 + a3 / 6   # error with the Taylor c2, c3
        A.append([float(a2 / scale), float(a3 / scale), -1.0])
        b.append(float(-b0 / scale))
        A.append([float(-a2 / scale), float(-a3 / scale), -1.0])
        b.append(float(b0 / scale))
    res = linprog([0, 0, 1], A_ub=A, b_ub=b, bounds=[(None, None)] * 3, method="highs")
    d2, d3, t = res.x
    c2, c3 = float(mp.mpf(1) / 2 + d2), float(mp.mpf(1) / 6 + d3)
    worst = max(abs((1 + r + c2 * r ** 2 + c3 * r ** 3) / mp.e ** r - 1)
                for r in [h * mp.mpf(k) / 2000 for k in range(-2000, 2001)])
    return c2, c3, float(worst)


def main():
    out = [
        "// Generated by gen_exp_table.py: tables 2^(j/2^B) (each the nearest double)",
        "// and polynomial coefficients of fexp (pjg_math.cuh).  Do not edit.",
        "#pragma once",
        "",
    ]
    for B in BITS:
        n = 1 << B
        vals = [float(mp.mpf(2) ** (mp.mpf(j) / n)) for j in range(n)]
        out.append("#if PJG_EXP_BITS == %d" % B)
        out.append("#define PJG_EXP_HAVE_TABLE 1")
        if B >= 10:
            c2, c3, worst = minimax_deg3(B)
            out.append("// minimax on |r| <= ln 2 / 2^%d: largest relative error %.2e" % (B + 1, worst))
            out.append("#define PJG_EXP_C2 %s" % float.hex(c2))
            out.append("#define PJG_EXP_C3 %s" % float.hex(c3))
        out.append("__device__ const double pjg_exp2_table[%d] = {" % n)
        for i in range(0, n, 4):
            out.append("    " + ", ".join(float.hex(v) for v in vals[i:i + 4]) + ",")
        out.append("};")
        out.append("#endif")
        out.append("")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pjg_exp_table.h")
    with open(path, "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
