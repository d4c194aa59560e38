"""Generate fp64_tables.h: the breakpoint tables of the FP64 logarithm and
arctangent in fp64_math.cuh, computed here at 60 significant digits with
mpmath and rounded to double.

* Logarithm -- the table-driven method of P. T. P. Tang, "Table-driven
  implementation of the logarithm function in IEEE floating-point
  arithmetic", ACM TOMS 16(4), 1990: breakpoints F_j = 1 + j/128
  (j = 0..128), 1/F_j, and log F_j split into a leading part that is a
  multiple of 2^-42 (so that k ln2_lead + lead_j is exact for |k| < 2048)
  and a trailing part.
* Arctangent -- breakpoints c_j = j/64 (j = 0..64) of t in [0, 1] with the
  Taylor coefficients of atan about c_j: atan(c_j + d) = a0 + a1 d + ... +
  a8 d^8 for |d| <= 1/128 (the truncation is below 2^-66); a0 is split into a
  rounded value and the rounded remainder.  The coefficients follow from
  atan'(x) = 1/(1 + x^2): with 1/(1 + (c + d)^2) = sum b_n d^n, multiplying
  out (1 + c^2 + 2 c d + d^2) sum b_n d^n = 1 gives b_0 = 1/(1 + c^2),
  b_n = -(2 c b_{n-1} + b_{n-2}) / (1 + c^2), and a_{n+1} = b_n / (n + 1).

Run:  python jif3d_gb300/csrc/gen_fp64_tables.py   (rewrites fp64_tables.h)
"""
import os

import mpmath as mp

mp.mp.dps = 60
HERE = os.path.dirname(os.path.abspath(__file__))
LOG_N, ATAN_N, ATAN_DEG = 128, 64, 8


def d(x):
    """Nearest double (mpmath rounds to nearest)."""
    return float(mp.mpf(x))


def lead(x, quantum):
    """x rounded to a multiple of quantum (nearest)."""
    return float(mp.nint(mp.mpf(x) / quantum) * quantum)


def fmt(v):
    return float(v).hex()


def main():
    q = mp.mpf(2) ** -42
    ln2 = mp.log(2)
    ln2_lead = lead(ln2, q)
    ln2_trail = d(ln2 - ln2_lead)
    log_rows = []
    for j in range(LOG_N + 1):
        F = 1 + mp.mpf(j) / LOG_N
        L = mp.log(F)
        Ll = lead(L, q)
        log_rows.append((d(1 / F), Ll, d(L - Ll)))
    atan_rows = []
    for j in range(ATAN_N + 1):
        c = mp.mpf(j) / ATAN_N
        q2 = 1 + c * c
        b = [1 / q2]
        for n in range(1, ATAN_DEG):
            b.append(-(2 * c * b[n - 1] + (b[n - 2] if n >= 2 else 0)) / q2)
        coeffs = [mp.atan(c)] + [b[n] / (n + 1) for n in range(ATAN_DEG)]
        check = mp.taylor(mp.atan, c, ATAN_DEG)
        assert all(abs(x - y) < mp.mpf(10) ** -40 for x, y in zip(coeffs, check))
        a0 = d(coeffs[0])
        atan_rows.append([a0, d(coeffs[0] - a0)] + [d(v) for v in coeffs[1:]])
    pio2 = mp.pi / 2
    lines = [
        "// fp64_tables.h -- generated by gen_fp64_tables.py; do not edit.",
        "// Breakpoint tables of the FP64 logarithm (Tang's table-driven method,",
        "// F_j = 1 + j/128: 1/F_j, lead and trail of log F_j) and arctangent",
        "// (c_j = j/64: atan(c_j) as value + remainder, then the Taylor",
        "// coefficients a1..a8 of atan about c_j), as exact hexadecimal doubles.",
        "#pragma once",
        "",
        "namespace j3g {",
        "namespace fp64tab {",
        "",
        f"constexpr int kLogN = {LOG_N};",
        f"constexpr int kAtanN = {ATAN_N};",
        f"constexpr int kAtanDeg = {ATAN_DEG};",
        f"constexpr double kLn2Lead = {fmt(ln2_lead)};",
        f"constexpr double kLn2Trail = {fmt(ln2_trail)};",
        f"constexpr double kPio2Hi = {fmt(d(pio2))};",
        f"constexpr double kPio2Lo = {fmt(d(pio2 - d(pio2)))};",
        f"constexpr double kPiHi = {fmt(d(mp.pi))};",
        f"constexpr double kPiLo = {fmt(d(mp.pi - d(mp.pi)))};",
        "// log(DBL_EPSILON) = -52 ln 2, rounded",
        f"constexpr double kLogDblEps = {fmt(d(-52 * ln2))};",
        "",
        "// {1/F_j, lead(log F_j), trail(log F_j)}",
        f"__device__ const double kLogTable[{LOG_N + 1}][3] = {{",
    ]
    lines += [f"    {{{fmt(a)}, {fmt(b)}, {fmt(c)}}}," for a, b, c in log_rows]
    lines += ["};", "", "// {atan(c_j), remainder, a1, ..., a8}",
              f"__device__ const double kAtanTable[{ATAN_N + 1}][{ATAN_DEG + 2}] = {{"]
    for row in atan_rows:
        lines.append("    {" + ", ".join(fmt(v) for v in row) + "},")
    lines += ["};", "", "}  // namespace fp64tab", "}  // namespace j3g", ""]
    with open(os.path.join(HERE, "fp64_tables.h"), "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
