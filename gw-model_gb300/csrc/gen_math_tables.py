"""Generates gw_math_tables.h: the tables of the engine's FP64 exp and log (gw_math64.cuh).

exp (Tang, ACM TOMS 15(2), 1989): 2^(j/64), j = 0..63, each as a lead double (the value rounded
to nearest) and a trail double (the rounding error of the lead), plus ln2/64 split the same way.
log (Tang, ACM TOMS 16(4), 1990): for j = 0..127, F_j = 1 + (j + 1/2)/128, invF_j = 1/F_j rounded
to nearest double, and -log(invF_j) as lead + trail doubles, plus ln2 split into lead + trail.
All values come from 60-digit decimal arithmetic (Python's decimal module).

Usage: python gen_math_tables.py > gw_math_tables.h
"""
from decimal import Decimal, getcontext

getcontext().prec = 60


def dbl(d: Decimal) -> float:
    return float(d)  # correctly rounded decimal -> double


def split(d: Decimal):
    lead = dbl(d)
    trail = dbl(d - Decimal(lead))
    return lead, trail


def main():
    ln2 = Decimal(2).ln()
    out = []
    out.append("// gw_math_tables.h -- generated by gen_math_tables.py; do not edit.")
    out.append("#pragma once")
    out.append("namespace gw {")
    out.append("namespace math64 {")
    l_hi, l_lo = split(ln2 / 64)
    out.append(f"constexpr double kLn2By64Hi = {l_hi.hex()};  // ln2/64, lead")
    out.append(f"constexpr double kLn2By64Lo = {l_lo.hex()};  // ln2/64 - lead")
    out.append(f"constexpr double k64ByLn2 = {dbl(64 / ln2).hex()};")
    n_hi, n_lo = split(ln2)
    out.append(f"constexpr double kLn2Hi = {n_hi.hex()};")
    out.append(f"constexpr double kLn2Lo = {n_lo.hex()};")
    out.append("// 2^(j/64): {lead, trail}")
    out.append("#define GW_EXP2_TABLE \\")
    out.append("    { \\")
    for j in range(64):
        v = (Decimal(j) / 64 * ln2).exp()
        a, b = split(v)
        out.append(f"        {{{a.hex()}, {b.hex()}}}, \\")
    out.append("    }")
    out.append("// j = 0..127: {invF_j, lead(-log(invF_j)), trail}, F_j = 1 + (j + 1/2)/128")
    out.append("#define GW_LOG_TABLE \\")
    out.append("    { \\")
    for j in range(128):
        F = 1 + (Decimal(j) + Decimal("0.5")) / 128
        inv = dbl(1 / F)
        L = -(Decimal(inv).ln())
        a, b = split(L)
        out.append(f"        {{{inv.hex()}, {a.hex()}, {b.hex()}}}, \\")
    out.append("    }")
    out.append("}  // namespace math64")
    out.append("}  // namespace gw")
    print("\n".join(out))


if __name__ == "__main__":
    main()
