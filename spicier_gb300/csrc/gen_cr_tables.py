#!/usr/bin/env python3
"""Generates cr_tables.h: the constants of the integer fixed-point ln and cos
in cr_math.cuh, computed with mpmath at 400 bits and rounded to nearest.

    python spicier_gb300/csrc/gen_cr_tables.py   # rewrites cr_tables.h

ln (format Q8.120, value = integer * 2^-120):
  for i in 0..255, c_i = ceil(2^16 / (1 + i/256)) / 2^16, so that for every
  mantissa m in [1 + i/256, 1 + (i+1)/256), r = m c_i - 1 lies in [0, 2^-7.8);
  the table holds C_i = c_i 2^16 and -ln(c_i); plus ln 2 and 1/j (j = 2..7).
  The tail coefficients 1/j (j = 8..15) are Q0.64.
exp (format Q2.126): exp(j/256) for j = -90..90, ln 2 (Q12.116) and 1/k!.
cos (format Q3.125):
  cos(j/512) and sin(j/512) for j = 0..403, pi/2, and the Taylor
  coefficients 1/k! of the cos (k = 2..10) and sin (k = 3..11) series.
fast paths (Q0.64): 1/j (j = 2..9) for ln; 1/k! (k = 2, 4, 6, 8) and
  (k = 3, 5, 7, 9) for cos and sin.
"""
import os

import mpmath as mp

mp.mp.prec = 400
HERE = os.path.dirname(os.path.abspath(__file__))
F_LN, F_COS, F_EXP = 120, 125, 126


def fixed(v, frac_bits, total_bits=128):
    q = int(mp.nint(mp.mpf(v) * mp.mpf(2) ** frac_bits))
    assert 0 <= q < 2 ** total_bits, (v, frac_bits)
    return q


def words(q):
    return f"0x{q >> 64:016x}ULL, 0x{q & (2**64 - 1):016x}ULL"


def main():
    out = []
    w = out.append
    w("// Generated by gen_cr_tables.py (mpmath, 400-bit arithmetic, round to nearest).")
    w("// Do not edit by hand.")
    w("#pragma once")
    w("#include <stdint.h>")
    w("")
    # ---------------------------------------------------------------- ln
    rows = []
    rmax = mp.mpf(0)
    for i in range(256):
        C = int(mp.ceil(mp.mpf(2) ** 16 / (1 + mp.mpf(i) / 256)))
        c = mp.mpf(C) / 2 ** 16
        lo, hi = 1 + mp.mpf(i) / 256, 1 + mp.mpf(i + 1) / 256
        assert lo * c >= 1
        rmax = max(rmax, hi * c - 1)
        T = fixed(-mp.log(c), F_LN)
        rows.append(f"    {{0x{C:016x}ULL, {words(T)}, 0ULL}},")
    assert rmax < mp.mpf(2) ** -7.8, rmax
    w(f"// ln: rows {{C_i, -ln(C_i/2^16) hi, lo, 0}}; max r = {mp.nstr(rmax, 6)}")
    w("#define SP_CR_LN_ROWS \\")
    w("    { \\")
    for r in rows:
        w(r + " \\")
    w("    }")
    w(f"#define SP_CR_LN2 {words(fixed(mp.log(2), F_LN))}")
    w("#define SP_CR_LN_INV128 \\")
    w("    { " + ", ".join(f"{{{words(fixed(mp.mpf(1) / j, F_LN))}}}" for j in range(2, 8)) + " }")
    w("#define SP_CR_LN_INV64 \\")
    w("    { " + ", ".join(f"0x{fixed(mp.mpf(1) / j, 64, 64):016x}ULL" for j in range(8, 16)) + " }")
    w("")
    # ---------------------------------------------------------------- cos
    rows = []
    for j in range(404):
        a = mp.mpf(j) / 512
        rows.append(f"    {{{words(fixed(mp.cos(a), F_COS))}, {words(fixed(mp.sin(a), F_COS))}}}, ")
    w("// cos: rows {cos(j/512) hi, lo, sin(j/512) hi, lo}, j = 0..403")
    w("#define SP_CR_COS_ROWS \\")
    w("    { \\")
    for r in rows:
        w(r + " \\")
    w("    }")
    w(f"#define SP_CR_PIO2 {words(fixed(mp.pi / 2, F_COS))}")
    w("// Taylor coefficients: 1/2!, 1/4!, 1/6! and 1/3!, 1/5!, 1/7! in Q3.125; the tails 1/8!, 1/10!")
    w("// and 1/9!, 1/11! in Q0.64")
    w("#define SP_CR_COS_COEF \\")
    w("    { " + ", ".join(f"{{{words(fixed(1 / mp.factorial(k), F_COS))}}}" for k in (2, 4, 6)) + " }")
    w("#define SP_CR_SIN_COEF \\")
    w("    { " + ", ".join(f"{{{words(fixed(1 / mp.factorial(k), F_COS))}}}" for k in (3, 5, 7)) + " }")
    w("#define SP_CR_COS_TAIL { " + ", ".join(f"0x{fixed(1 / mp.factorial(k), 64, 64):016x}ULL" for k in (8, 10)) + " }")
    w("#define SP_CR_SIN_TAIL { " + ", ".join(f"0x{fixed(1 / mp.factorial(k), 64, 64):016x}ULL" for k in (9, 11)) + " }")
    # ------------------------------------------------- fast paths (Q0.64)
    w("")
    w("// fast paths (64-bit Horner, Q0.64): ln(1+r) = r - r^2 P(r), P = 1/2 - r/3 + ... - r^7/9;")
    w("// 1 - cos d = w Pc(w), Pc = 1/2! - w/4! + w^2/6! - w^3/8!; sin d = d - d w Ps(w),")
    w("// Ps = 1/3! - w/5! + w^2/7! - w^3/9!  (w = d^2)")
    w("#define SP_CR_LN_FAST { " + ", ".join(f"0x{fixed(mp.mpf(1) / j, 64, 64):016x}ULL" for j in range(2, 10)) + " }")
    w("#define SP_CR_COS_FAST { " + ", ".join(f"0x{fixed(1 / mp.factorial(k), 64, 64):016x}ULL" for k in (2, 4, 6, 8)) + " }")
    w("#define SP_CR_SIN_FAST { " + ", ".join(f"0x{fixed(1 / mp.factorial(k), 64, 64):016x}ULL" for k in (3, 5, 7, 9)) + " }")
    # ---------------------------------------------------------------- exp
    w("")
    w("// exp: rows {exp(j/256) hi, lo} for j = -90..90 (Q2.126), ln 2 in Q12.116,")
    w("// and the Taylor coefficients 1/k! (k = 2..12, Q2.126)")
    w("#define SP_CR_EXP_ROWS \\")
    w("    { \\")
    for j in range(-90, 91):
        w(f"    {{{words(fixed(mp.exp(mp.mpf(j) / 256), F_EXP))}}}, \\")
    w("    }")
    w(f"#define SP_CR_EXP_LN2 {words(fixed(mp.log(2), 116))}")
    w("#define SP_CR_EXP_COEF \\")
    w("    { " + ", ".join(f"{{{words(fixed(1 / mp.factorial(k), F_EXP))}}}" for k in range(2, 13)) + " }")
    open(os.path.join(HERE, "cr_tables.h"), "w").write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
