"""Generate dd_tables.h: double-double tables for the correctly rounded
pow(x, 0.2) of the FP64 parity tracker (log via 1 + i/64 reduction, exp via
2^(j/64) reduction).  Values come from mpmath at 200 bits.

    python onekapy_gb300/csrc/gen_dd_tables.py > onekapy_gb300/csrc/dd_tables.h
"""
import mpmath as mp

mp.mp.prec = 200


def split(v):
    hi = float(v)
    lo = float(v - mp.mpf(hi))
    return hi, lo


def trunc_bits(v, bits):
    """Round v to `bits` significant bits (a double with trailing zeros)."""
    m, e = mp.frexp(v)
    return float(mp.ldexp(mp.nint(m * 2**bits), e - bits))


print("// Generated by gen_dd_tables.py -- double-double constants (hi, lo).")
print("#pragma once")
print("// log(1 + i/64), i = 0..64")
print("#define ONEKA_DD_LOG_TABLE \\")
for i in range(65):
    hi, lo = split(mp.log(1 + mp.mpf(i) / 64))
    print(f"    {hi!r}, {lo!r}," + (" \\" if i < 64 else ""))
print("// 2^(j/64), j = 0..63")
print("#define ONEKA_DD_EXP2_TABLE \\")
for j in range(64):
    hi, lo = split(mp.power(2, mp.mpf(j) / 64))
    print(f"    {hi!r}, {lo!r}," + (" \\" if j < 63 else ""))
ln2 = mp.log(2)
l2h = trunc_bits(ln2, 42)
l2l = float(ln2 - mp.mpf(l2h))
l64 = ln2 / 64
l64h = trunc_bits(l64, 38)
l64m = trunc_bits(l64 - mp.mpf(l64h), 38)
l64l = float(l64 - mp.mpf(l64h) - mp.mpf(l64m))
print(f"#define ONEKA_LN2_HI {l2h!r}   // 42 significant bits")
print(f"#define ONEKA_LN2_LO {l2l!r}")
print(f"#define ONEKA_LN2_64_HI {l64h!r}   // 38 significant bits")
print(f"#define ONEKA_LN2_64_MID {l64m!r}  // 38 significant bits")
print(f"#define ONEKA_LN2_64_LO {l64l!r}")
print(f"#define ONEKA_64_OVER_LN2 {float(64 / ln2)!r}")
