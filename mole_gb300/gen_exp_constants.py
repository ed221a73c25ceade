"""Derives the exponential's constants of mole_gb300/csrc/df64.cuh and fp64.cuh
from exact integer arithmetic, and prints them as C.

Tang's table-driven exponential (P. T. P. Tang, ACM TOMS 15(2), 1989) needs
ln2/64 split into a head with few significant bits (so that n times the head
is exact) and correctly rounded tails, the table 2^(j/64), j = 0..63, and the
FP32 value of 64/ln2 that picks n. ln 2 comes from the series
2 sum_k 1 / ((2k + 1) 3^(2k + 1)) = 2 atanh(1/3) in 480-bit fixed point, and
2^(j/64) = floor((2^j 2^(64 P))^(1/64)) by six nested integer square roots
(floor(sqrt(floor(sqrt(m)))) = floor(m^(1/4)) for integers m); every constant
is then rounded to nearest (even) at its precision from those exact values.
tests/test_exp_constants.py regenerates them and compares with the headers.

Usage: python -m mole_gb300.gen_exp_constants
"""
from __future__ import annotations

from fractions import Fraction
from math import isqrt

P = 480  # fixed-point bits


def ln2_fixed() -> int:
    """ln 2 * 2^P to within a few units."""
    one = 1 << (P + 16)
    term = one // 3
    total, k = 0, 0
    while term:
        total += term // (2 * k + 1)
        term //= 9
        k += 1
    return (2 * total) >> 16


def exp2_fixed(j: int) -> int:
    """floor(2^(j/64) * 2^P)."""
    m = 1 << (j + 64 * P)
    for _ in range(6):
        m = isqrt(m)
    return m


def round_bits(q: Fraction, bits: int) -> Fraction:
    """q rounded to nearest (ties to even) with `bits` significant bits."""
    if q == 0:
        return Fraction(0)
    sign = -1 if q < 0 else 1
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    scale = Fraction(2) ** (bits - 1 - e)  # a * scale in [2^(bits-1), 2^bits)
    v = a * scale
    n = v.numerator // v.denominator
    rem = v - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return sign * Fraction(n) / scale


def to_float(q: Fraction, bits: int) -> float:
    return float(round_bits(q, bits))


def constants() -> dict:
    ln2 = Fraction(ln2_fixed(), 1 << P)
    c64 = ln2 / 64
    out: dict = {}
    # FP64 exponential (fp64.cuh): 36-bit head as an integer times 2^-42
    m = round_bits(ln2 * 2 ** 36, 36)
    assert m.denominator == 1
    out["kExpL1Int"] = int(m)
    L1 = m / 2 ** 42
    out["L1"] = float(L1)
    out["kL2h"] = to_float(c64 - L1, 24)
    out["kL2l"] = to_float(c64 - L1 - Fraction(out["kL2h"]), 24)
    out["inv_ln2_64"] = to_float(64 / ln2, 24)
    sixth_h = to_float(Fraction(1, 6), 24)
    out["sixth"] = (sixth_h, to_float(Fraction(1, 6) - Fraction(sixth_h), 24))
    # double-float exponential (df64.cuh): 9-bit head so that n kL1 is exact in FP32
    h = Fraction(round(c64 * 2 ** 15), 2 ** 15)
    out["df_kL1"] = float(h)
    out["df_kL2"] = to_float(c64 - h, 24)
    out["df_kL3"] = to_float(c64 - h - Fraction(out["df_kL2"]), 24)
    tab, tabdf = [], []
    for j in range(64):
        t = Fraction(exp2_fixed(j), 1 << P)
        tab.append(to_float(t, 53))
        hi = to_float(t, 24)
        tabdf.append((hi, to_float(t - Fraction(hi), 24)))
    out["exp2_tab64"] = tab
    out["exp2_tab_df"] = tabdf
    return out


def main() -> None:
    c = constants()
    print(f"kExpL1Int = {c['kExpL1Int']:#X}  (L1 = {c['L1'].hex()})")
    print(f"kL2h = {c['kL2h'].hex()}f  kL2l = {c['kL2l'].hex()}f  64/ln2 = {c['inv_ln2_64'].hex()}f")
    print(f"1/6 = ({c['sixth'][0].hex()}f, {c['sixth'][1].hex()}f)")
    print(f"df: kL1 = {c['df_kL1'].hex()}f  kL2 = {c['df_kL2'].hex()}f  kL3 = {c['df_kL3'].hex()}f")
    print("kExp2Tab64 = {" + ", ".join(v.hex() for v in c["exp2_tab64"]) + "}")
    print("kExp2TabDF = {" + ", ".join(f"{{{a.hex()}f, {b.hex()}f}}" for a, b in c["exp2_tab_df"]) + "}")


if __name__ == "__main__":
    main()
