"""Generates shapes_sincos_tables.h: the constants of the correctly rounded
sine/cosine in shapes_sincos.h, computed with exact integer arithmetic.

    python shapes_gb300/csrc/gen_sincos_tables.py   # rewrites the header

Constants:
  - pi to 1600 bits by Machin's formula, pi = 16 atan(1/5) - 4 atan(1/239),
    each arctangent summed as its Taylor series in fixed point;
  - 2/pi as 20 words of 64 bits (1280 bits after the binary point), for the
    Payne-Hanek reduction of the accurate phase;
  - pi/2 in unsigned fixed point with 126 fractional bits (two words);
  - pi/512 split as P1 + P2 + P3 + P4 (29, 29, 53 and 53 significant bits),
    for the Cody-Waite reduction of the fast phase;
  - sin(i pi/512), i = 0..256, each as an unevaluated sum hi + lo of two
    doubles (hi = RN(v), lo = RN(v - hi));
  - 1/n!, n = 0..33, in unsigned fixed point with 127 fractional bits (the
    Taylor coefficients of the accurate phase), rounded to nearest.
The header is committed; tests/test_sincos.py regenerates it in memory and
checks that the committed file matches.
"""
from __future__ import annotations

from fractions import Fraction
from pathlib import Path

PREC = 1600  # working fixed-point bits


def _atan_inv(n: int, bits: int) -> int:
    """atan(1/n) * 2^bits, truncated series (error < a few units)."""
    one = 1 << bits
    term = one // n
    total = term
    n2 = n * n
    k = 1
    while term:
        term //= n2
        k += 2
        total += -(term // k) if (k // 2) % 2 else term // k
    return total


def pi_fixed(bits: int = PREC) -> int:
    """pi * 2^bits (error below 2^-(bits - 8))."""
    g = 16  # guard bits
    v = 16 * _atan_inv(5, bits + g) - 4 * _atan_inv(239, bits + g)
    return v >> g


def sin_fixed(num: int, den: int, pi_f: int, bits: int) -> int:
    """sin(num * pi / den) * 2^bits by its Taylor series (|arg| <= pi/2)."""
    x = (pi_f * num) // den  # x * 2^bits
    one = 1 << bits
    term = x
    total = x
    k = 1
    while term:
        term = -((term * x >> bits) * x >> bits) // ((k + 1) * (k + 2))
        k += 2
        total += term
    return total


def to_dd(v: int, bits: int) -> tuple[float, float]:
    """Nearest double to v/2^bits, then nearest double to the remainder."""
    fr = Fraction(v, 1 << bits)
    hi = float(fr)  # CPython rounds Fraction -> float correctly
    lo = float(fr - Fraction(hi))
    return hi, lo


def split_bits(value: Fraction, sig: int) -> float:
    """value truncated to `sig` significant bits, as an exact double."""
    if value == 0:
        return 0.0
    e = 0
    v = abs(value)
    while v >= 1:
        v /= 2
        e += 1
    while v < Fraction(1, 2):
        v *= 2
        e -= 1
    m = int(v * (1 << sig))  # truncation
    out = Fraction(m, 1 << sig) * (Fraction(2) ** e)
    f = float(out)
    assert Fraction(f) == out
    return f if value > 0 else -f


def hexf(x: float) -> str:
    return float.hex(x)


def generate() -> str:
    pi_f = pi_fixed()
    lines = []
    w = lines.append
    w("/* Generated by gen_sincos_tables.py (exact integer arithmetic); do not edit. */")
    w("#ifndef SHAPES_SINCOS_TABLES_H")
    w("#define SHAPES_SINCOS_TABLES_H")
    w("#include <stdint.h>")
    w("")
    # 2/pi words
    two_over_pi = (2 << (2 * PREC)) // pi_f  # (2/pi) * 2^PREC
    words = []
    for k in range(20):
        words.append((two_over_pi >> (PREC - 64 * (k + 1))) & ((1 << 64) - 1))
    w("/* 2/pi = sum_k W[k] 2^(-64(k+1)) (the first 1280 bits after the binary point) */")
    w("#define SHAPES_TWO_OVER_PI_WORDS { \\")
    for k in range(0, 20, 2):
        w(f"  0x{words[k]:016x}ull, 0x{words[k + 1]:016x}ull, \\")
    w("}")
    # pi/2 in Q2.126
    pio2 = (pi_f >> 1) >> (PREC - 126)
    w("/* pi/2 * 2^126, truncated: high and low 64-bit words */")
    w(f"#define SHAPES_PIO2_Q126_HI 0x{pio2 >> 64:016x}ull")
    w(f"#define SHAPES_PIO2_Q126_LO 0x{pio2 & ((1 << 64) - 1):016x}ull")
    # pi/512 split
    pi512 = Fraction(pi_f, 1 << PREC) / 512
    p1 = split_bits(pi512, 29)
    rem = pi512 - Fraction(p1)
    p2 = split_bits(rem, 29)
    rem -= Fraction(p2)
    p3 = split_bits(rem, 53)
    rem -= Fraction(p3)
    p4 = float(rem)
    w("/* pi/512 = P1 + P2 + P3 + P4 (+ < 2^-180): 29, 29, 53 and 53 significant bits */")
    w(f"#define SHAPES_PI512_P1 {hexf(p1)}")
    w(f"#define SHAPES_PI512_P2 {hexf(p2)}")
    w(f"#define SHAPES_PI512_P3 {hexf(p3)}")
    w(f"#define SHAPES_PI512_P4 {hexf(p4)}")
    inv = Fraction(1 << PREC, pi_f) * 512  # 512/pi
    w(f"#define SHAPES_512_OVER_PI {hexf(float(inv))}")
    # sin(i pi / 512)
    tb = 300
    pi_t = pi_f >> (PREC - tb)
    w("/* sin(i pi/512), i = 0..256: hi, lo pairs */")
    w("#define SHAPES_SIN_TABLE { \\")
    for i in range(257):
        if i == 0:
            hi, lo = 0.0, 0.0
        elif i == 256:
            hi, lo = 1.0, 0.0
        else:
            hi, lo = to_dd(sin_fixed(i, 512, pi_t, tb), tb)
        w(f"  {hexf(hi)}, {hexf(lo)}, \\")
    w("}")
    # 1/n! in Q1.127
    w("/* 1/n! * 2^127 rounded to nearest, n = 0..33: high and low 64-bit words */")
    w("#define SHAPES_INV_FACT_Q127 { \\")
    fact = 1
    for n in range(34):
        if n:
            fact *= n
        q = ((1 << 128) // fact + 1) >> 1  # round(2^127 / n!)
        assert q < (1 << 128)
        w(f"  0x{q >> 64:016x}ull, 0x{q & ((1 << 64) - 1):016x}ull, \\")
    w("}")
    w("")
    w("#endif /* SHAPES_SINCOS_TABLES_H */")
    return "\n".join(lines) + "\n"


OUT = Path(__file__).resolve().parent / "shapes_sincos_tables.h"

if __name__ == "__main__":
    OUT.write_text(generate())
    print(f"wrote {OUT}")
