"""The FP32 fixed-point constructions of the mixed deposit, checked with
exact rational arithmetic (no GPU):

- density (FixScale32::split in ecs_particles.cu, S = 38, B = 19): for
  |v 2^S| <= 2^38 the two FP32 additions of the bias 1.5 * 2^23 give
  H = rint(v 2^(S-B)) and rint(v 2^S - H 2^B), and H 2^B + rint(r) equals
  rint(v 2^S) (round half to even);
- flux (FixWord32::word, S = 22 - e_v): for |v 2^S| <= 2^22 one FP32
  multiply-add of the bias gives bits(bias) + rint(v 2^S), and 500 such words
  (the tile window's flush interval) sum without leaving int32.
"""
import random
from fractions import Fraction as F

import numpy as np

BIAS = F(12582912)  # 1.5 * 2^23
BIAS_BITS = 0x4B400000
B = 19


def rne_f32(x: F) -> F:
    """x rounded to the nearest FP32 value (ties to even), normal range."""
    if x == 0:
        return F(0)
    sign = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while F(2) ** e > a:
        e -= 1
    while F(2) ** (e + 1) <= a:
        e += 1
    ulp = F(2) ** (max(e, -126) - 23)
    q = a / ulp
    n = q.numerator // q.denominator
    rem = q - n
    if rem > F(1, 2) or (rem == F(1, 2) and n % 2 == 1):
        n += 1
    return sign * n * ulp


def rint_even(x: F) -> int:
    n = x.numerator // x.denominator
    rem = x - n
    if rem > F(1, 2) or (rem == F(1, 2) and n % 2 == 1):
        n += 1
    return n


def f32_bits(x: F) -> int:
    return int(np.float32(float(x)).view(np.uint32))


def split(v: F, S: int):
    h = rne_f32(v * F(2) ** (S - B) + BIAS)                 # fmaf(v, 2^(S-B), bias)
    r = rne_f32((h - BIAS) * (-(F(2) ** (B - S))) + v)       # fmaf(h - bias, -2^(B-S), v)
    low = rne_f32(r * F(2) ** S + BIAS)                     # fmaf(r, 2^S, bias)
    return f32_bits(h) - BIAS_BITS, f32_bits(low) - BIAS_BITS


def test_split_is_exact_rounding():
    rnd = random.Random(3)
    for S in (38, 33, 27):
        for t in range(1500):
            kind = t % 3
            if kind == 0:
                y = np.float32(rnd.uniform(-1, 1) * 2.0 ** rnd.randint(-40, 0))
            elif kind == 1:  # exact halves of the quantum: ties
                y = np.float32((rnd.randint(-2 ** 22, 2 ** 22) + 0.5) * 2.0 ** (-S + rnd.randint(0, 14)))
            else:
                y = np.float32(rnd.uniform(-1, 1))
            v = F(float(y))
            if abs(v) * F(2) ** S > F(2) ** 38:
                continue
            hi, lo = split(v, S)
            assert abs(hi) <= 2 ** 19 and abs(lo) <= 2 ** 18
            assert hi * 2 ** B + lo == rint_even(v * F(2) ** S)


S_FLUX = 22
WINDOW_MAX = 500


def word(v: F, S: int) -> int:
    # fmaf(v, 2^S, bias): the exact product plus the bias, rounded once
    return f32_bits(rne_f32(v * F(2) ** S + BIAS)) - BIAS_BITS


def test_flux_word_is_exact_rounding():
    rnd = random.Random(4)
    for S in (S_FLUX, 17, 12):
        for t in range(2000):
            kind = t % 3
            if kind == 0:
                y = np.float32(rnd.uniform(-1, 1) * 2.0 ** rnd.randint(-30, 0))
            elif kind == 1:  # exact halves of the quantum: ties
                y = np.float32((rnd.randint(-2 ** 20, 2 ** 20) + 0.5) * 2.0 ** -S)
            else:
                y = np.float32(rnd.uniform(-1, 1))
            v = F(float(y))
            if abs(v) * F(2) ** S > F(2) ** 22:
                continue
            assert word(v, S) == rint_even(v * F(2) ** S)


def test_flux_window_bound():
    # the largest flux contribution (|v w| at the velocity bound) is 2^22
    # quanta; a window node sums at most WINDOW_MAX of them
    assert word(F(1), S_FLUX) == 2 ** 22
    assert word(F(-1), S_FLUX) == -(2 ** 22)
    assert WINDOW_MAX * 2 ** 22 < 2 ** 31
