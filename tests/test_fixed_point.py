"""The FP32 fixed-point constructions of the mixed deposit, checked with
exact rational arithmetic (no GPU):

- density (FixScale32::split in ecs_particles.cu, S = 38, B = 19): for
  |v 2^S| <= 2^38 the two FP32 additions of the bias 1.5 * 2^23 give
  H = rint(v 2^(S-B)) and rint(v 2^S - H 2^B), and H 2^B + rint(r) equals
  rint(v 2^S) (round half to even);
- flux (FixWord32::word, S = 22 - e_v): for |v 2^S| <= 2^22 one FP32
  multiply-add of the bias gives bits(bias) + rint(v 2^S);
- the tile window (k_tiles32): an ion deposits there only when each velocity
  component is within vmax / 8, so its flux words are at most 2^19 quanta,
  and a chunk of kWindowMax ions (read from the kernel source) adds at most
  one word an ion to a node: the biased uint32 sums, less count * bits(bias)
  at the flush, are the exact int32 sums.
"""
import random
import re
from fractions import Fraction as F
from pathlib import Path

import numpy as np

KERNEL_SRC = Path(__file__).resolve().parents[1] / "ecsprt_gb300" / "csrc" / "ecs_particles.cu"

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


def window_max() -> int:
    m = re.search(r"constexpr int kWindowMax = (\d+);", KERNEL_SRC.read_text())
    assert m, "kWindowMax not found in the tile kernel"
    return int(m.group(1))


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
    # velocities in units of vmax = 2^e_v (S_FLUX = 22 for e_v = 0): the
    # largest contribution of an ion anywhere is 2^22 quanta (the int64 path),
    # of an ion within vmax / 8 (the window) 2^19; a window node sums at most
    # one word an ion of a chunk of kWindowMax ions
    wmax = window_max()
    assert word(F(1), S_FLUX) == 2 ** 22
    assert word(F(1, 8), S_FLUX) == 2 ** 19
    assert word(F(-1, 8), S_FLUX) == -(2 ** 19)
    assert wmax * 2 ** 19 < 2 ** 31  # flux words and the density's high words
    assert wmax * 2 ** 18 < 2 ** 31  # the density's low words


def test_biased_window_sums_are_exact():
    # each shared-memory word adds bits(bias) + value, wrapping in uint32; the
    # flush subtracts count * bits(bias) and reads the word as int32
    rng = np.random.default_rng(5)
    wmax = window_max()
    for trial in range(24):
        n = wmax if trial < 8 else int(rng.integers(1, wmax + 1))
        if trial % 4 == 0:
            vals = np.full(n, 2 ** 19, dtype=np.int64)
        elif trial % 4 == 1:
            vals = np.full(n, -(2 ** 19), dtype=np.int64)
        else:
            vals = rng.integers(-(2 ** 19), 2 ** 19 + 1, size=n)
        word_u32 = 0
        for v in vals.tolist():
            word_u32 = (word_u32 + BIAS_BITS + v) & 0xFFFFFFFF
        unbiased = (word_u32 - n * BIAS_BITS) & 0xFFFFFFFF
        as_int32 = unbiased - 2 ** 32 if unbiased >= 2 ** 31 else unbiased
        assert as_int32 == int(vals.sum())
