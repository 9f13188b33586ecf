"""The raster kernel's RGBA8 channel conversion, checked in exact arithmetic.

The kernel turns a texel channel v in [0, 255] into the float v / 255,
correctly rounded (what the oracle computes with an IEEE division), as
fl(v * hi + fl(v * lo)) with one fused multiply-add, where hi + lo is 1/255
in double-word form.  This test reads the two constants out of the kernel
source, checks that they are that split of 1/255, and checks the result for
all 256 inputs against v / 255 rounded to float, both sides in rationals."""
import math
import os
import re
from fractions import Fraction

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KERNELS = os.path.join(ROOT, "habitat-sim_gb300", "csrc", "kernels.cu")


def round_f32(x):
    """x rounded to the nearest binary32 value (ties to even), as a Fraction."""
    x = Fraction(x)
    if x == 0:
        return Fraction(0)
    sign = -1 if x < 0 else 1
    x = abs(x)
    e = math.floor(math.log2(x))
    while Fraction(2) ** e > x:
        e -= 1
    while Fraction(2) ** (e + 1) <= x:
        e += 1
    assert -126 <= e <= 127
    ulp = Fraction(2) ** (e - 23)
    q = x / ulp
    n = q.numerator // q.denominator
    r = q - n
    if r > Fraction(1, 2) or (r == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return sign * n * ulp


def kernel_constants():
    src = open(KERNELS).read()
    body = re.search(r"float chan\(uint32_t t, int c\) \{(.*?)\n\}", src, re.S).group(1)
    lits = re.findall(r"(-?0x[0-9a-fA-F.]+p[-+]?\d+)f", body)
    assert len(lits) == 2, lits
    hi, lo = (Fraction(float.fromhex(v)) for v in lits)
    return hi, lo


def test_constants_are_the_double_word_split_of_one_over_255():
    hi, lo = kernel_constants()
    assert hi == round_f32(Fraction(1, 255))
    assert lo == round_f32(Fraction(1, 255) - hi)
    assert round_f32(hi) == hi and round_f32(lo) == lo  # both exact binary32 values


def test_every_channel_value_is_correctly_rounded():
    hi, lo = kernel_constants()
    for v in range(256):
        got = round_f32(v * hi + round_f32(v * lo))  # fma(v, hi, v * lo)
        assert got == round_f32(Fraction(v, 255)), v


def test_single_product_would_not_be_exact():
    """Why two constants: v * fl(1/255) alone misrounds about half the inputs."""
    hi = round_f32(Fraction(1, 255))
    wrong = [v for v in range(256) if round_f32(v * hi) != round_f32(Fraction(v, 255))]
    assert len(wrong) > 100
