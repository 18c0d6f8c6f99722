"""The sampler's grey read divides a grey level k by 255 with no division and no table (grey_of in
lizard_gb300/csrc/sample_dev.cuh): q = RN(k r), r the float nearest 1 / 255, then q' = RN(q + r RN(k - 255 q)) with
both steps fused multiply-adds. Checked here in exact rational arithmetic for every k: q' is the correctly rounded
k / 255, the value the reference's table holds (liblizard/src/acquire.c:52, i / 255.0f)."""
from fractions import Fraction


def rn32(x):
    """A rational rounded to the nearest float32, ties to even (normal range), as a Fraction."""
    if x == 0:
        return Fraction(0)
    s = -1 if x < 0 else 1
    x = abs(x)
    e = 0
    while x >= 2:
        x /= 2
        e += 1
    while x < 1:
        x *= 2
        e -= 1
    m = x * (1 << 23)
    fl = m.numerator // m.denominator
    rem = m - fl
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and fl % 2 == 1):
        fl += 1
    return s * Fraction(fl, 1 << 23) * Fraction(2) ** e


def test_grey_division_is_correctly_rounded_for_every_level():
    r = rn32(Fraction(1, 255))
    assert float(r) == 0.003921568859368563   # the literal in grey_of
    for k in range(256):
        q = rn32(k * r)
        q2 = rn32(q + rn32(Fraction(k) - 255 * q) * r)
        assert q2 == rn32(Fraction(k, 255)), k
