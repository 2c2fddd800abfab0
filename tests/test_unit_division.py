"""The shaders' texel / 255 is computed as q = x * fl(1/255) followed by one correction with the
exact residual, q + fl(x - q*255) * fl(1/255), both steps single-rounded fused multiply-adds
(div255 in softglrender_gb300/csrc/sglc_device.cuh). This checks, in exact rational arithmetic with
IEEE binary32 round-to-nearest-even, that the result equals the correctly rounded quotient x / 255
for every RGBA8 channel value x = 0..255, the only inputs it receives."""
from fractions import Fraction

import numpy as np


def _rn32(x: Fraction) -> np.float32:
    """x rounded to the nearest binary32, ties to even (exact, no double rounding)."""
    f = np.float32(float(x))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        err = abs(Fraction(float(c)) - x)
        even = int(np.float32(c).view(np.uint32)) & 1 == 0
        key = (err, not even)
        if best is None or key < best[0]:
            best = (key, c)
    return np.float32(best[1])


def _fma(a: np.float32, b: np.float32, c: np.float32) -> np.float32:
    return _rn32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def test_div255_matches_ieee_quotient_for_every_byte():
    r = np.float32(1) / np.float32(255)
    assert Fraction(float(r)) == _rn32(Fraction(1, 255))
    for i in range(256):
        x = np.float32(i)
        q = np.float32(x * r)
        e = _fma(np.float32(-q), np.float32(255), x)
        got = _fma(e, r, q)
        want = _rn32(Fraction(i, 255))
        assert want == np.float32(x / np.float32(255))
        assert got.view(np.uint32) == want.view(np.uint32), i


def test_plain_product_is_not_enough():
    # why the correction step is there: the rounded product alone misses about half of the bytes
    r = np.float32(1) / np.float32(255)
    x = np.arange(256, dtype=np.float32)
    assert int(np.sum(x * r != x / np.float32(255))) > 100
