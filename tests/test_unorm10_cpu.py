"""The A2B10G10R10_UNORM read-back the kernels use (StoreRGB10A2 in radiance_device.cuh), checked
for every one of the 1024 codes without a GPU.

The kernels read a code q as r0 = q * c with c = RN(1/1023), then r1 = fma(fma(-r0, 1023, q), c, r0).
The format's value is q / 1023 rounded once to FP32 (what the oracle, the host and the reference
shader's shim compute with an IEEE division).  This test evaluates the kernels' sequence in exact
rational arithmetic, rounding to FP32 after each operation as the hardware does (a fused
multiply-add rounds once), and checks it equals q / 1023 for all codes; a plain product q * c
would not (24 codes differ), which is why the correction step is there.
"""
from fractions import Fraction

import numpy as np


def rn32(x: Fraction) -> np.float32:
    """x rounded to the nearest FP32 value, ties to even (exact, from the neighbours of float(x))."""
    c = np.float32(float(x))
    cands = [np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))]
    return min(cands, key=lambda y: (abs(Fraction(float(y)) - x), int(np.float32(y).view(np.uint32)) & 1))


def test_decode_sequence_is_exact_for_every_code():
    c = rn32(Fraction(1, 1023))
    assert int(c.view(np.uint32)) == 0x3A802008
    plain_differs = 0
    for q in range(1024):
        want = np.float32(q) / np.float32(1023)          # IEEE FP32 division, rounded once
        r0 = rn32(Fraction(q) * Fraction(float(c)))
        e = rn32(Fraction(q) - Fraction(float(r0)) * 1023)
        r1 = rn32(Fraction(float(e)) * Fraction(float(c)) + Fraction(float(r0)))
        assert r1 == want, q
        plain_differs += int(r0 != want)
    assert plain_differs > 0


def test_encode_rounds_to_nearest_even():
    import oracle
    v = np.array([0.0, 1.0, 0.5, 1.5 / 1023, 2.5 / 1023, -0.2, 1.7, np.nan], dtype=np.float32)
    got = oracle.quantize_unorm10(v)
    codes = np.rint(np.clip(np.nan_to_num(v), 0, 1) * np.float32(1023))
    assert np.array_equal(got, (codes / np.float32(1023)).astype(np.float32))
    assert got[0] == 0 and got[1] == 1 and got[5] == 0 and got[6] == 1 and got[7] == 0
