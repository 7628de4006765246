"""The kernels fold `c + a*b` into one fused multiply-add only where the product a*b is exact in
FP32, so that the fused form rounds the same single sum as the shader's two operations; and they
write the set-up's jitter 0.1*((r - 0.5)*2) as 0.2*(r - 0.5).  These checks pin the arithmetic
facts those rewrites rest on (numpy's float32 operations round to nearest like the kernels'
__fmul_rn / __fadd_rn); the GPU parity tests pin the kernels' results against the oracle.
"""
import numpy as np

F = np.float32


def test_point_two_is_exactly_twice_point_one():
    # 0.2f == 2 * 0.1f as real numbers: same mantissa, exponent one higher
    assert F(F(0.1) * F(2.0)) == F(0.2)
    assert int(F(0.2).view(np.uint32)) == int(F(0.1).view(np.uint32)) + (1 << 23)


def test_jitter_forms_round_alike():
    """fl(0.1 * fl(2t)) == fl(0.2 * t) for t = r - 0.5, r = u * 2^-32 as the hash forms it."""
    rng = np.random.default_rng(7)
    u = np.concatenate([rng.integers(0, 2**32, 2_000_000, dtype=np.uint64),
                        np.arange(0, 1 << 16, dtype=np.uint64),
                        2**32 - 1 - np.arange(0, 1 << 16, dtype=np.uint64),
                        (2**31 + np.arange(-(1 << 15), 1 << 15)).astype(np.uint64)])
    r = (u.astype(F) * F(2.3283064365386963e-10)).astype(F)
    t = (r - F(0.5)).astype(F)
    two_step = (F(0.1) * (t * F(2.0)).astype(F)).astype(F)
    one_step = (F(0.2) * t).astype(F)
    assert np.array_equal(two_step.view(np.uint32), one_step.view(np.uint32))


def test_scaled_products_are_exact():
    """The products the kernels fuse: trunc(p/16)*16 (an integer of at most |p|/16 times 16), a
    block index q*16 (q an int16) and (r - 0.5)*2: each equals its exact value, so fusing it with
    the following addition changes nothing."""
    rng = np.random.default_rng(8)
    p = np.concatenate([rng.uniform(-2.0**21, 2.0**21, 1_000_000), rng.uniform(-1e30, 1e30, 100_000)]).astype(F)
    tb = np.trunc((p * F(0.0625)).astype(F))
    assert np.array_equal((tb * F(16.0)).astype(np.float64), tb.astype(np.float64) * 16.0)
    q = np.arange(-32768, 32768, dtype=np.int16).astype(F)
    assert np.array_equal((q * F(16.0)).astype(np.float64), q.astype(np.float64) * 16.0)
    r = (rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(F) * F(2.3283064365386963e-10)).astype(F)
    t = (r - F(0.5)).astype(F)
    assert np.array_equal((t * F(2.0)).astype(np.float64), t.astype(np.float64) * 2.0)
