"""The fixed-point H1_adj conversion back to float (device.cuh from_fixed), restated in
numpy: the three float32 steps give the float nearest q 2^-34 (the float64 route) for
every accumulator value below 2^10 in magnitude, positive and negative.

Below 2^10 each step is an fmaf whose exact result is representable in float64 (argued
in device.cuh), so float64 arithmetic followed by one rounding to float32 reproduces it;
above, the restatement only bounds the result to one ulp."""
import numpy as np


def from_fixed_fp32_steps(q):
    q = np.asarray(q, dtype=np.int64)
    a = (q >> 44).astype(np.float64)
    b = ((q >> 22) & 0x3FFFFF).astype(np.float64)
    c = (q & 0x3FFFFF).astype(np.float64)
    t = (a * 1024.0 + b * 2.0 ** -12).astype(np.float32)  # fmaf(a, 1024, b / 4096)
    return (c * 2.0 ** -34 + t.astype(np.float64)).astype(np.float32)  # fmaf(c, 2^-34, t)


def test_from_fixed_is_correctly_rounded_below_2_to_10():
    rng = np.random.default_rng(7)
    mags = 2.0 ** rng.uniform(-34, 10, 200000)
    v = np.where(rng.random(mags.size) < 0.5, -mags, mags)
    q = np.round(v * 2.0 ** 34).astype(np.int64)
    q = np.concatenate([q, [0, 1, -1, 2 ** 22 - 1, -(2 ** 22), 2 ** 44 - 1, -(2 ** 44), 2 ** 43, -(2 ** 43) - 1]])
    q = q[np.abs(q) < 2 ** 44]
    ref = (q.astype(np.float64) * 2.0 ** -34).astype(np.float32)  # exact product, one rounding
    got = from_fixed_fp32_steps(q)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_from_fixed_within_one_ulp_above():
    rng = np.random.default_rng(8)
    v = rng.uniform(-2.0 ** 28, 2.0 ** 28, 100000)
    q = np.round(v * 2.0 ** 34).astype(np.int64)
    ref = (q.astype(np.float64) * 2.0 ** -34).astype(np.float32)
    got = from_fixed_fp32_steps(q)
    ulp = np.spacing(np.abs(ref))
    assert np.all(np.abs(got.astype(np.float64) - ref.astype(np.float64)) <= ulp)
