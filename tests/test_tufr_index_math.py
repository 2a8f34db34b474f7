"""Index arithmetic of the time unfolding's deramp staging (k_tufr_fused),
restated in numpy float32 and checked against exact integer division.

The staging maps a sample u of the T S-point deramp axis to its knot
interval floor(u (S - 1) / (T S - 1)) (the last sample in interval S - 2),
and an interval iv to its first sample ceil(iv (T S - 1) / (S - 1)), without
64-bit divisions: a float32 estimate (u * gk rounded toward zero, iv * rt
rounded up, gk and rt the float32 ratios) corrected by at most one step
with exact integer products.  The correction covers the estimate's error
only if that error is below one, which these tests check over every sample
and interval of burst geometries across the IW range, and at the kernel's
limit T S < 2^24."""
import numpy as np
import pytest


def knot_of_near(u, S, TS, gk):
    q = np.trunc(u.astype(np.float32) * np.float32(gk)).astype(np.int64)
    num = u.astype(np.int64) * (S - 1)
    q = np.where(q * (TS - 1) > num, q - 1, np.where((q + 1) * (TS - 1) <= num, q + 1, q))
    return np.minimum(q, S - 2)


def knot_first_near(iv, S, TS, rt):
    num = iv.astype(np.int64) * (TS - 1)
    n = np.ceil(iv.astype(np.float32) * np.float32(rt)).astype(np.int64)
    return np.where(n * (S - 1) < num, n + 1, np.where((n - 1) * (S - 1) >= num, n - 1, n))


def exact_knot_of(u, S, TS):
    return np.minimum(u.astype(np.int64) * (S - 1) // (TS - 1), S - 2)


def exact_knot_first(iv, S, TS):
    return -((-iv.astype(np.int64) * (TS - 1)) // (S - 1))


@pytest.mark.parametrize("S,T", [(6908, 6), (2760, 5), (6181, 7), (7403, 8), (4001, 4), (1201, 9)])
def test_interval_of_every_sample(S, T):
    TS = S * T
    gk = np.float32((S - 1) / (TS - 1))
    rt = np.float32((TS - 1) / (S - 1))
    u = np.arange(TS, dtype=np.int64)
    est = knot_of_near(u, S, TS, gk)
    np.testing.assert_array_equal(est, exact_knot_of(u, S, TS))
    # the float estimate alone is never off by more than one
    raw = np.trunc(u.astype(np.float32) * gk).astype(np.int64)
    assert np.abs(raw - u * (S - 1) // (TS - 1)).max() <= 1
    iv = np.arange(S - 1, dtype=np.int64)
    first = knot_first_near(iv, S, TS, rt)
    np.testing.assert_array_equal(first, exact_knot_first(iv, S, TS))
    # consistency: each interval's first sample maps back to it, the sample
    # before it to the interval before
    np.testing.assert_array_equal(exact_knot_of(first, S, TS), iv)
    np.testing.assert_array_equal(exact_knot_of(first[1:] - 1, S, TS), iv[:-1])


def test_estimates_at_the_kernel_limit():
    """T S just under 2^24 (the kernel rejects larger axes): sampled inputs."""
    rng = np.random.default_rng(3)
    for S, T in ((65521, 256), (2_000_003, 8), (559_240, 30)):
        TS = S * T
        assert TS < 1 << 24
        gk = np.float32((S - 1) / (TS - 1))
        rt = np.float32((TS - 1) / (S - 1))
        u = np.concatenate([rng.integers(0, TS, 200000), np.arange(TS - 1000, TS)])
        np.testing.assert_array_equal(knot_of_near(u, S, TS, gk), exact_knot_of(u, S, TS))
        iv = np.concatenate([rng.integers(0, S - 1, 200000), np.arange(max(0, S - 1001), S - 1)])
        np.testing.assert_array_equal(knot_first_near(iv, S, TS, rt), exact_knot_first(iv, S, TS))
