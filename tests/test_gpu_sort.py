"""The device sort (visacd_radix_sort_pairs: bitonic in one CTA up to 512
pairs, one CTA running every LSD pass up to 32768, three launches per pass
beyond) against numpy's stable sort, across the size boundaries, with many
equal keys (stability) and keys of every width the Morton orders use."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 3, 100, 511, 512, 513, 2000, 4096, 10242, 20480, 32767, 32768, 32769, 100003])
@pytest.mark.parametrize("key_bits", [30, 63])
def test_radix_sort_pairs_is_a_stable_sort(ctx, n, key_bits):
    rng = np.random.default_rng(n + key_bits)
    hi = 1 << key_bits
    keys = rng.integers(0, hi, n, dtype=np.uint64)
    keys[rng.random(n) < 0.3] = np.uint64(hi // 3)  # many equal keys
    keys[: n // 7] = keys[n // 7: 2 * (n // 7)]
    vals = rng.permutation(n).astype(np.uint32)
    k, v = ctx.radix_sort_pairs(keys, vals, key_bits)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])


def test_radix_sort_pairs_rejects_wide_keys(native, ctx):
    with pytest.raises(native.VisacdError):
        ctx.radix_sort_pairs(np.array([1 << 40, 3], np.uint64), np.array([0, 1], np.uint32), 30)
