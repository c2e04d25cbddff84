"""The oracle's restatement of pmwd's white-noise draw (JAX's Threefry-2x32
normal, pmwd/modes.py:33-36) against published known answers:

* Threefry-2x32 with 20 rounds: the three known-answer vectors of the
  Random123 distribution (Salmon et al. 2011), which JAX's own test suite
  also checks its hash against;
* the documented outputs of JAX for the key of seed 0 in the original
  counter layout: ``split(PRNGKey(0))`` and ``normal(PRNGKey(0), (10,))``
  and the scalar ``normal(PRNGKey(0))``, as printed in JAX's documentation;
* distribution properties of the uniform and the normal draws.
"""

import numpy as np
import pytest

from oracle import prng


@pytest.mark.parametrize('key, ctr, want', [
    ((0, 0), (0, 0), (0x6B200159, 0x99BA4EFE)),
    ((0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF), (0x1CB996FC, 0xBB002BE7)),
    ((0x13198A2E, 0x03707344), (0x243F6A88, 0x85A308D3), (0xC4923A9C, 0x483DF7A0)),
])
def test_threefry2x32_known_answers(key, ctr, want):
    y0, y1 = prng.threefry2x32(key, np.uint32([ctr[0]]), np.uint32([ctr[1]]))
    assert (int(y0[0]), int(y1[0])) == want


def test_prng_key_of_int64_seeds():
    assert prng.prng_key(0) == (0, 0)
    assert prng.prng_key(7) == (0, 7)
    assert prng.prng_key((3 << 32) + 5) == (3, 5)
    assert prng.prng_key(-1) == (0xFFFFFFFF, 0xFFFFFFFF)


def test_documented_jax_draws_of_seed_0():
    key = prng.prng_key(0)
    np.testing.assert_array_equal(prng.split(key), [[4146024105, 967050713],
                                                    [2718843009, 1272950319]])
    want = np.float32([-0.3721109, 0.26423115, -0.18252768, -0.7368197, -0.44030377,
                       -0.1521442, -0.67135346, -0.5908641, 0.73168886, 0.5673026])
    np.testing.assert_array_equal(prng.normal_f32(0, (10,)), want)
    np.testing.assert_array_equal(prng.normal_f32(0, ()).reshape(()), np.float32(-0.20584226))


def test_original_layout_pads_odd_counts():
    """Odd n hashes the counters (j, j + h) with h = (n + 1) / 2 and the
    last pair's second counter replaced by the pad 0; dropping that word."""
    key = prng.prng_key(11)
    n = 7
    y0, y1 = prng.threefry2x32(key, np.uint32([0, 1, 2, 3]), np.uint32([4, 5, 6, 0]))
    np.testing.assert_array_equal(prng.random_bits(key, n), np.concatenate([y0, y1[:3]]))
    # the first half of a longer draw is not the same as a shorter draw
    assert not np.array_equal(prng.random_bits(key, 8)[:4], prng.random_bits(key, 4))


def test_partitionable_layout_is_prefix_stable():
    """value i depends on i only: a longer draw extends a shorter one."""
    key = prng.prng_key(3)
    a = prng.random_bits(key, 1000, 'partitionable')
    b = prng.random_bits(key, 1500, 'partitionable')
    np.testing.assert_array_equal(a, b[:1000])
    y0, y1 = prng.threefry2x32(key, np.uint32([0]), np.uint32([999]))
    assert a[999] == y0[0] ^ y1[0]


@pytest.mark.parametrize('layout', ['original', 'partitionable'])
def test_uniform_and_normal_distribution(layout):
    bits = prng.random_bits(prng.prng_key(2), 1 << 20, layout)
    u = prng.uniform_f32(bits)
    lo = np.nextafter(np.float32(-1), np.float32(0))
    assert u.dtype == np.float32 and u.min() >= lo and u.max() < 1
    x = prng.normal_f32(2, (1 << 20,), layout)
    assert np.all(np.isfinite(x))
    assert abs(x.mean()) < 5e-3 and abs(x.std() - 1) < 5e-3
    # the tails: P(|x| > 3) = 2.70e-3
    assert abs(np.mean(np.abs(x) > 3) / 2.6998e-3 - 1) < 0.1


def test_erfinv_approximation_accuracy():
    """Giles' single-precision erfinv inverts erf to float32 accuracy on both
    branches (|x| below and above 0.9933, w = 5)."""
    from scipy.special import erf
    x = np.float32(np.concatenate([np.linspace(-0.9999, 0.9999, 20001), [-0.9999999, 0.9999999]]))
    y = prng.erfinv_f32(x)
    np.testing.assert_allclose(erf(y.astype(np.float64)), x.astype(np.float64), rtol=0,
                               atol=3e-7)
