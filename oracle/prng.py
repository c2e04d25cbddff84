"""NumPy restatement of the white-noise draw of pmwd (test infrastructure
only: the GPU kernels in libpmx are checked against it).

pmwd's ``white_noise`` (pmwd/modes.py:12-49) draws its modes with
``jax.random.normal(jax.random.PRNGKey(seed), shape, float32)``; pmwd turns
on 64-bit JAX types (pmwd/configuration.py:15), so the seed is an int64.
JAX is a third-party dependency absent here (pmwd/setup.py:28 asks for
``jax>=0.4.7``, unpinned), so its published algorithm is restated:

* the key of a seed is the pair (seed >> 32, seed & 0xffffffff) of uint32;
* the counter-based generator is Threefry-2x32 with 20 rounds (Salmon,
  Moraes, Dror & Shaw 2011, "Parallel random numbers: as easy as 1, 2, 3",
  the Random123 family): rotations 13 15 26 6 / 17 29 16 24, a key
  injection after every 4 rounds, key parity 0x1BD11BDA;
* 32 random bits per value, in one of JAX's two counter layouts:
  ``original`` (JAX's ``jax_threefry_partitionable=False``, the default
  before JAX 0.5): the counters 0..n-1 (padded with one 0 when n is odd)
  are split in halves, hashed pairwise, and the two output words are
  concatenated; ``partitionable`` (the default since JAX 0.5): value i
  hashes the 64-bit counter (i >> 32, i & 0xffffffff) and XORs the two
  output words;
* a uniform in [nextafter(-1, 0), 1): the top 23 bits as the mantissa of
  a float in [1, 2), minus 1, times (hi - lo), plus lo, clamped below at lo;
* a normal: sqrt(2) erfinv(u) with Giles' single-precision erfinv
  approximation (M. Giles, "Approximating the erfinv function", GPU
  Computing Gems Jade Edition, 2011): w = -log1p(-u^2), a degree-8
  polynomial in w - 2.5 for w < 5 and in sqrt(w) - 3 otherwise, each Horner
  step a fused multiply-add, times u; erfinv(+-1) = +-inf.
"""

import numpy as np

_ROT = (13, 15, 26, 6, 17, 29, 16, 24)
_PARITY = 0x1BD11BDA
_M32 = 0xFFFFFFFF

# Giles' single-precision erfinv coefficients, highest order first
_ERFINV_SMALL = (2.81022636e-08, 3.43273939e-07, -3.5233877e-06, -4.39150654e-06,
                 0.00021858087, -0.00125372503, -0.00417768164, 0.246640727, 1.50140941)
_ERFINV_LARGE = (-0.000200214257, 0.000100950558, 0.00134934322, -0.00367342844,
                 0.00573950773, -0.0076224613, 0.00943887047, 1.00167406, 2.83297682)


def threefry2x32(key, x0, x1):
    """Threefry-2x32, 20 rounds, on uint32 arrays x0, x1 with key (k0, k1)."""
    k0, k1 = np.uint32(key[0]), np.uint32(key[1])
    ks = (k0, k1, np.uint32(k0 ^ k1 ^ np.uint32(_PARITY)))
    x0 = np.asarray(x0, np.uint32) + ks[0]
    x1 = np.asarray(x1, np.uint32) + ks[1]
    with np.errstate(over='ignore'):
        for r in range(20):
            x0 = x0 + x1
            s = _ROT[r % 8]
            x1 = (x1 << np.uint32(s)) | (x1 >> np.uint32(32 - s))
            x1 = x1 ^ x0
            if r % 4 == 3:
                i = (r + 1) // 4
                x0 = x0 + ks[i % 3]
                x1 = x1 + ks[(i + 1) % 3] + np.uint32(i)
    return x0, x1


def prng_key(seed):
    """jax.random.PRNGKey of an int64 seed: (seed >> 32, seed & 0xffffffff)."""
    s = int(np.int64(seed)) & 0xFFFFFFFFFFFFFFFF
    return (np.uint32(s >> 32), np.uint32(s & _M32))


def split(key, num=2):
    """jax.random.split in the original counter layout: the hash of the
    counters 0..2 num-1, as num keys."""
    return random_bits(key, 2 * num, 'original').reshape(num, 2)


def random_bits(key, n, layout='original'):
    """n 32-bit random words of ``key`` in JAX's counter layout."""
    if layout == 'original':
        if n >= _M32:
            raise NotImplementedError('more than 2^32 - 2 values in the original layout')
        cnt = np.arange(n + (n & 1), dtype=np.uint32)
        if n & 1:
            cnt[-1] = 0
        h = len(cnt) // 2
        y0, y1 = threefry2x32(key, cnt[:h], cnt[h:])
        return np.concatenate([y0, y1])[:n]
    if layout == 'partitionable':
        i = np.arange(n, dtype=np.uint64)
        y0, y1 = threefry2x32(key, (i >> np.uint64(32)).astype(np.uint32),
                              (i & np.uint64(_M32)).astype(np.uint32))
        return y0 ^ y1
    raise ValueError(f'unknown counter layout {layout!r}')


def uniform_f32(bits):
    """Floats in [nextafter(-1, 0), 1) from 32-bit words, as JAX's uniform."""
    lo = np.nextafter(np.float32(-1), np.float32(0))
    f = ((bits >> np.uint32(9)) | np.uint32(0x3F800000)).view(np.float32) - np.float32(1)
    # (hi - lo) rounds to 2 in float32; f * 2 is exact, so one rounding
    u = f * (np.float32(1) - lo) + lo
    return np.maximum(lo, u)


def _fma32(a, b, c):
    # a b is exact in float64 for float32 a, b; one rounding of the sum to
    # float64 then float32 (a double rounding, off by one ulp in rare ties)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def erfinv_f32(x):
    """Giles' single-precision erfinv on float32 values in [-1, 1]."""
    x = np.asarray(x, np.float32)
    w = -np.log1p(-(x * x))
    small = w < np.float32(5)
    t = np.where(small, w - np.float32(2.5), np.sqrt(w) - np.float32(3)).astype(np.float32)
    p = np.where(small, np.float32(_ERFINV_SMALL[0]), np.float32(_ERFINV_LARGE[0]))
    for cs, cl in zip(_ERFINV_SMALL[1:], _ERFINV_LARGE[1:]):
        p = _fma32(p, t, np.where(small, np.float32(cs), np.float32(cl)))
    r = p * x
    with np.errstate(invalid='ignore', divide='ignore'):
        return np.where(np.abs(x) == 1, x * np.float32(np.inf), r)


def normal_f32(seed, shape, layout='original'):
    """jax.random.normal(PRNGKey(seed), shape, float32)."""
    n = int(np.prod(shape))
    u = uniform_f32(random_bits(prng_key(seed), n, layout))
    return (np.float32(np.sqrt(2)) * erfinv_f32(u)).reshape(shape)
