// White noise of pmwd's initial conditions (pmwd/modes.py:12-49), drawn on
// the GPU with the same values the reference draws.
//
// pmwd calls jax.random.normal(PRNGKey(seed), shape, float32).  JAX's
// published algorithm, restated here:
//  * the counter-based Threefry-2x32 hash, 20 rounds (Salmon et al. 2011,
//    the Random123 family): rotations 13 15 26 6 / 17 29 16 24, a key
//    injection after every 4 rounds, key parity 0x1BD11BDA;
//  * 32 random bits per value in one of two counter layouts.  ORIGINAL
//    (jax_threefry_partitionable off, JAX's default before 0.5): counters
//    0..n-1, padded with a 0 to even length, are hashed as the pairs
//    (j, j + h), h = half the padded length, and value j takes output word 0,
//    value j + h output word 1.  PARTITIONABLE: value i hashes the 64-bit
//    counter (i >> 32, i & 0xffffffff) and takes the XOR of the two words;
//  * a uniform u in [nextafter(-1, 0), 1): the top 23 bits as the mantissa
//    of a float in [1, 2), minus 1, times 2, plus nextafter(-1, 0);
//  * sqrt(2) erfinv(u), erfinv by Giles' single-precision approximation
//    (M. Giles, "Approximating the erfinv function", GPU Computing Gems Jade
//    Edition, 2011): w = -log1p(-u^2), then a degree-8 polynomial in
//    w - 2.5 (w < 5) or sqrt(w) - 3, each Horner step a fused multiply-add.
//
// Both layouts are one pass writing 4 bytes per value; the hash (about 90
// integer operations per pair) bounds it, not HBM.

#include "pmx_internal.cuh"

namespace pmx {
namespace {

constexpr int NT = 256;

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int s) { return __funnelshift_l(x, x, s); }

__device__ __forceinline__ void threefry2x32(uint32_t k0, uint32_t k1, uint32_t &x0,
                                             uint32_t &x1) {
    const uint32_t ks[3] = {k0, k1, k0 ^ k1 ^ 0x1BD11BDAu};
    constexpr int rot[8] = {13, 15, 26, 6, 17, 29, 16, 24};
    x0 += ks[0];
    x1 += ks[1];
#pragma unroll
    for (int r = 0; r < 20; ++r) {
        x0 += x1;
        x1 = rotl32(x1, rot[r % 8]);
        x1 ^= x0;
        if (r % 4 == 3) {
            const int i = (r + 1) / 4;
            x0 += ks[i % 3];
            x1 += ks[(i + 1) % 3] + (uint32_t)i;
        }
    }
}

__device__ __forceinline__ float bits_to_normal(uint32_t bits) {
    const float lo = -0.99999994f;  // nextafter(-1, 0)
    const float f = __uint_as_float((bits >> 9) | 0x3F800000u) - 1.0f;
    float u = fmaxf(lo, __fadd_rn(__fmul_rn(f, 2.0f), lo));  // f * 2 exact: one rounding
    // Giles' single-precision erfinv
    float w = -log1pf(-__fmul_rn(u, u));
    float p;
    if (w < 5.0f) {
        w = w - 2.5f;
        p = 2.81022636e-08f;
        p = fmaf(p, w, 3.43273939e-07f);
        p = fmaf(p, w, -3.5233877e-06f);
        p = fmaf(p, w, -4.39150654e-06f);
        p = fmaf(p, w, 0.00021858087f);
        p = fmaf(p, w, -0.00125372503f);
        p = fmaf(p, w, -0.00417768164f);
        p = fmaf(p, w, 0.246640727f);
        p = fmaf(p, w, 1.50140941f);
    } else {
        w = sqrtf(w) - 3.0f;
        p = -0.000200214257f;
        p = fmaf(p, w, 0.000100950558f);
        p = fmaf(p, w, 0.00134934322f);
        p = fmaf(p, w, -0.00367342844f);
        p = fmaf(p, w, 0.00573950773f);
        p = fmaf(p, w, -0.0076224613f);
        p = fmaf(p, w, 0.00943887047f);
        p = fmaf(p, w, 1.00167406f);
        p = fmaf(p, w, 2.83297682f);
    }
    const float e = fabsf(u) == 1.0f ? u * __int_as_float(0x7f800000) : __fmul_rn(p, u);
    return __fmul_rn(1.41421356f, e);
}

template <bool NORMAL>
__device__ __forceinline__ void store(void *out, int64_t i, uint32_t bits) {
    if (NORMAL)
        static_cast<float *>(out)[i] = bits_to_normal(bits);
    else
        static_cast<uint32_t *>(out)[i] = bits;
}

// original layout: thread j hashes the counter pair (j, j + h) and writes
// values j and j + h (coalesced in both halves); with n odd the last pair's
// second counter is the pad 0 and its second word is dropped
template <bool NORMAL>
__global__ void __launch_bounds__(NT) k_bits_original(uint32_t k0, uint32_t k1, int64_t n,
                                                      void *out) {
    const int64_t h = (n + 1) / 2;
    for (int64_t j = blockIdx.x * (int64_t)NT + threadIdx.x; j < h;
         j += (int64_t)gridDim.x * NT) {
        uint32_t x0 = (uint32_t)j;
        uint32_t x1 = j + h < n ? (uint32_t)(j + h) : 0u;
        threefry2x32(k0, k1, x0, x1);
        store<NORMAL>(out, j, x0);
        if (j + h < n) store<NORMAL>(out, j + h, x1);
    }
}

template <bool NORMAL>
__global__ void __launch_bounds__(NT) k_bits_partitionable(uint32_t k0, uint32_t k1, int64_t n,
                                                           void *out) {
    for (int64_t i = blockIdx.x * (int64_t)NT + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * NT) {
        uint32_t x0 = (uint32_t)((uint64_t)i >> 32), x1 = (uint32_t)i;
        threefry2x32(k0, k1, x0, x1);
        store<NORMAL>(out, i, x0 ^ x1);
    }
}

template <bool NORMAL>
int draw(uint32_t k0, uint32_t k1, int64_t n, int layout, void *out, void *stream) {
    clear_error();
    if (n < 0) return fail(PMX_ERR_ARG, "negative count");
    if (n == 0) return PMX_OK;
    if (!out) return fail(PMX_ERR_ARG, "null output");
    if (reinterpret_cast<uintptr_t>(out) % 4) return fail(PMX_ERR_ALIGN, "output not 4-byte aligned");
    cudaStream_t st = as_stream(stream);
    if (layout == PMX_PRNG_ORIGINAL) {
        // JAX draws more than 2^32 - 2 values of one key through split keys,
        // which this layout does not restate
        if (n >= (int64_t)0xFFFFFFFF)
            return fail(PMX_ERR_SHAPE, "the original counter layout covers at most 2^32 - 2 values");
        k_bits_original<NORMAL><<<stride_grid((n + 1) / 2, NT), NT, 0, st>>>(k0, k1, n, out);
    } else if (layout == PMX_PRNG_PARTITIONABLE) {
        k_bits_partitionable<NORMAL><<<stride_grid(n, NT), NT, 0, st>>>(k0, k1, n, out);
    } else {
        return fail(PMX_ERR_ARG, "unknown counter layout");
    }
    PMX_LAUNCH_CHECK("white noise");
    return PMX_OK;
}

}  // namespace
}  // namespace pmx

extern "C" int pmx_random_bits(uint32_t k0, uint32_t k1, int64_t n, int layout, uint32_t *out,
                               void *stream) {
    return pmx::draw<false>(k0, k1, n, layout, out, stream);
}

extern "C" int pmx_normal(uint32_t k0, uint32_t k1, int64_t n, int layout, float *out,
                          void *stream) {
    return pmx::draw<true>(k0, k1, n, layout, out, stream);
}
