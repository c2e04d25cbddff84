// Internal device/host helpers shared by the libpmx translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/pmx.h"

namespace pmx {

// ---------------------------------------------------------------------------
// error reporting (thread-local message behind pmx_last_error)
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
void clear_error();
int fail(int code, const std::string &msg);
int cuda_status(cudaError_t e, const char *what);

#define PMX_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) return ::pmx::cuda_status(e_, #call);          \
    } while (0)

#define PMX_LAUNCH_CHECK(what)                                                \
    do {                                                                      \
        cudaError_t e_ = cudaGetLastError();                                  \
        if (e_ != cudaSuccess) return ::pmx::cuda_status(e_, what);           \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

int device_sms();

// Grid for grid-stride kernels: enough blocks to fill every SM several times,
// never more than the work needs.
inline int stride_grid(int64_t work, int threads, int per_sm = 8) {
    int64_t need = (work + threads - 1) / threads;
    int64_t cap = (int64_t)device_sms() * per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

// ---------------------------------------------------------------------------
// enmesh parameters (pm_util.py:33-156), resolved on the host from
// pmx_enmesh_spec.  The kernels always work on 3 internal axes; a dim < 3
// problem is embedded as singleton leading axes (pmid 0, disp 0, shape 1),
// which reproduces the reference's fractions exactly (the padded factors
// are 1 and 0).
// ---------------------------------------------------------------------------
struct EmParams {
    int dim;           // user spatial dims
    int pad;           // 3 - dim: internal axes [0, pad) are singleton
    int wrap[3];       // s1 per internal axis (0: no wrapping, s1 = None)
    int drop;          // without wrapping: negative indices -> s2
    int64_t shape[3];  // s2 per internal axis
    int64_t stride[3]; // mesh cell stride per internal axis
    int f64;           // 1: non-default (float64) branch, pm_util.py:99-118
    // default branch (pm_util.py:119-137)
    float cellf;       // a1 as float32
    int i12[3];        // integer part of offset / a1 (jnp.divmod)
    float d12[3];      // remainder, cast to float32
    // float64 branch
    double a1d, a2d;
    double b12[3];
    double L[3];       // s1 * a1
    float a2f;
    // scatter/gather adjoints divide disp_cot by this (f32 of cell_size or
    // conf.cell_size), scatter.py:116 / gather.py:110
    float cot_div;
};

int make_em_params(const pmx_enmesh_spec *spec, EmParams *p);

// Fused x-axis pass of the Poisson solve (pmx_fft.cu).  Forward (adj =
// false): in = FFT_yz(rho) (n0, n1, n2h), out = the three gradient spectra
// (n0, 3, n1, n2h) after the inverse x transform.  Adjoint: in = FFT_yz of
// the three mesh cotangents (n0, 3, n1, n2h), out = (n0, n1, n2h).
// Complex rows hold n2h values at a stride of rs >= n2h elements.
bool xpass_supported(int64_t n0);
int xpass(bool adj, const float2 *in, float2 *out, const float *kt, const float2 *tw, int64_t n0,
          int64_t n1, int64_t n2h, int64_t rs, float c, cudaStream_t st);
// n2h rounded up to a multiple of 4 complex values (32 bytes): the complex
// row stride of the plane-kernel path, so every column tile of a plane
// covers whole 32-byte sectors (HBM3e has no byte-masked writes).
inline int64_t padded_row(int64_t n2h) { return (n2h + 3) & ~(int64_t)3; }
void xpass_twiddles(int64_t n, float2 *host);

// 2-D (y, z) transforms of consecutive planes (pmx_fft.cu): forward real
// (n1, n2) -> complex (n1, n2/2+1) at row stride padded_row(n2/2+1); inverse
// complex -> real through a scratch plane per cluster (n1 * padded_row
// complex values each, plane_max_clusters of them).  One thread-block cluster
// per plane.  ptw holds plane_twiddles(n1, n2) (2 n1 + 1 entries).
bool plane_supported(int64_t n1, int64_t n2);
// c16: clusters of 16 CTAs (non-portable size) instead of 8.
int plane_max_clusters(int64_t n1, int64_t n2, bool c16, int *ncl);
int plane_fft(bool inv, const void *in, void *out, const float2 *ptw, int64_t nplanes, int64_t n1,
              int64_t n2, float2 *scratch, int max_clusters, bool c16, cudaStream_t st);
void plane_twiddles(int64_t n1, int64_t n2, float2 *host);

__device__ __forceinline__ int pymod(int x, int m) {
    int r = x % m;
    return r < 0 ? r + m : r;
}

__device__ __forceinline__ float sgnf(float x) {
    // jnp.sign: -1, 0 (signed), +1
    return x > 0.f ? 1.f : (x < 0.f ? -1.f : x);
}

// jnp.remainder for doubles (sign of divisor)
__device__ __forceinline__ double pyfmod(double x, double m) {
    double t = fmod(x, m);
    if (t != 0.0 && ((t < 0.0) != (m < 0.0))) t = __dadd_rn(t, m);
    return t;
}

// jnp.floor_divide for doubles (CPython float_divmod + round half away)
__device__ __forceinline__ double floordiv(double x, double y) {
    double mod = fmod(x, y);
    double div = __ddiv_rn(__dsub_rn(x, mod), y);
    if (mod != 0.0 && ((y < 0.0) != (mod < 0.0))) div = __dsub_rn(div, 1.0);
    return round(div);
}

// Per-axis neighbour data: indices (wrapped by s1, not dropped), fractions
// and the signs sign(-d2) used by the fraction gradients.
struct Axis {
    int i[2];
    float w[2];
    float s[2];
    int u;  // unwrapped index of the lower neighbour (hot path only)
};

__device__ __forceinline__ void enmesh_axis(const EmParams &p, int a, int pm, float d,
                                            Axis &ax) {
    if (a < p.pad) {
        ax.i[0] = 0; ax.i[1] = 0;
        ax.w[0] = 1.f; ax.w[1] = 0.f;
        ax.s[0] = 0.f; ax.s[1] = 1.f;
        return;
    }
    if (!p.f64) {
        int ip = pm - p.i12[a];
        float x = __fdiv_rn(__fsub_rn(d, p.d12[a]), p.cellf);
        int fl = (int)floorf(x);
#pragma unroll
        for (int nb = 0; nb < 2; ++nb) {
            int ii = fl + nb;
            float d2 = __fsub_rn(x, (float)ii);
            ax.w[nb] = __fsub_rn(1.f, fabsf(d2));
            ax.s[nb] = sgnf(-d2);
            // without wrapping, the reference's int16 sum (two's complement)
            ax.i[nb] = p.wrap[a] ? pymod(ii + ip, p.wrap[a]) : (int)(short)(ii + ip);
        }
    } else {
        double P = __dsub_rn(__dadd_rn(__dmul_rn((double)pm, p.a1d), (double)d), p.b12[a]);
#pragma unroll
        for (int nb = 0; nb < 2; ++nb) {
            double x = nb ? __dadd_rn(P, p.a2d) : P;
            if (p.wrap[a]) x = pyfmod(x, p.L[a]);
            double q = floordiv(x, p.a2d);
            double d2 = __dsub_rn(P, __dmul_rn(q, p.a2d));
            if (p.wrap[a]) d2 = __dsub_rn(d2, __dmul_rn(rint(__ddiv_rn(d2, p.L[a])), p.L[a]));
            float d2f = __fdiv_rn((float)d2, p.a2f);
            ax.w[nb] = __fsub_rn(1.f, fabsf(d2f));
            ax.s[nb] = sgnf(-d2f);
            ax.i[nb] = (int)(short)(int)q;
        }
    }
    // pm_util.py:139-140: without wrapping, negative indices are set to s2
    if (!p.wrap[a] && p.drop) {
#pragma unroll
        for (int nb = 0; nb < 2; ++nb)
            if (ax.i[nb] < 0) ax.i[nb] = (int)p.shape[a];
    }
}

// Loads one particle (3 internal axes) from row-major (n, dim) arrays.
template <typename IT>
__device__ __forceinline__ void load_particle(const EmParams &p, const IT *pmid,
                                              const float *disp, int64_t q,
                                              int pm[3], float dd[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int u = a - p.pad;
        if (u >= 0) {
            pm[a] = (int)pmid[q * p.dim + u];
            dd[a] = disp[q * p.dim + u];
        } else {
            pm[a] = 0;
            dd[a] = 0.f;
        }
    }
}

// Raveled cell of neighbour k (bit a of k selects neighbour along internal
// axis a, matching pm_util.py:95-97), or -1 when dropped (index >= s2).
__device__ __forceinline__ int64_t cell_of(const EmParams &p, const Axis ax[3], int k) {
    int64_t off = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int ii = ax[a].i[(k >> a) & 1];
        // wrapped indices are never negative; a negative one can only come
        // from int16 overflow of a huge displacement and is dropped
        if (ii < 0 || (int64_t)ii >= p.shape[a]) return -1;
        off += (int64_t)ii * p.stride[a];
    }
    return off;
}

__device__ __forceinline__ float frac_of(const Axis ax[3], int k) {
    return __fmul_rn(__fmul_rn(ax[0].w[k & 1], ax[1].w[(k >> 1) & 1]), ax[2].w[(k >> 2) & 1]);
}

// d frac / d (x_a / cell): sign(-d2_a) times the product of the other axes'
// fractions in the reference's order (a+1, ..., dim-1, 0, ..., a-1).
__device__ __forceinline__ void frac_grad_of(const Axis ax[3], int k, float g[3]) {
    float w0 = ax[0].w[k & 1], w1 = ax[1].w[(k >> 1) & 1], w2 = ax[2].w[(k >> 2) & 1];
    g[0] = __fmul_rn(ax[0].s[k & 1], __fmul_rn(w1, w2));
    g[1] = __fmul_rn(ax[1].s[(k >> 1) & 1], __fmul_rn(w2, w0));
    g[2] = __fmul_rn(ax[2].s[(k >> 2) & 1], __fmul_rn(w0, w1));
}

// Deterministic block sum of one double per thread; thread 0 gets the total.
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < THREADS / 32; ++w) t += sh[w];
    }
    __syncthreads();
    return t;
}

}  // namespace pmx
