// Fused x-axis pass of the Poisson solve for power-of-two meshes.
//
// The 3-D transforms of the force are split by axis: cuFFT does the 2-D
// (y, z) transforms of slabs of x-planes (so each slab's intermediate stays
// in the 129 MB L2), and this file does the x axis -- the slowest, strided
// one -- fused with the Fourier-space operators of pmwd/gravity.py:9-72:
//
//   forward force:  H = FFT_yz(rho)  ->  per (ky, kz) column:
//       P   = -(c / k^2) FFT_x(H)                       (laplace, k=0 -> 0)
//       G_0 = IFFT_x(-i kx P)                            (neg_grad, axis 0)
//       Q   = IFFT_x(P);  G_1 = -i ky Q;  G_2 = -i kz Q   (axes 1, 2: ky, kz are
//                                                         constant along x)
//     then g_j = IFFT_yz(G_j).  Two inverse x-transforms instead of three.
//   force VJP (transpose):  C_j = FFT_yz(mcot_j) ->
//       S = -(c / k^2) [ i kx FFT_x(C_0) + FFT_x(i ky C_1 + i kz C_2) ]
//       rho_cot = IFFT_yz(IFFT_x(S)).
// k components are the Nyquist-masked ones of neg_grad (gravity.py:37-44);
// c = 1.5 Omega_m / N folds in the real-space scale and irfftn's 1/N.
//
// One CTA transforms T columns (fixed ky, T consecutive kz) of length n0
// held in shared memory as padded complex (float2) buffers.  The length-n0
// FFT is a six-step transform n0 = R1 * R2: R2-strided DFTs of length R1
// with twiddles, then contiguous DFTs of length R2; each DFT runs in
// registers (radix-2, unrolled).  The second step, the Fourier-space
// operator and the first inverse step all act on the same contiguous group
// of R2 values, so one thread does them back to back in registers; the
// spectrum never needs natural order and no reordering pass exists.

#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <utility>

#include "pmx_internal.cuh"

namespace pmx {

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;

// cos/sin by their Taylor series on [-pi, pi], evaluated at compile time;
// used only for the exact small-radix twiddles exp(-2 pi i k / R), R <= 32.
constexpr double taylor_cos(double x) {
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 24; ++i) {
        term *= -x * x / ((2.0 * i - 1.0) * (2.0 * i));
        sum += term;
    }
    return sum;
}
constexpr double taylor_sin(double x) {
    double term = x, sum = x;
    for (int i = 1; i < 24; ++i) {
        term *= -x * x / ((2.0 * i) * (2.0 * i + 1.0));
        sum += term;
    }
    return sum;
}

struct Twiddle32 {
    float c[32], s[32];  // cos / sin of 2 pi k / 32
    constexpr Twiddle32() : c(), s() {
        for (int k = 0; k < 32; ++k) {
            double a = 2.0 * kPi * k / 32.0;
            if (a > kPi) a -= 2.0 * kPi;
            c[k] = (float)taylor_cos(a);
            s[k] = (float)taylor_sin(a);
        }
    }
};

__constant__ Twiddle32 c_tw32 = Twiddle32();

template <int R>
struct Log2 {
    static constexpr int v = R <= 1 ? 0 : 1 + Log2<R / 2>::v;
};
template <>
struct Log2<1> {
    static constexpr int v = 0;
};

// In-register DFT of length R (power of two, <= 32): natural-order input,
// output in bit-reversed order (element k holds frequency brev(k)); radix-2
// decimation in frequency.  The butterflies are generated by fold
// expressions so every register index is a compile-time constant (the
// arrays stay in registers).  INV selects exp(+2 pi i ...) (unnormalised).
template <int R, bool INV, int S, int J>
__device__ __forceinline__ void bfly(float (&re)[R], float (&im)[R]) {
    constexpr int half = 1 << (S - 1), len = 1 << S;
    constexpr int g = J / half, k = J % half;
    constexpr int a = g * len + k, b = a + half, ti = k * (32 >> S);
    const float ur = re[a], ui = im[a], vr = re[b], vi = im[b];
    re[a] = ur + vr;
    im[a] = ui + vi;
    const float dr = ur - vr, di = ui - vi;
    const float wc = c_tw32.c[ti];
    const float ws = INV ? c_tw32.s[ti] : -c_tw32.s[ti];
    re[b] = dr * wc - di * ws;
    im[b] = dr * ws + di * wc;
}

template <int R, bool INV, int S, int... Js>
__device__ __forceinline__ void dft_stage(float (&re)[R], float (&im)[R],
                                          std::integer_sequence<int, Js...>) {
    (bfly<R, INV, S, Js>(re, im), ...);
}

template <int R, bool INV, int... Ss>
__device__ __forceinline__ void dft_stages(float (&re)[R], float (&im)[R],
                                           std::integer_sequence<int, Ss...>) {
    (dft_stage<R, INV, Log2<R>::v - Ss>(re, im, std::make_integer_sequence<int, R / 2>{}), ...);
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float (&re)[R], float (&im)[R]) {
    dft_stages<R, INV>(re, im, std::make_integer_sequence<int, Log2<R>::v>{});
}

// bit reversal of the low `bits` bits
__device__ __forceinline__ int brev(int k, int bits) { return (int)(__brev((unsigned)k) >> (32 - bits)); }


constexpr int cbrev(int k, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((k >> b) & 1) << (bits - 1 - b);
    return r;
}

// out[i] = in[brev(i)]: bit-reversed register order -> natural order, with
// compile-time indices (fold expression).
template <int R, int... Is>
__device__ __forceinline__ void unbrev_impl(const float2 (&in)[R], float2 (&out)[R],
                                            std::integer_sequence<int, Is...>) {
    ((out[Is] = in[cbrev(Is, Log2<R>::v)]), ...);
}
template <int R>
__device__ __forceinline__ void unbrev(const float2 (&in)[R], float2 (&out)[R]) {
    unbrev_impl<R>(in, out, std::make_integer_sequence<int, R>{});
}

// float2 wrappers of the split-array register DFT
template <int R, bool INV, int... Is>
__device__ __forceinline__ void dft2_impl(float2 (&v)[R], std::integer_sequence<int, Is...>) {
    float re[R], im[R];
    ((re[Is] = v[Is].x, im[Is] = v[Is].y), ...);
    dft<R, INV>(re, im);
    ((v[Is] = make_float2(re[Is], im[Is])), ...);
}
template <int R, bool INV>
__device__ __forceinline__ void dft2(float2 (&v)[R]) {
    dft2_impl<R, INV>(v, std::make_integer_sequence<int, R>{});
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

template <int N>
struct Split;  // N = R1 * R2
template <> struct Split<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Split<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Split<256> { static constexpr int R1 = 16, R2 = 16; };
template <> struct Split<512> { static constexpr int R1 = 32, R2 = 16; };
template <> struct Split<1024> { static constexpr int R1 = 32, R2 = 32; };

constexpr int XT = 256;  // threads per x-pass CTA

// Column buffers of complex (float2) values: column t at t*CS, logical
// position p at p + p/R2 (one pad per R2 values keeps the strided and the
// contiguous DFT steps free of bank conflicts for 8-byte accesses; the +1
// per column does the same for the tile loads and stores).
template <int N>
struct XCfg {
    static constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2;
    static constexpr int RM = R1 > R2 ? R1 : R2;
    static constexpr int T = XT / RM;  // columns per CTA
    static constexpr int CS = N + N / R2 + 1;
    static constexpr int BUF = T * CS;  // float2 per buffer
    __device__ static __forceinline__ int at(int t, int p) { return t * CS + p + p / R2; }
};

// Forward step 1 on one buffer: R2-strided radix-R1 DFTs + twiddles,
// natural order -> "transposed" positions k1*R2 + b.
template <int N>
__device__ __forceinline__ void fwd_step1(float2 *buf, const float2 *tw) {
    using C = XCfg<N>;
    constexpr int R1 = C::R1, R2 = C::R2;
    for (int it = threadIdx.x; it < C::T * R2; it += XT) {
        const int t = it / R2, b = it % R2;
        float2 v[R1];
#pragma unroll
        for (int a = 0; a < R1; ++a) v[a] = buf[C::at(t, a * R2 + b)];
        dft2<R1, false>(v);
#pragma unroll
        for (int k = 0; k < R1; ++k) {
            const int k1 = brev(k, Log2<R1>::v);
            buf[C::at(t, k1 * R2 + b)] = cmul(v[k], tw[b * k1]);
        }
    }
}

// Inverse step 1 (the last inverse step) on one buffer: radix-R1 inverse
// DFTs over k1 at fixed b -> natural order.
template <int N>
__device__ __forceinline__ void inv_step1(float2 *buf) {
    using C = XCfg<N>;
    constexpr int R1 = C::R1, R2 = C::R2;
    for (int it = threadIdx.x; it < C::T * R2; it += XT) {
        const int t = it / R2, b = it % R2;
        float2 v[R1];
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) v[k1] = buf[C::at(t, k1 * R2 + b)];
        dft2<R1, true>(v);
#pragma unroll
        for (int k = 0; k < R1; ++k) buf[C::at(t, brev(k, Log2<R1>::v) * R2 + b)] = v[k];
    }
}

// Inverse step 2 on a register group in bit-reversed k2 order (as the
// forward step 2 leaves it), twiddle, store to positions k1*R2 + b.
template <int N>
__device__ __forceinline__ void inv_step2_store(float2 (&v)[XCfg<N>::R2], float2 *buf, int t,
                                                int k1, const float2 *tw) {
    using C = XCfg<N>;
    constexpr int R2 = C::R2;
    float2 u[R2];
    unbrev<R2>(v, u);           // natural k2 order
    dft2<R2, true>(u);          // element k holds b = brev(k)
#pragma unroll
    for (int k = 0; k < R2; ++k) {
        const int b = brev(k, Log2<R2>::v);
        buf[C::at(t, k1 * R2 + b)] = cmulc(u[k], tw[b * k1]);
    }
}

struct XGeom {
    int64_t n1, n2h;
    int64_t ncol_tiles;   // ceil(n2h / T)
    float c;              // 1.5 Omega_m / N
};

// Loads the column tile (fixed ky row j, kz in [l0, l0+T), all x) of a
// complex array laid out (x, ncomp, n1, n2h), component `comp`; optionally
// combines two components: out = (i k1m) in1 + (i k2m) in2.
template <int N>
__device__ __forceinline__ void load_tile(const float2 *__restrict__ src, int ncomp, int comp,
                                          int64_t j, int64_t l0, const XGeom &g, float2 *buf) {
    using C = XCfg<N>;
    constexpr int T = C::T;
    constexpr int PER = N * T / XT;
    constexpr int CH = PER < 16 ? PER : 16;
    const int t = threadIdx.x % T;
    const int x0 = threadIdx.x / T;
    const int64_t l = l0 + t;
    const bool ok = l < g.n2h;
    const float2 *base = src + ((int64_t)comp * g.n1 + j) * g.n2h + l;
    const int64_t xs = (int64_t)ncomp * g.n1 * g.n2h;
#pragma unroll
    for (int b = 0; b < PER; b += CH) {
        float2 v[CH];
#pragma unroll
        for (int r = 0; r < CH; ++r) {
            const int x = x0 + (b + r) * (XT / T);
            v[r] = ok ? __ldg(base + x * xs) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < CH; ++r) buf[C::at(t, x0 + (b + r) * (XT / T))] = v[r];
    }
}

template <int N>
__global__ void __launch_bounds__(XT) k_xpass_fwd(const float2 *__restrict__ H,
                                                  float2 *__restrict__ G,
                                                  const float *__restrict__ kt,
                                                  const float2 *__restrict__ twg, XGeom g,
                                                  int64_t n0) {
    using C = XCfg<N>;
    constexpr int T = C::T, R1 = C::R1, R2 = C::R2;
    extern __shared__ __align__(16) float2 smem2[];
    float2 *A = smem2, *B = smem2 + C::BUF;
    float2 *tw = smem2 + 2 * C::BUF;
    for (int m = threadIdx.x; m < N; m += XT) tw[m] = twg[m];

    const int64_t tot = n0 + g.n1 + g.n2h;
    const float *kx = kt, *ky = kt + n0, *kz = kt + n0 + g.n1;
    const float *mx = kt + tot, *my = kt + tot + n0, *mz = kt + tot + n0 + g.n1;

    for (int64_t tile = blockIdx.x; tile < g.n1 * g.ncol_tiles; tile += gridDim.x) {
        const int64_t j = tile / g.ncol_tiles;
        const int64_t l0 = (tile % g.ncol_tiles) * T;
        __syncthreads();  // buffers free (also orders the twiddle fill)
        load_tile<N>(H, 1, 0, j, l0, g, A);
        __syncthreads();
        fwd_step1<N>(A, tw);
        __syncthreads();
        // fused: forward step 2, Green + gradient, inverse step 2 of P and of
        // B = -i kx P, all on one thread's contiguous group
        const float kyj = __ldg(ky + j), myj = __ldg(my + j);
        const float ky2 = __fmul_rn(kyj, kyj);
        for (int it = threadIdx.x; it < T * R1; it += XT) {
            const int t = it / R1, k1 = it % R1;
            const int64_t l = l0 + t;
            const float kzl = l < g.n2h ? __ldg(kz + l) : 0.f;
            const float kz2 = __fmul_rn(kzl, kzl);
            float2 v[R2];
#pragma unroll
            for (int b = 0; b < R2; ++b) v[b] = A[C::at(t, k1 * R2 + b)];
            dft2<R2, false>(v);          // element k: kx index k1 + R1*brev(k)
            float2 w[R2];
#pragma unroll
            for (int k = 0; k < R2; ++k) {
                const int ix = k1 + R1 * brev(k, Log2<R2>::v);
                const float kxi = __ldg(kx + ix), mxi = __ldg(mx + ix);
                const float k2v = __fadd_rn(__fadd_rn(__fmul_rn(kxi, kxi), ky2), kz2);
                float pr = 0.f, pi = 0.f;
                if (k2v != 0.f) {
                    pr = -__fdiv_rn(__fmul_rn(v[k].x, g.c), k2v);
                    pi = -__fdiv_rn(__fmul_rn(v[k].y, g.c), k2v);
                }
                v[k] = make_float2(pr, pi);
                w[k] = make_float2(__fmul_rn(mxi, pi), -__fmul_rn(mxi, pr));  // -i kx P
            }
            inv_step2_store<N>(v, A, t, k1, tw);
            inv_step2_store<N>(w, B, t, k1, tw);
        }
        __syncthreads();
        inv_step1<N>(A);
        inv_step1<N>(B);
        __syncthreads();
        // G_0 = B; G_1 = -i ky Q; G_2 = -i kz Q  (Q in A); layout (x, 3, n1, n2h)
        for (int it = threadIdx.x; it < N * T; it += XT) {
            const int t = it % T, x = it / T;
            const int64_t l = l0 + t;
            if (l >= g.n2h) continue;
            const int q = C::at(t, x);
            const float2 Q = A[q];
            const float mzl = __ldg(mz + l);
            float2 *o = G + ((int64_t)x * 3 * g.n1 + j) * g.n2h + l;
            o[0] = B[q];
            o[g.n1 * g.n2h] = make_float2(__fmul_rn(myj, Q.y), -__fmul_rn(myj, Q.x));
            o[2 * g.n1 * g.n2h] = make_float2(__fmul_rn(mzl, Q.y), -__fmul_rn(mzl, Q.x));
        }
    }
}

template <int N>
__global__ void __launch_bounds__(XT) k_xpass_adj(const float2 *__restrict__ Cin,
                                                  float2 *__restrict__ S,
                                                  const float *__restrict__ kt,
                                                  const float2 *__restrict__ twg, XGeom g,
                                                  int64_t n0) {
    using C = XCfg<N>;
    constexpr int T = C::T, R1 = C::R1, R2 = C::R2;
    extern __shared__ __align__(16) float2 smem2[];
    float2 *A = smem2, *B = smem2 + C::BUF;
    float2 *tw = smem2 + 2 * C::BUF;
    for (int m = threadIdx.x; m < N; m += XT) tw[m] = twg[m];

    const int64_t tot = n0 + g.n1 + g.n2h;
    const float *kx = kt, *ky = kt + n0, *kz = kt + n0 + g.n1;
    const float *mx = kt + tot, *my = kt + tot + n0, *mz = kt + tot + n0 + g.n1;

    for (int64_t tile = blockIdx.x; tile < g.n1 * g.ncol_tiles; tile += gridDim.x) {
        const int64_t j = tile / g.ncol_tiles;
        const int64_t l0 = (tile % g.ncol_tiles) * T;
        const float myj = __ldg(my + j);
        __syncthreads();
        // A = C_0;  B = i ky C_1 + i kz C_2   (i k (a + i b) = (-k b, k a))
        load_tile<N>(Cin, 3, 0, j, l0, g, A);
        {
            constexpr int PER = N * T / XT;
            constexpr int CH = PER < 8 ? PER : 8;
            const int t = threadIdx.x % T, x0 = threadIdx.x / T;
            const int64_t l = l0 + t;
            const bool ok = l < g.n2h;
            const float mzl = ok ? __ldg(mz + l) : 0.f;
            const int64_t cs = g.n1 * g.n2h, xs = 3 * cs;
            const float2 *base = Cin + j * g.n2h + l;
#pragma unroll
            for (int b = 0; b < PER; b += CH) {
                float2 c1[CH], c2[CH];
#pragma unroll
                for (int r = 0; r < CH; ++r) {
                    const int x = x0 + (b + r) * (XT / T);
                    c1[r] = ok ? __ldg(base + x * xs + cs) : make_float2(0.f, 0.f);
                    c2[r] = ok ? __ldg(base + x * xs + 2 * cs) : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int r = 0; r < CH; ++r)
                    B[C::at(t, x0 + (b + r) * (XT / T))] =
                        make_float2(-__fadd_rn(__fmul_rn(myj, c1[r].y), __fmul_rn(mzl, c2[r].y)),
                                    __fadd_rn(__fmul_rn(myj, c1[r].x), __fmul_rn(mzl, c2[r].x)));
            }
        }
        __syncthreads();
        fwd_step1<N>(A, tw);
        fwd_step1<N>(B, tw);
        __syncthreads();
        const float kyj = __ldg(ky + j);
        const float ky2 = __fmul_rn(kyj, kyj);
        for (int it = threadIdx.x; it < T * R1; it += XT) {
            const int t = it / R1, k1 = it % R1;
            const int64_t l = l0 + t;
            const float kzl = l < g.n2h ? __ldg(kz + l) : 0.f;
            const float kz2 = __fmul_rn(kzl, kzl);
            float2 v[R2], w[R2];
#pragma unroll
            for (int b = 0; b < R2; ++b) v[b] = A[C::at(t, k1 * R2 + b)];
            dft2<R2, false>(v);
#pragma unroll
            for (int b = 0; b < R2; ++b) w[b] = B[C::at(t, k1 * R2 + b)];
            dft2<R2, false>(w);
#pragma unroll
            for (int k = 0; k < R2; ++k) {
                const int ix = k1 + R1 * brev(k, Log2<R2>::v);
                const float kxi = __ldg(kx + ix), mxi = __ldg(mx + ix);
                const float k2v = __fadd_rn(__fadd_rn(__fmul_rn(kxi, kxi), ky2), kz2);
                const float re = __fadd_rn(-__fmul_rn(mxi, v[k].y), w[k].x);
                const float im = __fadd_rn(__fmul_rn(mxi, v[k].x), w[k].y);
                float sr = 0.f, si = 0.f;
                if (k2v != 0.f) {
                    sr = -__fdiv_rn(__fmul_rn(re, g.c), k2v);
                    si = -__fdiv_rn(__fmul_rn(im, g.c), k2v);
                }
                v[k] = make_float2(sr, si);
            }
            inv_step2_store<N>(v, A, t, k1, tw);
        }
        __syncthreads();
        inv_step1<N>(A);
        __syncthreads();
        for (int it = threadIdx.x; it < N * T; it += XT) {
            const int t = it % T, x = it / T;
            const int64_t l = l0 + t;
            if (l >= g.n2h) continue;
            S[((int64_t)x * g.n1 + j) * g.n2h + l] = A[C::at(t, x)];
        }
    }
}

template <int N>
size_t xpass_smem() {
    return (size_t)(2 * XCfg<N>::BUF + N) * sizeof(float2);
}

template <int N>
int launch_xpass(bool adj, const float2 *in, float2 *out, const float *kt, const float2 *tw,
                 int64_t n1, int64_t n2h, float c, cudaStream_t st) {
    XGeom g;
    g.n1 = n1;
    g.n2h = n2h;
    g.ncol_tiles = (n2h + XCfg<N>::T - 1) / XCfg<N>::T;
    g.c = c;
    const size_t sm = xpass_smem<N>();
    const int64_t tiles = n1 * g.ncol_tiles;
    const int per_sm = sm > 110 * 1024 ? 1 : (sm > 72 * 1024 ? 2 : 3);
    const int64_t cap = (int64_t)device_sms() * per_sm;
    const int grid = (int)(tiles < cap ? tiles : cap);
    if (adj) {
        PMX_CUDA(cudaFuncSetAttribute(k_xpass_adj<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sm));
        k_xpass_adj<N><<<grid, XT, sm, st>>>(in, out, kt, tw, g, (int64_t)N);
        PMX_LAUNCH_CHECK("k_xpass_adj");
    } else {
        PMX_CUDA(cudaFuncSetAttribute(k_xpass_fwd<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sm));
        k_xpass_fwd<N><<<grid, XT, sm, st>>>(in, out, kt, tw, g, (int64_t)N);
        PMX_LAUNCH_CHECK("k_xpass_fwd");
    }
    return PMX_OK;
}

}  // namespace

bool xpass_supported(int64_t n0) {
    return n0 == 64 || n0 == 128 || n0 == 256 || n0 == 512 || n0 == 1024;
}

int xpass(bool adj, const float2 *in, float2 *out, const float *kt, const float2 *tw, int64_t n0,
          int64_t n1, int64_t n2h, float c, cudaStream_t st) {
    switch (n0) {
        case 64: return launch_xpass<64>(adj, in, out, kt, tw, n1, n2h, c, st);
        case 128: return launch_xpass<128>(adj, in, out, kt, tw, n1, n2h, c, st);
        case 256: return launch_xpass<256>(adj, in, out, kt, tw, n1, n2h, c, st);
        case 512: return launch_xpass<512>(adj, in, out, kt, tw, n1, n2h, c, st);
        case 1024: return launch_xpass<1024>(adj, in, out, kt, tw, n1, n2h, c, st);
        default: return fail(PMX_ERR_SHAPE, "x-pass needs n0 in {64, 128, 256, 512, 1024}");
    }
}

// exp(-2 pi i m / n) for m in [0, n), in float64 on the host, then float32.
void xpass_twiddles(int64_t n, float2 *host) {
    for (int64_t m = 0; m < n; ++m) {
        double a = -2.0 * kPi * (double)m / (double)n;
        host[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
}

}  // namespace pmx
