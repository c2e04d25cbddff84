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
// held in shared memory as split re/im float arrays.  The length-n0 FFT is
// a six-step transform n0 = R1 * R2: R2-strided DFTs of length R1 with
// twiddles, then contiguous DFTs of length R2; each DFT runs in registers
// (radix-2, unrolled).  The forward leaves the spectrum in the transposed
// order p = k1*R2 + k2 <-> kx = k1 + R1*k2, which the inverse consumes
// directly and returns to natural order, so no reordering pass is needed.

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

// Column buffer geometry: column t of length N stored at t*CS, logical
// position p at p + p/R2 (one pad float per R2 values, so both the strided
// and the contiguous DFT steps are free of bank conflicts).
template <int N, int R2>
struct Col {
    static constexpr int CS = N + N / R2;
    __device__ static __forceinline__ int at(int t, int p) { return t * CS + p + p / R2; }
};

template <int N>
struct Split;  // N = R1 * R2
template <> struct Split<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Split<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Split<256> { static constexpr int R1 = 16, R2 = 16; };
template <> struct Split<512> { static constexpr int R1 = 32, R2 = 16; };
template <> struct Split<1024> { static constexpr int R1 = 32, R2 = 32; };

constexpr int XT = 256;  // threads per x-pass CTA

template <int N>
struct XCfg {
    static constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2;
    static constexpr int RM = R1 > R2 ? R1 : R2;
    static constexpr int T = XT / RM;  // columns per CTA
    static constexpr int CS = Col<N, R2>::CS;
    static constexpr int BUF = T * CS;  // floats per re (or im) buffer
};

// Forward FFT (natural -> transposed order) of the T columns in (re, im).
// tw = exp(-2 pi i m / N), m in [0, N).
template <int N>
__device__ __forceinline__ void fft_fwd(float *re, float *im, const float2 *tw) {
    using C = XCfg<N>;
    constexpr int R1 = C::R1, R2 = C::R2;
    for (int it = threadIdx.x; it < C::T * R2; it += XT) {
        const int t = it / R2, b = it % R2;
        float xr[R1], xi[R1];
#pragma unroll
        for (int a = 0; a < R1; ++a) {
            const int q = Col<N, R2>::at(t, a * R2 + b);
            xr[a] = re[q];
            xi[a] = im[q];
        }
        dft<R1, false>(xr, xi);
#pragma unroll
        for (int k = 0; k < R1; ++k) {
            const int k1 = brev(k, Log2<R1>::v);
            const float2 w = tw[(b * k1) & (N - 1)];
            const float r = xr[k] * w.x - xi[k] * w.y;
            const float i = xr[k] * w.y + xi[k] * w.x;
            const int q = Col<N, R2>::at(t, k1 * R2 + b);
            re[q] = r;
            im[q] = i;
        }
    }
    __syncthreads();
    for (int it = threadIdx.x; it < C::T * R1; it += XT) {
        const int t = it / R1, k1 = it % R1;
        float xr[R2], xi[R2];
#pragma unroll
        for (int b = 0; b < R2; ++b) {
            const int q = Col<N, R2>::at(t, k1 * R2 + b);
            xr[b] = re[q];
            xi[b] = im[q];
        }
        dft<R2, false>(xr, xi);
#pragma unroll
        for (int k = 0; k < R2; ++k) {
            const int q = Col<N, R2>::at(t, k1 * R2 + brev(k, Log2<R2>::v));
            re[q] = xr[k];
            im[q] = xi[k];
        }
    }
    __syncthreads();
}

// Unnormalised inverse FFT (transposed -> natural order), the exact
// reversal of fft_fwd's index maps.
template <int N>
__device__ __forceinline__ void fft_inv(float *re, float *im, const float2 *tw) {
    using C = XCfg<N>;
    constexpr int R1 = C::R1, R2 = C::R2;
    for (int it = threadIdx.x; it < C::T * R1; it += XT) {
        const int t = it / R1, k1 = it % R1;
        float xr[R2], xi[R2];
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
            const int q = Col<N, R2>::at(t, k1 * R2 + k2);
            xr[k2] = re[q];
            xi[k2] = im[q];
        }
        dft<R2, true>(xr, xi);
#pragma unroll
        for (int k = 0; k < R2; ++k) {
            const int b = brev(k, Log2<R2>::v);
            const float2 w = tw[(b * k1) & (N - 1)];  // conj(w) below
            const float r = xr[k] * w.x + xi[k] * w.y;
            const float i = xi[k] * w.x - xr[k] * w.y;
            const int q = Col<N, R2>::at(t, k1 * R2 + b);
            re[q] = r;
            im[q] = i;
        }
    }
    __syncthreads();
    for (int it = threadIdx.x; it < C::T * R2; it += XT) {
        const int t = it / R2, b = it % R2;
        float xr[R1], xi[R1];
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) {
            const int q = Col<N, R2>::at(t, k1 * R2 + b);
            xr[k1] = re[q];
            xi[k1] = im[q];
        }
        dft<R1, true>(xr, xi);
#pragma unroll
        for (int k = 0; k < R1; ++k) {
            const int q = Col<N, R2>::at(t, brev(k, Log2<R1>::v) * R2 + b);
            re[q] = xr[k];
            im[q] = xi[k];
        }
    }
    __syncthreads();
}

struct XGeom {
    int64_t n1, n2h;
    int64_t ncol_tiles;   // ceil(n2h / T)
    float c;              // 1.5 Omega_m / N
};

// Loads column tile (fixed ky row j, kz in [l0, l0+T)) of a complex array
// laid out (x, comp, n1, n2h) with `ncomp` components; component `comp`.
template <int N>
__device__ __forceinline__ void load_tile(const float2 *__restrict__ src, int ncomp, int comp,
                                          int64_t j, int64_t l0, const XGeom &g, float *re,
                                          float *im) {
    using C = XCfg<N>;
    constexpr int T = C::T;
    constexpr int PER = N * T / XT;          // elements per thread
    constexpr int CH = PER < 16 ? PER : 16;  // loads kept in flight per batch
    const int t = threadIdx.x % T;           // this thread's column
    const int x0 = threadIdx.x / T;          // and its first x (stride XT/T)
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
        for (int r = 0; r < CH; ++r) {
            const int q = Col<N, C::R2>::at(t, x0 + (b + r) * (XT / T));
            re[q] = v[r].x;
            im[q] = v[r].y;
        }
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
    extern __shared__ float smem[];
    float *are = smem, *aim = smem + C::BUF;
    float *bre = smem + 2 * C::BUF, *bim = smem + 3 * C::BUF;
    float2 *tw = reinterpret_cast<float2 *>(smem + 4 * C::BUF);
    for (int m = threadIdx.x; m < N; m += XT) tw[m] = twg[m];

    const int64_t tot = n0 + g.n1 + g.n2h;
    const float *kx = kt, *ky = kt + n0, *kz = kt + n0 + g.n1;
    const float *mx = kt + tot, *my = kt + tot + n0, *mz = kt + tot + n0 + g.n1;

    for (int64_t tile = blockIdx.x; tile < g.n1 * g.ncol_tiles; tile += gridDim.x) {
        const int64_t j = tile / g.ncol_tiles;
        const int64_t l0 = (tile % g.ncol_tiles) * T;
        __syncthreads();  // previous tile's buffers are free
        load_tile<N>(H, 1, 0, j, l0, g, are, aim);
        __syncthreads();
        fft_fwd<N>(are, aim, tw);
        // P = -(c/k^2) F in A;  B = -i kx P
        const float kyj = __ldg(ky + j), myj = __ldg(my + j);
        const float ky2 = __fmul_rn(kyj, kyj);
        for (int it = threadIdx.x; it < N * T; it += XT) {
            const int t = it / N, p = it % N;
            const int k1 = p / R2, k2 = p % R2;
            const int ix = k1 + R1 * k2;
            const int64_t l = l0 + t;
            const float kxi = __ldg(kx + ix), mxi = __ldg(mx + ix);
            const float kzl = l < g.n2h ? __ldg(kz + l) : 0.f;
            const float k2v = __fadd_rn(__fadd_rn(__fmul_rn(kxi, kxi), ky2), __fmul_rn(kzl, kzl));
            const int q = Col<N, R2>::at(t, p);
            float pr = 0.f, pi = 0.f;
            if (k2v != 0.f) {
                pr = -__fdiv_rn(__fmul_rn(are[q], g.c), k2v);
                pi = -__fdiv_rn(__fmul_rn(aim[q], g.c), k2v);
            }
            are[q] = pr;
            aim[q] = pi;
            // (-i k)(pr + i pi) = (k pi, -k pr)
            bre[q] = __fmul_rn(mxi, pi);
            bim[q] = -__fmul_rn(mxi, pr);
        }
        __syncthreads();
        fft_inv<N>(bre, bim, tw);
        fft_inv<N>(are, aim, tw);
        // G_0 = B; G_1 = -i ky Q; G_2 = -i kz Q  (Q in A), layout (x, 3, n1, n2h)
        for (int it = threadIdx.x; it < N * T; it += XT) {
            const int t = it % T, x = it / T;
            const int64_t l = l0 + t;
            if (l >= g.n2h) continue;
            const int q = Col<N, R2>::at(t, x);
            const float qr = are[q], qi = aim[q];
            const float mzl = __ldg(mz + l);
            float2 *o = G + ((int64_t)x * 3 * g.n1 + j) * g.n2h + l;
            o[0] = make_float2(bre[q], bim[q]);
            o[g.n1 * g.n2h] = make_float2(__fmul_rn(myj, qi), -__fmul_rn(myj, qr));
            o[2 * g.n1 * g.n2h] = make_float2(__fmul_rn(mzl, qi), -__fmul_rn(mzl, qr));
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
    extern __shared__ float smem[];
    float *are = smem, *aim = smem + C::BUF;
    float *bre = smem + 2 * C::BUF, *bim = smem + 3 * C::BUF;
    float2 *tw = reinterpret_cast<float2 *>(smem + 4 * C::BUF);
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
        load_tile<N>(Cin, 3, 0, j, l0, g, are, aim);
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
                for (int r = 0; r < CH; ++r) {
                    const int q = Col<N, R2>::at(t, x0 + (b + r) * (XT / T));
                    bre[q] = -__fadd_rn(__fmul_rn(myj, c1[r].y), __fmul_rn(mzl, c2[r].y));
                    bim[q] = __fadd_rn(__fmul_rn(myj, c1[r].x), __fmul_rn(mzl, c2[r].x));
                }
            }
        }
        __syncthreads();
        fft_fwd<N>(are, aim, tw);
        fft_fwd<N>(bre, bim, tw);
        const float kyj = __ldg(ky + j);
        const float ky2 = __fmul_rn(kyj, kyj);
        for (int it = threadIdx.x; it < N * T; it += XT) {
            const int t = it / N, p = it % N;
            const int k1 = p / R2, k2 = p % R2;
            const int ix = k1 + R1 * k2;
            const int64_t l = l0 + t;
            const float kxi = __ldg(kx + ix), mxi = __ldg(mx + ix);
            const float kzl = l < g.n2h ? __ldg(kz + l) : 0.f;
            const float k2v = __fadd_rn(__fadd_rn(__fmul_rn(kxi, kxi), ky2), __fmul_rn(kzl, kzl));
            const int q = Col<N, R2>::at(t, p);
            const float re = __fadd_rn(-__fmul_rn(mxi, aim[q]), bre[q]);
            const float im = __fadd_rn(__fmul_rn(mxi, are[q]), bim[q]);
            float sr = 0.f, si = 0.f;
            if (k2v != 0.f) {
                sr = -__fdiv_rn(__fmul_rn(re, g.c), k2v);
                si = -__fdiv_rn(__fmul_rn(im, g.c), k2v);
            }
            are[q] = sr;
            aim[q] = si;
        }
        __syncthreads();
        fft_inv<N>(are, aim, tw);
        for (int it = threadIdx.x; it < N * T; it += XT) {
            const int t = it % T, x = it / T;
            const int64_t l = l0 + t;
            if (l >= g.n2h) continue;
            const int q = Col<N, R2>::at(t, x);
            S[((int64_t)x * g.n1 + j) * g.n2h + l] = make_float2(are[q], aim[q]);
        }
    }
}

template <int N>
size_t xpass_smem() {
    return (size_t)4 * XCfg<N>::BUF * sizeof(float) + (size_t)N * sizeof(float2);
}

template <int N>
int launch_xpass(bool adj, const float2 *in, float2 *out, const float *kt, const float2 *tw,
                 int64_t n1, int64_t n2h, float c, cudaStream_t st) {
    XGeom g;
    g.n1 = n1;
    g.n2h = n2h;
    g.ncol_tiles = (n2h + XCfg<N>::T - 1) / XCfg<N>::T;
    g.c = c;
    size_t sm = xpass_smem<N>();
    int64_t tiles = n1 * g.ncol_tiles;
    int64_t cap = (int64_t)device_sms() * (sm > 110 * 1024 ? 1 : 2);
    int grid = (int)(tiles < cap ? tiles : cap);
    if (adj) {
        static bool attr = false;
        if (!attr) {
            PMX_CUDA(cudaFuncSetAttribute(k_xpass_adj<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sm));
            attr = true;
        }
        k_xpass_adj<N><<<grid, XT, sm, st>>>(in, out, kt, tw, g, (int64_t)N);
        PMX_LAUNCH_CHECK("k_xpass_adj");
    } else {
        static bool attr = false;
        if (!attr) {
            PMX_CUDA(cudaFuncSetAttribute(k_xpass_fwd<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sm));
            attr = true;
        }
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
