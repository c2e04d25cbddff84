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

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <mutex>
#include <cstdlib>
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
constexpr Twiddle32 kTw32 = Twiddle32();

template <int R, bool INV, int S, int J>
__device__ __forceinline__ void bfly(float (&re)[R], float (&im)[R]) {
    constexpr int half = 1 << (S - 1), len = 1 << S;
    constexpr int g = J / half, k = J % half;
    constexpr int a = g * len + k, b = a + half, ti = k * (32 >> S);
    const float ur = re[a], ui = im[a], vr = re[b], vi = im[b];
    re[a] = ur + vr;
    im[a] = ui + vi;
    const float dr = ur - vr, di = ui - vi;
    // twiddle exp(-+2 pi i ti / 32), a compile-time constant; 1 and -+i exactly
    if constexpr (ti == 0) {
        re[b] = dr;
        im[b] = di;
    } else if constexpr (ti == 8) {
        re[b] = INV ? -di : di;
        im[b] = INV ? dr : -dr;
    } else {
        constexpr float wc = kTw32.c[ti];
        constexpr float ws = INV ? kTw32.s[ti] : -kTw32.s[ti];
        re[b] = dr * wc - di * ws;
        im[b] = dr * ws + di * wc;
    }
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
template <> struct Split<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Split<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Split<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Split<256> { static constexpr int R1 = 16, R2 = 16; };
template <> struct Split<512> { static constexpr int R1 = 32, R2 = 16; };
template <> struct Split<1024> { static constexpr int R1 = 32, R2 = 32; };

constexpr int XTF = 256;  // threads per forward x-pass CTA
constexpr int XTA = 256;  // threads per adjoint x-pass CTA

// Column stride of the padded tile buffers.  One pad per R2 values keeps the
// strided and the contiguous DFT steps free of bank conflicts for 8-byte
// accesses.  The tile loads and stores walk (column t, row x) with t fastest;
// 16 lanes (one 128-byte wavefront) then cover T columns x 16/T rows, which
// hit 16 distinct bank pairs when CS = 16/T (mod 16) for T <= 16, or CS odd.
constexpr int pad_cs(int n, int r2, int t) {
    int cs = n + n / r2 + 1;
    if (t > 16) return cs | 1;
    while (cs % 16 != 16 / t) ++cs;
    return cs;
}

// Tile geometry: T columns (fixed ky, consecutive kz) of length N, column t
// at t*CS, logical position p at p + p/R2.
template <int N, int XTH>
struct XCfg {
    static constexpr int TH = XTH;
    static constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2;
    static constexpr int RM = R1 > R2 ? R1 : R2;
    static constexpr int T = XTH / RM;  // columns per CTA
    static constexpr int CS = pad_cs(N, R2, T);
    static constexpr int BUF = T * CS;  // float2 per buffer
    static constexpr int PER = N * T / XTH;  // tile elements per thread
    static constexpr int TWP = R1 * (R2 + 1);  // padded twiddle table entries
    __device__ static __forceinline__ int at(int t, int p) { return t * CS + p + p / R2; }
};

// 8-byte asynchronous global -> shared copy; ok == false writes zeros and
// reads nothing (src must still be a valid address).
__device__ __forceinline__ void cp_async8(float2 *dst, const float2 *src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = ok ? 8 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_group1() {
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}

// Twiddles w^(b k1) (w = exp(-2 pi i / n0), b < R2, k1 < R1) in a padded
// table twP[k1 (R2 + 1) + b]: step 1 reads it with the lanes on b
// (consecutive entries), the inverse step 2 with the lanes on k1 (an odd
// stride of 8-byte entries), so neither has shared-memory bank conflicts.
// A flat table read at b k1 has power-of-two strides in both.
template <class C>
__device__ __forceinline__ void fill_twiddles(const float2 *__restrict__ twg, float2 *twP) {
    for (int m = threadIdx.x; m < C::R1 * (C::R2 + 1); m += C::TH) {
        const int k1 = m / (C::R2 + 1), b = m % (C::R2 + 1);
        twP[m] = b < C::R2 ? twg[b * k1] : make_float2(0.f, 0.f);
    }
}

// Forward step 1 on one buffer: R2-strided radix-R1 DFTs + twiddles,
// natural order -> "transposed" positions k1*R2 + b.
template <class C>
__device__ __forceinline__ void fwd_step1(float2 *buf, const float2 *twP) {
    constexpr int R1 = C::R1, R2 = C::R2;
    for (int it = threadIdx.x; it < C::T * R2; it += C::TH) {
        const int t = it / R2, b = it % R2;
        float2 *col = buf + t * C::CS + b;  // position a*R2 + b at col[a*(R2+1)]
        float2 v[R1];
#pragma unroll
        for (int a = 0; a < R1; ++a) v[a] = col[a * (R2 + 1)];
        dft2<R1, false>(v);
#pragma unroll
        for (int k = 0; k < R1; ++k) {
            const int k1 = brev(k, Log2<R1>::v);
            col[k1 * (R2 + 1)] = cmul(v[k], twP[k1 * (R2 + 1) + b]);
        }
    }
}

// Inverse step 1 (the last inverse step) on one buffer: radix-R1 inverse
// DFTs over k1 at fixed b -> natural order.
template <class C>
__device__ __forceinline__ void inv_step1(float2 *buf) {
    constexpr int R1 = C::R1, R2 = C::R2;
    for (int it = threadIdx.x; it < C::T * R2; it += C::TH) {
        const int t = it / R2, b = it % R2;
        float2 *col = buf + t * C::CS + b;
        float2 v[R1];
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) v[k1] = col[k1 * (R2 + 1)];
        dft2<R1, true>(v);
#pragma unroll
        for (int k = 0; k < R1; ++k) col[brev(k, Log2<R1>::v) * (R2 + 1)] = v[k];
    }
}

// Inverse step 2 on a register group in bit-reversed k2 order (as the
// forward step 2 leaves it), twiddle, store to positions k1*R2 + b.
template <class C>
__device__ __forceinline__ void inv_step2_store(float2 (&v)[C::R2], float2 *buf, int t, int k1,
                                                const float2 *twP) {
    constexpr int R2 = C::R2;
    float2 u[R2];
    unbrev<R2>(v, u);           // natural k2 order
    dft2<R2, true>(u);          // element k holds b = brev(k)
    float2 *grp = buf + t * C::CS + k1 * (R2 + 1);  // position k1*R2 + b at grp[b]
#pragma unroll
    for (int k = 0; k < R2; ++k) {
        const int b = brev(k, Log2<R2>::v);
        grp[b] = cmulc(u[k], twP[k1 * (R2 + 1) + b]);
    }
}

// Column tiles of a ky row j start at l0 = s_j + (k - 1) T, k < ncol_tiles,
// with s_j = (-j rs) mod 4 (rs the row stride): every tile but the first and
// last of a row then covers whole 32-byte sectors of every x-plane (the plane
// size n1 rs is a multiple of 4 then).  HBM3e has no byte-masked writes, so partial-sector
// stores would cost read-modify-writes.  Columns outside [0, n2h) are idle.
struct XGeom {
    int64_t n1, n2h;
    int64_t rs;           // row stride of the complex arrays (>= n2h)
    int64_t ncol_tiles;   // ceil(n2h / T) + 1
    int align;            // 1: shift rows as above (n1 rs % 4 == 0)
    float c;              // 1.5 Omega_m / N
    __device__ __forceinline__ int64_t row(int64_t tile) const { return tile / ncol_tiles; }
    __device__ __forceinline__ int64_t col0(int64_t tile, int T) const {
        const int64_t j = tile / ncol_tiles, k = tile % ncol_tiles;
        const int64_t sj = align ? (4 - (j * rs) % 4) % 4 : 0;
        return sj + (k - 1) * T;
    }
};

// Starts the asynchronous load of the column tile (fixed ky row j, kz in
// [l0, l0+T), all x) of component `comp` of a complex array laid out
// (x, ncomp, n1, rs); columns outside [0, n2h) read as zero.
template <class C>
__device__ __forceinline__ void issue_tile(const float2 *__restrict__ src, int ncomp, int comp,
                                           int64_t j, int64_t l0, const XGeom &g, float2 *buf) {
    constexpr int T = C::T, XS = C::TH / C::T;
    const int t = threadIdx.x % T, x0 = threadIdx.x / T;
    const int64_t l = l0 + t;
    const bool ok = l >= 0 && l < g.n2h;
    const float2 *base = src + ((int64_t)comp * g.n1 + j) * g.rs + (ok ? l : 0);
    const int64_t xs = (int64_t)ncomp * g.n1 * g.rs;
#pragma unroll 8
    for (int r = 0; r < C::PER; ++r) {
        const int x = x0 + r * XS;
        cp_async8(buf + C::at(t, x), base + x * xs, ok);
    }
}

// Both kernels are software pipelined: while a CTA transforms one tile, the
// cp.async copies of its next tile are in flight into a second buffer set,
// so the HBM reads overlap the shared-memory FFT work and the stores.

template <int N>
__global__ void __launch_bounds__(XTF, 1) k_xpass_fwd(const float2 *__restrict__ H,
                                                      float2 *__restrict__ G,
                                                      const float *__restrict__ kt,
                                                      const float2 *__restrict__ twg, XGeom g,
                                                      int64_t n0) {
    using C = XCfg<N, XTF>;
    constexpr int T = C::T, R1 = C::R1, R2 = C::R2;
    extern __shared__ __align__(16) float2 smem2[];
    float2 *A0 = smem2, *A1 = smem2 + C::BUF, *B = smem2 + 2 * C::BUF;
    float2 *twP = smem2 + 3 * C::BUF;
    float *kxs = reinterpret_cast<float *>(twP + C::TWP), *mxs = kxs + N;

    const int64_t tot = n0 + g.n1 + g.n2h;
    const float *ky = kt + n0, *kz = kt + n0 + g.n1;
    const float *my = kt + tot + n0, *mz = kt + tot + n0 + g.n1;
    fill_twiddles<C>(twg, twP);
    for (int m = threadIdx.x; m < N; m += XTF) {
        kxs[m] = kt[m];
        mxs[m] = kt[tot + m];
    }

    const int64_t ntiles = g.n1 * g.ncol_tiles;
    int64_t tile = blockIdx.x;
    if (tile < ntiles) issue_tile<C>(H, 1, 0, g.row(tile), g.col0(tile, T), g, A0);
    cp_async_commit();
    for (int cur = 0; tile < ntiles; tile += gridDim.x, cur ^= 1) {
        float2 *A = cur ? A1 : A0;
        const int64_t j = g.row(tile);
        const int64_t l0 = g.col0(tile, T);
        cp_async_wait_all();
        // this tile is in A; the previous tile's store phase (reads of the
        // other A buffer and of B) is over; the tables are filled
        __syncthreads();
        const int64_t nxt = tile + gridDim.x;
        if (nxt < ntiles) issue_tile<C>(H, 1, 0, g.row(nxt), g.col0(nxt, T), g, cur ? A0 : A1);
        cp_async_commit();
        fwd_step1<C>(A, twP);
        __syncthreads();
        // fused: forward step 2, Green + gradient, inverse step 2 of P and of
        // B = -i kx P, all on one thread's contiguous group
        const float kyj = __ldg(ky + j), myj = __ldg(my + j);
        const float ky2 = __fmul_rn(kyj, kyj);
        for (int it = threadIdx.x; it < T * R1; it += XTF) {
            const int t = it / R1, k1 = it % R1;
            const int64_t l = l0 + t;
            const float kzl = l >= 0 && l < g.n2h ? __ldg(kz + l) : 0.f;
            const float kz2 = __fmul_rn(kzl, kzl);
            float2 v[R2];
#pragma unroll
            for (int b = 0; b < R2; ++b) v[b] = A[t * C::CS + k1 * (R2 + 1) + b];
            dft2<R2, false>(v);          // element k: kx index k1 + R1*brev(k)
            float2 w[R2];
#pragma unroll
            for (int k = 0; k < R2; ++k) {
                const int ix = k1 + R1 * brev(k, Log2<R2>::v);
                const float kxi = kxs[ix], mxi = mxs[ix];
                const float k2v = __fadd_rn(__fadd_rn(__fmul_rn(kxi, kxi), ky2), kz2);
                // laplace (k = 0 -> 0); c / k^2 to within 2 ulp
                const float rk = k2v != 0.f ? __fdividef(g.c, k2v) : 0.f;
                const float pr = -__fmul_rn(v[k].x, rk), pi = -__fmul_rn(v[k].y, rk);
                v[k] = make_float2(pr, pi);
                w[k] = make_float2(__fmul_rn(mxi, pi), -__fmul_rn(mxi, pr));  // -i kx P
            }
            inv_step2_store<C>(v, A, t, k1, twP);
            inv_step2_store<C>(w, B, t, k1, twP);
        }
        __syncthreads();
        inv_step1<C>(A);
        inv_step1<C>(B);
        __syncthreads();
        // G_0 = B; G_1 = -i ky Q; G_2 = -i kz Q  (Q in A); layout (x, 3, n1, rs)
        {
            constexpr int XS = XTF / T;
            const int t = threadIdx.x % T;
            const int64_t l = l0 + t;
            if (l >= 0 && l < g.n2h) {
                const float mzl = __ldg(mz + l);
                const int64_t cs = g.n1 * g.rs, xs = 3 * cs;
                float2 *o = G + j * g.rs + l;
                for (int x = threadIdx.x / T; x < N; x += XS) {
                    const int q = C::at(t, x);
                    const float2 Q = A[q];
                    float2 *ox = o + x * xs;
                    ox[0] = B[q];
                    ox[cs] = make_float2(__fmul_rn(myj, Q.y), -__fmul_rn(myj, Q.x));
                    ox[2 * cs] = make_float2(__fmul_rn(mzl, Q.y), -__fmul_rn(mzl, Q.x));
                }
            }
        }
    }
    cp_async_wait_all();
}

// Loads B = i ky C_1 + i kz C_2 of a column tile (components 1, 2 of the
// (x, 3, n1, rs) array) synchronously, in register batches.
template <class C>
__device__ __forceinline__ void load_comb(const float2 *__restrict__ Cin, int64_t j, int64_t l0,
                                          float myj, const float *__restrict__ mz,
                                          const XGeom &g, float2 *buf) {
    constexpr int T = C::T, XS = C::TH / C::T, PER = C::PER, CH = PER < 8 ? PER : 8;
    const int t = threadIdx.x % T, x0 = threadIdx.x / T;
    const int64_t l = l0 + t;
    const bool ok = l >= 0 && l < g.n2h;
    const float mzl = ok ? __ldg(mz + l) : 0.f;
    const int64_t cs = g.n1 * g.rs, xs = 3 * cs;
    const float2 *base = Cin + j * g.rs + (ok ? l : 0);
#pragma unroll
    for (int b = 0; b < PER; b += CH) {
        float2 c1[CH], c2[CH];
#pragma unroll
        for (int r = 0; r < CH; ++r) {
            const int x = x0 + (b + r) * XS;
            c1[r] = ok ? __ldg(base + x * xs + cs) : make_float2(0.f, 0.f);
            c2[r] = ok ? __ldg(base + x * xs + 2 * cs) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < CH; ++r)  // i k (a + i b) = (-k b, k a)
            buf[C::at(t, x0 + (b + r) * XS)] =
                make_float2(-__fadd_rn(__fmul_rn(myj, c1[r].y), __fmul_rn(mzl, c2[r].y)),
                            __fadd_rn(__fmul_rn(myj, c1[r].x), __fmul_rn(mzl, c2[r].x)));
    }
}

template <int N>
__global__ void __launch_bounds__(XTA, 1) k_xpass_adj(const float2 *__restrict__ Cin,
                                                      float2 *__restrict__ S,
                                                      const float *__restrict__ kt,
                                                      const float2 *__restrict__ twg, XGeom g,
                                                      int64_t n0) {
    using C = XCfg<N, XTA>;
    constexpr int T = C::T, R1 = C::R1, R2 = C::R2;
    extern __shared__ __align__(16) float2 smem2[];
    float2 *A0 = smem2, *A1 = smem2 + C::BUF, *B = smem2 + 2 * C::BUF;
    float2 *twP = smem2 + 3 * C::BUF;
    float *kxs = reinterpret_cast<float *>(twP + C::TWP), *mxs = kxs + N;

    const int64_t tot = n0 + g.n1 + g.n2h;
    const float *ky = kt + n0, *kz = kt + n0 + g.n1;
    const float *my = kt + tot + n0, *mz = kt + tot + n0 + g.n1;
    fill_twiddles<C>(twg, twP);
    for (int m = threadIdx.x; m < N; m += XTA) {
        kxs[m] = kt[m];
        mxs[m] = kt[tot + m];
    }

    const int64_t ntiles = g.n1 * g.ncol_tiles;
    int64_t tile = blockIdx.x;
    if (tile < ntiles) issue_tile<C>(Cin, 3, 0, g.row(tile), g.col0(tile, T), g, A0);
    cp_async_commit();
    for (int cur = 0; tile < ntiles; tile += gridDim.x, cur ^= 1) {
        float2 *A = cur ? A1 : A0;
        const int64_t j = g.row(tile);
        const int64_t l0 = g.col0(tile, T);
        // the previous tile's store phase (reads of the other A buffer) is over
        __syncthreads();
        const int64_t nxt = tile + gridDim.x;
        if (nxt < ntiles) issue_tile<C>(Cin, 3, 0, g.row(nxt), g.col0(nxt, T), g, cur ? A0 : A1);
        cp_async_commit();
        const float myj = __ldg(my + j);
        load_comb<C>(Cin, j, l0, myj, mz, g, B);
        cp_async_wait_group1();  // this tile's C_0 (the next tile's may stay in flight)
        __syncthreads();
        fwd_step1<C>(A, twP);
        fwd_step1<C>(B, twP);
        __syncthreads();
        const float kyj = __ldg(ky + j);
        const float ky2 = __fmul_rn(kyj, kyj);
        for (int it = threadIdx.x; it < T * R1; it += XTA) {
            const int t = it / R1, k1 = it % R1;
            const int64_t l = l0 + t;
            const float kzl = l >= 0 && l < g.n2h ? __ldg(kz + l) : 0.f;
            const float kz2 = __fmul_rn(kzl, kzl);
            float2 v[R2], w[R2];
#pragma unroll
            for (int b = 0; b < R2; ++b) v[b] = A[t * C::CS + k1 * (R2 + 1) + b];
            dft2<R2, false>(v);
#pragma unroll
            for (int b = 0; b < R2; ++b) w[b] = B[t * C::CS + k1 * (R2 + 1) + b];
            dft2<R2, false>(w);
#pragma unroll
            for (int k = 0; k < R2; ++k) {
                const int ix = k1 + R1 * brev(k, Log2<R2>::v);
                const float kxi = kxs[ix], mxi = mxs[ix];
                const float k2v = __fadd_rn(__fadd_rn(__fmul_rn(kxi, kxi), ky2), kz2);
                const float re = __fadd_rn(-__fmul_rn(mxi, v[k].y), w[k].x);
                const float im = __fadd_rn(__fmul_rn(mxi, v[k].x), w[k].y);
                const float rk = k2v != 0.f ? __fdividef(g.c, k2v) : 0.f;
                v[k] = make_float2(-__fmul_rn(re, rk), -__fmul_rn(im, rk));
            }
            inv_step2_store<C>(v, A, t, k1, twP);
        }
        __syncthreads();
        inv_step1<C>(A);
        __syncthreads();
        {
            constexpr int XS = XTA / T;
            const int t = threadIdx.x % T;
            const int64_t l = l0 + t;
            if (l >= 0 && l < g.n2h) {
                float2 *o = S + j * g.rs + l;
                const int64_t xs = g.n1 * g.rs;
                for (int x = threadIdx.x / T; x < N; x += XS) o[x * xs] = A[C::at(t, x)];
            }
        }
    }
    cp_async_wait_all();
}

template <int N>
size_t xpass_smem(bool adj) {
    using CF = XCfg<N, XTF>;
    using CA = XCfg<N, XTA>;
    const size_t tables = (size_t)CF::TWP * sizeof(float2) + (size_t)N * 2 * sizeof(float);
    return (size_t)3 * (adj ? CA::BUF : CF::BUF) * sizeof(float2) + tables;
}

template <int N>
int launch_xpass(bool adj, const float2 *in, float2 *out, const float *kt, const float2 *tw,
                 int64_t n1, int64_t n2h, int64_t rs, float c, cudaStream_t st) {
    XGeom g;
    g.n1 = n1;
    g.n2h = n2h;
    g.rs = rs;
    g.c = c;
    const size_t sm = xpass_smem<N>(adj);
    const void *fn = adj ? (const void *)k_xpass_adj<N> : (const void *)k_xpass_fwd<N>;
    const int threads = adj ? XTA : XTF;
    const int T = adj ? XCfg<N, XTA>::T : XCfg<N, XTF>::T;
    g.ncol_tiles = (n2h + T - 1) / T + 1;
    g.align = (n1 * rs) % 4 == 0;
    // the shared-memory opt-in and the occupancy query once per device and
    // kernel: a small mesh's force is short enough for them to show
    int per_sm = 0;
    {
        static std::mutex mu;
        static std::map<std::pair<int, bool>, int> known;
        int dev = 0;
        PMX_CUDA(cudaGetDevice(&dev));
        std::lock_guard<std::mutex> lock(mu);
        auto it = known.find({dev, adj});
        if (it != known.end()) {
            per_sm = it->second;
        } else {
            PMX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            PMX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, sm));
            known[{dev, adj}] = per_sm;
        }
    }
    if (per_sm < 1) return fail(PMX_ERR_CUDA, "x-pass kernel does not fit on an SM");
    const int64_t tiles = n1 * g.ncol_tiles;
    const int64_t cap = (int64_t)device_sms() * per_sm;
    const int grid = (int)(tiles < cap ? tiles : cap);
    if (adj) {
        k_xpass_adj<N><<<grid, XTA, sm, st>>>(in, out, kt, tw, g, (int64_t)N);
        PMX_LAUNCH_CHECK("k_xpass_adj");
    } else {
        k_xpass_fwd<N><<<grid, XTF, sm, st>>>(in, out, kt, tw, g, (int64_t)N);
        PMX_LAUNCH_CHECK("k_xpass_fwd");
    }
    return PMX_OK;
}

// ---------------------------------------------------------------------------
// Plane (y, z) transforms.  The 3-D r2c / c2r transforms of the force are
// the x pass above plus, per x-plane (and component), a 2-D transform over
// (y, z): real rows of n2 values along z (contiguous) and complex columns of
// n1 values along y.  Complex rows are stored at the padded stride
// RS = padded_row(n2h), so every 8-column tile covers whole 32-byte sectors.
// One thread-block cluster of CL CTAs owns a plane at a time: each CTA
// transforms n1/CL rows, the cluster synchronises (barrier.cluster:
// release/acquire at cluster scope, so the rows written by the other CTAs
// are visible), then each CTA transforms every CL-th tile of T columns.
// Between the two phases the plane (n1 * RS * 8 bytes, 4.2 MB at 1024^2)
// sits in L2, so HBM sees one read of the input and one write of the output
// per plane:
//   r2c: rows -> the output plane (stores marked L2 evict_last), columns in
//        place (the final stores evict_first);
//   c2r: columns of the input -> a per-cluster scratch plane that is
//        rewritten for every plane (evict_last: it stays in L2 and is never
//        written back), rows of the scratch -> the real output (evict_first).
//
// Rows use the half-length complex FFT: z[m] = x[2m] + i x[2m+1],
// Z = FFT_L(z) (L = n2/2), then X[k] = E[k] + w_N^k O[k] with
// E[k] = (Z[k] + conj Z[L-k]) / 2, O[k] = (Z[k] - conj Z[L-k]) / 2i.  The
// inverse rebuilds Zc[k] = (X[k] + conj X[L-k]) + i w_N^-k (X[k] - conj X[L-k])
// (imaginary parts of X[0] and X[L] ignored, as c2r does) and z = IFFT_L(Zc).
// All transforms are unnormalised, like cuFFT's.
// ---------------------------------------------------------------------------

namespace cg = cooperative_groups;

constexpr int PTH = 256;  // threads per plane CTA

// L2 cache policies (createpolicy) for the eviction-priority hints.
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}
// cp_async8 with an L2 eviction policy
__device__ __forceinline__ void cp_async8_pol(float2 *dst, const float2 *src, bool ok, uint64_t pol) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = ok ? 8 : 0;
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2, %3;\n" ::"r"(d),
                 "l"(src), "r"(n), "l"(pol)
                 : "memory");
}
// 8-byte global store with an L2 eviction policy
__device__ __forceinline__ void st8_pol(float2 *p, float2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;\n" ::"l"(p), "f"(v.x),
                 "f"(v.y), "l"(pol)
                 : "memory");
}

// Length-N FFT (N = R1 * R2) of the T columns of a padded tile buffer, in
// place, natural order in and out; INV selects exp(+2 pi i ...).  Step 2
// gives each thread exactly one group (T * R1 == threads), which lets the
// reordering to natural order happen in place after a barrier.
template <class C, bool INV>
__device__ __forceinline__ void fft_cols(float2 *buf, const float2 *tw) {
    constexpr int R1 = C::R1, R2 = C::R2;
    static_assert(C::T * R1 == C::TH, "one step-2 group per thread");
    for (int it = threadIdx.x; it < C::T * R2; it += C::TH) {
        const int t = it / R2, b = it % R2;
        float2 *col = buf + t * C::CS + b;
        float2 v[R1];
#pragma unroll
        for (int a = 0; a < R1; ++a) v[a] = col[a * (R2 + 1)];
        dft2<R1, INV>(v);
#pragma unroll
        for (int k = 0; k < R1; ++k) {
            const int k1 = brev(k, Log2<R1>::v);
            col[k1 * (R2 + 1)] = INV ? cmulc(v[k], tw[b * k1]) : cmul(v[k], tw[b * k1]);
        }
    }
    __syncthreads();
    const int t = threadIdx.x / R1, k1 = threadIdx.x % R1;
    float2 v[R2];
    const float2 *grp = buf + t * C::CS + k1 * (R2 + 1);
#pragma unroll
    for (int b = 0; b < R2; ++b) v[b] = grp[b];
    dft2<R2, INV>(v);  // element k: frequency k1 + R1 * brev(k)
    __syncthreads();
    // natural position f = k1 + R1 k2 at t*CS + k1 + k1/R2 + k2 (R1 + R1/R2)
    float2 *nat = buf + t * C::CS + k1 + k1 / R2;
#pragma unroll
    for (int k = 0; k < R2; ++k) nat[brev(k, Log2<R2>::v) * (R1 + R1 / R2)] = v[k];
    __syncthreads();
}

// Asynchronous load of T columns [l0, l0+T) (those < ncol valid, the rest
// zero) of ROWS rows with row stride rs (float2) into a tile buffer.
template <class C, int ROWS>
__device__ __forceinline__ void issue_cols(const float2 *src, int64_t rs, int l0, int ncol,
                                           float2 *buf, uint64_t pol) {
    constexpr int T = C::T, XS = C::TH / C::T;
    const int t = threadIdx.x % T, y0 = threadIdx.x / T;
    const bool ok = l0 + t < ncol;
    const float2 *base = src + (ok ? l0 + t : 0);
#pragma unroll 8
    for (int r = 0; r < ROWS / XS; ++r) {
        const int y = y0 + r * XS;
        cp_async8_pol(buf + C::at(t, y), base + y * rs, ok, pol);
    }
}

// Stores T columns of a tile buffer (columns >= ncol skipped).
template <class C, int ROWS>
__device__ __forceinline__ void store_cols(float2 *dst, int64_t rs, int l0, int ncol,
                                           const float2 *buf, uint64_t pol) {
    constexpr int T = C::T, XS = C::TH / C::T;
    const int t = threadIdx.x % T;
    if (l0 + t >= ncol) return;
    for (int y = threadIdx.x / T; y < ROWS; y += XS)
        st8_pol(dst + (int64_t)y * rs + l0 + t, buf[C::at(t, y)], pol);
}

struct PGeom {
    int64_t nplanes;
    float2 *scratch;  // c2r: one plane (N1 x RS complex) per cluster
};

template <int L>
struct PRow {
    static constexpr int N2H = L + 1;
    static constexpr int RS = (N2H + 3) & ~3;  // padded_row(N2H)
};

// Forward plane transform: real planes (n1, 2L) -> complex planes (n1, RS).
// Twiddles in ptw: [exp(-2 pi i m / N1), m < N1 | exp(-2 pi i m / L), m < L |
// exp(-2 pi i k / 2L), k <= L].
template <int N1, int L, int CL>
__global__ void __launch_bounds__(PTH, 1) k_plane_r2c(const float *__restrict__ in,
                                                      float2 *__restrict__ out,
                                                      const float2 *__restrict__ ptw, PGeom g) {
    using ZC = XCfg<L, PTH>;
    using YC = XCfg<N1, PTH>;
    constexpr int N2 = 2 * L, N2H = L + 1, RS = PRow<L>::RS, RPC = N1 / CL;
    constexpr int ZT = ZC::T, NB = (RPC + ZT - 1) / ZT;
    constexpr int YT = YC::T, NTILE = (N2H + YT - 1) / YT;
    constexpr int ZREG = 2 * ZC::BUF, YREG = 2 * YC::BUF;
    constexpr int REG = ZREG > YREG ? ZREG : YREG;
    extern __shared__ __align__(16) float2 smem2[];
    float2 *twY = smem2 + REG, *twL = twY + N1, *twN = twL + L;
    for (int m = threadIdx.x; m < N1 + L + N2H; m += PTH) twY[m] = ptw[m];
    const uint64_t pfirst = policy_evict_first(), plast = policy_evict_last();

    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int64_t cid = blockIdx.x / CL, ncl = gridDim.x / CL;
    const int yb = rank * RPC;

    for (int64_t p = cid; p < g.nplanes; p += ncl) {
        const float2 *src = reinterpret_cast<const float2 *>(in + p * (int64_t)N1 * N2);
        float2 *dst = out + p * (int64_t)N1 * RS;
        // rows [yb, yb + RPC): half-length FFT, then the real-input split
        auto issue_rows = [&](int b, float2 *buf) {
            for (int it = threadIdx.x; it < ZT * L; it += PTH) {
                const int t = it / L, m = it % L, y = b * ZT + t;
                const bool ok = y < RPC;
                cp_async8_pol(buf + ZC::at(t, m), src + (int64_t)(yb + (ok ? y : 0)) * L + m, ok,
                              pfirst);
            }
        };
        issue_rows(0, smem2);
        cp_async_commit();
        for (int b = 0; b < NB; ++b) {
            float2 *buf = smem2 + (b & 1) * ZC::BUF;
            cp_async_wait_all();
            __syncthreads();
            if (b + 1 < NB) issue_rows(b + 1, smem2 + ((b + 1) & 1) * ZC::BUF);
            cp_async_commit();
            fft_cols<ZC, false>(buf, twL);
            for (int it = threadIdx.x; it < ZT * N2H; it += PTH) {
                const int t = it / N2H, k = it % N2H, y = b * ZT + t;
                if (y >= RPC) continue;
                const float2 zk = buf[ZC::at(t, k == L ? 0 : k)];
                const float2 zm = buf[ZC::at(t, k == 0 ? 0 : L - k)];
                const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
                const float2 o = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
                const float2 w = twN[k];
                st8_pol(dst + (int64_t)(yb + y) * RS + k,
                        make_float2(e.x + (w.x * o.x - w.y * o.y), e.y + (w.x * o.y + w.y * o.x)),
                        plast);
            }
        }
        cp_async_wait_all();
        cl.sync();  // every row of the plane is written (and visible)
        // columns in place: tiles rank, rank + CL, ...
        int tl = rank;
        if (tl < NTILE) issue_cols<YC, N1>(dst, RS, tl * YT, N2H, smem2, pfirst);
        cp_async_commit();
        for (int i = 0; tl < NTILE; tl += CL, ++i) {
            float2 *buf = smem2 + (i & 1) * YC::BUF;
            cp_async_wait_all();
            __syncthreads();
            if (tl + CL < NTILE)
                issue_cols<YC, N1>(dst, RS, (tl + CL) * YT, N2H, smem2 + ((i + 1) & 1) * YC::BUF,
                                   pfirst);
            cp_async_commit();
            fft_cols<YC, false>(buf, twY);
            store_cols<YC, N1>(dst, RS, tl * YT, N2H, buf, pfirst);
        }
        cp_async_wait_all();
        __syncthreads();  // tile buffers free before the next plane's rows
    }
}

// Inverse plane transform: complex planes (n1, RS) -> real planes (n1, 2L),
// through the cluster's scratch plane (the input is left unchanged).
template <int N1, int L, int CL>
__global__ void __launch_bounds__(PTH, 1) k_plane_c2r(const float2 *__restrict__ in,
                                                      float *__restrict__ out,
                                                      const float2 *__restrict__ ptw, PGeom g) {
    using ZC = XCfg<L, PTH>;
    using YC = XCfg<N1, PTH>;
    constexpr int N2 = 2 * L, N2H = L + 1, RS = PRow<L>::RS, RPC = N1 / CL;
    constexpr int ZT = ZC::T, NB = (RPC + ZT - 1) / ZT;
    constexpr int YT = YC::T, NTILE = (N2H + YT - 1) / YT;
    constexpr int XRS = N2H + 1;  // raw row stride in shared memory
    constexpr int ZREG = 2 * ZT * XRS + ZC::BUF, YREG = 2 * YC::BUF;
    constexpr int REG = ZREG > YREG ? ZREG : YREG;
    extern __shared__ __align__(16) float2 smem2[];
    float2 *twY = smem2 + REG, *twL = twY + N1, *twN = twL + L;
    for (int m = threadIdx.x; m < N1 + L + N2H; m += PTH) twY[m] = ptw[m];
    const uint64_t pfirst = policy_evict_first(), plast = policy_evict_last();

    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int64_t cid = blockIdx.x / CL, ncl = gridDim.x / CL;
    const int yb = rank * RPC;
    float2 *scr = g.scratch + cid * (int64_t)N1 * RS;

    for (int64_t p = cid; p < g.nplanes; p += ncl) {
        const float2 *cpl = in + p * (int64_t)N1 * RS;
        float2 *rpl = reinterpret_cast<float2 *>(out + p * (int64_t)N1 * N2);
        // columns first (inverse along y) into the scratch plane
        int tl = rank;
        if (tl < NTILE) issue_cols<YC, N1>(cpl, RS, tl * YT, N2H, smem2, pfirst);
        cp_async_commit();
        for (int i = 0; tl < NTILE; tl += CL, ++i) {
            float2 *buf = smem2 + (i & 1) * YC::BUF;
            cp_async_wait_all();
            __syncthreads();
            if (tl + CL < NTILE)
                issue_cols<YC, N1>(cpl, RS, (tl + CL) * YT, N2H, smem2 + ((i + 1) & 1) * YC::BUF,
                                   pfirst);
            cp_async_commit();
            fft_cols<YC, true>(buf, twY);
            store_cols<YC, N1>(scr, RS, tl * YT, N2H, buf, plast);
        }
        cp_async_wait_all();
        cl.sync();  // every column of the plane is in the scratch (and visible)
        // rows [yb, yb + RPC): Hermitian rebuild, half-length inverse FFT
        float2 *F = smem2 + 2 * ZT * XRS;
        auto issue_rows = [&](int b, float2 *raw) {
            for (int it = threadIdx.x; it < ZT * N2H; it += PTH) {
                const int t = it / N2H, k = it % N2H, y = b * ZT + t;
                const bool ok = y < RPC;
                cp_async8_pol(raw + t * XRS + k, scr + (int64_t)(yb + (ok ? y : 0)) * RS + k, ok,
                              plast);
            }
        };
        issue_rows(0, smem2);
        cp_async_commit();
        for (int b = 0; b < NB; ++b) {
            const float2 *raw = smem2 + (b & 1) * ZT * XRS;
            cp_async_wait_all();
            __syncthreads();
            if (b + 1 < NB) issue_rows(b + 1, smem2 + ((b + 1) & 1) * ZT * XRS);
            cp_async_commit();
            for (int it = threadIdx.x; it < ZT * L; it += PTH) {
                const int t = it / L, k = it % L;
                float2 xk = raw[t * XRS + k], xm = raw[t * XRS + (L - k)];
                if (k == 0) {
                    xk.y = 0.f;
                    xm.y = 0.f;
                }
                const float2 s = make_float2(xk.x + xm.x, xk.y - xm.y);  // X[k] + conj X[L-k]
                const float2 d = make_float2(xk.x - xm.x, xk.y + xm.y);  // X[k] - conj X[L-k]
                const float2 w = twN[k];                                  // w_N^k; use conj
                const float2 dw = make_float2(d.x * w.x + d.y * w.y, d.y * w.x - d.x * w.y);
                F[ZC::at(t, k)] = make_float2(s.x - dw.y, s.y + dw.x);    // s + i d conj(w)
            }
            __syncthreads();
            fft_cols<ZC, true>(F, twL);
            for (int it = threadIdx.x; it < ZT * L; it += PTH) {
                const int t = it / L, m = it % L, y = b * ZT + t;
                if (y < RPC) st8_pol(rpl + (int64_t)(yb + y) * L + m, F[ZC::at(t, m)], pfirst);
            }
        }
        cp_async_wait_all();
        // the scratch rows are read: the cluster may overwrite it next plane
        cl.sync();
    }
}

template <int N1, int L>
size_t plane_smem(bool inv) {
    using ZC = XCfg<L, PTH>;
    using YC = XCfg<N1, PTH>;
    const int zreg = inv ? 2 * ZC::T * (L + 2) + ZC::BUF : 2 * ZC::BUF;
    const int yreg = 2 * YC::BUF;
    const int reg = zreg > yreg ? zreg : yreg;
    return (size_t)(reg + N1 + L + L + 1) * sizeof(float2);
}

template <int N1, int L, int CL>
cudaError_t plane_config(bool inv, cudaLaunchConfig_t *cfg, cudaLaunchAttribute *attr, int *ncl) {
    const size_t sm = plane_smem<N1, L>(inv);
    const void *fn = inv ? (const void *)k_plane_c2r<N1, L, CL> : (const void *)k_plane_r2c<N1, L, CL>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess && CL > 8)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    *cfg = cudaLaunchConfig_t{};
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg->blockDim = dim3(PTH);
    cfg->dynamicSmemBytes = sm;
    cfg->attrs = attr;
    cfg->numAttrs = 1;
    cfg->gridDim = dim3(CL);
    return cudaOccupancyMaxActiveClusters(ncl, fn, cfg);
}

template <int N1, int L, int CL>
int launch_plane(bool inv, const void *in, void *out, const float2 *ptw, int64_t nplanes,
                 float2 *scratch, int max_clusters, cudaStream_t st) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    int ncl = 0;
    PMX_CUDA((plane_config<N1, L, CL>(inv, &cfg, attr, &ncl)));
    if (ncl < 1) return fail(PMX_ERR_CUDA, "plane transform cluster does not fit on the GPU");
    if (ncl > max_clusters) ncl = max_clusters;
    if (ncl > nplanes) ncl = (int)nplanes;
    cfg.gridDim = dim3(ncl * CL);
    cfg.stream = st;
    PGeom g;
    g.nplanes = nplanes;
    g.scratch = scratch;
    if (inv) {
        PMX_CUDA(cudaLaunchKernelEx(&cfg, k_plane_c2r<N1, L, CL>, (const float2 *)in, (float *)out,
                                    ptw, g));
        PMX_LAUNCH_CHECK("k_plane_c2r");
    } else {
        PMX_CUDA(cudaLaunchKernelEx(&cfg, k_plane_r2c<N1, L, CL>, (const float *)in, (float2 *)out,
                                    ptw, g));
        PMX_LAUNCH_CHECK("k_plane_r2c");
    }
    return PMX_OK;
}

}  // namespace

bool xpass_supported(int64_t n0) {
    return n0 == 64 || n0 == 128 || n0 == 256 || n0 == 512 || n0 == 1024;
}

int xpass(bool adj, const float2 *in, float2 *out, const float *kt, const float2 *tw, int64_t n0,
          int64_t n1, int64_t n2h, int64_t rs, float c, cudaStream_t st) {
    switch (n0) {
        case 64: return launch_xpass<64>(adj, in, out, kt, tw, n1, n2h, rs, c, st);
        case 128: return launch_xpass<128>(adj, in, out, kt, tw, n1, n2h, rs, c, st);
        case 256: return launch_xpass<256>(adj, in, out, kt, tw, n1, n2h, rs, c, st);
        case 512: return launch_xpass<512>(adj, in, out, kt, tw, n1, n2h, rs, c, st);
        case 1024: return launch_xpass<1024>(adj, in, out, kt, tw, n1, n2h, rs, c, st);
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


bool plane_supported(int64_t n1, int64_t n2) {
    return n1 == n2 && (n1 == 64 || n1 == 128 || n1 == 256 || n1 == 512 || n1 == 1024);
}

int plane_max_clusters(int64_t n1, int64_t n2, bool c16, int *ncl) {
    if (!plane_supported(n1, n2)) return fail(PMX_ERR_SHAPE, "plane transform needs square power-of-two planes 64..1024");
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    int a = 0, b = 0;
    cudaError_t e = cudaSuccess;
#define PMX_PLANE_Q(N1_, L_)                                                                       \
    if (c16) {                                                                                      \
        e = plane_config<N1_, L_, 16>(false, &cfg, attr, &a);                                       \
        if (e == cudaSuccess) e = plane_config<N1_, L_, 16>(true, &cfg, attr, &b);                  \
    } else {                                                                                        \
        e = plane_config<N1_, L_, 8>(false, &cfg, attr, &a);                                        \
        if (e == cudaSuccess) e = plane_config<N1_, L_, 8>(true, &cfg, attr, &b);                   \
    }
    switch (n1) {
        case 64: PMX_PLANE_Q(64, 32) break;
        case 128: PMX_PLANE_Q(128, 64) break;
        case 256: PMX_PLANE_Q(256, 128) break;
        case 512: PMX_PLANE_Q(512, 256) break;
        default: PMX_PLANE_Q(1024, 512) break;
    }
#undef PMX_PLANE_Q
    if (e != cudaSuccess) return cuda_status(e, "plane kernel occupancy");
    *ncl = a > b ? a : b;
    if (*ncl < 1) return fail(PMX_ERR_CUDA, "plane transform cluster does not fit on the GPU");
    return PMX_OK;
}

int plane_fft(bool inv, const void *in, void *out, const float2 *ptw, int64_t nplanes, int64_t n1,
              int64_t n2, float2 *scratch, int max_clusters, bool c16, cudaStream_t st) {
    if (!plane_supported(n1, n2)) return fail(PMX_ERR_SHAPE, "plane transform needs square power-of-two planes 64..1024");
    if (nplanes < 1) return PMX_OK;
#define PMX_PLANE_L(N1_, L_)                                                                       \
    return c16 ? launch_plane<N1_, L_, 16>(inv, in, out, ptw, nplanes, scratch, max_clusters, st)  \
               : launch_plane<N1_, L_, 8>(inv, in, out, ptw, nplanes, scratch, max_clusters, st);
    switch (n1) {
        case 64: PMX_PLANE_L(64, 32)
        case 128: PMX_PLANE_L(128, 64)
        case 256: PMX_PLANE_L(256, 128)
        case 512: PMX_PLANE_L(512, 256)
        default: PMX_PLANE_L(1024, 512)
    }
#undef PMX_PLANE_L
}

// [exp(-2 pi i m / n1), m < n1 | exp(-2 pi i m / L), m < L | exp(-2 pi i k / n2), k <= L],
// L = n2 / 2; float64 on the host, then float32.
void plane_twiddles(int64_t n1, int64_t n2, float2 *host) {
    const int64_t L = n2 / 2;
    int64_t o = 0;
    for (int64_t m = 0; m < n1; ++m, ++o) {
        double a = -2.0 * kPi * (double)m / (double)n1;
        host[o] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    for (int64_t m = 0; m < L; ++m, ++o) {
        double a = -2.0 * kPi * (double)m / (double)L;
        host[o] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    for (int64_t k = 0; k <= L; ++k, ++o) {
        double a = -2.0 * kPi * (double)k / (double)n2;
        host[o] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
}

}  // namespace pmx
