// Power-spectrum binning of half spectra (pmwd/spec_util.py:50-147).
//
// The reference builds |k|, P and the Hermitian multiplicity as full-mesh
// float64 arrays, digitizes |k| against the bin edges and sums with
// bincount.  Here one pass reads the complex64 spectrum (and the second one
// of a cross spectrum) once: every thread computes |k| from the float64
// wavenumber tables in the reference's order ((kx^2 + ky^2) + kz^2), the bin
// with numpy digitize semantics, P in float64 (|F|^2 from the widened parts,
// or F conj(G) formed in complex64 and widened, as the reference does), the
// optional sinc^-deconv window, and accumulates k N, P N and N per bin:
// warp shuffle sums per distinct bin, then shared-memory float64 sums merged
// once per block.

#include <cuda_runtime.h>

#include <algorithm>

#include "pmx_internal.cuh"

namespace pmx {
namespace {

constexpr int ST = 256;
constexpr int SMEM_BINS = 2048;  // per-block shared accumulators up to this many bins

// numpy.digitize(x, edges, right): right = 0 -> count of edges <= x,
// right = 1 -> count of edges < x (edges increasing).
__device__ __forceinline__ int digitize(double x, const double *e, int ne, int right) {
    int lo = 0, hi = ne;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const bool go = right ? (e[mid] < x) : (e[mid] <= x);
        if (go) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// sinc(x) = sin(pi x) / (pi x), 1 at 0 (torch.sinc / jnp.sinc)
__device__ __forceinline__ double sincd(double x) {
    return x == 0.0 ? 1.0 : sinpi(x) / (3.141592653589793238462643383279502884 * x);
}

struct SpecArgs {
    const float2 *F, *G;
    int64_t nb, n0, n1, n2h, Mc;
    int nyq_z;                    // 1: the last z index is the Nyquist plane (even n2)
    const double *kx, *ky, *kz;   // cycles per sample (fftfreq / rfftfreq)
    const double *edges;
    int ne, right, nbin;
    double deconv;                // 0: none
    double *ksum, *psum, *nsum;   // nbin, 2 nbin (re, im), nbin
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Each warp takes 32 consecutive cells (mostly one or two bins: |k| varies
// slowly along a row), sums its lanes per distinct bin with shuffles, and
// one lane adds each bin's sums to the block's shared accumulators (SH) or
// to global memory.
template <bool SH>
__global__ void __launch_bounds__(ST) k_powspec(SpecArgs a) {
    extern __shared__ double sb[];  // SH: 4 doubles per bin (k N, P_re N, P_im N, N)
    if (SH) {
        for (int i = threadIdx.x; i < 4 * a.nbin; i += ST) sb[i] = 0.0;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    for (int64_t c0 = blockIdx.x * (int64_t)ST + (threadIdx.x & ~31); c0 < a.Mc;
         c0 += (int64_t)gridDim.x * ST) {  // warp-uniform
        const int64_t c = c0 + lane;
        int b = a.nbin;  // "no bin"
        double kn = 0.0, prn = 0.0, pin = 0.0, N = 0.0;
        if (c < a.Mc) {
            const int64_t l = c % a.n2h, r = c / a.n2h;
            const int64_t j = r % a.n1, i = r / a.n1;
            const double kxi = a.kx[i], kyj = a.ky[j], kzl = a.kz[l];
            const double k = sqrt(
                __dadd_rn(__dadd_rn(__dmul_rn(kxi, kxi), __dmul_rn(kyj, kyj)), __dmul_rn(kzl, kzl)));
            b = digitize(k, a.edges, a.ne, a.right);
            if (b < a.nbin) {
                N = (l == 0 || (a.nyq_z && l == a.n2h - 1)) ? 1.0 : 2.0;
                double pr = 0.0, pi = 0.0;
                for (int64_t t = 0; t < a.nb; ++t) {
                    const float2 f = a.F[t * a.Mc + c];
                    if (a.G) {
                        const float2 gg = a.G[t * a.Mc + c];
                        // F * conj(G) in complex64, then widened
                        pr += (double)__fadd_rn(__fmul_rn(f.x, gg.x), __fmul_rn(f.y, gg.y));
                        pi += (double)__fsub_rn(__fmul_rn(f.y, gg.x), __fmul_rn(f.x, gg.y));
                    } else {
                        pr += __dadd_rn(__dmul_rn((double)f.x, (double)f.x),
                                        __dmul_rn((double)f.y, (double)f.y));
                    }
                }
                if (a.deconv != 0.0) {
                    const double w = pow(sincd(kxi), -a.deconv) * pow(sincd(kyj), -a.deconv) *
                                     pow(sincd(kzl), -a.deconv);
                    pr *= w;
                    pi *= w;
                }
                kn = k * N;
                prn = pr * N;
                pin = pi * N;
            } else {
                b = a.nbin;
            }
        }
        // per distinct bin of the warp: shuffle sums, one add
        unsigned pending = __ballot_sync(0xffffffffu, b < a.nbin);
        while (pending) {
            const int src = __ffs(pending) - 1;
            const int bb = __shfl_sync(0xffffffffu, b, src);
            const bool mine = b == bb;
            const double s0 = warp_sum(mine ? kn : 0.0), s1 = warp_sum(mine ? prn : 0.0);
            const double s2 = a.G ? warp_sum(mine ? pin : 0.0) : 0.0;
            const double s3 = warp_sum(mine ? N : 0.0);
            if (lane == src) {
                if (SH) {
                    atomicAdd(sb + 4 * bb, s0);
                    atomicAdd(sb + 4 * bb + 1, s1);
                    if (a.G) atomicAdd(sb + 4 * bb + 2, s2);
                    atomicAdd(sb + 4 * bb + 3, s3);
                } else {
                    atomicAdd(a.ksum + bb, s0);
                    atomicAdd(a.psum + 2 * bb, s1);
                    if (a.G) atomicAdd(a.psum + 2 * bb + 1, s2);
                    atomicAdd(a.nsum + bb, s3);
                }
            }
            pending &= ~__ballot_sync(0xffffffffu, mine);
        }
    }
    if (SH) {
        __syncthreads();
        for (int b = threadIdx.x; b < a.nbin; b += ST) {
            if (sb[4 * b + 3] == 0.0) continue;
            atomicAdd(a.ksum + b, sb[4 * b]);
            atomicAdd(a.psum + 2 * b, sb[4 * b + 1]);
            if (a.G) atomicAdd(a.psum + 2 * b + 1, sb[4 * b + 2]);
            atomicAdd(a.nsum + b, sb[4 * b + 3]);
        }
    }
}

// ---------------------------------------------------------------------------
// Power-of-two grids.  fftfreq values are i/n exactly, so k^2 = i^2/n0^2 +
// j^2/n1^2 + l^2/n2^2 is exact in float64 (multiples of 1/D, D = max(n)^2)
// whatever the summation order, and k = sqrt(m / D) with the integer
// m = i^2 D/n0^2 + j^2 D/n1^2 + l^2 D/n2^2: |k| and its bin depend on m only.
// Tables of k(m) and bin(m) (built once per call, float64 as the reference)
// replace the per-cell float64 |k|.  GB300's float64 rate is low, so this
// path keeps float64 out of the per-cell work: P N is formed in float32 and
// summed per bin with warp shuffles before one float64 add.  The sums k N
// and N depend on the grid alone; they are accumulated (float64 per cell)
// only when ksum / nsum are given, so a caller can compute them once per
// grid and bins and pass NULL afterwards.
// ---------------------------------------------------------------------------

struct Pow2Args {
    const float2 *F, *G;
    int64_t nb, n0, n1, n2h, Mc;
    int nyq_z;
    int64_t ax, ay, az;            // D / n_a^2
    int h0, h1;                    // n0, n1 (signed index: i' = i <= n/2 ? i : i - n)
    const double *ktab;            // k(m)
    const int *btab;               // bin(m), nbin = none
    const float *wx, *wy, *wz;     // sinc^-deconv per axis, or NULL
    int nbin;
    int zm;                        // 1: layout (n2h, n0, n1), y contiguous
    double *ksum, *psum, *nsum;
};

__global__ void k_pow2_tables(int64_t mmax, double D, const double *edges, int ne, int right,
                              int nbin, double *ktab, int *btab) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m <= mmax;
         m += (int64_t)gridDim.x * blockDim.x) {
        const double k = sqrt((double)m / D);  // exact quotient (D a power of two)
        ktab[m] = k;
        const int b = digitize(k, edges, ne, right);
        btab[m] = b < nbin ? b : nbin;
    }
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One warp per (x, y) row of n2h cells, lanes on consecutive kz (coalesced
// loads); per 32 cells, shuffle sums per distinct bin (usually one or two)
// and one float64 shared-memory add per bin.  CROSS: F conj(G); GEOM: also
// the sums of k N and N; WIN: sinc^-deconv windows.  PRIV (few bins): every
// warp owns its own bin array, so the per-bin adds are plain stores of one
// lane instead of float64 atomics that all warps of the block contend for;
// the arrays are summed at the end.
constexpr int PRIV_BINS = 64;

template <bool CROSS, bool GEOM, bool WIN, bool PRIV>
__global__ void __launch_bounds__(ST, 6) k_powspec_rows(Pow2Args a) {
    extern __shared__ double sbase[];  // 4 doubles per bin (per warp with PRIV)
    const int nacc = (PRIV ? ST / 32 : 1) * 4 * a.nbin;
    for (int i = threadIdx.x; i < nacc; i += ST) sbase[i] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    double *sb = PRIV ? sbase + (threadIdx.x >> 5) * 4 * a.nbin : sbase;
    const int n2h = (int)a.n2h, az = (int)a.az;
    // rows of contiguous cells: (x, y) rows along kz for the (n0, n1, n2h)
    // layout; with zm, (kz, x) rows along y of the (n2h, n0, n1) layout that
    // torch's CUDA rfftn returns, which this kernel serves only for n1 < 32
    // or n1 not a multiple of 32 (k_powspec_runs takes the others)
    // every index below fits in 32 bits (grids up to 2048: rows < 2^22,
    // bin-table indices < 2^31)
    const int n0 = (int)a.n0, n1 = (int)a.n1, h0 = a.h0, h1 = a.h1;
    const int ax = (int)a.ax, ay = (int)a.ay;
    const int nrows = a.zm ? n2h * n0 : n0 * n1;
    const int nlane = a.zm ? n1 : n2h;
    const int wstride = gridDim.x * (ST / 32);
    for (int row = blockIdx.x * (ST / 32) + (threadIdx.x >> 5); row < nrows;
         row += wstride) {  // warp-uniform
        int i, j = 0, lr = 0, mrow;
        if (a.zm) {
            lr = row / n0;
            i = row - lr * n0;
            const int si = i <= h0 / 2 ? i : i - h0;
            mrow = si * si * ax + lr * lr * az;
        } else {
            i = row / n1;
            j = row - i * n1;
            const int si = i <= h0 / 2 ? i : i - h0, sj = j <= h1 / 2 ? j : j - h1;
            mrow = si * si * ax + sj * sj * ay;
        }
        const float2 *Fr = a.F + (int64_t)row * nlane;
        const float2 *Gr = CROSS ? a.G + (int64_t)row * nlane : nullptr;
        for (int c0 = 0; c0 < nlane; c0 += 32) {
            const int c = c0 + lane;   // kz, or y with zm
            int b = a.nbin;
            float pr = 0.f, pi = 0.f;
            double kn = 0.0, nn = 0.0;
            if (c < nlane) {
                int m, l, jj;
                if (a.zm) {
                    const int sjj = c <= h1 / 2 ? c : c - h1;
                    m = mrow + sjj * sjj * ay;
                    l = lr;
                    jj = c;
                } else {
                    m = mrow + c * c * az;
                    l = c;
                    jj = j;
                }
                b = a.btab[m];
                if (b < a.nbin) {
                    for (int64_t t = 0; t < a.nb; ++t) {
                        const float2 f = Fr[t * a.Mc + c];
                        if (CROSS) {
                            const float2 gg = Gr[t * a.Mc + c];
                            pr += __fadd_rn(__fmul_rn(f.x, gg.x), __fmul_rn(f.y, gg.y));
                            pi += __fsub_rn(__fmul_rn(f.y, gg.x), __fmul_rn(f.x, gg.y));
                        } else {
                            pr += fmaf(f.x, f.x, f.y * f.y);
                        }
                    }
                    if (WIN) {  // ((P wx) wy) wz
                        const float w = (a.wx[i] * a.wy[jj]) * a.wz[l];
                        pr *= w;
                        pi *= w;
                    }
                    const bool two = !(l == 0 || (a.nyq_z && l == n2h - 1));
                    if (two) {
                        pr += pr;
                        pi += pi;
                    }
                    if (GEOM) {
                        const double k = a.ktab[m];
                        kn = two ? k + k : k;
                        nn = two ? 2.0 : 1.0;
                    }
                }
            }
            // many distinct bins in these 32 cells (fine linear bins): each
            // lane adds its own values; few: shuffle sums per bin
            const unsigned peers = __match_any_sync(0xffffffffu, b);
            const int ndist = __popc(__ballot_sync(0xffffffffu, lane == __ffs(peers) - 1));
            if (ndist > 4) {
                if (b < a.nbin) {
                    atomicAdd(sb + 4 * b + 1, (double)pr);
                    if (CROSS) atomicAdd(sb + 4 * b + 2, (double)pi);
                    if (GEOM) {
                        atomicAdd(sb + 4 * b, kn);
                        atomicAdd(sb + 4 * b + 3, nn);
                    }
                }
                continue;
            }
            unsigned pending = __ballot_sync(0xffffffffu, b < a.nbin);
            while (pending) {
                const int src = __ffs(pending) - 1;
                const int bb = __shfl_sync(0xffffffffu, b, src);
                const bool mine = b == bb;
                const float spr = warp_sumf(mine ? pr : 0.f);
                const float spi = CROSS ? warp_sumf(mine ? pi : 0.f) : 0.f;
                double sk = 0.0, sn = 0.0;
                if (GEOM) {
                    sk = warp_sum(mine ? kn : 0.0);
                    sn = warp_sum(mine ? nn : 0.0);
                }
                if (lane == src) {
                    if (PRIV) {  // this warp's array: one lane at a time
                        sb[4 * bb + 1] += (double)spr;
                        if (CROSS) sb[4 * bb + 2] += (double)spi;
                        if (GEOM) {
                            sb[4 * bb] += sk;
                            sb[4 * bb + 3] += sn;
                        }
                    } else {
                        atomicAdd(sb + 4 * bb + 1, (double)spr);
                        if (CROSS) atomicAdd(sb + 4 * bb + 2, (double)spi);
                        if (GEOM) {
                            atomicAdd(sb + 4 * bb, sk);
                            atomicAdd(sb + 4 * bb + 3, sn);
                        }
                    }
                }
                pending &= ~__ballot_sync(0xffffffffu, mine);
            }
            if (PRIV) __syncwarp();  // the next chunk's adds see these
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < a.nbin; b += ST) {
        double acc[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[c] = sbase[4 * b + c];
        if (PRIV)
            for (int w = 1; w < ST / 32; ++w)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[c] += sbase[w * 4 * a.nbin + 4 * b + c];
        if (GEOM) {
            atomicAdd(a.ksum + b, acc[0]);
            atomicAdd(a.nsum + b, acc[3]);
        }
        atomicAdd(a.psum + 2 * b, acc[1]);
        if (CROSS) atomicAdd(a.psum + 2 * b + 1, acc[2]);
    }
}

// Half-axis-major spectra with n1 a multiple of 32: the warp takes row
// (kz, x) and lane r walks the contiguous run y in [r n1/32, (r+1) n1/32),
// keeping the sums of its current bin in registers.  The bins are shells in
// |k|, so a run changes bin rarely: then the lane adds its sums to the bin
// array, and at the end of the row the lanes holding the same bin are
// merged by shuffles and added once.  Every shared-memory add is atomic.
template <bool CROSS, bool GEOM, bool WIN, bool PRIV>
__global__ void __launch_bounds__(ST, 6) k_powspec_runs(Pow2Args a) {
    extern __shared__ double sbase[];  // 4 doubles per bin (per warp with PRIV)
    const int nacc = (PRIV ? ST / 32 : 1) * 4 * a.nbin;
    for (int i = threadIdx.x; i < nacc; i += ST) sbase[i] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    double *sb = PRIV ? sbase + (threadIdx.x >> 5) * 4 * a.nbin : sbase;
    const int n2h = (int)a.n2h, n0 = (int)a.n0, n1 = (int)a.n1, h0 = a.h0, h1 = a.h1;
    const int ax = (int)a.ax, ay = (int)a.ay, az = (int)a.az, nbin = a.nbin;
    const int R = n1 / 32, nrows = n2h * n0;
    const int wstride = gridDim.x * (ST / 32);
    auto add = [&](int b, double pr, double pi, double kn, double nn) {
        atomicAdd(sb + 4 * b + 1, pr);
        if (CROSS) atomicAdd(sb + 4 * b + 2, pi);
        if (GEOM) {
            atomicAdd(sb + 4 * b, kn);
            atomicAdd(sb + 4 * b + 3, nn);
        }
    };
    for (int row = blockIdx.x * (ST / 32) + (threadIdx.x >> 5); row < nrows;
         row += wstride) {  // warp-uniform
        const int l = row / n0, i = row - l * n0;
        const int si = i <= h0 / 2 ? i : i - h0;
        const int mrow = si * si * ax + l * l * az;
        const bool two = !(l == 0 || (a.nyq_z && l == n2h - 1));
        const int j0 = lane * R;
        const float2 *Fr = a.F + (int64_t)row * n1 + j0;
        const float2 *Gr = CROSS ? a.G + (int64_t)row * n1 + j0 : nullptr;
        int cur = nbin;
        // a run holds up to n1/32 cells: its sums are float64, so a long
        // run rounds like the row kernel's per-32-cell float sums
        double ar = 0.0, ai = 0.0, ak = 0.0, an = 0.0;
        for (int r = 0; r < R; ++r) {
            const int j = j0 + r;
            const int sj = j <= h1 / 2 ? j : j - h1;
            const int m = mrow + sj * sj * ay;
            const int b = a.btab[m];
            if (b != cur) {
                if (cur < nbin) add(cur, ar, ai, ak, an);
                cur = b;
                ar = ai = ak = an = 0.0;
            }
            if (b < nbin) {
                float pr = 0.f, pi = 0.f;
                for (int64_t t = 0; t < a.nb; ++t) {
                    const float2 f = Fr[t * a.Mc + r];
                    if (CROSS) {
                        const float2 gg = Gr[t * a.Mc + r];
                        pr += __fadd_rn(__fmul_rn(f.x, gg.x), __fmul_rn(f.y, gg.y));
                        pi += __fsub_rn(__fmul_rn(f.y, gg.x), __fmul_rn(f.x, gg.y));
                    } else {
                        pr += fmaf(f.x, f.x, f.y * f.y);
                    }
                }
                if (WIN) {  // ((P wx) wy) wz
                    const float w = (a.wx[i] * a.wy[j]) * a.wz[l];
                    pr *= w;
                    pi *= w;
                }
                if (two) {
                    pr += pr;
                    pi += pi;
                }
                ar += pr;
                ai += pi;
                if (GEOM) {
                    const double k = a.ktab[m];
                    ak += two ? k + k : k;
                    an += two ? 2.0 : 1.0;
                }
            }
        }
        __syncwarp();
        // end of row: lanes still holding sums merge per bin
        const int b = cur;
        const unsigned peers = __match_any_sync(0xffffffffu, b);
        const int ndist = __popc(__ballot_sync(0xffffffffu, lane == __ffs(peers) - 1));
        if (ndist > 4) {
            if (b < nbin) add(b, ar, ai, ak, an);
        } else {
            unsigned pending = __ballot_sync(0xffffffffu, b < nbin);
            while (pending) {
                const int src = __ffs(pending) - 1;
                const int bb = __shfl_sync(0xffffffffu, b, src);
                const bool mine = b == bb;
                const double spr = warp_sum(mine ? ar : 0.0);
                const double spi = CROSS ? warp_sum(mine ? ai : 0.0) : 0.0;
                double sk = 0.0, sn = 0.0;
                if (GEOM) {
                    sk = warp_sum(mine ? ak : 0.0);
                    sn = warp_sum(mine ? an : 0.0);
                }
                if (lane == src) add(bb, spr, spi, sk, sn);
                pending &= ~__ballot_sync(0xffffffffu, mine);
            }
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < a.nbin; b += ST) {
        double acc[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[c] = sbase[4 * b + c];
        if (PRIV)
            for (int w = 1; w < ST / 32; ++w)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[c] += sbase[w * 4 * a.nbin + 4 * b + c];
        if (GEOM) {
            atomicAdd(a.ksum + b, acc[0]);
            atomicAdd(a.nsum + b, acc[3]);
        }
        atomicAdd(a.psum + 2 * b, acc[1]);
        if (CROSS) atomicAdd(a.psum + 2 * b + 1, acc[2]);
    }
}

// Dynamic shared memory above the default 48 KB needs the opt-in attribute.
template <class K>
void allow_smem(K *kern, size_t sm) {
    if (sm > 48 * 1024)
        cudaFuncSetAttribute(reinterpret_cast<const void *>(kern),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
}

template <bool CROSS, bool GEOM, bool PRIV>
void launch_rows_p(const Pow2Args &p, cudaStream_t s) {
    const size_t sm = (PRIV ? ST / 32 : 1) * 4 * (size_t)p.nbin * sizeof(double);
    if (p.zm && p.n1 >= 32 && p.n1 % 32 == 0) {   // contiguous runs per lane
        const int grid = stride_grid(p.n2h * p.n0 * 32, ST, 6);
        if (p.wx) {
            allow_smem(k_powspec_runs<CROSS, GEOM, true, PRIV>, sm);
            k_powspec_runs<CROSS, GEOM, true, PRIV><<<grid, ST, sm, s>>>(p);
        } else {
            allow_smem(k_powspec_runs<CROSS, GEOM, false, PRIV>, sm);
            k_powspec_runs<CROSS, GEOM, false, PRIV><<<grid, ST, sm, s>>>(p);
        }
        return;
    }
    const int grid = stride_grid(p.n0 * p.n1 * 32, ST, 8);
    if (p.wx) {
        allow_smem(k_powspec_rows<CROSS, GEOM, true, PRIV>, sm);
        k_powspec_rows<CROSS, GEOM, true, PRIV><<<grid, ST, sm, s>>>(p);
    } else {
        allow_smem(k_powspec_rows<CROSS, GEOM, false, PRIV>, sm);
        k_powspec_rows<CROSS, GEOM, false, PRIV><<<grid, ST, sm, s>>>(p);
    }
}

template <bool CROSS, bool GEOM>
void launch_rows(const Pow2Args &p, cudaStream_t s) {
    if (p.nbin <= PRIV_BINS)
        launch_rows_p<CROSS, GEOM, true>(p, s);
    else
        launch_rows_p<CROSS, GEOM, false>(p, s);
}

bool is_pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

__global__ void k_sinc_tab(const double *k, int64_t n, double deconv, float *w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        w[i] = (float)pow(sincd(k[i]), -deconv);
}

}  // namespace
}  // namespace pmx

using namespace pmx;

static int powspec_bin(const float *F, const float *G, int64_t nbatch, const int64_t grid_shape[3],
                       const double *kx, const double *ky, const double *kz, const double *edges,
                       int32_t nedges, int32_t right, int32_t nbin, double deconv, double *ksum,
                       double *psum, double *nsum, void *stream, bool zm) {
    clear_error();
    if (!F || !grid_shape || !kx || !ky || !kz || !edges || !psum)
        return fail(PMX_ERR_ARG, "null argument");
    if (!ksum != !nsum) return fail(PMX_ERR_ARG, "ksum and nsum are both given or both NULL");
    if (nbatch < 1 || nedges < 1 || nbin < 1 || nbin > nedges)
        return fail(PMX_ERR_ARG, "need nbatch >= 1 and 1 <= nbin <= nedges");
    for (int a = 0; a < 3; ++a)
        if (grid_shape[a] < 1) return fail(PMX_ERR_SHAPE, "bad grid shape");
    SpecArgs a;
    a.F = reinterpret_cast<const float2 *>(F);
    a.G = reinterpret_cast<const float2 *>(G);
    a.nb = nbatch;
    a.n0 = grid_shape[0];
    a.n1 = grid_shape[1];
    a.n2h = grid_shape[2] / 2 + 1;
    a.Mc = a.n0 * a.n1 * a.n2h;
    a.nyq_z = grid_shape[2] % 2 == 0;
    a.kx = kx;
    a.ky = ky;
    a.kz = kz;
    a.edges = edges;
    a.ne = nedges;
    a.right = right != 0;
    a.nbin = nbin;
    a.deconv = deconv;
    a.ksum = ksum;
    a.psum = psum;
    a.nsum = nsum;
    cudaStream_t s = as_stream(stream);
    const int64_t nmax = std::max(grid_shape[0], std::max(grid_shape[1], grid_shape[2]));
    if (is_pow2(grid_shape[0]) && is_pow2(grid_shape[1]) && is_pow2(grid_shape[2]) && nmax <= 2048 &&
        nbin <= SMEM_BINS) {
        // tables of k(m), bin(m) and the per-axis windows: stream-ordered
        // scratch, freed after the launch (the stream keeps them alive)
        Pow2Args p;
        p.zm = zm;
        p.F = a.F;
        p.G = a.G;
        p.nb = a.nb;
        p.n0 = a.n0;
        p.n1 = a.n1;
        p.n2h = a.n2h;
        p.Mc = a.Mc;
        p.nyq_z = a.nyq_z;
        const int64_t D = nmax * nmax;
        p.ax = D / (grid_shape[0] * grid_shape[0]);
        p.ay = D / (grid_shape[1] * grid_shape[1]);
        p.az = D / (grid_shape[2] * grid_shape[2]);
        p.h0 = (int)grid_shape[0];
        p.h1 = (int)grid_shape[1];
        const int64_t i0 = grid_shape[0] / 2, j0 = grid_shape[1] / 2, l0 = a.n2h - 1;
        const int64_t mmax = i0 * i0 * p.ax + j0 * j0 * p.ay + l0 * l0 * p.az;
        p.nbin = nbin;
        p.ksum = ksum;
        p.psum = psum;
        p.nsum = nsum;
        char *scr = nullptr;
        const size_t tb = (size_t)(mmax + 1) * (sizeof(double) + sizeof(int));
        const size_t wb = deconv != 0.0 ? (size_t)(a.n0 + a.n1 + a.n2h) * sizeof(float) : 0;
        PMX_CUDA(cudaMallocAsync((void **)&scr, tb + wb, s));
        double *ktab = reinterpret_cast<double *>(scr);
        int *btab = reinterpret_cast<int *>(scr + (size_t)(mmax + 1) * sizeof(double));
        p.ktab = ktab;
        p.btab = btab;
        p.wx = p.wy = p.wz = nullptr;
        k_pow2_tables<<<stride_grid(mmax + 1, 256, 4), 256, 0, s>>>(mmax, (double)D, edges, nedges,
                                                                     a.right, nbin, ktab, btab);
        if (wb) {
            float *w = reinterpret_cast<float *>(scr + tb);
            k_sinc_tab<<<1, 256, 0, s>>>(kx, a.n0, deconv, w);
            k_sinc_tab<<<1, 256, 0, s>>>(ky, a.n1, deconv, w + a.n0);
            k_sinc_tab<<<1, 256, 0, s>>>(kz, a.n2h, deconv, w + a.n0 + a.n1);
            p.wx = w;
            p.wy = w + a.n0;
            p.wz = w + a.n0 + a.n1;
        }
        if (a.G) {
            if (ksum) launch_rows<true, true>(p, s);
            else launch_rows<true, false>(p, s);
        } else {
            if (ksum) launch_rows<false, true>(p, s);
            else launch_rows<false, false>(p, s);
        }
        PMX_LAUNCH_CHECK("k_powspec_rows");
        PMX_CUDA(cudaFreeAsync(scr, s));
        return PMX_OK;
    }
    if (zm) return fail(PMX_ERR_SHAPE, "the (n2h, n0, n1) layout needs a power-of-two grid <= 2048");
    if (!ksum) return fail(PMX_ERR_ARG, "ksum/nsum may be NULL only for power-of-two grids <= 2048");
    const int grid = stride_grid(a.Mc, ST, 4);
    if (nbin <= SMEM_BINS) {
        allow_smem(k_powspec<true>, 4 * nbin * sizeof(double));
        k_powspec<true><<<grid, ST, 4 * nbin * sizeof(double), s>>>(a);
    } else {
        k_powspec<false><<<grid, ST, 0, s>>>(a);
    }
    PMX_LAUNCH_CHECK("k_powspec");
    return PMX_OK;
}

extern "C" int pmx_powspec_bin(const float *F, const float *G, int64_t nbatch,
                               const int64_t grid_shape[3], const double *kx, const double *ky,
                               const double *kz, const double *edges, int32_t nedges,
                               int32_t right, int32_t nbin, double deconv, double *ksum,
                               double *psum, double *nsum, void *stream) {
    return powspec_bin(F, G, nbatch, grid_shape, kx, ky, kz, edges, nedges, right, nbin, deconv,
                       ksum, psum, nsum, stream, false);
}

extern "C" int pmx_powspec_bin_zmajor(const float *F, const float *G, int64_t nbatch,
                                      const int64_t grid_shape[3], const double *kx,
                                      const double *ky, const double *kz, const double *edges,
                                      int32_t nedges, int32_t right, int32_t nbin, double deconv,
                                      double *ksum, double *psum, double *nsum, void *stream) {
    return powspec_bin(F, G, nbatch, grid_shape, kx, ky, kz, edges, nedges, right, nbin, deconv,
                       ksum, psum, nsum, stream, true);
}
