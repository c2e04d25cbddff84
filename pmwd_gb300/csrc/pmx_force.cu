// Poisson force, leapfrog and reversible-adjoint kernels (the hot path).
//
// Reference: pmwd/gravity.py:47-72 (gravity), pmwd/nbody.py:39-162
// (drift/kick/force, their adjoints and the symplectic step).  All kernels
// here are specialised for the path the N-body loop takes: 3-D, default
// enmesh branch (offset 0, cell_size None), one channel, scalar value
// conf.mesh_size / conf.ptcl_num.
//
// Device layout of a workspace (float32 unless noted):
//   dens  M           CIC density (initialised to -1, so it holds the overdensity)
//   ck    3 * Mc      complex64 half spectra (r2c output; the Fourier kernel
//                     writes the three gradient spectra over it)
//   g     3 * M       real acceleration meshes (planar, one per axis)
//   mcot  3 * M       cotangents of g (adjoint workspaces only)
//   ktab  2*(n0+n1+n2h) angular wavenumbers, plain and Nyquist-masked
//   part  4 * pstride float64 per-block partial sums of the dot products
// with M = n0*n1*n2 and Mc = n0*n1*(n2/2+1).

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "pmx_internal.cuh"

using namespace pmx;

namespace {

constexpr int PMAX = 4096;       // max blocks of the stand-alone dot kernels (partials)
// Per-block partial sums per dot slot of a workspace: one per block of a
// particle kernel, whose grids reach one particle per thread up to 2^27
// particles (512^3) in a single-simulation workspace; 2^16 per simulation
// of a batched one.
constexpr int64_t PART_ONE = int64_t(1) << 19;
constexpr int64_t PART_SLOT = int64_t(1) << 16;
constexpr int BMAX = 16;         // most simulations of one batched call
constexpr int NSLOT = 4;         // dot-product slots
constexpr int PT = 256;          // threads per particle kernel
constexpr double PI = 3.141592653589793;

const char *cufft_name(cufftResult r) {
    switch (r) {
        case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
        case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
        case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
        case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
        case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
        case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
        case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
        case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
        default: return "cuFFT error";
    }
}

#define PMX_CUFFT(call)                                                                   \
    do {                                                                                  \
        cufftResult r_ = (call);                                                          \
        if (r_ != CUFFT_SUCCESS)                                                          \
            return fail(PMX_ERR_CUFFT, std::string(#call) + ": " + cufft_name(r_));       \
    } while (0)

}  // namespace

namespace pmx {
namespace slabs {
constexpr int KMAX = 4;  // most concurrent slab chains
// One slab-wise 2-D transform: a cuFFT plan (with its own work area) per
// chain, and the captured graph of the whole slab loop.
constexpr int GMAX = 16;  // captured slab graphs per transform (one per slot count)
struct SlabXf {
    cufftHandle plan[KMAX] = {};
    bool have[KMAX] = {};
    void *work[KMAX] = {};
    bool r2c = true;
    // the captured slab loop of each slot count (1..GMAX), with the buffers
    // it was captured with
    cudaGraphExec_t exec[GMAX + 1] = {};
    const void *in[GMAX + 1] = {};
    void *out[GMAX + 1] = {};
};
}  // namespace slabs
}  // namespace pmx
using pmx::slabs::SlabXf;
using pmx::slabs::KMAX;
using pmx::slabs::GMAX;

struct pmx_workspace {
    int dev = 0;
    int flags = 0;
    int64_t n0 = 0, n1 = 0, n2 = 0, n2h = 0, M = 0, Mc = 0;
    // simulations one call can carry (batched workspaces): every mesh
    // buffer below holds `slots` consecutive copies, slot-major
    int slots = 1;
    // per-block partial sums per dot slot (and per simulation slot) in part
    int64_t pstride = 0;
    float *dens = nullptr;
    float2 *ck = nullptr;
    float *g = nullptr;
    float *mcot = nullptr;
    float *ktab = nullptr;
    double *part = nullptr;
    void *fft_work = nullptr;
    size_t fft_work_bytes = 0;
    cufftHandle r2c1 = 0, c2r3 = 0, r2c3 = 0, c2r1 = 0;
    bool have_r2c1 = false, have_c2r3 = false, have_r2c3 = false, have_c2r1 = false;
    double ktab_cell = -1.0;
    // power-of-two meshes: slab-wise 2-D cuFFT over (y, z) plus the fused
    // x pass of pmx_fft.cu; meshes are then plane-interleaved (x, 3, n1, n2)
    bool xfast = false;
    bool win = false;           // warp-window deposits (n2 % 4 == 0)
    int64_t slab = 0;           // x-planes per 2-D cuFFT execution
    float2 *tw = nullptr;       // exp(-2 pi i m / n0)
    // square power-of-two planes: the (y, z) transforms are the cluster
    // plane kernels of pmx_fft.cu instead of 2-D cuFFT
    bool plane = false;
    bool plane16 = false;       // clusters of 16 CTAs instead of 8
    bool vec = false;           // vector z-pair reductions (n2 % 4 == 0)
    bool agg = false;           // warp-aggregated deposits
    bool tma = false;           // TMA-staged forward gathers (tmap describes g)
    CUtensorMap tmap;
    int *err = nullptr;         // device word: a TMA wait gave up (kernels then read global)
    float2 *ptw = nullptr;      // plane_twiddles(n1, n2)
    float2 *pscr = nullptr;     // c2r scratch: one n1 x n2p plane per cluster
    int pcl = 0;                // clusters the scratch serves
    int64_t n2p = 0;            // complex row stride: padded_row(n2h) for the plane kernels
    // slab-wise 2-D cuFFT: kinds 0..3 = r2c of the density, c2r of the three
    // gradient spectra, r2c of the three mesh cotangents, c2r of the adjoint
    SlabXf sx[4];
    int nbranch = 1;            // concurrent slab chains (streams)
    bool graphs = false;        // slab loops captured as CUDA graphs
    cudaStream_t cap = nullptr, aux[KMAX] = {};
    cudaEvent_t fork = nullptr, join[KMAX] = {};
    // the adjoint's density cotangent (rho_cot), in g behind the complex
    // spectra the last inverse transform reads (b slots of n0 n1 n2p
    // complex values for a call over b slots, then b meshes): the density
    // itself stays free, so a multi-step run can deposit the next step's
    // density while it gathers rho_cot
    float *rcot_of(int b) const { return g + 2 * b * n0 * n1 * n2p; }
    // stage profiler: CUDA events around every stage while enabled
    bool prof_on = false;
    struct Rec {
        int stage;
        cudaEvent_t b, e;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    int64_t launches = 0;  // launches of libpmx kernels (cuFFT's not counted)
};

namespace {

const char *const kStageNames[PMX_PROF_STAGES] = {
    "fill", "deposit_fwd", "r2c", "poisson_fwd", "c2r_x3", "gather3_kick",
    "kick_drift_adj_deposit", "gather3_adj", "r2c_x3", "poisson_adj", "c2r", "scatter_adj_kick",
    "finish", "gather3_kick_kick_drift_deposit", "scatter_adj_kick_kick_drift_adj_deposit"};

cudaEvent_t prof_event(pmx_workspace *ws) {
    if (!ws->pool.empty()) {
        cudaEvent_t e = ws->pool.back();
        ws->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// Brackets one stage with events when profiling is on; counts libpmx
// kernel launches (nk per stage) always.
struct Stage {
    pmx_workspace *ws;
    int id;
    cudaStream_t s;
    cudaEvent_t b = nullptr;
    Stage(pmx_workspace *w, int stage, cudaStream_t st, int nk) : ws(w), id(stage), s(st) {
        ws->launches += nk;
        if (ws->prof_on && (b = prof_event(ws))) cudaEventRecord(b, s);
    }
    ~Stage() {
        if (!b) return;
        cudaEvent_t e = prof_event(ws);
        if (!e) {
            ws->pool.push_back(b);
            return;
        }
        cudaEventRecord(e, s);
        ws->recs.push_back({id, b, e});
    }
};

}  // namespace

namespace pmx {

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------

__global__ void k_fill(float *p, float v, int64_t n) {
    int64_t n4 = n >> 2;
    float4 v4 = make_float4(v, v, v, v);
    float4 *p4 = reinterpret_cast<float4 *>(p);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
         i += (int64_t)gridDim.x * blockDim.x)
        p4[i] = v4;
    for (int64_t i = (n4 << 2) + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Angular wavenumbers of pm_util.py:159-199 (fftfreq * 2*pi/spacing in
// float64, cast to float32), plain and with the Nyquist entries zeroed as
// neg_grad does (gravity.py:37-44).
__global__ void k_ktab(float *kt, int n0, int n1, int n2, double period, float nyq, float eps) {
    int n2h = n2 / 2 + 1;
    int tot = n0 + n1 + n2h;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
        int n, i;
        long fi;
        if (t < n0) {
            n = n0; i = t; fi = i < (n + 1) / 2 ? i : i - n;
        } else if (t < n0 + n1) {
            n = n1; i = t - n0; fi = i < (n + 1) / 2 ? i : i - n;
        } else {
            n = n2; i = t - n0 - n1; fi = i;  // rfftfreq
        }
        double f = __ddiv_rn((double)fi, (double)n);
        float k = (float)__dmul_rn(f, period);
        kt[t] = k;
        float dk = fabsf(__fsub_rn(fabsf(k), nyq));
        kt[tot + t] = dk <= eps ? 0.f : k;
    }
}

// Forward Fourier kernel, fused laplace + neg_grad for the three axes
// (gravity.py:9-16, 37-44, 58-62): reads the r2c spectrum of the overdensity
// and writes -i k_j * (-(F c)/k^2) for j = 0,1,2 (k = 0 -> 0), c = 1.5
// Omega_m / N folding in the real-space scale and irfftn's 1/N.
// One warp per (i, j) row of n2h complex values.
__global__ void k_poisson_fwd(float2 *ck, int64_t n0, int64_t n1, int64_t n2h, int64_t Mc,
                              const float *__restrict__ kt, float c) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const float *kx = kt, *ky = kt + n0, *kz = kt + n0 + n1;
    const int64_t tot = n0 + n1 + n2h;
    const float *mx = kt + tot, *my = kt + tot + n0, *mz = kt + tot + n0 + n1;
    for (int64_t row = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
         row < n0 * n1; row += warps) {
        int64_t i = row / n1, j = row - i * n1;
        float kxi = __ldg(kx + i), kyj = __ldg(ky + j);
        float mxi = __ldg(mx + i), myj = __ldg(my + j);
        float kxy = __fadd_rn(__fmul_rn(kxi, kxi), __fmul_rn(kyj, kyj));
        float2 *r0 = ck + row * n2h;
        for (int64_t l = lane; l < n2h; l += 32) {
            float kzl = __ldg(kz + l), mzl = __ldg(mz + l);
            float k2 = __fadd_rn(kxy, __fmul_rn(kzl, kzl));
            float2 F = r0[l];
            float pr = 0.f, pi = 0.f;
            if (k2 != 0.f) {
                pr = -__fdiv_rn(__fmul_rn(F.x, c), k2);
                pi = -__fdiv_rn(__fmul_rn(F.y, c), k2);
            }
            // (-i k)(pr + i pi) = (k pi, -k pr)
            r0[l] = make_float2(__fmul_rn(mxi, pi), -__fmul_rn(mxi, pr));
            r0[Mc + l] = make_float2(__fmul_rn(myj, pi), -__fmul_rn(myj, pr));
            r0[2 * Mc + l] = make_float2(__fmul_rn(mzl, pi), -__fmul_rn(mzl, pr));
        }
    }
}

// Adjoint Fourier kernel: the real transpose of the forward operator
// irfftn o (-i k_j)(-1/k^2) o rfftn is irfftn o (+i k_j)(-1/k^2) o rfftn;
// summed over the three axes: S = -(c/k^2) sum_j i k_j G_j, written over
// the first spectrum.
__global__ void k_poisson_adj(float2 *ck, int64_t n0, int64_t n1, int64_t n2h, int64_t Mc,
                              const float *__restrict__ kt, float c) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const float *kx = kt, *ky = kt + n0, *kz = kt + n0 + n1;
    const int64_t tot = n0 + n1 + n2h;
    const float *mx = kt + tot, *my = kt + tot + n0, *mz = kt + tot + n0 + n1;
    for (int64_t row = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
         row < n0 * n1; row += warps) {
        int64_t i = row / n1, j = row - i * n1;
        float kxi = __ldg(kx + i), kyj = __ldg(ky + j);
        float mxi = __ldg(mx + i), myj = __ldg(my + j);
        float kxy = __fadd_rn(__fmul_rn(kxi, kxi), __fmul_rn(kyj, kyj));
        float2 *r0 = ck + row * n2h;
        for (int64_t l = lane; l < n2h; l += 32) {
            float kzl = __ldg(kz + l), mzl = __ldg(mz + l);
            float k2 = __fadd_rn(kxy, __fmul_rn(kzl, kzl));
            float2 G0 = r0[l], G1 = r0[Mc + l], G2 = r0[2 * Mc + l];
            // i k (a + i b) = (-k b, k a)
            float re = -__fadd_rn(__fadd_rn(__fmul_rn(mxi, G0.y), __fmul_rn(myj, G1.y)),
                                  __fmul_rn(mzl, G2.y));
            float im = __fadd_rn(__fadd_rn(__fmul_rn(mxi, G0.x), __fmul_rn(myj, G1.x)),
                                 __fmul_rn(mzl, G2.x));
            float sr = 0.f, si = 0.f;
            if (k2 != 0.f) {
                sr = -__fdiv_rn(__fmul_rn(re, c), k2);
                si = -__fdiv_rn(__fmul_rn(im, c), k2);
            }
            r0[l] = make_float2(sr, si);
        }
    }
}

// ---------------------------------------------------------------------------
// particle kernels of the hot path (3-D, default enmesh branch)
// ---------------------------------------------------------------------------

struct Hot {
    int wrap[3];
    int64_t stride[3];
    float cell;   // f32(conf.cell_size), also the disp_cot divisor
    float val;    // f32(mesh_size / ptcl_num)
    // component j of the acceleration meshes (and their cotangents) at cell
    // c with x index x lives at c + x*gxs + j*gjs: planar (0, M) or
    // plane-interleaved (x, 3, n1, n2) = (2 n1 n2, n1 n2)
    int64_t gxs, gjs;
    // optional Kahan compensation terms of disp and vel (n, 3); NULL = plain
    float *dcomp, *vcomp;
    // deposit through per-warp shared-memory windows (needs n2 % 4 == 0)
    bool win;
    // n2 % 4 == 0: every mesh row starts on 16 bytes, so z-neighbour pairs
    // inside one aligned group of four floats take one vector reduction
    bool vec;
    // warp-aggregated deposits (mesh indices below 2^32 - 32)
    bool agg;
    // per-block partial sums: slot s of block b at part[s * pstride + b]
    int64_t pstride;
};

__device__ __forceinline__ void hot_axis(const Hot &h, int a, int pm, float d, Axis &ax) {
    float x = __fdiv_rn(d, h.cell);
    int fl = (int)floorf(x);
#pragma unroll
    for (int nb = 0; nb < 2; ++nb) {
        int ii = fl + nb;
        float d2 = __fsub_rn(x, (float)ii);
        ax.w[nb] = __fsub_rn(1.f, fabsf(d2));
        ax.s[nb] = sgnf(-d2);
        ax.i[nb] = pymod(ii + pm, h.wrap[a]);
    }
    ax.u = fl + pm;
}

__device__ __forceinline__ int64_t hot_cell(const Hot &h, const Axis ax[3], int k) {
    return (int64_t)ax[0].i[k & 1] * h.stride[0] + (int64_t)ax[1].i[(k >> 1) & 1] * h.stride[1] +
           (int64_t)ax[2].i[(k >> 2) & 1];
}

__device__ __forceinline__ float3 ld3(const float *p, int64_t q) {
    return make_float3(p[3 * q], p[3 * q + 1], p[3 * q + 2]);
}
__device__ __forceinline__ void st3(float *p, int64_t q, float3 v) {
    p[3 * q] = v.x;
    p[3 * q + 1] = v.y;
    p[3 * q + 2] = v.z;
}
__device__ __forceinline__ float3 axpy3(float3 y, float3 x, float a) {  // y + x*a, unfused
    return make_float3(__fadd_rn(y.x, __fmul_rn(x.x, a)), __fadd_rn(y.y, __fmul_rn(x.y, a)),
                       __fadd_rn(y.z, __fmul_rn(x.z, a)));
}
__device__ __forceinline__ float3 axmy3(float3 y, float3 x, float a) {  // y - x*a, unfused
    return make_float3(__fsub_rn(y.x, __fmul_rn(x.x, a)), __fsub_rn(y.y, __fmul_rn(x.y, a)),
                       __fsub_rn(y.z, __fmul_rn(x.z, a)));
}
// y + x*a with Kahan compensation kept in comp[3q..3q+2] (comp == NULL:
// the plain float32 update of the reference).
__device__ __forceinline__ float3 kahan_axpy(float3 y, float3 x, float a, float *comp, int64_t q) {
    if (!comp) return axpy3(y, x, a);
    float3 c = ld3(comp, q);
    float3 u = make_float3(__fsub_rn(__fmul_rn(x.x, a), c.x), __fsub_rn(__fmul_rn(x.y, a), c.y),
                           __fsub_rn(__fmul_rn(x.z, a), c.z));
    float3 t = make_float3(__fadd_rn(y.x, u.x), __fadd_rn(y.y, u.y), __fadd_rn(y.z, u.z));
    c = make_float3(__fsub_rn(__fsub_rn(t.x, y.x), u.x), __fsub_rn(__fsub_rn(t.y, y.y), u.y),
                    __fsub_rn(__fsub_rn(t.z, y.z), u.z));
    st3(comp, q, c);
    return t;
}

__device__ __forceinline__ double dot3d(float3 a, float3 b) {
    return (double)a.x * (double)b.x + (double)a.y * (double)b.y + (double)a.z * (double)b.z;
}

__device__ __forceinline__ void hot_enmesh(const Hot &h, const int16_t *pmid, int64_t q, float3 d,
                                           Axis ax[3]) {
    hot_axis(h, 0, pmid[3 * q], d.x, ax[0]);
    hot_axis(h, 1, pmid[3 * q + 1], d.y, ax[1]);
    hot_axis(h, 2, pmid[3 * q + 2], d.z, ax[2]);
}

// Adds a at z index i0 and b at z index i1 (a particle's two z neighbours)
// of one mesh row: one 16-byte red.global.add.v4.f32 (the other two lanes
// add zero) when both cells lie in the same aligned group of four floats,
// else two scalar atomics.  3 of 4 lower-neighbour positions qualify.
__device__ __forceinline__ void zpair_add(float *row, int i0, int i1, float a, float b, bool vec) {
    const int r = i0 & 3;
    if (vec && i1 == i0 + 1 && r != 3) {
        const float4 v = make_float4(r == 0 ? a : 0.f, r == 0 ? b : (r == 1 ? a : 0.f),
                                     r == 1 ? b : (r == 2 ? a : 0.f), r == 2 ? b : 0.f);
        atomicAdd(reinterpret_cast<float4 *>(row + (i0 - r)), v);
    } else {
        atomicAdd(row + i0, a);
        atomicAdd(row + i1, b);
    }
}

// Offset of the (x, y) mesh row of neighbour pair p (bit 0: x, bit 1: y).
__device__ __forceinline__ int64_t hot_row(const Hot &h, const Axis ax[3], int p) {
    return (int64_t)ax[0].i[p & 1] * h.stride[0] + (int64_t)ax[1].i[(p >> 1) & 1] * h.stride[1];
}

// CIC deposit of val * frac_k, frac_k = (w_x w_y) w_z as frac_of.
__device__ __forceinline__ void hot_deposit(const Hot &h, const Axis ax[3], float *dens) {
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const float fxy = __fmul_rn(ax[0].w[p & 1], ax[1].w[(p >> 1) & 1]);
        zpair_add(dens + hot_row(h, ax, p), ax[2].i[0], ax[2].i[1],
                  __fmul_rn(h.val, __fmul_rn(fxy, ax[2].w[0])),
                  __fmul_rn(h.val, __fmul_rn(fxy, ax[2].w[1])), h.vec);
    }
}

// ---------------------------------------------------------------------------
// Warp-aggregated deposits for clustered particles.  Two particles with the
// same base cell (the wrapped lower neighbour on every axis) share all eight
// neighbour cells.  A warp first matches its lanes' base cells; when no two
// lanes share one (the nearly uniform early steps) it deposits directly,
// as hot_deposit.  Otherwise every lane adds its NC x 8 contributions into a
// shared-memory slot of its group's lowest lane, and that lane issues one
// global reduction per cell and component for the whole group: in a halo,
// where many particles of a warp fall into the same cell, the contended L2
// reductions drop by the group size.  Only the order of the float32 sums
// changes.  Needs a warp-uniform loop (every lane calls it) and mesh
// indices below 2^32 - 32 (Hot::agg).
// ---------------------------------------------------------------------------

constexpr int AGG_SLOT = 8;  // floats per lane and component in the warp buffer

// Adds s[c] * frac_k to component c of neighbour k for NC components:
// component c of cell (row, z) at base + row + z + c * cs, the row of
// neighbour pair p at hot_row(h, ax, p) + x_p * xs.
template <int NC>
__device__ __forceinline__ void agg_deposit(const Hot &h, bool act, const Axis ax[3],
                                            const float s[NC], float *base, int64_t xs,
                                            int64_t cs, float *wbuf) {
    const int lane = threadIdx.x & 31;
    const unsigned key =
        act ? (unsigned)((int64_t)ax[0].i[0] * h.stride[0] + (int64_t)ax[1].i[0] * h.stride[1] +
                         ax[2].i[0])
            : 0xFFFFFFFFu - (unsigned)lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (!__any_sync(0xffffffffu, (peers & (peers - 1)) != 0)) {   // no shared base cell
        if (act) {
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const float fxy = __fmul_rn(ax[0].w[p & 1], ax[1].w[(p >> 1) & 1]);
                const float fa = __fmul_rn(fxy, ax[2].w[0]), fb = __fmul_rn(fxy, ax[2].w[1]);
                float *row = base + hot_row(h, ax, p) + (int64_t)ax[0].i[p & 1] * xs;
#pragma unroll
                for (int c = 0; c < NC; ++c)
                    zpair_add(row + c * cs, ax[2].i[0], ax[2].i[1], __fmul_rn(s[c], fa),
                              __fmul_rn(s[c], fb), h.vec);
            }
        }
        return;
    }
    const int leader = __ffs(peers) - 1;
    float *slot = wbuf + leader * (AGG_SLOT * NC);
    if (act) {
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const float fxy = __fmul_rn(ax[0].w[p & 1], ax[1].w[(p >> 1) & 1]);
            const float fa = __fmul_rn(fxy, ax[2].w[0]), fb = __fmul_rn(fxy, ax[2].w[1]);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                atomicAdd(slot + (2 * p) * NC + c, __fmul_rn(s[c], fa));
                atomicAdd(slot + (2 * p + 1) * NC + c, __fmul_rn(s[c], fb));
            }
        }
    }
    __syncwarp();
    if (act && lane == leader) {
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            float *row = base + hot_row(h, ax, p) + (int64_t)ax[0].i[p & 1] * xs;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                float *a = slot + (2 * p) * NC + c, *b = slot + (2 * p + 1) * NC + c;
                zpair_add(row + c * cs, ax[2].i[0], ax[2].i[1], *a, *b, h.vec);
                *a = 0.f;
                *b = 0.f;
            }
        }
    }
    __syncwarp();
}

// This warp's zeroed aggregation buffer (32 lanes x 8 neighbours x NC).
template <int NC>
__device__ __forceinline__ float *agg_buffer() {
    __shared__ float buf[PT / 32][32 * AGG_SLOT * NC];
    float *w = buf[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < 32 * AGG_SLOT * NC; i += 32) w[i] = 0.f;
    __syncwarp();
    return w;
}

// ---------------------------------------------------------------------------
// Warp deposit windows.  Particles are in Lagrangian (pmid-raveled) order, so
// the 32 particles of a warp sit along one z row and their 8 neighbour cells
// span 3 x 3 (x, y) rows of a short z range.  Each warp accumulates into a
// shared-memory window of WROWS rows x WZ cells (z origin aligned to 4) with
// shared atomics, then flushes it with one 16-byte red.global.add.v4.f32 per
// four cells instead of one global atomic per contribution.  Contributions
// outside the window go straight to global memory, so any particle order is
// correct; the window only changes speed.  Needs n2 % 4 == 0 (16-byte groups).
// ---------------------------------------------------------------------------

constexpr int WZ = 80;      // window width along z (multiple of 4)
constexpr int WROWS = 9;    // 3 x 3 (x, y) rows
constexpr size_t WIN1_SMEM = (PT / 32) * WROWS * WZ * sizeof(float);  // one component
constexpr size_t WIN3_SMEM = 3 * WIN1_SMEM;                           // three components

struct Win {
    int x0, y0, z0;         // unwrapped origin (z0 multiple of 4)
    int nx, ny, ng;         // rows and 4-cell groups the warp can have touched
};

__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Origin and extent of the warp's window from the lower-neighbour unwrapped
// indices of its active lanes (each particle also touches index + 1).
__device__ __forceinline__ Win win_origin(bool act, const Axis ax[3]) {
    Win w;
    w.x0 = warp_min(act ? ax[0].u : INT_MAX);
    w.y0 = warp_min(act ? ax[1].u : INT_MAX);
    const int zm = warp_min(act ? ax[2].u : INT_MAX);
    w.z0 = zm & ~3;  // floor to a multiple of 4 (two's complement)
    const int xM = warp_max(act ? ax[0].u : INT_MIN);
    const int yM = warp_max(act ? ax[1].u : INT_MIN);
    const int zM = warp_max(act ? ax[2].u : INT_MIN);
    w.nx = min(3, xM - w.x0 + 2);
    w.ny = min(3, yM - w.y0 + 2);
    w.ng = min(WZ / 4, (zM + 1 - w.z0) / 4 + 1);
    return w;
}

// Adds v to neighbour k of this particle: into the warp window `buf`
// (component stride WROWS*WZ) when inside it, else to global memory at
// `gaddr`.
__device__ __forceinline__ void win_add(float *buf, const Win &w, const Axis ax[3], int k, float v,
                                        float *gaddr) {
    const int dx = ax[0].u + (k & 1) - w.x0;
    const int dy = ax[1].u + ((k >> 1) & 1) - w.y0;
    const int dz = ax[2].u + ((k >> 2) & 1) - w.z0;
    if ((unsigned)dx < 3u && (unsigned)dy < 3u && (unsigned)dz < (unsigned)WZ)
        atomicAdd(buf + (dx * 3 + dy) * WZ + dz, v);
    else
        atomicAdd(gaddr, v);
}

// Flushes NC component windows of one warp to global memory with vector
// reductions and zeroes them.  Global address of component c, cell
// (x, y, z): c * cstride + x * xstride + y * n2 + z (wrapped), which covers
// the density (NC = 1) and both mesh layouts of the cotangent meshes.
template <int NC>
__device__ __forceinline__ void win_flush(float *buf, const Win &w, const Hot &h, float *base,
                                          int64_t xstride, int64_t cstride) {
    const int lane = threadIdx.x & 31;
    const int ng = w.ng, nrow = w.nx * w.ny;
    for (int idx = lane; idx < NC * nrow * ng; idx += 32) {
        const int c = idx / (nrow * ng);
        const int rr = (idx / ng) % nrow;
        const int r = (rr / w.ny) * 3 + rr % w.ny;   // window row (dx * 3 + dy)
        const int g = idx % ng;
        float4 *p = reinterpret_cast<float4 *>(buf + (c * WROWS + r) * WZ) + g;
        const float4 v = *p;
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
            const int x = pymod(w.x0 + r / 3, h.wrap[0]);
            const int y = pymod(w.y0 + r % 3, h.wrap[1]);
            const int z = pymod(w.z0 + 4 * g, h.wrap[2]);
            float *a = base + c * cstride + (int64_t)x * xstride + (int64_t)y * h.stride[1] + z;
            atomicAdd(reinterpret_cast<float4 *>(a), v);
            *p = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

__device__ __forceinline__ void win_zero(float *buf, int nfloats) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < nfloats; i += 32) buf[i] = 0.f;
}

// Forward: optional kick (vel += acc*K1) and drift (disp += vel*D), then the
// CIC density deposit of the (new) positions.
// WIN: deposit through the warp windows; KAHAN: compensated updates (the
// compensation arrays in h are then non-NULL).  Both are template arguments
// so the default path carries neither their registers nor their branches.
template <bool KD, bool WIN, bool KAHAN, bool AGG = false>
__device__ __forceinline__ void kds_body(Hot h, const int16_t *__restrict__ pmid, float *disp,
                                            float *vel, const float *__restrict__ acc, int64_t n,
                                            float K1, float D, float *dens) {
    extern __shared__ __align__(16) float wsm[];
    const int lane = threadIdx.x & 31;
    float *buf = wsm + (threadIdx.x >> 5) * (WROWS * WZ);
    float *const vcomp = KAHAN ? h.vcomp : nullptr, *const dcomp = KAHAN ? h.dcomp : nullptr;
    float *abuf = nullptr;
    if constexpr (AGG) abuf = agg_buffer<1>();
    if (WIN) win_zero(buf, WROWS * WZ);
    __syncwarp();
    // warp-uniform loop: each warp takes 32 consecutive particles
    for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); q0 < n;
         q0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = q0 + lane;
        const bool act = q < n;
        Axis ax[3];
        if (act) {
            float3 d = ld3(disp, q);
            if (KD) {
                float3 v = kahan_axpy(ld3(vel, q), ld3(acc, q), K1, vcomp, q);
                d = kahan_axpy(d, v, D, dcomp, q);
                st3(vel, q, v);
                st3(disp, q, d);
            }
            hot_enmesh(h, pmid, q, d, ax);
        }
        if constexpr (AGG) {
            const float sv[1] = {h.val};
            agg_deposit<1>(h, act, ax, sv, dens, 0, 0, abuf);
            continue;
        }
        if (!WIN) {
            if (act) hot_deposit(h, ax, dens);
            continue;
        }
        const Win w = win_origin(act, ax);
        if (act) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                win_add(buf, w, ax, k, __fmul_rn(h.val, frac_of(ax, k)), dens + hot_cell(h, ax, k));
        }
        __syncwarp();
        win_flush<1>(buf, w, h, dens, h.stride[0], 0);
        __syncwarp();
    }
}

template <bool KD, bool WIN, bool KAHAN, bool AGG = false>
__global__ void __launch_bounds__(PT) k_kds(Hot h, const int16_t *__restrict__ pmid, float *disp,
                                            float *vel, const float *__restrict__ acc, int64_t n,
                                            float K1, float D, float *dens) {
    kds_body<KD, WIN, KAHAN, AGG>(h, pmid, disp, vel, acc, n, K1, D, dens);
}

// ---------------------------------------------------------------------------
// TMA-staged gather (workspaces with PMX_WS_TMA, plane-interleaved meshes).
// Each warp takes 32 consecutive particles; their lower neighbour cells span
// a small box of the (x, 3, n1, n2) acceleration meshes (Lagrangian order:
// one z row of the particle grid).  One lane loads that box -- TBX x-planes
// x 3 components x TBY rows x TBZ cells -- into the warp's shared-memory
// buffer with one cp.async.bulk.tensor copy completing on an mbarrier, and
// the 8-point interpolation then reads shared memory.  A warp whose cells do
// not fit the box, or whose box would cross the periodic boundary (the
// copy fills out-of-range cells with zeros), reads global memory instead, as
// k_gather3 does; both paths add the same products in the same order.
// ---------------------------------------------------------------------------

constexpr int TBX = 3, TBY = 3, TBZ = 72;            // box: x-planes, y rows, z cells
constexpr int TBOX = TBX * 3 * TBY * TBZ;            // floats a box copy writes
constexpr int TBOX_PAD = (TBOX + 31) & ~31;          // box stride: 128-byte aligned
constexpr size_t TMA_SMEM = (PT / 32) * (TBOX_PAD * 4 + 8);
constexpr int TMA_WAIT_LIMIT = 1 << 24;              // mbarrier polls before giving up

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

// Waits for the mbarrier phase `parity`; false after TMA_WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    const unsigned a = smem_addr(bar);
    for (int i = 0; i < TMA_WAIT_LIMIT; ++i) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <bool KICK>
__global__ void __launch_bounds__(PT) k_gather3_tma(Hot h, const __grid_constant__ CUtensorMap tmap,
                                                    const int16_t *__restrict__ pmid,
                                                    const float *__restrict__ disp, float *vel,
                                                    float *acc, int64_t n,
                                                    const float *__restrict__ g, float K2,
                                                    int *err) {
    extern __shared__ __align__(128) float tbuf[];   // PT/32 boxes, then PT/32 mbarriers
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *box = tbuf + warp * TBOX_PAD;
    uint64_t *bar = reinterpret_cast<uint64_t *>(tbuf + (PT / 32) * TBOX_PAD) + warp;
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();
    unsigned parity = 0;
    bool tma_ok = true;   // false after a wait gave up: the warp then reads global memory
    for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); q0 < n;
         q0 += (int64_t)gridDim.x * blockDim.x) {   // warp-uniform
        const int64_t q = q0 + lane;
        const bool act = q < n;
        Axis ax[3];
        if (act) hot_enmesh(h, pmid, q, ld3(disp, q), ax);
        // the warp's box: unwrapped lower-neighbour indices, z origin on 16 bytes
        const int x0 = warp_min(act ? ax[0].u : INT_MAX), y0 = warp_min(act ? ax[1].u : INT_MAX);
        const int z0 = warp_min(act ? ax[2].u : INT_MAX) & ~3;
        const int x1 = warp_max(act ? ax[0].u : INT_MIN) + 2;
        const int y1 = warp_max(act ? ax[1].u : INT_MIN) + 2;
        const int z1 = warp_max(act ? ax[2].u : INT_MIN) + 2;
        const bool fits = tma_ok && x0 >= 0 && y0 >= 0 && z0 >= 0 && x1 - x0 <= TBX &&
                          y1 - y0 <= TBY && z1 - z0 <= TBZ && x1 <= h.wrap[0] &&
                          y1 <= h.wrap[1] && z1 <= h.wrap[2];
        bool staged = false;
        if (fits) {   // warp-uniform
            if (lane == 0) {
                const unsigned b = smem_addr(bar);
                // the box's earlier reads (generic proxy) before the copy's writes
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b),
                             "r"((unsigned)(TBOX * 4))
                             : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_addr(box)),
                    "l"(&tmap), "r"(z0), "r"(y0), "r"(0), "r"(x0), "r"(b)
                    : "memory");
            }
            staged = __all_sync(0xffffffffu, mbar_wait(bar, parity));
            parity ^= 1u;
            if (!staged) {   // record, wait once more for the copy in flight, then go direct
                if (lane == 0) atomicExch(err, 1);
                mbar_wait(bar, parity ^ 1u);
                tma_ok = false;
            }
        }
        if (act) {
            float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float f = frac_of(ax, k);
                float m0, m1, m2;
                if (staged) {
                    const int xi = ax[0].u + (k & 1) - x0, yi = ax[1].u + ((k >> 1) & 1) - y0;
                    const int zi = ax[2].u + ((k >> 2) & 1) - z0;
                    const float *b = box + ((xi * 3) * TBY + yi) * TBZ + zi;
                    m0 = b[0];
                    m1 = b[TBY * TBZ];
                    m2 = b[2 * TBY * TBZ];
                } else {
                    const float *gc = g + hot_cell(h, ax, k) + (int64_t)ax[0].i[k & 1] * h.gxs;
                    m0 = __ldg(gc);
                    m1 = __ldg(gc + h.gjs);
                    m2 = __ldg(gc + 2 * h.gjs);
                }
                a0 = __fadd_rn(a0, __fmul_rn(m0, f));
                a1 = __fadd_rn(a1, __fmul_rn(m1, f));
                a2 = __fadd_rn(a2, __fmul_rn(m2, f));
            }
            float3 a = make_float3(a0, a1, a2);
            st3(acc, q, a);
            if (KICK) st3(vel, q, axpy3(ld3(vel, q), a, K2));
        }
        __syncwarp();   // every lane's reads of the box are done before it is refilled
    }
}

// Forward: gather the three acceleration meshes, optionally kick with K2.
template <bool KICK, bool KAHAN>
__device__ __forceinline__ void gather3_body(Hot h, const int16_t *__restrict__ pmid,
                                                const float *__restrict__ disp, float *vel,
                                                float *acc, int64_t n, int64_t M,
                                                const float *__restrict__ g, float K2) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        Axis ax[3];
        hot_enmesh(h, pmid, q, ld3(disp, q), ax);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t c = hot_cell(h, ax, k);
            float f = frac_of(ax, k);
            const float *gc = g + c + (int64_t)ax[0].i[k & 1] * h.gxs;
            a0 = __fadd_rn(a0, __fmul_rn(__ldg(gc), f));
            a1 = __fadd_rn(a1, __fmul_rn(__ldg(gc + h.gjs), f));
            a2 = __fadd_rn(a2, __fmul_rn(__ldg(gc + 2 * h.gjs), f));
        }
        float3 a = make_float3(a0, a1, a2);
        st3(acc, q, a);
        if (KICK) st3(vel, q, kahan_axpy(ld3(vel, q), a, K2, KAHAN ? h.vcomp : nullptr, q));
    }
}

template <bool KICK, bool KAHAN>
__global__ void __launch_bounds__(PT) k_gather3(Hot h, const int16_t *__restrict__ pmid,
                                                const float *__restrict__ disp, float *vel,
                                                float *acc, int64_t n, int64_t M,
                                                const float *__restrict__ g, float K2) {
    gather3_body<KICK, KAHAN>(h, pmid, disp, vel, acc, n, M, g, K2);
}

// Adjoint: kick_adj(K1) then drift_adj(D) (nbody.py:80-99, 49-67), then the
// density deposit of the reconstructed positions.  Partial dots:
// slot 0 = sum(vel_cot*acc), slot 1 = sum(disp_cot*vel).
template <bool KD, bool WIN, bool KAHAN, bool AGG = false>
__device__ __forceinline__ void ka_body(Hot h, const int16_t *__restrict__ pmid, float *disp,
                                           float *vel, const float *__restrict__ acc,
                                           float *disp_cot, float *vel_cot,
                                           const float *__restrict__ alpha, int64_t n, float K1,
                                           float D, float *dens, double *part) {
    __shared__ double sh[PT / 32];
    extern __shared__ __align__(16) float wsm[];
    const int lane = threadIdx.x & 31;
    float *buf = wsm + (threadIdx.x >> 5) * (WROWS * WZ);
    float *const vcomp = KAHAN ? h.vcomp : nullptr, *const dcomp = KAHAN ? h.dcomp : nullptr;
    float *abuf = nullptr;
    if constexpr (AGG) abuf = agg_buffer<1>();
    if (WIN) win_zero(buf, WROWS * WZ);
    __syncwarp();
    double s0 = 0.0, s1 = 0.0;
    for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); q0 < n;
         q0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = q0 + lane;
        const bool act = q < n;
        Axis ax[3];
        if (act) {
            float3 d = ld3(disp, q);
            if (KD) {
                float3 a = ld3(acc, q);
                float3 vc = ld3(vel_cot, q);
                float3 v = kahan_axpy(ld3(vel, q), a, K1, vcomp, q);
                float3 dc = axmy3(ld3(disp_cot, q), ld3(alpha, q), K1);
                s0 += dot3d(vc, a);
                d = kahan_axpy(d, v, D, dcomp, q);
                vc = axmy3(vc, dc, D);
                s1 += dot3d(dc, v);
                st3(vel, q, v);
                st3(disp, q, d);
                st3(disp_cot, q, dc);
                st3(vel_cot, q, vc);
            }
            hot_enmesh(h, pmid, q, d, ax);
        }
        if constexpr (AGG) {
            const float sv[1] = {h.val};
            agg_deposit<1>(h, act, ax, sv, dens, 0, 0, abuf);
            continue;
        }
        if (!WIN) {
            if (act) hot_deposit(h, ax, dens);
            continue;
        }
        const Win w = win_origin(act, ax);
        if (act) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                win_add(buf, w, ax, k, __fmul_rn(h.val, frac_of(ax, k)), dens + hot_cell(h, ax, k));
        }
        __syncwarp();
        win_flush<1>(buf, w, h, dens, h.stride[0], 0);
        __syncwarp();
    }
    if (KD) {
        double t0 = block_sum<PT>(s0, sh);
        double t1 = block_sum<PT>(s1, sh);
        if (threadIdx.x == 0) {
            part[0 * h.pstride + blockIdx.x] = t0;
            part[1 * h.pstride + blockIdx.x] = t1;
        }
    }
}

template <bool KD, bool WIN, bool KAHAN, bool AGG = false>
__global__ void __launch_bounds__(PT) k_ka(Hot h, const int16_t *__restrict__ pmid, float *disp,
                                           float *vel, const float *__restrict__ acc,
                                           float *disp_cot, float *vel_cot,
                                           const float *__restrict__ alpha, int64_t n, float K1,
                                           float D, float *dens, double *part) {
    ka_body<KD, WIN, KAHAN, AGG>(h, pmid, disp, vel, acc, disp_cot, vel_cot, alpha, n, K1, D, dens,
                                 part);
}

// Adjoint: gather the three acceleration meshes (new acc), the gather VJP
// disp_cot term sum_j vc_j sum_k g_j[k] dfrac_k / cell (into alpha), and the
// gather VJP mesh term mcot_j[k] += vc_j frac_k.  Partial dot slot 2 =
// sum(vel_cot * acc_new).
template <bool WIN, bool AGG = false>
__device__ __forceinline__ void g3adj_body(Hot h, const int16_t *__restrict__ pmid,
                                              const float *__restrict__ disp,
                                              const float *__restrict__ vel_cot, float *acc,
                                              float *alpha, int64_t n, int64_t M,
                                              const float *__restrict__ g, float *mcot,
                                              double *part) {
    __shared__ double sh[PT / 32];
    extern __shared__ __align__(16) float wsm[];
    const int lane = threadIdx.x & 31;
    float *buf = wsm + (threadIdx.x >> 5) * (3 * WROWS * WZ);
    float *abuf = nullptr;
    if constexpr (AGG) abuf = agg_buffer<3>();
    if (WIN) win_zero(buf, 3 * WROWS * WZ);
    __syncwarp();
    double s2 = 0.0;
    for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); q0 < n;
         q0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = q0 + lane;
        const bool act = q < n;
        Axis ax[3];
        float3 vc = make_float3(0.f, 0.f, 0.f);
        if (act) {
            hot_enmesh(h, pmid, q, ld3(disp, q), ax);
            vc = ld3(vel_cot, q);
            float a0 = 0.f, a1 = 0.f, a2 = 0.f;
            float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                int64_t c = hot_cell(h, ax, k);
                float f = frac_of(ax, k);
                float fg[3];
                frac_grad_of(ax, k, fg);
                const int64_t gc = c + (int64_t)ax[0].i[k & 1] * h.gxs;
                float m0 = __ldg(g + gc), m1 = __ldg(g + gc + h.gjs), m2 = __ldg(g + gc + 2 * h.gjs);
                a0 = __fadd_rn(a0, __fmul_rn(m0, f));
                a1 = __fadd_rn(a1, __fmul_rn(m1, f));
                a2 = __fadd_rn(a2, __fmul_rn(m2, f));
                float t = __fadd_rn(__fadd_rn(__fmul_rn(vc.x, m0), __fmul_rn(vc.y, m1)),
                                    __fmul_rn(vc.z, m2));
                c0 = __fadd_rn(c0, __fmul_rn(t, fg[0]));
                c1 = __fadd_rn(c1, __fmul_rn(t, fg[1]));
                c2 = __fadd_rn(c2, __fmul_rn(t, fg[2]));
            }
            if (!WIN && !AGG) {
                // gather-VJP mesh term mcot_j[k] += vc_j frac_k
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    const float fxy = __fmul_rn(ax[0].w[p & 1], ax[1].w[(p >> 1) & 1]);
                    const float fa = __fmul_rn(fxy, ax[2].w[0]), fb = __fmul_rn(fxy, ax[2].w[1]);
                    float *row = mcot + hot_row(h, ax, p) + (int64_t)ax[0].i[p & 1] * h.gxs;
                    const int i0 = ax[2].i[0], i1 = ax[2].i[1];
                    zpair_add(row, i0, i1, __fmul_rn(vc.x, fa), __fmul_rn(vc.x, fb), h.vec);
                    zpair_add(row + h.gjs, i0, i1, __fmul_rn(vc.y, fa), __fmul_rn(vc.y, fb), h.vec);
                    zpair_add(row + 2 * h.gjs, i0, i1, __fmul_rn(vc.z, fa), __fmul_rn(vc.z, fb),
                              h.vec);
                }
            }
            float3 a = make_float3(a0, a1, a2);
            st3(acc, q, a);
            st3(alpha, q, make_float3(__fdiv_rn(c0, h.cell), __fdiv_rn(c1, h.cell),
                                      __fdiv_rn(c2, h.cell)));
            s2 += dot3d(vc, a);
        }
        if constexpr (AGG) {
            const float sv[3] = {vc.x, vc.y, vc.z};
            agg_deposit<3>(h, act, ax, sv, mcot, h.gxs, h.gjs, abuf);
            continue;
        }
        if (!WIN) continue;
        // gather-VJP mesh term through the warp window, three components
        const Win w = win_origin(act, ax);
        if (act) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float f = frac_of(ax, k);
                const int64_t gc = hot_cell(h, ax, k) + (int64_t)ax[0].i[k & 1] * h.gxs;
                win_add(buf, w, ax, k, __fmul_rn(vc.x, f), mcot + gc);
                win_add(buf + WROWS * WZ, w, ax, k, __fmul_rn(vc.y, f), mcot + gc + h.gjs);
                win_add(buf + 2 * WROWS * WZ, w, ax, k, __fmul_rn(vc.z, f), mcot + gc + 2 * h.gjs);
            }
        }
        __syncwarp();
        win_flush<3>(buf, w, h, mcot, h.stride[0] + h.gxs, h.gjs);
        __syncwarp();
    }
    double t2 = block_sum<PT>(s2, sh);
    if (threadIdx.x == 0) part[2 * h.pstride + blockIdx.x] = t2;
}

template <bool WIN, bool AGG = false>
__global__ void __launch_bounds__(PT) k_g3adj(Hot h, const int16_t *__restrict__ pmid,
                                              const float *__restrict__ disp,
                                              const float *__restrict__ vel_cot, float *acc,
                                              float *alpha, int64_t n, int64_t M,
                                              const float *__restrict__ g, float *mcot,
                                              double *part) {
    g3adj_body<WIN, AGG>(h, pmid, disp, vel_cot, acc, alpha, n, M, g, mcot, part);
}

// Adjoint: scatter VJP disp_cot term sum_k (rho_cot[k] val) dfrac_k / cell
// added into alpha, then optionally kick_adj(K2): vel += acc*K2,
// disp_cot -= alpha*K2.
template <bool KICK, bool KAHAN>
__device__ __forceinline__ void sadj_body(Hot h, const int16_t *__restrict__ pmid,
                                             const float *__restrict__ disp, float *vel,
                                             const float *__restrict__ acc, float *disp_cot,
                                             float *alpha, int64_t n,
                                             const float *__restrict__ rho_cot, float K2) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        Axis ax[3];
        hot_enmesh(h, pmid, q, ld3(disp, q), ax);
        float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t c = hot_cell(h, ax, k);
            float fg[3];
            frac_grad_of(ax, k, fg);
            float t = __fmul_rn(__ldg(rho_cot + c), h.val);
            c0 = __fadd_rn(c0, __fmul_rn(t, fg[0]));
            c1 = __fadd_rn(c1, __fmul_rn(t, fg[1]));
            c2 = __fadd_rn(c2, __fmul_rn(t, fg[2]));
        }
        float3 al = ld3(alpha, q);
        al = make_float3(__fadd_rn(al.x, __fdiv_rn(c0, h.cell)),
                         __fadd_rn(al.y, __fdiv_rn(c1, h.cell)),
                         __fadd_rn(al.z, __fdiv_rn(c2, h.cell)));
        st3(alpha, q, al);
        if (KICK) {
            st3(vel, q, kahan_axpy(ld3(vel, q), ld3(acc, q), K2, KAHAN ? h.vcomp : nullptr, q));
            st3(disp_cot, q, axmy3(ld3(disp_cot, q), al, K2));
        }
    }
}

template <bool KICK, bool KAHAN>
__global__ void __launch_bounds__(PT) k_sadj(Hot h, const int16_t *__restrict__ pmid,
                                             const float *__restrict__ disp, float *vel,
                                             const float *__restrict__ acc, float *disp_cot,
                                             float *alpha, int64_t n,
                                             const float *__restrict__ rho_cot, float K2) {
    sadj_body<KICK, KAHAN>(h, pmid, disp, vel, acc, disp_cot, alpha, n, rho_cot, K2);
}

// ---------------------------------------------------------------------------
// Kernels that join two consecutive steps of a multi-step run: the last
// particle pass of step i and the first of step i+1 have no FFT between them,
// so they run as one pass over the particles, with the same float32 updates
// in the same order as the two kernels they replace (default path: no
// windows, no compensation).
// ---------------------------------------------------------------------------

// k_gather3<true> of step i, then k_kds<true> of step i+1: gather, kick K2,
// kick K1n, drift Dn, deposit.  acc is not stored: the next force rewrites it
// before anything reads it.
// One particle of k_gk_kds up to the deposit: ax holds its new neighbours.
__device__ __forceinline__ void gk_kds_particle(const Hot &h, const int16_t *__restrict__ pmid,
                                                float *disp, float *vel,
                                                const float *__restrict__ g, float K2, float K1n,
                                                float Dn, int64_t q, Axis ax[3]) {
    {
        float3 d = ld3(disp, q);
        hot_enmesh(h, pmid, q, d, ax);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t c = hot_cell(h, ax, k);
            float f = frac_of(ax, k);
            const float *gc = g + c + (int64_t)ax[0].i[k & 1] * h.gxs;
            a0 = __fadd_rn(a0, __fmul_rn(__ldg(gc), f));
            a1 = __fadd_rn(a1, __fmul_rn(__ldg(gc + h.gjs), f));
            a2 = __fadd_rn(a2, __fmul_rn(__ldg(gc + 2 * h.gjs), f));
        }
        const float3 a = make_float3(a0, a1, a2);
        float3 v = axpy3(ld3(vel, q), a, K2);   // kick, step i
        v = axpy3(v, a, K1n);                   // kick, step i+1
        d = axpy3(d, v, Dn);                    // drift, step i+1
        st3(vel, q, v);
        st3(disp, q, d);
        hot_enmesh(h, pmid, q, d, ax);
    }
}

template <bool AGG = false>
__device__ __forceinline__ void gk_kds_body(Hot h, const int16_t *__restrict__ pmid, float *disp,
                                            float *vel, int64_t n, const float *__restrict__ g,
                                            float K2, float K1n, float Dn, float *dens) {
    if constexpr (!AGG) {
        for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
             q += (int64_t)gridDim.x * blockDim.x) {
            Axis ax[3];
            gk_kds_particle(h, pmid, disp, vel, g, K2, K1n, Dn, q, ax);
            hot_deposit(h, ax, dens);
        }
    } else {
        float *abuf = agg_buffer<1>();
        const float sv[1] = {h.val};
        for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); q0 < n;
             q0 += (int64_t)gridDim.x * blockDim.x) {   // warp-uniform
            const int64_t q = q0 + (threadIdx.x & 31);
            Axis ax[3];
            if (q < n) gk_kds_particle(h, pmid, disp, vel, g, K2, K1n, Dn, q, ax);
            agg_deposit<1>(h, q < n, ax, sv, dens, 0, 0, abuf);
        }
    }
}

template <bool AGG = false>
__global__ void __launch_bounds__(PT) k_gk_kds(Hot h, const int16_t *__restrict__ pmid, float *disp,
                                               float *vel, int64_t n, const float *__restrict__ g,
                                               float K2, float K1n, float Dn, float *dens) {
    gk_kds_body<AGG>(h, pmid, disp, vel, n, g, K2, K1n, Dn, dens);
}

// k_sadj<true> of adjoint step i, then k_ka<true> of adjoint step i+1: the
// scatter-VJP term into alpha, kick_adj K2, kick_adj K1n, drift_adj Dn,
// deposit; partial dots of step i+1 into slots 0, 1.  alpha is not stored:
// the next gather VJP rewrites it before anything reads it.
// One particle of k_sa_ka up to the deposit (dots into s0, s1).
__device__ __forceinline__ void sa_ka_particle(const Hot &h, const int16_t *__restrict__ pmid,
                                               float *disp, float *vel,
                                               const float *__restrict__ acc, float *disp_cot,
                                               float *vel_cot, const float *__restrict__ alpha,
                                               const float *__restrict__ rho_cot, float K2,
                                               float K1n, float Dn, int64_t q, Axis ax[3],
                                               double &s0, double &s1) {
    {
        float3 d = ld3(disp, q);
        hot_enmesh(h, pmid, q, d, ax);
        float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t c = hot_cell(h, ax, k);
            float fg[3];
            frac_grad_of(ax, k, fg);
            float t = __fmul_rn(__ldg(rho_cot + c), h.val);
            c0 = __fadd_rn(c0, __fmul_rn(t, fg[0]));
            c1 = __fadd_rn(c1, __fmul_rn(t, fg[1]));
            c2 = __fadd_rn(c2, __fmul_rn(t, fg[2]));
        }
        float3 al = ld3(alpha, q);
        al = make_float3(__fadd_rn(al.x, __fdiv_rn(c0, h.cell)),
                         __fadd_rn(al.y, __fdiv_rn(c1, h.cell)),
                         __fadd_rn(al.z, __fdiv_rn(c2, h.cell)));
        const float3 a = ld3(acc, q);
        float3 v = axpy3(ld3(vel, q), a, K2);            // kick_adj, step i
        float3 dc = axmy3(ld3(disp_cot, q), al, K2);
        float3 vc = ld3(vel_cot, q);
        v = axpy3(v, a, K1n);                            // kick_adj, step i+1
        dc = axmy3(dc, al, K1n);
        s0 += dot3d(vc, a);
        d = axpy3(d, v, Dn);                             // drift_adj, step i+1
        vc = axmy3(vc, dc, Dn);
        s1 += dot3d(dc, v);
        st3(vel, q, v);
        st3(disp, q, d);
        st3(disp_cot, q, dc);
        st3(vel_cot, q, vc);
        hot_enmesh(h, pmid, q, d, ax);
    }
}

template <bool AGG = false>
__device__ __forceinline__ void sa_ka_body(Hot h, const int16_t *__restrict__ pmid,
                                           float *disp, float *vel,
                                           const float *__restrict__ acc, float *disp_cot,
                                           float *vel_cot, const float *__restrict__ alpha,
                                           int64_t n, const float *__restrict__ rho_cot,
                                           float K2, float K1n, float Dn, float *dens,
                                           double *part) {
    __shared__ double sh[PT / 32];
    double s0 = 0.0, s1 = 0.0;
    if constexpr (!AGG) {
        for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
             q += (int64_t)gridDim.x * blockDim.x) {
            Axis ax[3];
            sa_ka_particle(h, pmid, disp, vel, acc, disp_cot, vel_cot, alpha, rho_cot, K2, K1n,
                           Dn, q, ax, s0, s1);
            hot_deposit(h, ax, dens);
        }
    } else {
        float *abuf = agg_buffer<1>();
        const float sv[1] = {h.val};
        for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); q0 < n;
             q0 += (int64_t)gridDim.x * blockDim.x) {   // warp-uniform
            const int64_t q = q0 + (threadIdx.x & 31);
            Axis ax[3];
            if (q < n)
                sa_ka_particle(h, pmid, disp, vel, acc, disp_cot, vel_cot, alpha, rho_cot, K2,
                               K1n, Dn, q, ax, s0, s1);
            agg_deposit<1>(h, q < n, ax, sv, dens, 0, 0, abuf);
        }
    }
    double t0 = block_sum<PT>(s0, sh);
    double t1 = block_sum<PT>(s1, sh);
    if (threadIdx.x == 0) {
        part[0 * h.pstride + blockIdx.x] = t0;
        part[1 * h.pstride + blockIdx.x] = t1;
    }
}

template <bool AGG = false>
__global__ void __launch_bounds__(PT) k_sa_ka(Hot h, const int16_t *__restrict__ pmid,
                                              float *disp, float *vel,
                                              const float *__restrict__ acc, float *disp_cot,
                                              float *vel_cot, const float *__restrict__ alpha,
                                              int64_t n, const float *__restrict__ rho_cot,
                                              float K2, float K1n, float Dn, float *dens,
                                              double *part) {
    sa_ka_body<AGG>(h, pmid, disp, vel, acc, disp_cot, vel_cot, alpha, n, rho_cot, K2, K1n, Dn,
                    dens, part);
}

// Sums the per-block partials in a fixed order: dots[s] = sum of slot s for
// s < nslots (dots may be NULL), and *om_out = om_scale * sum of slot 2
// (om_out may be NULL).  Slot 2 holds nblk2 partials (the gather VJP's
// grid), the other slots nblk; slot s starts at part + s * pstride.
__global__ void k_finish(const double *part, int64_t pstride, int nblk, int nblk2, double *dots,
                         int nslots, double *om_out, double om_scale) {
    __shared__ double sh[32];
    int last = nslots > 3 ? nslots : 3;
    for (int s = 0; s < last; ++s) {
        bool want = (dots && s < nslots) || (om_out && s == 2);
        if (!want) continue;
        const int nb = s == 2 ? nblk2 : nblk;
        const double *p = part + s * pstride;
        // eight independent partial sums per thread of the 1024 (a fixed
        // order), so the loads of a large grid's partials overlap
        double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        int b = threadIdx.x;
        for (; b + 7 * 1024 < nb; b += 8 * 1024) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] += p[b + u * 1024];
        }
        for (; b < nb; b += 1024) a[0] += p[b];
        double v = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
        double t = block_sum<1024>(v, sh);
        if (threadIdx.x == 0) {
            if (dots && s < nslots) dots[s] = t;
            if (om_out && s == 2) *om_out = om_scale * t;
        }
    }
}

// ---------------------------------------------------------------------------
// Batched simulations: one launch serves up to BMAX simulations that share a
// mesh shape and cell size.  blockIdx.y selects the simulation; its particle
// arrays, particle count, CIC value and this launch's leapfrog factors come
// from a table passed by value (__grid_constant__: read in place from the
// parameter space), its meshes are slot blockIdx.y of the workspace buffers.
// Each body is the one the single-simulation kernels run, so a simulation's
// arithmetic is the same alone and in a batch.
// ---------------------------------------------------------------------------

struct SimB {
    const int16_t *pmid;
    float *disp, *vel, *acc, *dcot, *vcot, *alpha;
    int64_t n;
    float val;     // f32(mesh_size / ptcl_num) of this simulation
    float f[3];    // this launch's leapfrog factors (meaning per kernel)
};
struct BatchTab {
    SimB s[BMAX];
};

// Slot b's share of a slot-major buffer of `per` elements per slot.
template <typename T>
__device__ __forceinline__ T *slot_ptr(T *base, int64_t per) {
    return base + blockIdx.y * per;
}

__device__ __forceinline__ Hot sim_hot(const Hot &h, const SimB &sb) {
    Hot hh = h;
    hh.val = sb.val;
    return hh;
}

template <bool KD, bool AGG>
__global__ void __launch_bounds__(PT) k_kds_b(Hot h, const __grid_constant__ BatchTab t,
                                              float *dens, int64_t M) {
    const SimB &sb = t.s[blockIdx.y];
    kds_body<KD, false, false, AGG>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vel, sb.acc, sb.n, sb.f[0],
                               sb.f[1], slot_ptr(dens, M));
}

template <bool KICK>
__global__ void __launch_bounds__(PT) k_gather3_b(Hot h, const __grid_constant__ BatchTab t,
                                                  int64_t M, const float *g) {
    const SimB &sb = t.s[blockIdx.y];
    gather3_body<KICK, false>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vel, sb.acc, sb.n, M,
                              slot_ptr(g, 3 * M), sb.f[0]);
}

template <bool AGG>
__global__ void __launch_bounds__(PT) k_gk_kds_b(Hot h, const __grid_constant__ BatchTab t,
                                                 int64_t M, const float *g, float *dens) {
    const SimB &sb = t.s[blockIdx.y];
    gk_kds_body<AGG>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vel, sb.n, slot_ptr(g, 3 * M), sb.f[0],
                sb.f[1], sb.f[2], slot_ptr(dens, M));
}

template <bool KD, bool AGG>
__global__ void __launch_bounds__(PT) k_ka_b(Hot h, const __grid_constant__ BatchTab t,
                                             int64_t M, float *dens, double *part) {
    const SimB &sb = t.s[blockIdx.y];
    ka_body<KD, false, false, AGG>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vel, sb.acc, sb.dcot, sb.vcot,
                              sb.alpha, sb.n, sb.f[0], sb.f[1], slot_ptr(dens, M),
                              slot_ptr(part, NSLOT * h.pstride));
}

// acc_cot: the simulation's vel_cot (steps) or the given cotangent of acc
// (the force VJP, where it is also vel_cot)
template <bool AGG>
__global__ void __launch_bounds__(PT) k_g3adj_b(Hot h, const __grid_constant__ BatchTab t,
                                                int64_t M, const float *g, float *mcot,
                                                double *part) {
    const SimB &sb = t.s[blockIdx.y];
    g3adj_body<false, AGG>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vcot, sb.acc, sb.alpha, sb.n, M,
                      slot_ptr(g, 3 * M), slot_ptr(mcot, 3 * M),
                      slot_ptr(part, NSLOT * h.pstride));
}

template <bool KICK>
__global__ void __launch_bounds__(PT) k_sadj_b(Hot h, const __grid_constant__ BatchTab t,
                                               int64_t M, const float *rcot) {
    const SimB &sb = t.s[blockIdx.y];
    sadj_body<KICK, false>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vel, sb.acc, sb.dcot, sb.alpha,
                           sb.n, slot_ptr(rcot, M), sb.f[0]);
}

template <bool AGG>
__global__ void __launch_bounds__(PT) k_sa_ka_b(Hot h, const __grid_constant__ BatchTab t,
                                                int64_t M, const float *rcot, float *dens,
                                                double *part) {
    const SimB &sb = t.s[blockIdx.y];
    sa_ka_body<AGG>(sim_hot(h, sb), sb.pmid, sb.disp, sb.vel, sb.acc, sb.dcot, sb.vcot, sb.alpha, sb.n,
               slot_ptr(rcot, M), sb.f[0], sb.f[1], sb.f[2], slot_ptr(dens, M),
               slot_ptr(part, NSLOT * h.pstride));
}

// k_finish of every simulation of a batch (block b: slot b): dots[b][0..3)
// and the Omega_m term into dots[b][3], or only the latter (ndots 0).
struct FinishTab {
    double *dots[BMAX];
    double oms[BMAX];
};
__global__ void k_finish_b(const double *part, int64_t pstride, int nblk,
                           const __grid_constant__ FinishTab t, int ndots) {
    __shared__ double sh[32];
    const double *pp = part + blockIdx.x * NSLOT * pstride;
    double *dots = t.dots[blockIdx.x];
    for (int s = 0; s < 3; ++s) {
        if (s >= ndots && s != 2) continue;
        double v = 0.0;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += pp[s * pstride + b];
        double tt = block_sum<1024>(v, sh);
        if (threadIdx.x == 0) {
            if (s < ndots) dots[s] = tt;
            if (s == 2) dots[3] = t.oms[blockIdx.x] * tt;
        }
    }
}

// Elementwise leapfrog kernels of the generic API.
__global__ void k_axpy(float *y, const float *__restrict__ x, int64_t n, float a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __fadd_rn(y[i], __fmul_rn(x[i], a));
}

// y += x*a; z -= w*a; partial sum(u * x) (u may equal the updated y/z: it
// is read before any update of this element).  Covers kick_adj (y=vel,
// x=acc, z=disp_cot, w=alpha, u=vel_cot) and drift_adj (y=disp, x=vel,
// z=vel_cot, w=disp_cot, dot of the updated disp_cot... see callers).
__global__ void k_kick_adj(float *vel, const float *__restrict__ acc, float *disp_cot,
                           const float *__restrict__ alpha, const float *__restrict__ vel_cot,
                           int64_t n, float K, double *part) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float a = acc[i];
        vel[i] = __fadd_rn(vel[i], __fmul_rn(a, K));
        disp_cot[i] = __fsub_rn(disp_cot[i], __fmul_rn(alpha[i], K));
        s += (double)vel_cot[i] * (double)a;
    }
    double t = block_sum<PT>(s, sh);
    if (part && threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_drift_adj(float *disp, const float *__restrict__ vel, float *vel_cot,
                            const float *__restrict__ disp_cot, int64_t n, float D, double *part) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float v = vel[i];
        float dc = disp_cot[i];
        disp[i] = __fadd_rn(disp[i], __fmul_rn(v, D));
        vel_cot[i] = __fsub_rn(vel_cot[i], __fmul_rn(dc, D));
        s += (double)dc * (double)v;
    }
    double t = block_sum<PT>(s, sh);
    if (part && threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_dot(const float *__restrict__ x, const float *__restrict__ y, int64_t n,
                      double *part) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s += (double)x[i] * (double)y[i];
    double t = block_sum<PT>(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_reduce1(const double *part, int nblk, double *out) {
    __shared__ double sh[32];
    double v = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += part[b];
    double t = block_sum<1024>(v, sh);
    if (threadIdx.x == 0) *out = t;
}

}  // namespace pmx

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

namespace {

int grid_fill(int64_t n) { return stride_grid((n + 3) / 4, 256, 16); }

// Blocks of a grid-stride particle kernel: one particle per thread, or at
// most per_sm blocks per SM, and never more than the workspace holds
// partial sums for.  Many short blocks beat a few long-running ones: the
// block scheduler starts a new block whenever one ends, so warps slowed by
// contended atomics (the halos of the late, clustered steps) hold up only
// their own block, not a fixed share of the particles.  Measured on the
// 512^3-particle / 1024^3-mesh run, ms per forward + adjoint step pair over
// all 100 + 100 steps (over the first 10 + 10): one particle per thread
// 112.8 (90.1); 65536 blocks 121.3 (90.7); 64 blocks per SM 130 (91.4); 8
// per SM 140 (93.8); one resident wave of blocks slower still.
int ptcl_grid(const pmx_workspace *ws, int64_t n, int per_sm = 1 << 30) {
    const int64_t g = stride_grid(n, PT, per_sm);
    return (int)(g < ws->pstride ? g : ws->pstride);
}
// The kernels that also sum two dot products per block (the adjoint's
// kick/drift passes) measured best at 64 blocks per SM: k_sa_ka 5.59 ms per
// launch vs 5.84 at 65536 blocks, k_ka 0.56 vs 0.80 ms at one particle per
// thread.
constexpr int DOT2_PER_SM = 64;

// Per-device reduction scratch for the stand-alone dot entry points,
// allocated once at their first use on a device.
std::mutex g_scratch_mu;
double *g_scratch[64] = {nullptr};

int device_scratch(double **out) {
    int dev = 0;
    PMX_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(PMX_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch[dev]) {
        if (cudaMalloc(&g_scratch[dev], PMAX * sizeof(double)) != cudaSuccess) {
            g_scratch[dev] = nullptr;
            cudaGetLastError();
            return fail(PMX_ERR_NOMEM, "cannot allocate reduction scratch");
        }
    }
    *out = g_scratch[dev];
    return PMX_OK;
}

// Launches KERNEL<KD, WIN, KAHAN> for the Hot's window and compensation
// settings (dynamic shared memory only with windows).
#define PMX_WIN_LAUNCH(h, KERNEL, KD, grid, wsmem, st, args)                                   \
    do {                                                                                       \
        if ((h).win) {                                                                         \
            if ((h).vcomp) KERNEL<PMX_UNPAREN KD, true, true><<<grid, PT, wsmem, st>>> args;   \
            else KERNEL<PMX_UNPAREN KD, true, false><<<grid, PT, wsmem, st>>> args;            \
        } else {                                                                               \
            if ((h).vcomp) KERNEL<PMX_UNPAREN KD, false, true><<<grid, PT, 0, st>>> args;      \
            else if ((h).agg) KERNEL<PMX_UNPAREN KD, false, false, true><<<grid, PT, 0, st>>> args; \
            else KERNEL<PMX_UNPAREN KD, false, false><<<grid, PT, 0, st>>> args;               \
        }                                                                                      \
    } while (0)
#define PMX_UNPAREN(...) __VA_ARGS__

int check_hot(pmx_workspace *ws, const pmx_enmesh_spec *spec, const void *pmid, const void *disp,
              int64_t n, int64_t ptcl_num, Hot *h) {
    if (!ws) return fail(PMX_ERR_ARG, "null workspace");
    if (!spec) return fail(PMX_ERR_ARG, "null spec");
    if (spec->dim != 3) return fail(PMX_ERR_ARG, "the force path is 3-D");
    if (spec->cell_size > 0 || spec->offset[0] != 0 || spec->offset[1] != 0 || spec->offset[2] != 0)
        return fail(PMX_ERR_ARG, "the force path uses the default enmesh (offset 0, cell_size None)");
    if (spec->mesh_shape[0] != ws->n0 || spec->mesh_shape[1] != ws->n1 || spec->mesh_shape[2] != ws->n2 ||
        spec->wrap_shape[0] != ws->n0 || spec->wrap_shape[1] != ws->n1 || spec->wrap_shape[2] != ws->n2)
        return fail(PMX_ERR_SHAPE, "mesh shape differs from the workspace's");
    if (!(spec->conf_cell_size > 0)) return fail(PMX_ERR_ARG, "conf_cell_size must be > 0");
    if (n < 0 || ptcl_num <= 0) return fail(PMX_ERR_ARG, "bad particle counts");
    if (n > 0 && (!pmid || !disp)) return fail(PMX_ERR_ARG, "null pmid/disp");
    int dev = 0;
    PMX_CUDA(cudaGetDevice(&dev));
    if (dev != ws->dev) return fail(PMX_ERR_ARG, "workspace belongs to another device");
    for (int a = 0; a < 3; ++a) h->wrap[a] = spec->wrap_shape[a];
    h->stride[2] = 1;
    h->stride[1] = ws->n2;
    h->stride[0] = ws->n1 * ws->n2;
    h->cell = (float)spec->conf_cell_size;
    h->val = (float)((double)ws->M / (double)ptcl_num);
    h->dcomp = nullptr;
    h->vcomp = nullptr;
    h->win = ws->win;
    // measured slower on GB300 (the v4 reductions with two zero lanes cost
    // more than the scalar atomics they replace): opt-in, PMX_WS_VEC
    h->vec = ws->vec;
    h->agg = ws->agg;
    h->pstride = ws->pstride;
    if (ws->xfast) {
        h->gxs = 2 * ws->n1 * ws->n2;
        h->gjs = ws->n1 * ws->n2;
    } else {
        h->gxs = 0;
        h->gjs = ws->M;
    }
    return PMX_OK;
}

int ensure_ktab(pmx_workspace *ws, double cell, cudaStream_t st) {
    if (ws->ktab_cell == cell) return PMX_OK;
    double period = 2 * PI / cell;
    float nyq = (float)(PI / cell);
    float eps = nyq * 1.1920928955078125e-07f;
    int tot = (int)(ws->n0 + ws->n1 + ws->n2h);
    k_ktab<<<(tot + 255) / 256, 256, 0, st>>>(ws->ktab, (int)ws->n0, (int)ws->n1, (int)ws->n2,
                                              period, nyq, eps);
    PMX_LAUNCH_CHECK("k_ktab");
    ws->ktab_cell = cell;
    return PMX_OK;
}

int poisson_grid(pmx_workspace *ws) {
    int64_t rows = ws->n0 * ws->n1;
    int64_t blocks = (rows + 7) / 8;  // 8 warps per block
    int64_t cap = (int64_t)device_sms() * 16;
    return (int)(blocks < cap ? blocks : cap);
}

// Issues the slab loop of transform `kind` on stream s0: slab i (S x-planes
// of one component) runs on chain i % nbranch, each chain on its own stream
// with its own plan, forked from and joined back into s0.
int slab_issue(pmx_workspace *ws, int kind, int nslot, const void *in, void *out,
               cudaStream_t s0) {
    SlabXf &x = ws->sx[kind];
    const int64_t pr = ws->n1 * ws->n2, pc = ws->n1 * ws->n2h, S = ws->slab;
    const int64_t np = nslot * ((kind == 1 || kind == 2) ? 3 * ws->n0 : ws->n0);
    const int K = ws->nbranch;
    if (K > 1) {
        PMX_CUDA(cudaEventRecord(ws->fork, s0));
        for (int k = 1; k < K; ++k) PMX_CUDA(cudaStreamWaitEvent(ws->aux[k], ws->fork, 0));
    }
    for (int64_t p = 0, i = 0; p < np; p += S, ++i) {
        const int k = (int)(i % K);
        PMX_CUFFT(cufftSetStream(x.plan[k], k ? ws->aux[k] : s0));
        if (x.r2c)
            PMX_CUFFT(cufftExecR2C(x.plan[k], (float *)in + p * pr, (cufftComplex *)out + p * pc));
        else
            PMX_CUFFT(cufftExecC2R(x.plan[k], (cufftComplex *)in + p * pc, (float *)out + p * pr));
    }
    for (int k = 1; k < K; ++k) {
        PMX_CUDA(cudaEventRecord(ws->join[k], ws->aux[k]));
        PMX_CUDA(cudaStreamWaitEvent(s0, ws->join[k], 0));
    }
    return PMX_OK;
}

// Runs transform `kind` (in -> out, all planes of nslot slots) on st:
// directly, or by launching the CUDA graph of its slab loop, captured on
// first use for this slot count (and again if the buffers change).
int slab_run(pmx_workspace *ws, int kind, int nslot, const void *in, void *out,
             cudaStream_t st) {
    if (!ws->graphs || nslot > GMAX) return slab_issue(ws, kind, nslot, in, out, st);
    SlabXf &x = ws->sx[kind];
    cudaGraphExec_t &ex = x.exec[nslot];
    if (ex && (x.in[nslot] != in || x.out[nslot] != out)) {
        cudaGraphExecDestroy(ex);
        ex = nullptr;
    }
    if (!ex) {
        PMX_CUDA(cudaStreamBeginCapture(ws->cap, cudaStreamCaptureModeThreadLocal));
        int e = slab_issue(ws, kind, nslot, in, out, ws->cap);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(ws->cap, &g);
        if (e) {
            if (g) cudaGraphDestroy(g);
            return e;
        }
        if (ce != cudaSuccess) return cuda_status(ce, "slab graph capture");
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            ex = nullptr;
            return cuda_status(ce, "slab graph instantiate");
        }
        x.in[nslot] = in;
        x.out[nslot] = out;
    }
    PMX_CUDA(cudaGraphLaunch(ex, st));
    return PMX_OK;
}

// Green's function constant of the Poisson solve: -(1.5 Omega_m) / M in
// the reference's float32 rounding (gravity.py:56-60).
float green_c(const pmx_workspace *ws, double omega_m) {
    float s = (float)(1.5 * (double)(float)omega_m);
    return (float)((double)s / (double)ws->M);
}

// Forward force up to the three acceleration meshes in ws->g, for the
// densities of the first nslot slots (slot b: Green's constant c[b]); the
// slots' spectra and meshes are consecutive, so each plane transform runs
// over all their planes at once.
int force_meshes_b(pmx_workspace *ws, int nslot, const float *c, cudaStream_t st) {
    if (ws->xfast) {
        float2 *H = reinterpret_cast<float2 *>(ws->g);  // g is free until the c2r
        const int64_t pc = ws->n0 * ws->n1 * ws->n2p;  // complex values per slot spectrum
        if (ws->plane) {
            Stage sg(ws, 2, st, 1);
            int st2 = plane_fft(false, ws->dens, H, ws->ptw, nslot * ws->n0, ws->n1, ws->n2,
                                ws->pscr, ws->pcl, ws->plane16, st);
            if (st2) return st2;
        } else {
            Stage sg(ws, 2, st, 0);
            int st2 = slab_run(ws, 0, nslot, ws->dens, H, st);
            if (st2) return st2;
        }
        {
            Stage sg(ws, 3, st, nslot);
            for (int b = 0; b < nslot; ++b) {
                int st2 = xpass(false, H + b * pc, ws->ck + 3 * b * pc, ws->ktab, ws->tw, ws->n0,
                                ws->n1, ws->n2h, ws->n2p, c[b], st);
                if (st2) return st2;
            }
        }
        if (ws->plane) {
            Stage sg(ws, 4, st, 1);
            int st2 = plane_fft(true, ws->ck, ws->g, ws->ptw, 3 * nslot * ws->n0, ws->n1, ws->n2,
                                ws->pscr, ws->pcl, ws->plane16, st);
            if (st2) return st2;
        } else {
            Stage sg(ws, 4, st, 0);
            int st2 = slab_run(ws, 1, nslot, ws->ck, ws->g, st);
            if (st2) return st2;
        }
        return PMX_OK;
    }
    if (nslot != 1) return fail(PMX_ERR_SHAPE, "batched calls need the fused x-pass path");
    const float c0 = c[0];
    {
        Stage sg(ws, 2, st, 0);
        PMX_CUFFT(cufftSetStream(ws->r2c1, st));
        PMX_CUFFT(cufftExecR2C(ws->r2c1, ws->dens, reinterpret_cast<cufftComplex *>(ws->ck)));
    }
    {
        Stage sg(ws, 3, st, 1);
        k_poisson_fwd<<<poisson_grid(ws), 256, 0, st>>>(ws->ck, ws->n0, ws->n1, ws->n2h, ws->Mc,
                                                         ws->ktab, c0);
        PMX_LAUNCH_CHECK("k_poisson_fwd");
    }
    {
        Stage sg(ws, 4, st, 0);
        PMX_CUFFT(cufftSetStream(ws->c2r3, st));
        PMX_CUFFT(cufftExecC2R(ws->c2r3, reinterpret_cast<cufftComplex *>(ws->ck), ws->g));
    }
    return PMX_OK;
}

// The force VJP tail after k_g3adj has filled the mesh cotangents of the
// first nslot slots: r2c of the three cotangent meshes, adjoint Fourier
// operator, c2r into rcot_of(nslot) (then rho_cot of each slot, scale
// folded in).
int force_adj_meshes_b(pmx_workspace *ws, int nslot, const float *c, cudaStream_t st) {
    if (ws->xfast) {
        float2 *Sk = reinterpret_cast<float2 *>(ws->g);  // g is dead after k_g3adj
        float *rcot = ws->rcot_of(nslot);
        const int64_t pc = ws->n0 * ws->n1 * ws->n2p;
        if (ws->plane) {
            Stage sg(ws, 8, st, 1);
            int st2 = plane_fft(false, ws->mcot, ws->ck, ws->ptw, 3 * nslot * ws->n0, ws->n1,
                                ws->n2, ws->pscr, ws->pcl, ws->plane16, st);
            if (st2) return st2;
        } else {
            Stage sg(ws, 8, st, 0);
            int st2 = slab_run(ws, 2, nslot, ws->mcot, ws->ck, st);
            if (st2) return st2;
        }
        {
            Stage sg(ws, 9, st, nslot);
            for (int b = 0; b < nslot; ++b) {
                int st2 = xpass(true, ws->ck + 3 * b * pc, Sk + b * pc, ws->ktab, ws->tw, ws->n0,
                                ws->n1, ws->n2h, ws->n2p, c[b], st);
                if (st2) return st2;
            }
        }
        if (ws->plane) {
            Stage sg(ws, 10, st, 1);
            int st2 = plane_fft(true, Sk, rcot, ws->ptw, nslot * ws->n0, ws->n1, ws->n2,
                                ws->pscr, ws->pcl, ws->plane16, st);
            if (st2) return st2;
        } else {
            Stage sg(ws, 10, st, 0);
            int st2 = slab_run(ws, 3, nslot, Sk, rcot, st);
            if (st2) return st2;
        }
        return PMX_OK;
    }
    if (nslot != 1) return fail(PMX_ERR_SHAPE, "batched calls need the fused x-pass path");
    const float c0 = c[0];
    {
        Stage sg(ws, 8, st, 0);
        PMX_CUFFT(cufftSetStream(ws->r2c3, st));
        PMX_CUFFT(cufftExecR2C(ws->r2c3, ws->mcot, reinterpret_cast<cufftComplex *>(ws->ck)));
    }
    {
        Stage sg(ws, 9, st, 1);
        k_poisson_adj<<<poisson_grid(ws), 256, 0, st>>>(ws->ck, ws->n0, ws->n1, ws->n2h, ws->Mc,
                                                         ws->ktab, c0);
        PMX_LAUNCH_CHECK("k_poisson_adj");
    }
    {
        Stage sg(ws, 10, st, 0);
        PMX_CUFFT(cufftSetStream(ws->c2r1, st));
        PMX_CUFFT(cufftExecC2R(ws->c2r1, reinterpret_cast<cufftComplex *>(ws->ck), ws->rcot_of(1)));
    }
    return PMX_OK;
}

// One simulation (slot 0) of the workspace.
int force_meshes(pmx_workspace *ws, const Hot &, double omega_m, cudaStream_t st) {
    const float c = green_c(ws, omega_m);
    return force_meshes_b(ws, 1, &c, st);
}
int force_adj_meshes(pmx_workspace *ws, double omega_m, cudaStream_t st) {
    const float c = green_c(ws, omega_m);
    return force_adj_meshes_b(ws, 1, &c, st);
}

double om_scale(double omega_m) {
    float s = (float)(1.5 * (double)(float)omega_m);
    return 1.5 / (double)s;
}

int make_plan(cufftHandle *plan, const int64_t shape[3], cufftType type, int64_t batch,
              size_t *work) {
    PMX_CUFFT(cufftCreate(plan));
    PMX_CUFFT(cufftSetAutoAllocation(*plan, 0));
    long long n[3] = {shape[0], shape[1], shape[2]};
    size_t w = 0;
    PMX_CUFFT(cufftMakePlanMany64(*plan, 3, n, nullptr, 1, 0, nullptr, 1, 0, type, batch, &w));
    *work = w;
    return PMX_OK;
}

int make_plan2d(cufftHandle *plan, int64_t n1, int64_t n2, cufftType type, int64_t batch,
                size_t *work) {
    PMX_CUFFT(cufftCreate(plan));
    PMX_CUFFT(cufftSetAutoAllocation(*plan, 0));
    long long n[2] = {n1, n2};
    size_t w = 0;
    PMX_CUFFT(cufftMakePlanMany64(*plan, 2, n, nullptr, 1, 0, nullptr, 1, 0, type, batch, &w));
    *work = w;
    return PMX_OK;
}

// x-planes per slab execution of the (y, z) plane transforms: the smallest
// power of two >= 8 whose complex planes reach 32 MB (8 planes at 1024^2,
// every plane of meshes up to 128^3), so small meshes take a few large
// cuFFT launches instead of many tiny ones.  A nonzero log2 (the
// PMX_WS_SLAB_LOG2 field of the flags) sets it instead.
int64_t choose_slab(int64_t n0, int64_t n1, int64_t n2, int log2) {
    int64_t S = log2 > 0 ? (int64_t)1 << log2 : 0;
    if (S <= 0) {
        const int64_t plane = n1 * (n2 / 2 + 1) * 8;
        S = 8;
        while (S < n0 && S * plane < ((int64_t)32 << 20)) S *= 2;
    }
    if (S > n0) S = n0;
    while (S > 1 && n0 % S) S /= 2;
    if (S < 1) S = 1;
    return S;
}

void ws_free(pmx_workspace *ws) {
    if (!ws) return;
    if (ws->have_r2c1) cufftDestroy(ws->r2c1);
    if (ws->have_c2r3) cufftDestroy(ws->c2r3);
    if (ws->have_r2c3) cufftDestroy(ws->r2c3);
    if (ws->have_c2r1) cufftDestroy(ws->c2r1);
    for (auto &x : ws->sx) {
        for (auto e : x.exec)
            if (e) cudaGraphExecDestroy(e);
        for (int k = 0; k < KMAX; ++k) {
            if (x.have[k]) cufftDestroy(x.plan[k]);
            cudaFree(x.work[k]);
        }
    }
    for (int k = 0; k < KMAX; ++k) {
        if (ws->aux[k]) cudaStreamDestroy(ws->aux[k]);
        if (ws->join[k]) cudaEventDestroy(ws->join[k]);
    }
    if (ws->cap) cudaStreamDestroy(ws->cap);
    if (ws->fork) cudaEventDestroy(ws->fork);
    cudaFree(ws->tw);
    cudaFree(ws->ptw);
    cudaFree(ws->pscr);
    cudaFree(ws->dens);
    cudaFree(ws->ck);
    cudaFree(ws->g);
    cudaFree(ws->mcot);
    cudaFree(ws->ktab);
    cudaFree(ws->part);
    cudaFree(ws->err);
    cudaFree(ws->fft_work);
    for (auto &r : ws->recs) {
        cudaEventDestroy(r.b);
        cudaEventDestroy(r.e);
    }
    for (auto e : ws->pool) cudaEventDestroy(e);
    delete ws;
}

size_t buffers_bytes(const int64_t s[3], int32_t flags, int32_t slots) {
    int64_t M = s[0] * s[1] * s[2], Mc = s[0] * s[1] * (s[2] / 2 + 1);
    size_t b = (size_t)M * 4 + (size_t)Mc * 8 * 3 + (size_t)M * 4 * 3;
    if (flags & PMX_WS_ADJOINT) b += (size_t)M * 4 * 3;
    b += (size_t)NSLOT * (slots == 1 ? PART_ONE : PART_SLOT) * 8;
    return b * (size_t)slots + (size_t)2 * (s[0] + s[1] + s[2] / 2 + 1) * 4;
}

// The tensor map of the plane-interleaved acceleration meshes g, (x, 3, n1,
// n2) float32, for k_gather3_tma's (TBX, 3, TBY, TBZ) boxes.  The encoder is
// a driver entry point, looked up through the runtime.
int encode_gather_map(pmx_workspace *ws) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!encode) {
            cudaDriverEntryPointQueryResult q;
            void *fn = nullptr;
            cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                             cudaEnableDefault, &q);
            if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
                return fail(PMX_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        }
    }
    if (ws->n2 % 4) return fail(PMX_ERR_SHAPE, "TMA gathers need n2 % 4 == 0");
    const cuuint64_t dims[4] = {(cuuint64_t)ws->n2, (cuuint64_t)ws->n1, 3, (cuuint64_t)ws->n0};
    const cuuint64_t strides[3] = {(cuuint64_t)ws->n2 * 4, (cuuint64_t)(ws->n1 * ws->n2) * 4,
                                   (cuuint64_t)(3 * ws->n1 * ws->n2) * 4};
    const cuuint32_t box[4] = {TBZ, TBY, 3, TBX};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = encode(&ws->tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, ws->g, dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(PMX_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return PMX_OK;
}

int check_shape(const int64_t s[3]) {
    for (int a = 0; a < 3; ++a)
        if (s[a] < 1 || s[a] > (1 << 20)) return fail(PMX_ERR_SHAPE, "bad mesh shape");
    return PMX_OK;
}

}  // namespace

extern "C" int pmx_workspace_bytes(const int64_t mesh_shape[3], int32_t flags, size_t *bytes) {
    if (!mesh_shape || !bytes) return fail(PMX_ERR_ARG, "null argument");
    int st = check_shape(mesh_shape);
    if (st) return st;
    size_t total = buffers_bytes(mesh_shape, flags, 1), wmax = 0;
    cufftType types[4] = {CUFFT_R2C, CUFFT_C2R, CUFFT_R2C, CUFFT_C2R};
    int64_t batches[4] = {1, 3, 3, 1};
    int nplans = (flags & PMX_WS_ADJOINT) ? 4 : 2;
    for (int i = 0; i < nplans; ++i) {
        int n[3] = {(int)mesh_shape[0], (int)mesh_shape[1], (int)mesh_shape[2]};
        size_t w = 0;
        PMX_CUFFT(cufftEstimateMany(3, n, nullptr, 1, 0, nullptr, 1, 0, types[i],
                                    (int)batches[i], &w));
        if (w > wmax) wmax = w;
    }
    *bytes = total + wmax;
    return PMX_OK;
}

static int ws_create(const int64_t mesh_shape[3], int32_t flags, int32_t slots,
                     pmx_workspace **out) {
    if (!mesh_shape || !out) return fail(PMX_ERR_ARG, "null argument");
    int st = check_shape(mesh_shape);
    if (st) return st;
    if (slots < 1 || slots > BMAX) return fail(PMX_ERR_ARG, "slots must be in 1..16");
    pmx_workspace *ws = new pmx_workspace();
    ws->flags = flags;
    ws->slots = slots;
    ws->pstride = slots == 1 ? PART_ONE : PART_SLOT;
    ws->n0 = mesh_shape[0];
    ws->n1 = mesh_shape[1];
    ws->n2 = mesh_shape[2];
    ws->n2h = ws->n2 / 2 + 1;
    ws->M = ws->n0 * ws->n1 * ws->n2;
    ws->Mc = ws->n0 * ws->n1 * ws->n2h;
    if (cudaGetDevice(&ws->dev) != cudaSuccess) {
        delete ws;
        return fail(PMX_ERR_CUDA, "cudaGetDevice failed");
    }
    auto alloc = [&](void **p, size_t b) -> int {
        if (cudaMalloc(p, b) != cudaSuccess) {
            cudaGetLastError();
            *p = nullptr;
            return fail(PMX_ERR_NOMEM, "workspace allocation of " + std::to_string(b) + " bytes failed");
        }
        return PMX_OK;
    };
    ws->xfast = xpass_supported(ws->n0) && !(flags & PMX_WS_CUFFT3D);
    ws->plane = ws->xfast && plane_supported(ws->n1, ws->n2) && (flags & PMX_WS_PLANE);
    ws->plane16 = (flags & PMX_WS_PLANE16) != 0;
    ws->vec = ws->n2 % 4 == 0 && (flags & PMX_WS_VEC);
    ws->agg = (flags & PMX_WS_AGG) && (uint64_t)ws->M * (uint64_t)slots < 0xFFFFFFE0ull;
    ws->n2p = ws->plane ? padded_row(ws->n2h) : ws->n2h;
    int64_t ktn = 2 * (ws->n0 + ws->n1 + ws->n2h);
    const int64_t B = slots;
    if ((st = alloc((void **)&ws->dens, B * ws->M * 4)) ||
        (st = alloc((void **)&ws->ck, B * ws->n0 * ws->n1 * ws->n2p * 8 * 3)) ||
        (st = alloc((void **)&ws->g, B * ws->M * 4 * 3)) || (st = alloc((void **)&ws->ktab, ktn * 4)) ||
        (st = alloc((void **)&ws->part, B * NSLOT * ws->pstride * 8)) ||
        ((flags & PMX_WS_ADJOINT) && (st = alloc((void **)&ws->mcot, B * ws->M * 4 * 3)))) {
        ws_free(ws);
        return st;
    }
    ws->win = (ws->n2 % 4 == 0) && (flags & PMX_WS_WINDOW);
    if (ws->win) {
        cudaError_t e = cudaFuncSetAttribute(k_g3adj<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)WIN3_SMEM);
        if (e != cudaSuccess) {
            ws_free(ws);
            return cuda_status(e, "cudaFuncSetAttribute(k_g3adj)");
        }
    }
    size_t wk[4] = {0, 0, 0, 0};
    cufftHandle *ph[4];
    bool *hv[4];
    if (ws->plane) {
        if ((st = plane_max_clusters(ws->n1, ws->n2, ws->plane16, &ws->pcl)) ||
            (st = alloc((void **)&ws->pscr, (size_t)ws->pcl * ws->n1 * ws->n2p * sizeof(float2)))) {
            ws_free(ws);
            return st;
        }
        const int64_t np = 2 * ws->n1 + 1;
        std::vector<float2> ptw(np);
        plane_twiddles(ws->n1, ws->n2, ptw.data());
        if ((st = alloc((void **)&ws->ptw, np * sizeof(float2)))) { ws_free(ws); return st; }
        if (cudaMemcpy(ws->ptw, ptw.data(), np * sizeof(float2), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            ws_free(ws);
            return fail(PMX_ERR_CUDA, "plane twiddle upload failed");
        }
    }
    if (ws->xfast) {
        ws->slab = choose_slab(ws->n0, ws->n1, ws->n2, (flags >> PMX_WS_SLAB_SHIFT) & 15);
        const int64_t S = ws->slab;
        if (!ws->plane) {
            const int kf = (flags >> PMX_WS_CHAINS_SHIFT) & 7;
            const int K = kf ? kf : 2;   // two concurrent chains measured best
            ws->nbranch = K > KMAX ? KMAX : K;
            ws->graphs = !(flags & PMX_WS_NO_GRAPH);
            auto mk_stream = [&](cudaStream_t *sp) -> int {
                cudaError_t e = cudaStreamCreateWithFlags(sp, cudaStreamNonBlocking);
                return e == cudaSuccess ? PMX_OK : cuda_status(e, "cudaStreamCreate");
            };
            auto mk_event = [&](cudaEvent_t *ep) -> int {
                cudaError_t e = cudaEventCreateWithFlags(ep, cudaEventDisableTiming);
                return e == cudaSuccess ? PMX_OK : cuda_status(e, "cudaEventCreate");
            };
            if ((st = mk_stream(&ws->cap)) || (st = mk_event(&ws->fork))) { ws_free(ws); return st; }
            for (int k = 1; k < ws->nbranch; ++k)
                if ((st = mk_stream(&ws->aux[k])) || (st = mk_event(&ws->join[k]))) { ws_free(ws); return st; }
            const int nkind = (flags & PMX_WS_ADJOINT) ? 4 : 2;
            for (int kind = 0; kind < nkind; ++kind) {
                SlabXf &x = ws->sx[kind];
                x.r2c = kind == 0 || kind == 2;
                for (int k = 0; k < ws->nbranch; ++k) {
                    size_t w = 0;
                    if ((st = make_plan2d(&x.plan[k], ws->n1, ws->n2, x.r2c ? CUFFT_R2C : CUFFT_C2R, S, &w))) { ws_free(ws); return st; }
                    x.have[k] = true;
                    if (w > 0 && (st = alloc(&x.work[k], w))) { ws_free(ws); return st; }
                    cufftResult r = cufftSetWorkArea(x.plan[k], x.work[k]);
                    if (r != CUFFT_SUCCESS) {
                        ws_free(ws);
                        return fail(PMX_ERR_CUFFT, std::string("cufftSetWorkArea: ") + cufft_name(r));
                    }
                }
            }
        }
        std::vector<float2> tw(ws->n0);
        xpass_twiddles(ws->n0, tw.data());
        if ((st = alloc((void **)&ws->tw, ws->n0 * sizeof(float2)))) { ws_free(ws); return st; }
        if (cudaMemcpy(ws->tw, tw.data(), ws->n0 * sizeof(float2), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            ws_free(ws);
            return fail(PMX_ERR_CUDA, "twiddle upload failed");
        }
        for (int i = 0; i < 4; ++i) {
            ph[i] = nullptr;
            hv[i] = nullptr;
        }
    } else {
        int64_t shp[3] = {ws->n0, ws->n1, ws->n2};
        if ((st = make_plan(&ws->r2c1, shp, CUFFT_R2C, 1, &wk[0]))) { ws_free(ws); return st; }
        ws->have_r2c1 = true;
        if ((st = make_plan(&ws->c2r3, shp, CUFFT_C2R, 3, &wk[1]))) { ws_free(ws); return st; }
        ws->have_c2r3 = true;
        if (flags & PMX_WS_ADJOINT) {
            if ((st = make_plan(&ws->r2c3, shp, CUFFT_R2C, 3, &wk[2]))) { ws_free(ws); return st; }
            ws->have_r2c3 = true;
            if ((st = make_plan(&ws->c2r1, shp, CUFFT_C2R, 1, &wk[3]))) { ws_free(ws); return st; }
            ws->have_c2r1 = true;
        }
        ph[0] = &ws->r2c1; ph[1] = &ws->c2r3; ph[2] = &ws->r2c3; ph[3] = &ws->c2r1;
        hv[0] = &ws->have_r2c1; hv[1] = &ws->have_c2r3; hv[2] = &ws->have_r2c3; hv[3] = &ws->have_c2r1;
    }
    if ((flags & PMX_WS_TMA) && ws->xfast && slots == 1) {
        if ((st = alloc((void **)&ws->err, sizeof(int)))) { ws_free(ws); return st; }
        if (cudaMemset(ws->err, 0, sizeof(int)) != cudaSuccess) {
            ws_free(ws);
            return fail(PMX_ERR_CUDA, "error word reset failed");
        }
        if ((st = encode_gather_map(ws))) { ws_free(ws); return st; }
        cudaError_t e = cudaFuncSetAttribute(k_gather3_tma<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TMA_SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_gather3_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)TMA_SMEM);
        if (e != cudaSuccess) { ws_free(ws); return cuda_status(e, "cudaFuncSetAttribute(k_gather3_tma)"); }
        ws->tma = true;
    }
    size_t wmax = 0;
    for (int i = 0; i < 4; ++i)
        if (wk[i] > wmax) wmax = wk[i];
    if (wmax > 0 && (st = alloc(&ws->fft_work, wmax))) { ws_free(ws); return st; }
    ws->fft_work_bytes = wmax;
    for (int i = 0; i < 4; ++i) {
        if (!hv[i] || !*hv[i]) continue;
        cufftResult r = cufftSetWorkArea(*ph[i], ws->fft_work);
        if (r != CUFFT_SUCCESS) {
            ws_free(ws);
            return fail(PMX_ERR_CUFFT, std::string("cufftSetWorkArea: ") + cufft_name(r));
        }
    }
    *out = ws;
    return PMX_OK;
}

extern "C" int pmx_workspace_create(const int64_t mesh_shape[3], int32_t flags,
                                    pmx_workspace **out) {
    return ws_create(mesh_shape, flags, 1, out);
}

extern "C" int pmx_workspace_create_batch(const int64_t mesh_shape[3], int32_t flags,
                                          int32_t slots, pmx_workspace **out) {
    return ws_create(mesh_shape, flags, slots, out);
}

extern "C" int pmx_workspace_destroy(pmx_workspace *ws) {
    if (!ws) return PMX_OK;
    cudaDeviceSynchronize();
    ws_free(ws);
    return PMX_OK;
}

extern "C" int pmx_force(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                         const float *disp, int64_t n, int64_t ptcl_num, double omega_m,
                         float *acc, void *stream) {
    Hot h;
    int st = check_hot(ws, spec, pmid, disp, n, ptcl_num, &h);
    if (st) return st;
    if (n > 0 && !acc) return fail(PMX_ERR_ARG, "null acc");
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    {
        Stage sg(ws, 0, s, 1);
        k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
        PMX_LAUNCH_CHECK("k_fill");
    }
    if (n > 0) {
        {
            Stage sg(ws, 1, s, 1);
            PMX_WIN_LAUNCH(h, k_kds, (false), ptcl_grid(ws, n), WIN1_SMEM, s,
                           (h, pmid, const_cast<float *>(disp), nullptr, nullptr, n, 0.f, 0.f,
                            ws->dens));
            PMX_LAUNCH_CHECK("k_kds");
        }
    }
    if ((st = force_meshes(ws, h, omega_m, s))) return st;
    if (n > 0) {
        {
            Stage sg(ws, 5, s, 1);
            if (ws->tma)
                k_gather3_tma<false><<<ptcl_grid(ws, n), PT, TMA_SMEM, s>>>(
                    h, ws->tmap, pmid, disp, nullptr, acc, n, ws->g, 0.f, ws->err);
            else
                k_gather3<false, false><<<ptcl_grid(ws, n), PT, 0, s>>>(h, pmid, disp, nullptr,
                                                                    acc, n, ws->M, ws->g, 0.f);
            PMX_LAUNCH_CHECK("k_gather3");
        }
    }
    return PMX_OK;
}

extern "C" int pmx_force_vjp(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                             const float *disp, int64_t n, int64_t ptcl_num, double omega_m,
                             const float *acc_cot, float *acc, float *disp_cot,
                             double *omega_m_cot, void *stream) {
    Hot h;
    int st = check_hot(ws, spec, pmid, disp, n, ptcl_num, &h);
    if (st) return st;
    if (!(ws->flags & PMX_WS_ADJOINT)) return fail(PMX_ERR_ARG, "workspace lacks PMX_WS_ADJOINT");
    if (n > 0 && (!acc_cot || !acc || !disp_cot)) return fail(PMX_ERR_ARG, "null acc_cot/acc/disp_cot");
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    {
        Stage sg(ws, 0, s, 2);
        k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
        k_fill<<<grid_fill(3 * ws->M), 256, 0, s>>>(ws->mcot, 0.f, 3 * ws->M);
        PMX_LAUNCH_CHECK("k_fill");
    }
    const int G = ptcl_grid(ws, n);
    if (n > 0) {
        {
            Stage sg(ws, 1, s, 1);
            PMX_WIN_LAUNCH(h, k_kds, (false), G, WIN1_SMEM, s,
                           (h, pmid, const_cast<float *>(disp), nullptr, nullptr, n, 0.f, 0.f,
                            ws->dens));
            PMX_LAUNCH_CHECK("k_kds");
        }
    }
    if ((st = force_meshes(ws, h, omega_m, s))) return st;
    if (n > 0) {
        {
            Stage sg(ws, 7, s, 1);
            if (h.win)
                k_g3adj<true><<<G, PT, WIN3_SMEM, s>>>(h, pmid, disp, acc_cot, acc, disp_cot, n, ws->M,
                                                       ws->g, ws->mcot, ws->part);
            else if (h.agg)
                k_g3adj<false, true><<<G, PT, 0, s>>>(h, pmid, disp, acc_cot, acc, disp_cot, n, ws->M,
                                                      ws->g, ws->mcot, ws->part);
            else
                k_g3adj<false><<<G, PT, 0, s>>>(h, pmid, disp, acc_cot, acc, disp_cot, n, ws->M, ws->g,
                                                ws->mcot, ws->part);
            PMX_LAUNCH_CHECK("k_g3adj");
        }
    }
    if ((st = force_adj_meshes(ws, omega_m, s))) return st;
    if (n > 0) {
        {
            Stage sg(ws, 11, s, 1);
            k_sadj<false, false><<<G, PT, 0, s>>>(h, pmid, disp, nullptr, nullptr, nullptr, disp_cot,
                                                  n, ws->rcot_of(1), 0.f);
            PMX_LAUNCH_CHECK("k_sadj");
        }
    }
    if (omega_m_cot) {
        if (n == 0) {
            PMX_CUDA(cudaMemsetAsync(omega_m_cot, 0, sizeof(double), s));
        } else {
            {
                Stage sg(ws, 12, s, 1);
                k_finish<<<1, 1024, 0, s>>>(ws->part, ws->pstride, G, G, nullptr, 0, omega_m_cot,
                                            om_scale(omega_m));
                PMX_LAUNCH_CHECK("k_finish");
            }
        }
    }
    return PMX_OK;
}

// ---------------------------------------------------------------------------
// leapfrog entry points
// ---------------------------------------------------------------------------

extern "C" int pmx_kick(float *vel, const float *acc, int64_t n3, float factor, void *stream) {
    if (n3 < 0) return fail(PMX_ERR_ARG, "negative size");
    if (n3 == 0) return PMX_OK;
    if (!vel || !acc) return fail(PMX_ERR_ARG, "null vel/acc");
    k_axpy<<<stride_grid(n3, PT), PT, 0, as_stream(stream)>>>(vel, acc, n3, factor);
    PMX_LAUNCH_CHECK("k_axpy");
    return PMX_OK;
}

extern "C" int pmx_drift(float *disp, const float *vel, int64_t n3, float factor, void *stream) {
    if (n3 < 0) return fail(PMX_ERR_ARG, "negative size");
    if (n3 == 0) return PMX_OK;
    if (!disp || !vel) return fail(PMX_ERR_ARG, "null disp/vel");
    k_axpy<<<stride_grid(n3, PT), PT, 0, as_stream(stream)>>>(disp, vel, n3, factor);
    PMX_LAUNCH_CHECK("k_axpy");
    return PMX_OK;
}

extern "C" int pmx_kick_adj(float *vel, const float *acc, float *disp_cot, const float *acc_cot,
                            const float *vel_cot, int64_t n3, float factor, double *dot,
                            void *stream) {
    if (n3 < 0) return fail(PMX_ERR_ARG, "negative size");
    cudaStream_t s = as_stream(stream);
    if (n3 == 0) {
        if (dot) PMX_CUDA(cudaMemsetAsync(dot, 0, sizeof(double), s));
        return PMX_OK;
    }
    if (!vel || !acc || !disp_cot || !acc_cot || !vel_cot) return fail(PMX_ERR_ARG, "null array");
    double *scr = nullptr;
    int st;
    if (dot && (st = device_scratch(&scr))) return st;
    int G = stride_grid(n3, PT);
    if (G > PMAX) G = PMAX;
    k_kick_adj<<<G, PT, 0, s>>>(vel, acc, disp_cot, acc_cot, vel_cot, n3, factor, scr);
    PMX_LAUNCH_CHECK("k_kick_adj");
    if (dot) {
        k_reduce1<<<1, 1024, 0, s>>>(scr, G, dot);
        PMX_LAUNCH_CHECK("k_reduce1");
    }
    return PMX_OK;
}

extern "C" int pmx_drift_adj(float *disp, const float *vel, float *vel_cot, const float *disp_cot,
                             int64_t n3, float factor, double *dot, void *stream) {
    if (n3 < 0) return fail(PMX_ERR_ARG, "negative size");
    cudaStream_t s = as_stream(stream);
    if (n3 == 0) {
        if (dot) PMX_CUDA(cudaMemsetAsync(dot, 0, sizeof(double), s));
        return PMX_OK;
    }
    if (!disp || !vel || !vel_cot || !disp_cot) return fail(PMX_ERR_ARG, "null array");
    double *scr = nullptr;
    int st;
    if (dot && (st = device_scratch(&scr))) return st;
    int G = stride_grid(n3, PT);
    if (G > PMAX) G = PMAX;
    k_drift_adj<<<G, PT, 0, s>>>(disp, vel, vel_cot, disp_cot, n3, factor, scr);
    PMX_LAUNCH_CHECK("k_drift_adj");
    if (dot) {
        k_reduce1<<<1, 1024, 0, s>>>(scr, G, dot);
        PMX_LAUNCH_CHECK("k_reduce1");
    }
    return PMX_OK;
}

extern "C" int pmx_dot(const float *x, const float *y, int64_t n, double *out, void *stream) {
    if (n < 0 || !out) return fail(PMX_ERR_ARG, "bad dot arguments");
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        PMX_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
        return PMX_OK;
    }
    if (!x || !y) return fail(PMX_ERR_ARG, "null x/y");
    double *scr = nullptr;
    int st;
    if ((st = device_scratch(&scr))) return st;
    int G = stride_grid(n, PT);
    if (G > PMAX) G = PMAX;
    k_dot<<<G, PT, 0, s>>>(x, y, n, scr);
    PMX_LAUNCH_CHECK("k_dot");
    k_reduce1<<<1, 1024, 0, s>>>(scr, G, out);
    PMX_LAUNCH_CHECK("k_reduce1");
    return PMX_OK;
}

static int nbody_step(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                      float *disp, float *vel, float *acc, int64_t n, int64_t ptcl_num,
                      const float factors[3], double omega_m, float *dcomp, float *vcomp,
                      void *stream) {
    Hot h;
    int st = check_hot(ws, spec, pmid, disp, n, ptcl_num, &h);
    if (st) return st;
    h.dcomp = dcomp;
    h.vcomp = vcomp;
    if (!factors) return fail(PMX_ERR_ARG, "null factors");
    if (n > 0 && (!vel || !acc)) return fail(PMX_ERR_ARG, "null vel/acc");
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    {
        Stage sg(ws, 0, s, 1);
        k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
        PMX_LAUNCH_CHECK("k_fill");
    }
    const int G = ptcl_grid(ws, n);
    if (n > 0) {
        {
            Stage sg(ws, 1, s, 1);
            PMX_WIN_LAUNCH(h, k_kds, (true), G, WIN1_SMEM, s,
                           (h, pmid, disp, vel, acc, n, factors[0], factors[1], ws->dens));
            PMX_LAUNCH_CHECK("k_kds");
        }
    }
    if ((st = force_meshes(ws, h, omega_m, s))) return st;
    if (n > 0) {
        {
            Stage sg(ws, 5, s, 1);
            if (h.vcomp)
                k_gather3<true, true><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, n, ws->M, ws->g,
                                                       factors[2]);
            else if (ws->tma)
                k_gather3_tma<true><<<G, PT, TMA_SMEM, s>>>(h, ws->tmap, pmid, disp, vel, acc, n,
                                                            ws->g, factors[2], ws->err);
            else
                k_gather3<true, false><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, n, ws->M, ws->g,
                                                        factors[2]);
            PMX_LAUNCH_CHECK("k_gather3");
        }
    }
    return PMX_OK;
}

static int nbody_adj_step(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                          float *disp, float *vel, float *acc, float *disp_cot, float *vel_cot,
                          float *acc_cot, int64_t n, int64_t ptcl_num, const float factors[3],
                          double omega_m, double *dots, float *dcomp, float *vcomp,
                          void *stream) {
    Hot h;
    int st = check_hot(ws, spec, pmid, disp, n, ptcl_num, &h);
    if (st) return st;
    h.dcomp = dcomp;
    h.vcomp = vcomp;
    if (!(ws->flags & PMX_WS_ADJOINT)) return fail(PMX_ERR_ARG, "workspace lacks PMX_WS_ADJOINT");
    if (!factors || !dots) return fail(PMX_ERR_ARG, "null factors/dots");
    if (n > 0 && (!vel || !acc || !disp_cot || !vel_cot || !acc_cot))
        return fail(PMX_ERR_ARG, "null particle array");
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    {
        Stage sg(ws, 0, s, 2);
        k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
        k_fill<<<grid_fill(3 * ws->M), 256, 0, s>>>(ws->mcot, 0.f, 3 * ws->M);
        PMX_LAUNCH_CHECK("k_fill");
    }
    if (n == 0) {
        PMX_CUDA(cudaMemsetAsync(dots, 0, 4 * sizeof(double), s));
        return PMX_OK;
    }
    const int G = ptcl_grid(ws, n), G2 = ptcl_grid(ws, n, DOT2_PER_SM);
    {
        Stage sg(ws, 6, s, 1);
        PMX_WIN_LAUNCH(h, k_ka, (true), G2, WIN1_SMEM, s,
                       (h, pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot, n, factors[0],
                        factors[1], ws->dens, ws->part));
        PMX_LAUNCH_CHECK("k_ka");
    }
    if ((st = force_meshes(ws, h, omega_m, s))) return st;
    {
        Stage sg(ws, 7, s, 1);
        if (h.win)
            k_g3adj<true><<<G, PT, WIN3_SMEM, s>>>(h, pmid, disp, vel_cot, acc, acc_cot, n, ws->M,
                                                   ws->g, ws->mcot, ws->part);
        else if (h.agg)
            k_g3adj<false, true><<<G, PT, 0, s>>>(h, pmid, disp, vel_cot, acc, acc_cot, n, ws->M,
                                                  ws->g, ws->mcot, ws->part);
        else
            k_g3adj<false><<<G, PT, 0, s>>>(h, pmid, disp, vel_cot, acc, acc_cot, n, ws->M, ws->g,
                                            ws->mcot, ws->part);
        PMX_LAUNCH_CHECK("k_g3adj");
    }
    if ((st = force_adj_meshes(ws, omega_m, s))) return st;
    {
        Stage sg(ws, 11, s, 1);
        if (h.vcomp)
            k_sadj<true, true><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot, acc_cot, n,
                                                ws->rcot_of(1), factors[2]);
        else
            k_sadj<true, false><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot, acc_cot, n,
                                                 ws->rcot_of(1), factors[2]);
        PMX_LAUNCH_CHECK("k_sadj");
    }
    {
        Stage sg(ws, 12, s, 1);
        k_finish<<<1, 1024, 0, s>>>(ws->part, ws->pstride, G2, G, dots, 3, dots + 3,
                                    om_scale(omega_m));
        PMX_LAUNCH_CHECK("k_finish");
    }
    return PMX_OK;
}

extern "C" int pmx_nbody_step(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                              float *disp, float *vel, float *acc, int64_t n, int64_t ptcl_num,
                              const float factors[3], double omega_m, void *stream) {
    return nbody_step(ws, spec, pmid, disp, vel, acc, n, ptcl_num, factors, omega_m, nullptr,
                      nullptr, stream);
}

extern "C" int pmx_nbody_step_kahan(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                                    const int16_t *pmid, float *disp, float *vel, float *acc,
                                    float *disp_comp, float *vel_comp, int64_t n,
                                    int64_t ptcl_num, const float factors[3], double omega_m,
                                    void *stream) {
    if (n > 0 && (!disp_comp || !vel_comp)) return fail(PMX_ERR_ARG, "null compensation arrays");
    return nbody_step(ws, spec, pmid, disp, vel, acc, n, ptcl_num, factors, omega_m, disp_comp,
                      vel_comp, stream);
}

extern "C" int pmx_nbody_adj_step(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                                  const int16_t *pmid, float *disp, float *vel, float *acc,
                                  float *disp_cot, float *vel_cot, float *acc_cot, int64_t n,
                                  int64_t ptcl_num, const float factors[3], double omega_m,
                                  double *dots, void *stream) {
    return nbody_adj_step(ws, spec, pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot, n, ptcl_num,
                          factors, omega_m, dots, nullptr, nullptr, stream);
}

extern "C" int pmx_nbody_adj_step_kahan(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                                        const int16_t *pmid, float *disp, float *vel, float *acc,
                                        float *disp_cot, float *vel_cot, float *acc_cot,
                                        float *disp_comp, float *vel_comp, int64_t n,
                                        int64_t ptcl_num, const float factors[3],
                                        double omega_m, double *dots, void *stream) {
    if (n > 0 && (!disp_comp || !vel_comp)) return fail(PMX_ERR_ARG, "null compensation arrays");
    return nbody_adj_step(ws, spec, pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot, n, ptcl_num,
                          factors, omega_m, dots, disp_comp, vel_comp, stream);
}

// ---------------------------------------------------------------------------
// stage profiler
// ---------------------------------------------------------------------------

// Multi-step runs: nsteps consecutive steps in one call, joining the last
// particle pass of each step with the first of the next (k_gk_kds,
// k_sa_ka).  With windows or compensation the steps run one by one.
static int nbody_steps(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                       float *disp, float *vel, float *acc, int64_t n, int64_t ptcl_num,
                       int32_t nsteps, const float *factors, double omega_m, void *stream) {
    if (nsteps < 0 || (nsteps > 0 && !factors)) return fail(PMX_ERR_ARG, "bad nsteps/factors");
    if (nsteps == 0) return PMX_OK;
    Hot h;
    int st = check_hot(ws, spec, pmid, disp, n, ptcl_num, &h);
    if (st) return st;
    if (n > 0 && (!vel || !acc)) return fail(PMX_ERR_ARG, "null vel/acc");
    if (h.win || n == 0) {
        for (int32_t i = 0; i < nsteps; ++i)
            if ((st = nbody_step(ws, spec, pmid, disp, vel, acc, n, ptcl_num, factors + 3 * i,
                                 omega_m, nullptr, nullptr, stream)))
                return st;
        return PMX_OK;
    }
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    const int G = ptcl_grid(ws, n);
    {
        Stage sg(ws, 0, s, 1);
        k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
        PMX_LAUNCH_CHECK("k_fill");
    }
    {
        Stage sg(ws, 1, s, 1);
        if (h.agg)
            k_kds<true, false, false, true><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, n, factors[0],
                                                             factors[1], ws->dens);
        else
            k_kds<true, false, false><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, n, factors[0],
                                                         factors[1], ws->dens);
        PMX_LAUNCH_CHECK("k_kds");
    }
    for (int32_t i = 0; i < nsteps; ++i) {
        const float *f = factors + 3 * i;
        if ((st = force_meshes(ws, h, omega_m, s))) return st;
        if (i + 1 < nsteps) {
            {
                Stage sg(ws, 0, s, 1);
                k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
                PMX_LAUNCH_CHECK("k_fill");
            }
            Stage sg(ws, 13, s, 1);
            if (h.agg)
                k_gk_kds<true><<<G, PT, 0, s>>>(h, pmid, disp, vel, n, ws->g, f[2], f[3], f[4],
                                                ws->dens);
            else
                k_gk_kds<<<G, PT, 0, s>>>(h, pmid, disp, vel, n, ws->g, f[2], f[3], f[4], ws->dens);
            PMX_LAUNCH_CHECK("k_gk_kds");
        } else {
            Stage sg(ws, 5, s, 1);
            if (ws->tma)
                k_gather3_tma<true><<<G, PT, TMA_SMEM, s>>>(h, ws->tmap, pmid, disp, vel, acc, n,
                                                            ws->g, f[2], ws->err);
            else
                k_gather3<true, false><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, n, ws->M, ws->g,
                                                        f[2]);
            PMX_LAUNCH_CHECK("k_gather3");
        }
    }
    return PMX_OK;
}

static int nbody_adj_steps(pmx_workspace *ws, const pmx_enmesh_spec *spec, const int16_t *pmid,
                           float *disp, float *vel, float *acc, float *disp_cot, float *vel_cot,
                           float *acc_cot, int64_t n, int64_t ptcl_num, int32_t nsteps,
                           const float *factors, double omega_m, double *dots, void *stream) {
    if (nsteps < 0 || (nsteps > 0 && (!factors || !dots)))
        return fail(PMX_ERR_ARG, "bad nsteps/factors/dots");
    if (nsteps == 0) return PMX_OK;
    Hot h;
    int st = check_hot(ws, spec, pmid, disp, n, ptcl_num, &h);
    if (st) return st;
    if (!(ws->flags & PMX_WS_ADJOINT)) return fail(PMX_ERR_ARG, "workspace lacks PMX_WS_ADJOINT");
    if (n > 0 && (!vel || !acc || !disp_cot || !vel_cot || !acc_cot))
        return fail(PMX_ERR_ARG, "null particle array");
    if (h.win || n == 0) {
        for (int32_t i = 0; i < nsteps; ++i)
            if ((st = nbody_adj_step(ws, spec, pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot, n,
                                     ptcl_num, factors + 3 * i, omega_m, dots + 4 * i, nullptr,
                                     nullptr, stream)))
                return st;
        return PMX_OK;
    }
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    const int G = ptcl_grid(ws, n), G2 = ptcl_grid(ws, n, DOT2_PER_SM);
    int nb01 = G2;  // blocks of the kernel that last wrote dot slots 0 and 1
    {
        Stage sg(ws, 0, s, 2);
        k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
        k_fill<<<grid_fill(3 * ws->M), 256, 0, s>>>(ws->mcot, 0.f, 3 * ws->M);
        PMX_LAUNCH_CHECK("k_fill");
    }
    {
        Stage sg(ws, 6, s, 1);
        if (h.agg)
            k_ka<true, false, false, true><<<G2, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot,
                                                             vel_cot, acc_cot, n, factors[0],
                                                             factors[1], ws->dens, ws->part);
        else
            k_ka<true, false, false><<<G2, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot, vel_cot,
                                                         acc_cot, n, factors[0], factors[1],
                                                         ws->dens, ws->part);
        PMX_LAUNCH_CHECK("k_ka");
    }
    for (int32_t i = 0; i < nsteps; ++i) {
        const float *f = factors + 3 * i;
        if ((st = force_meshes(ws, h, omega_m, s))) return st;
        {
            Stage sg(ws, 7, s, 1);
            if (h.agg)
                k_g3adj<false, true><<<G, PT, 0, s>>>(h, pmid, disp, vel_cot, acc, acc_cot, n, ws->M,
                                                      ws->g, ws->mcot, ws->part);
            else
                k_g3adj<false><<<G, PT, 0, s>>>(h, pmid, disp, vel_cot, acc, acc_cot, n, ws->M,
                                                ws->g, ws->mcot, ws->part);
            PMX_LAUNCH_CHECK("k_g3adj");
        }
        {
            Stage sg(ws, 12, s, 1);
            k_finish<<<1, 1024, 0, s>>>(ws->part, ws->pstride, nb01, G, dots + 4 * i, 3,
                                        dots + 4 * i + 3,
                                        om_scale(omega_m));
            PMX_LAUNCH_CHECK("k_finish");
        }
        if ((st = force_adj_meshes(ws, omega_m, s))) return st;
        if (i + 1 < nsteps) {
            {
                Stage sg(ws, 0, s, 2);
                k_fill<<<grid_fill(ws->M), 256, 0, s>>>(ws->dens, -1.f, ws->M);
                k_fill<<<grid_fill(3 * ws->M), 256, 0, s>>>(ws->mcot, 0.f, 3 * ws->M);
                PMX_LAUNCH_CHECK("k_fill");
            }
            Stage sg(ws, 14, s, 1);
            if (h.agg)
                k_sa_ka<true><<<G2, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot, vel_cot,
                                                   acc_cot, n, ws->rcot_of(1), f[2], f[3], f[4],
                                                   ws->dens, ws->part);
            else
                k_sa_ka<<<G2, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot,
                                             n, ws->rcot_of(1), f[2], f[3], f[4], ws->dens,
                                             ws->part);
            PMX_LAUNCH_CHECK("k_sa_ka");
            nb01 = G2;
        } else {
            Stage sg(ws, 11, s, 1);
            k_sadj<true, false><<<G, PT, 0, s>>>(h, pmid, disp, vel, acc, disp_cot, acc_cot, n,
                                                 ws->rcot_of(1), f[2]);
            PMX_LAUNCH_CHECK("k_sadj");
        }
    }
    return PMX_OK;
}

extern "C" int pmx_nbody_steps(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                               const int16_t *pmid, float *disp, float *vel, float *acc,
                               int64_t n, int64_t ptcl_num, int32_t nsteps, const float *factors,
                               double omega_m, void *stream) {
    return nbody_steps(ws, spec, pmid, disp, vel, acc, n, ptcl_num, nsteps, factors, omega_m,
                       stream);
}

extern "C" int pmx_nbody_adj_steps(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                                   const int16_t *pmid, float *disp, float *vel, float *acc,
                                   float *disp_cot, float *vel_cot, float *acc_cot, int64_t n,
                                   int64_t ptcl_num, int32_t nsteps, const float *factors,
                                   double omega_m, double *dots, void *stream) {
    return nbody_adj_steps(ws, spec, pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot, n,
                           ptcl_num, nsteps, factors, omega_m, dots, stream);
}

// ---------------------------------------------------------------------------
// batched simulations (equal mesh shape and cell size, one slot each)
// ---------------------------------------------------------------------------

namespace {

struct BatchCall {
    Hot h;
    BatchTab tab;
    float c[BMAX];       // Green's constant per simulation
    FinishTab fin;
    int nb = 0;
    int G = 1;           // blocks per simulation
};

// Every host-side check of a batched call, before anything is launched.
int batch_prepare(pmx_workspace *ws, const pmx_enmesh_spec *spec, int32_t nsim,
                  const pmx_sim *sims, bool adjoint, int32_t nsteps, BatchCall *bc) {
    if (nsteps < 0) return fail(PMX_ERR_ARG, "negative nsteps");
    if (!ws) return fail(PMX_ERR_ARG, "null workspace");
    if (!sims || nsim < 1) return fail(PMX_ERR_ARG, "no simulations");
    if (nsim > ws->slots || nsim > BMAX)
        return fail(PMX_ERR_ARG, "more simulations than the workspace's slots");
    if (!ws->xfast) return fail(PMX_ERR_SHAPE, "batched calls need the fused x-pass path");
    if (ws->win) return fail(PMX_ERR_ARG, "batched calls use the plain deposits (no windows)");
    if (adjoint && !(ws->flags & PMX_WS_ADJOINT))
        return fail(PMX_ERR_ARG, "workspace lacks PMX_WS_ADJOINT");
    int st = check_hot(ws, spec, sims[0].pmid, sims[0].disp, sims[0].n, sims[0].ptcl_num, &bc->h);
    if (st) return st;
    bc->nb = nsim;
    int64_t nmax = 0;
    for (int b = 0; b < nsim; ++b) {
        const pmx_sim &q = sims[b];
        if (q.n < 0 || q.ptcl_num <= 0) return fail(PMX_ERR_ARG, "bad particle counts");
        if (q.n > 0 && (!q.pmid || !q.disp || !q.vel || !q.acc))
            return fail(PMX_ERR_ARG, "null particle array");
        if (adjoint && q.n > 0 && (!q.disp_cot || !q.vel_cot || !q.acc_cot))
            return fail(PMX_ERR_ARG, "null cotangent array");
        if (adjoint && !q.dots) return fail(PMX_ERR_ARG, "null dots");
        if (nsteps > 0 && !q.factors) return fail(PMX_ERR_ARG, "null factors");
        SimB &sb = bc->tab.s[b];
        sb.pmid = q.pmid;
        sb.disp = q.disp;
        sb.vel = q.vel;
        sb.acc = q.acc;
        sb.dcot = q.disp_cot;
        sb.vcot = q.vel_cot;
        sb.alpha = q.acc_cot;
        sb.n = q.n;
        sb.val = (float)((double)ws->M / (double)q.ptcl_num);
        bc->c[b] = green_c(ws, q.omega_m);
        bc->fin.dots[b] = q.dots;
        bc->fin.oms[b] = om_scale(q.omega_m);
        if (q.n > nmax) nmax = q.n;
    }
    bc->G = ptcl_grid(ws, nmax);
    return PMX_OK;
}

// Sets every simulation's launch factors f[0..2] from its factor table:
// f[j] = factors[3 i + off + j] for j < cnt (else 0).
int batch_factors(BatchCall *bc, const pmx_sim *sims, int i, int off, int cnt) {
    for (int b = 0; b < bc->nb; ++b) {
        for (int j = 0; j < 3; ++j)
            bc->tab.s[b].f[j] = j < cnt ? sims[b].factors[3 * i + off + j] : 0.f;
    }
    return PMX_OK;
}

}  // namespace

extern "C" int pmx_nbody_steps_batch(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                                     int32_t nsim, const pmx_sim *sims, int32_t init_force,
                                     int32_t nsteps, void *stream) {
    BatchCall bc;
    int st = batch_prepare(ws, spec, nsim, sims, false, nsteps, &bc);
    if (st) return st;
    if (!init_force && nsteps == 0) return PMX_OK;
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    const int64_t M = ws->M, nb = bc.nb;
    const dim3 grid(bc.G, bc.nb);
    auto fill_dens = [&]() -> int {
        Stage sg(ws, 0, s, 1);
        k_fill<<<grid_fill(nb * M), 256, 0, s>>>(ws->dens, -1.f, nb * M);
        PMX_LAUNCH_CHECK("k_fill");
        return PMX_OK;
    };
    if ((st = fill_dens())) return st;
    if (init_force) {   // acc = F(disp), as pmx_force
        {
            Stage sg(ws, 1, s, 1);
            if (bc.h.agg) k_kds_b<false, true><<<grid, PT, 0, s>>>(bc.h, bc.tab, ws->dens, M);
            else k_kds_b<false, false><<<grid, PT, 0, s>>>(bc.h, bc.tab, ws->dens, M);
            PMX_LAUNCH_CHECK("k_kds_b");
        }
        if ((st = force_meshes_b(ws, bc.nb, bc.c, s))) return st;
        {
            Stage sg(ws, 5, s, 1);
            k_gather3_b<false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g);
            PMX_LAUNCH_CHECK("k_gather3_b");
        }
        if (nsteps == 0) return PMX_OK;
        if ((st = fill_dens())) return st;
    }
    if ((st = batch_factors(&bc, sims, 0, 0, 2))) return st;
    {
        Stage sg(ws, 1, s, 1);
        if (bc.h.agg) k_kds_b<true, true><<<grid, PT, 0, s>>>(bc.h, bc.tab, ws->dens, M);
        else k_kds_b<true, false><<<grid, PT, 0, s>>>(bc.h, bc.tab, ws->dens, M);
        PMX_LAUNCH_CHECK("k_kds_b");
    }
    for (int32_t i = 0; i < nsteps; ++i) {
        if ((st = force_meshes_b(ws, bc.nb, bc.c, s))) return st;
        if (i + 1 < nsteps) {
            if ((st = fill_dens())) return st;
            if ((st = batch_factors(&bc, sims, i, 2, 3))) return st;   // K2_i, K1_i+1, D_i+1
            Stage sg(ws, 13, s, 1);
            if (bc.h.agg) k_gk_kds_b<true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g, ws->dens);
            else k_gk_kds_b<false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g, ws->dens);
            PMX_LAUNCH_CHECK("k_gk_kds_b");
        } else {
            if ((st = batch_factors(&bc, sims, i, 2, 1))) return st;   // K2_i
            Stage sg(ws, 5, s, 1);
            k_gather3_b<true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g);
            PMX_LAUNCH_CHECK("k_gather3_b");
        }
    }
    return PMX_OK;
}

extern "C" int pmx_nbody_adj_steps_batch(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                                         int32_t nsim, const pmx_sim *sims, int32_t init_vjp,
                                         int32_t nsteps, void *stream) {
    BatchCall bc;
    int st = batch_prepare(ws, spec, nsim, sims, true, nsteps, &bc);
    if (st) return st;
    if (!init_vjp && nsteps == 0) return PMX_OK;
    cudaStream_t s = as_stream(stream);
    if ((st = ensure_ktab(ws, spec->conf_cell_size, s))) return st;
    const int64_t M = ws->M, nb = bc.nb;
    const dim3 grid(bc.G, bc.nb);
    float *rcot = ws->rcot_of(bc.nb);
    auto fills = [&]() -> int {
        Stage sg(ws, 0, s, 2);
        k_fill<<<grid_fill(nb * M), 256, 0, s>>>(ws->dens, -1.f, nb * M);
        k_fill<<<grid_fill(3 * nb * M), 256, 0, s>>>(ws->mcot, 0.f, 3 * nb * M);
        PMX_LAUNCH_CHECK("k_fill");
        return PMX_OK;
    };
    auto finish = [&](int64_t row, int ndots) -> int {
        FinishTab ft = bc.fin;
        for (int b = 0; b < bc.nb; ++b) ft.dots[b] = bc.fin.dots[b] + 4 * row;
        Stage sg(ws, 12, s, 1);
        k_finish_b<<<bc.nb, 1024, 0, s>>>(ws->part, ws->pstride, bc.G, ft, ndots);
        PMX_LAUNCH_CHECK("k_finish_b");
        return PMX_OK;
    };
    if (init_vjp) {   // the force VJP of acc_cot = vel_cot, as pmx_force_vjp
        if ((st = fills())) return st;
        {
            Stage sg(ws, 1, s, 1);
            if (bc.h.agg) k_kds_b<false, true><<<grid, PT, 0, s>>>(bc.h, bc.tab, ws->dens, M);
            else k_kds_b<false, false><<<grid, PT, 0, s>>>(bc.h, bc.tab, ws->dens, M);
            PMX_LAUNCH_CHECK("k_kds_b");
        }
        if ((st = force_meshes_b(ws, bc.nb, bc.c, s))) return st;
        {
            Stage sg(ws, 7, s, 1);
            if (bc.h.agg) k_g3adj_b<true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g, ws->mcot, ws->part);
            else k_g3adj_b<false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g, ws->mcot, ws->part);
            PMX_LAUNCH_CHECK("k_g3adj_b");
        }
        if ((st = force_adj_meshes_b(ws, bc.nb, bc.c, s))) return st;
        {
            Stage sg(ws, 11, s, 1);
            k_sadj_b<false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, rcot);
            PMX_LAUNCH_CHECK("k_sadj_b");
        }
        if ((st = finish(nsteps, 0))) return st;
        if (nsteps == 0) return PMX_OK;
    }
    if ((st = fills())) return st;
    if ((st = batch_factors(&bc, sims, 0, 0, 2))) return st;
    {
        Stage sg(ws, 6, s, 1);
        if (bc.h.agg) k_ka_b<true, true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->dens, ws->part);
        else k_ka_b<true, false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->dens, ws->part);
        PMX_LAUNCH_CHECK("k_ka_b");
    }
    for (int32_t i = 0; i < nsteps; ++i) {
        if ((st = force_meshes_b(ws, bc.nb, bc.c, s))) return st;
        {
            Stage sg(ws, 7, s, 1);
            if (bc.h.agg) k_g3adj_b<true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g, ws->mcot, ws->part);
            else k_g3adj_b<false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, ws->g, ws->mcot, ws->part);
            PMX_LAUNCH_CHECK("k_g3adj_b");
        }
        if ((st = finish(i, 3))) return st;
        if ((st = force_adj_meshes_b(ws, bc.nb, bc.c, s))) return st;
        if (i + 1 < nsteps) {
            if ((st = fills())) return st;
            if ((st = batch_factors(&bc, sims, i, 2, 3))) return st;
            Stage sg(ws, 14, s, 1);
            if (bc.h.agg) k_sa_ka_b<true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, rcot, ws->dens, ws->part);
            else k_sa_ka_b<false><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, rcot, ws->dens, ws->part);
            PMX_LAUNCH_CHECK("k_sa_ka_b");
        } else {
            if ((st = batch_factors(&bc, sims, i, 2, 1))) return st;
            Stage sg(ws, 11, s, 1);
            k_sadj_b<true><<<grid, PT, 0, s>>>(bc.h, bc.tab, M, rcot);
            PMX_LAUNCH_CHECK("k_sadj_b");
        }
    }
    return PMX_OK;
}

extern "C" int pmx_workspace_tma_status(pmx_workspace *ws, int32_t *gave_up) {
    if (!ws || !gave_up) return fail(PMX_ERR_ARG, "null argument");
    *gave_up = 0;
    if (!ws->err) return PMX_OK;
    int v = 0;
    PMX_CUDA(cudaMemcpy(&v, ws->err, sizeof(int), cudaMemcpyDeviceToHost));
    *gave_up = v;
    return PMX_OK;
}

extern "C" int pmx_workspace_slots(const pmx_workspace *ws, int32_t *slots) {
    if (!ws || !slots) return fail(PMX_ERR_ARG, "null argument");
    *slots = ws->slots;
    return PMX_OK;
}

extern "C" int pmx_profile_enable(pmx_workspace *ws, int on) {
    if (!ws) return fail(PMX_ERR_ARG, "null workspace");
    ws->prof_on = on != 0;
    return PMX_OK;
}

extern "C" int pmx_profile_read(pmx_workspace *ws, double *ms, int64_t *calls, int64_t *launches) {
    if (!ws) return fail(PMX_ERR_ARG, "null workspace");
    double acc[PMX_PROF_STAGES] = {0};
    int64_t cnt[PMX_PROF_STAGES] = {0};
    int st = PMX_OK;
    for (auto &r : ws->recs) {
        float t = 0.f;
        cudaError_t e = cudaEventSynchronize(r.e);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.b, r.e);
        if (e != cudaSuccess && st == PMX_OK) st = cuda_status(e, "pmx_profile_read");
        acc[r.stage] += t;
        cnt[r.stage] += 1;
        ws->pool.push_back(r.b);
        ws->pool.push_back(r.e);
    }
    ws->recs.clear();
    for (int i = 0; i < PMX_PROF_STAGES; ++i) {
        if (ms) ms[i] = acc[i];
        if (calls) calls[i] = cnt[i];
    }
    if (launches) *launches = ws->launches;
    ws->launches = 0;
    return st;
}

extern "C" const char *pmx_profile_stage_name(int i) {
    if (i < 0 || i >= PMX_PROF_STAGES) return nullptr;
    return kStageNames[i];
}

// ---------------------------------------------------------------------------
// Dot product that allocates nothing
//
// Some callers cannot let a library call cudaMalloc: a JAX/XLA process that
// has preallocated most of the GPU for its own pool (pmwd's notebooks set
// XLA_PYTHON_CLIENT_MEM_FRACTION=.95), or a framework custom call that must
// not allocate outside the framework's allocator.  pmx_dot_noalloc serves
// them: its per-block partial sums live in the file-scope array below, which
// the module places in device memory when the library is loaded (64 KiB on
// every GPU that loads libpmx, held until the process exits).  Host code
// must not pass the array's name to a kernel -- on the host it is only a
// stand-in -- so the device address is looked up once per device with
// cudaGetSymbolAddress and passed as an argument.
// ---------------------------------------------------------------------------

namespace {

constexpr int64_t NOALLOC_CHUNK = int64_t(1) << 17;  // elements summed per block
constexpr int NOALLOC_BLOCKS = 8192;                 // partial sums the array holds

__device__ __align__(256) double g_noalloc_partials[NOALLOC_BLOCKS];

std::mutex g_noalloc_mu;
double *g_noalloc_addr[64] = {nullptr};

// Device address of g_noalloc_partials on the current device, looked up at
// the first call on that device (with that device current).
int noalloc_partials(double **out) {
    int dev = 0;
    PMX_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(PMX_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_partials)");
        g_noalloc_addr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_addr[dev];
    return PMX_OK;
}

// Block b sums x*y over elements [b*CHUNK, (b+1)*CHUNK) into part[b].
__global__ void __launch_bounds__(PT) k_dot_chunks(const float *__restrict__ x,
                                                   const float *__restrict__ y, int64_t n,
                                                   double *part) {
    __shared__ double sh[PT / 32];
    int64_t beg = (int64_t)blockIdx.x * NOALLOC_CHUNK;
    int64_t end = beg + NOALLOC_CHUNK < n ? beg + NOALLOC_CHUNK : n;
    double s = 0.0;
    for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) s += (double)x[i] * (double)y[i];
    double t = block_sum<PT>(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

}  // namespace

extern "C" int pmx_dot_noalloc(const float *x, const float *y, int64_t n, double *out,
                               void *stream) {
    if (n < 0 || !out) return fail(PMX_ERR_ARG, "pmx_dot_noalloc: bad arguments");
    if (n > NOALLOC_CHUNK * NOALLOC_BLOCKS)
        return fail(PMX_ERR_SHAPE, "pmx_dot_noalloc: n = " + std::to_string(n) +
                                       " exceeds its maximum of 2^30 elements (8192 static "
                                       "partial sums of 2^17 elements each); use pmx_dot");
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        PMX_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
        return PMX_OK;
    }
    if (!x || !y) return fail(PMX_ERR_ARG, "pmx_dot_noalloc: null x/y");
    double *part = nullptr;
    int st = noalloc_partials(&part);
    if (st) return st;
    int blocks = (int)((n + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK);
    // every block overwrites its own partial, so no clearing is needed
    k_dot_chunks<<<blocks, PT, 0, s>>>(x, y, n, part);
    PMX_LAUNCH_CHECK("k_dot_chunks");
    k_reduce1<<<1, 1024, 0, s>>>(part, blocks, out);
    PMX_LAUNCH_CHECK("k_reduce1");
    return PMX_OK;
}
