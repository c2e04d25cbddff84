// Generic CIC mesh operators: enmesh, scatter, gather and their VJPs.
//
// These back the general pmwd signatures (any dim 1..3, channels, offset,
// non-default cell size): pmwd/scatter.py:8-150, pmwd/gather.py:8-144,
// pmwd/particles.py:212-254.  The Poisson-force hot path uses the fused,
// specialised kernels in pmx_force.cu.
//
// One thread per particle, grid-stride.  Scatter-type updates use float32
// global reductions (red.global.add.f32 through atomicAdd with the result
// unused), like the reference's XLA scatter-add.

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "pmx_internal.cuh"

namespace pmx {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }
void clear_error() { g_err.clear(); }
int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}
int cuda_status(cudaError_t e, const char *what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return PMX_ERR_CUDA;
}

int device_sms() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = 152;
        cached[dev] = v;
    }
    return cached[dev];
}

// jnp.divmod(b12, a1) for floats, done once on the host (pm_util.py:120).
static void host_float_divmod(double x, double y, double *div, double *mod) {
    double m = std::fmod(x, y);
    double d = (x - m) / y;
    if (m != 0.0 && ((y < 0.0) != (m < 0.0))) {
        m += y;
        d -= 1.0;
    }
    *div = std::round(d);  // half away from zero, like lax.round
    *mod = m;
}

int make_em_params(const pmx_enmesh_spec *s, EmParams *p) {
    if (!s) return fail(PMX_ERR_ARG, "null enmesh spec");
    if (s->dim < 1 || s->dim > 3) return fail(PMX_ERR_ARG, "dim must be 1, 2 or 3");
    if (!(s->conf_cell_size > 0)) return fail(PMX_ERR_ARG, "conf_cell_size must be > 0");
    p->dim = s->dim;
    p->pad = 3 - s->dim;
    // all wrap_shape entries 0: no periodic wrapping (s1 = None)
    bool nowrap = true;
    for (int u = 0; u < s->dim; ++u) nowrap = nowrap && s->wrap_shape[u] == 0;
    p->drop = nowrap && s->drop;
    for (int a = 0; a < 3; ++a) {
        int u = a - p->pad;
        if (u < 0) {
            p->wrap[a] = 1;
            p->shape[a] = 1;
        } else if (nowrap) {
            if (s->mesh_shape[u] <= 0) return fail(PMX_ERR_ARG, "mesh_shape must be > 0");
            p->wrap[a] = 0;
            p->shape[a] = s->mesh_shape[u];
        } else {
            if (s->wrap_shape[u] <= 0) return fail(PMX_ERR_ARG, "wrap_shape must be > 0 (or all 0)");
            if (s->mesh_shape[u] <= 0) return fail(PMX_ERR_ARG, "mesh_shape must be > 0");
            p->wrap[a] = s->wrap_shape[u];
            p->shape[a] = s->mesh_shape[u];
        }
    }
    p->stride[2] = 1;
    p->stride[1] = p->shape[2];
    p->stride[0] = p->shape[1] * p->shape[2];
    p->f64 = s->cell_size > 0 ? 1 : 0;
    p->cellf = (float)s->conf_cell_size;
    p->a1d = s->conf_cell_size;
    p->a2d = s->cell_size > 0 ? s->cell_size : s->conf_cell_size;
    p->a2f = (float)p->a2d;
    for (int a = 0; a < 3; ++a) {
        int u = a - p->pad;
        double off = u >= 0 ? s->offset[u] : 0.0;
        double div, mod;
        host_float_divmod(off, (double)p->cellf, &div, &mod);
        p->i12[a] = (int)(int16_t)(int64_t)div;
        p->d12[a] = (float)mod;
        p->b12[a] = off;
        p->L[a] = (double)p->wrap[a] * p->a1d;
    }
    p->cot_div = (float)(s->cell_size > 0 ? s->cell_size : s->conf_cell_size);
    return PMX_OK;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

__global__ void k_enmesh(EmParams p, const int16_t *__restrict__ pmid,
                         const float *__restrict__ disp, int64_t n, int32_t *ind,
                         float *frac, float *frac_grad) {
    const int nk = 1 << p.dim;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        int pm[3];
        float dd[3];
        load_particle(p, pmid, disp, q, pm, dd);
        Axis ax[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) enmesh_axis(p, a, pm[a], dd[a], ax[a]);
        for (int ku = 0; ku < nk; ++ku) {
            int k = ku << p.pad;  // user neighbour bits -> internal bits
            frac[q * nk + ku] = frac_of(ax, k);
            if (ind) {
                for (int u = 0; u < p.dim; ++u) {
                    int a = u + p.pad;
                    ind[(q * nk + ku) * p.dim + u] = ax[a].i[(k >> a) & 1];
                }
            }
            if (frac_grad) {
                float g[3];
                frac_grad_of(ax, k, g);
                for (int u = 0; u < p.dim; ++u)
                    frac_grad[(q * nk + ku) * p.dim + u] = g[u + p.pad];
            }
        }
    }
}

__global__ void k_scatter(EmParams p, const int16_t *__restrict__ pmid,
                          const float *__restrict__ disp, int64_t n,
                          const float *__restrict__ val, float val_scalar, int64_t chan,
                          float *mesh) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        int pm[3];
        float dd[3];
        load_particle(p, pmid, disp, q, pm, dd);
        Axis ax[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) enmesh_axis(p, a, pm[a], dd[a], ax[a]);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t cell = cell_of(p, ax, k);
            if (cell < 0) continue;
            float f = frac_of(ax, k);
            if (val) {
                for (int64_t c = 0; c < chan; ++c)
                    atomicAdd(mesh + cell * chan + c, __fmul_rn(val[q * chan + c], f));
            } else {
                atomicAdd(mesh + cell, __fmul_rn(val_scalar, f));
            }
        }
    }
}

__global__ void k_scatter_adj(EmParams p, const int16_t *__restrict__ pmid,
                              const float *__restrict__ disp, int64_t n,
                              const float *__restrict__ val, float val_scalar, int64_t chan,
                              const float *__restrict__ mesh_cot, float *disp_cot,
                              float *val_cot) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        int pm[3];
        float dd[3];
        load_particle(p, pmid, disp, q, pm, dd);
        Axis ax[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) enmesh_axis(p, a, pm[a], dd[a], ax[a]);
        float dc[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 8; ++k) {
            int64_t cell = cell_of(p, ax, k);
            float g[3];
            frac_grad_of(ax, k, g);
            float f = frac_of(ax, k);
            float s = 0.f;
            for (int64_t c = 0; c < chan; ++c) {
                float m = cell >= 0 ? mesh_cot[cell * chan + c] : 0.f;
                float v = val ? val[q * chan + c] : val_scalar;
                s = __fadd_rn(s, __fmul_rn(m, v));
                if (val_cot) {
                    float *o = val_cot + q * chan + c;
                    float prev = k == 0 ? 0.f : *o;
                    *o = __fadd_rn(prev, __fmul_rn(m, f));
                }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) dc[a] = __fadd_rn(dc[a], __fmul_rn(s, g[a]));
        }
        for (int u = 0; u < p.dim; ++u)
            disp_cot[q * p.dim + u] = __fdiv_rn(dc[u + p.pad], p.cot_div);
    }
}

__global__ void k_gather(EmParams p, const int16_t *__restrict__ pmid,
                         const float *__restrict__ disp, int64_t n,
                         const float *__restrict__ mesh, int64_t chan,
                         const float *__restrict__ val, float val_scalar, float *out) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        int pm[3];
        float dd[3];
        load_particle(p, pmid, disp, q, pm, dd);
        Axis ax[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) enmesh_axis(p, a, pm[a], dd[a], ax[a]);
        int64_t cells[8];
        float fr[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cells[k] = cell_of(p, ax, k);
            fr[k] = frac_of(ax, k);
        }
        for (int64_t c = 0; c < chan; ++c) {
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                float m = cells[k] >= 0 ? mesh[cells[k] * chan + c] : 0.f;
                s = __fadd_rn(s, __fmul_rn(m, fr[k]));
            }
            float v = val ? val[q * chan + c] : val_scalar;
            out[q * chan + c] = __fadd_rn(v, s);
        }
    }
}

__global__ void k_gather_adj(EmParams p, const int16_t *__restrict__ pmid,
                             const float *__restrict__ disp, int64_t n,
                             const float *__restrict__ mesh, int64_t chan,
                             const float *__restrict__ val_cot, float *disp_cot,
                             float *mesh_cot) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        int pm[3];
        float dd[3];
        load_particle(p, pmid, disp, q, pm, dd);
        Axis ax[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) enmesh_axis(p, a, pm[a], dd[a], ax[a]);
        float dc[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 8; ++k) {
            int64_t cell = cell_of(p, ax, k);
            float g[3];
            frac_grad_of(ax, k, g);
            float f = frac_of(ax, k);
            float s = 0.f;
            for (int64_t c = 0; c < chan; ++c) {
                float vc = val_cot[q * chan + c];
                float m = cell >= 0 ? mesh[cell * chan + c] : 0.f;
                s = __fadd_rn(s, __fmul_rn(vc, m));
                if (cell >= 0) atomicAdd(mesh_cot + cell * chan + c, __fmul_rn(vc, f));
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) dc[a] = __fadd_rn(dc[a], __fmul_rn(s, g[a]));
        }
        for (int u = 0; u < p.dim; ++u)
            disp_cot[q * p.dim + u] = __fdiv_rn(dc[u + p.pad], p.cot_div);
    }
}

}  // namespace pmx

using namespace pmx;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" int pmx_version(void) { return 200; }

extern "C" const char *pmx_last_error(void) { return g_err.c_str(); }

extern "C" int pmx_device_sms(int *sms) {
    if (!sms) return fail(PMX_ERR_ARG, "null sms");
    *sms = device_sms();
    return PMX_OK;
}

extern "C" int pmx_stream_create(int device, void **stream) {
    if (!stream) return fail(PMX_ERR_ARG, "null stream");
    *stream = nullptr;
    int prev = 0;
    PMX_CUDA(cudaGetDevice(&prev));
    PMX_CUDA(cudaSetDevice(device));
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamCreateWithFlags");
    *stream = reinterpret_cast<void *>(s);
    return PMX_OK;
}

extern "C" int pmx_stream_destroy(void *stream) {
    if (!stream) return PMX_OK;
    PMX_CUDA(cudaStreamDestroy(reinterpret_cast<cudaStream_t>(stream)));
    return PMX_OK;
}

static int check_common(const pmx_enmesh_spec *spec, const void *pmid, const void *disp,
                        int64_t n, EmParams *p) {
    int st = make_em_params(spec, p);
    if (st) return st;
    if (n < 0) return fail(PMX_ERR_ARG, "negative particle count");
    if (n > 0 && (!pmid || !disp)) return fail(PMX_ERR_ARG, "null pmid/disp");
    return PMX_OK;
}

extern "C" int pmx_enmesh(const pmx_enmesh_spec *spec, const int16_t *pmid, const float *disp,
                          int64_t n, int32_t *ind, float *frac, float *frac_grad, void *stream) {
    EmParams p;
    int st = check_common(spec, pmid, disp, n, &p);
    if (st) return st;
    if (n == 0) return PMX_OK;
    if (!frac) return fail(PMX_ERR_ARG, "null frac");
    const int T = 256;
    k_enmesh<<<stride_grid(n, T), T, 0, as_stream(stream)>>>(p, pmid, disp, n, ind, frac, frac_grad);
    PMX_LAUNCH_CHECK("k_enmesh");
    return PMX_OK;
}

extern "C" int pmx_scatter(const pmx_enmesh_spec *spec, const int16_t *pmid, const float *disp,
                           int64_t n, const float *val, float val_scalar, int64_t channels,
                           float *mesh, void *stream) {
    EmParams p;
    int st = check_common(spec, pmid, disp, n, &p);
    if (st) return st;
    if (channels < 1) return fail(PMX_ERR_ARG, "channels must be >= 1");
    if (!val && channels != 1) return fail(PMX_ERR_SHAPE, "scalar val needs channels == 1");
    if (!mesh) return fail(PMX_ERR_ARG, "null mesh");
    if (n == 0) return PMX_OK;
    const int T = 256;
    k_scatter<<<stride_grid(n, T), T, 0, as_stream(stream)>>>(p, pmid, disp, n, val, val_scalar,
                                                              channels, mesh);
    PMX_LAUNCH_CHECK("k_scatter");
    return PMX_OK;
}

extern "C" int pmx_scatter_adj(const pmx_enmesh_spec *spec, const int16_t *pmid,
                               const float *disp, int64_t n, const float *val, float val_scalar,
                               int64_t channels, const float *mesh_cot, float *disp_cot,
                               float *val_cot, void *stream) {
    EmParams p;
    int st = check_common(spec, pmid, disp, n, &p);
    if (st) return st;
    if (channels < 1) return fail(PMX_ERR_ARG, "channels must be >= 1");
    if (!val && channels != 1) return fail(PMX_ERR_SHAPE, "scalar val needs channels == 1");
    if (!mesh_cot || (n > 0 && !disp_cot)) return fail(PMX_ERR_ARG, "null mesh_cot/disp_cot");
    if (n == 0) return PMX_OK;
    const int T = 256;
    k_scatter_adj<<<stride_grid(n, T), T, 0, as_stream(stream)>>>(
        p, pmid, disp, n, val, val_scalar, channels, mesh_cot, disp_cot, val_cot);
    PMX_LAUNCH_CHECK("k_scatter_adj");
    return PMX_OK;
}

extern "C" int pmx_gather(const pmx_enmesh_spec *spec, const int16_t *pmid, const float *disp,
                          int64_t n, const float *mesh, int64_t channels, const float *val,
                          float val_scalar, float *out, void *stream) {
    EmParams p;
    int st = check_common(spec, pmid, disp, n, &p);
    if (st) return st;
    if (channels < 1) return fail(PMX_ERR_ARG, "channels must be >= 1");
    if (!mesh || (n > 0 && !out)) return fail(PMX_ERR_ARG, "null mesh/out");
    if (n == 0) return PMX_OK;
    const int T = 256;
    k_gather<<<stride_grid(n, T), T, 0, as_stream(stream)>>>(p, pmid, disp, n, mesh, channels,
                                                             val, val_scalar, out);
    PMX_LAUNCH_CHECK("k_gather");
    return PMX_OK;
}

extern "C" int pmx_gather_adj(const pmx_enmesh_spec *spec, const int16_t *pmid,
                              const float *disp, int64_t n, const float *mesh, int64_t channels,
                              const float *val_cot, float *disp_cot, float *mesh_cot,
                              void *stream) {
    EmParams p;
    int st = check_common(spec, pmid, disp, n, &p);
    if (st) return st;
    if (channels < 1) return fail(PMX_ERR_ARG, "channels must be >= 1");
    if (!mesh || !mesh_cot || (n > 0 && (!val_cot || !disp_cot)))
        return fail(PMX_ERR_ARG, "null mesh/mesh_cot/val_cot/disp_cot");
    if (n == 0) return PMX_OK;
    const int T = 256;
    k_gather_adj<<<stride_grid(n, T), T, 0, as_stream(stream)>>>(
        p, pmid, disp, n, mesh, channels, val_cot, disp_cot, mesh_cot);
    PMX_LAUNCH_CHECK("k_gather_adj");
    return PMX_OK;
}
