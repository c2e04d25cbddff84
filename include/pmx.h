/*
 * pmx.h -- C ABI of the GB300 particle-mesh library (libpmx.so).
 *
 * Replaces the compute underneath pmwd's Python operators; each entry point
 * names the reference function (path:line inside the pmwd project) whose
 * behaviour it reproduces.  Conventions:
 *
 *  - All array arguments are caller-owned DEVICE pointers, row-major:
 *    pmid int16 (n, dim), disp/vel/acc/cotangents float32 (n, dim),
 *    meshes float32 (mesh_shape..., channels).
 *  - Every call is asynchronous on the given CUDA stream (cudaStream_t passed
 *    as void*; NULL = legacy default stream) and never synchronises the host.
 *  - Every call returns PMX_OK (0) or a negative status; pmx_last_error()
 *    returns a thread-local message describing the last failure.
 *  - No C++ exception crosses this boundary.  Re-entrant: calls on different
 *    workspaces / streams may run concurrently.
 */
#ifndef PMX_H
#define PMX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMX_OK          0
#define PMX_ERR_ARG    -1   /* bad argument value or null pointer          */
#define PMX_ERR_SHAPE  -2   /* inconsistent shapes                         */
#define PMX_ERR_ALIGN  -3   /* pointer alignment requirement violated      */
#define PMX_ERR_CUDA   -4   /* CUDA runtime error                          */
#define PMX_ERR_CUFFT  -5   /* cuFFT error                                 */
#define PMX_ERR_NOMEM  -6   /* device allocation failed                    */

/* Geometry of one enmesh (pm_util.py:33-156 ``enmesh``) as scatter/gather
 * call it: grid 1 is the particle grid of conf (cell size a1 =
 * conf.cell_size, periodic shape s1 = conf.mesh_shape); grid 2 is the target
 * mesh with spatial shape mesh_shape, origin offset b12 and cell size a2
 * (cell_size <= 0 means the reference's ``cell_size=None``).  All
 * wrap_shape entries 0 means s1 = None (no periodic wrapping,
 * particles.py:212-254 with wrap=False); then `drop` != 0 replaces negative
 * indices by mesh_shape, as the reference does with s2 given. */
typedef struct pmx_enmesh_spec {
    int32_t dim;             /* spatial dimension, 1..3                    */
    int32_t wrap_shape[3];   /* conf.mesh_shape (s1), first `dim` used;
                                all 0: no wrapping                         */
    int64_t mesh_shape[3];   /* spatial shape of the mesh array (s2)       */
    double  conf_cell_size;  /* conf.cell_size (a1)                        */
    double  offset[3];       /* offset of mesh to particle grid (b12)      */
    double  cell_size;       /* mesh cell size a2, <= 0 for None           */
    int32_t drop;            /* without wrapping: negative indices -> s2   */
} pmx_enmesh_spec;

/* Library version (major*10000 + minor*100 + patch). */
int pmx_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char *pmx_last_error(void);

/* Number of SMs of the current device, used to size persistent grids. */
int pmx_device_sms(int *sms);

/* A non-blocking CUDA stream of the library's own on `device`, and its
 * release.  No counterpart in the reference (JAX owns its streams).  For
 * host code whose stream API hands out streams from a fixed pool --
 * torch.cuda.Stream() draws from 32 per device -- and that captures CUDA
 * graphs from several threads: a capture on a pooled stream would also
 * record the work another thread launches on that same stream. */
int pmx_stream_create(int device, void **stream);
int pmx_stream_destroy(void *stream);

/* --------------------------------------------------------------------------
 * Mesh operators
 * ------------------------------------------------------------------------ */

/* Multilinear indices, fractions and fraction gradients of every particle,
 * pmwd/particles.py:212-254 ``ptcl_enmesh`` -> pm_util.py:33-156.
 * ind (n, 2^dim, dim) int32, frac (n, 2^dim), frac_grad (n, 2^dim, dim);
 * ind and frac_grad may be NULL.  Indices are bit-exact with the reference's
 * int16 indices: wrapped by s1, or without wrapping the int16 sums, negative
 * ones replaced by s2 when spec->drop is set. */
int pmx_enmesh(const pmx_enmesh_spec *spec, const int16_t *pmid,
               const float *disp, int64_t n, int32_t *ind, float *frac,
               float *frac_grad, void *stream);

/* mesh[i_k, c] += val[p, c] * frac_k for the 2^dim neighbours of each
 * particle, out-of-range neighbours dropped; pmwd/scatter.py:8-83.
 * val == NULL uses val_scalar for every particle (channels must be 1).
 * mesh is accumulated in place (the caller zeroes it for a fresh scatter). */
int pmx_scatter(const pmx_enmesh_spec *spec, const int16_t *pmid,
                const float *disp, int64_t n, const float *val,
                float val_scalar, int64_t channels, float *mesh, void *stream);

/* Scatter VJP, pmwd/scatter.py:86-148 (``_scatter_chunk_adj``):
 * disp_cot (n, dim) = sum_k (mesh_cot[i_k] . val) dfrac_k / cell  (overwritten),
 * val_cot  (n, channels) = sum_k mesh_cot[i_k] frac_k  (overwritten, may be NULL).
 * The mesh cotangent passes through unchanged (the caller keeps it). */
int pmx_scatter_adj(const pmx_enmesh_spec *spec, const int16_t *pmid,
                    const float *disp, int64_t n, const float *val,
                    float val_scalar, int64_t channels, const float *mesh_cot,
                    float *disp_cot, float *val_cot, void *stream);

/* out[p, c] = val[p, c] + sum_k mesh[i_k, c] frac_k, out-of-range neighbours
 * read as 0; pmwd/gather.py:8-77.  val == NULL uses val_scalar. */
int pmx_gather(const pmx_enmesh_spec *spec, const int16_t *pmid,
               const float *disp, int64_t n, const float *mesh,
               int64_t channels, const float *val, float val_scalar,
               float *out, void *stream);

/* Gather VJP, pmwd/gather.py:80-144 (``_gather_chunk_adj``):
 * disp_cot (n, dim) = sum_k (val_cot . mesh[i_k]) dfrac_k / cell (overwritten),
 * mesh_cot[i_k, c] += val_cot[p, c] frac_k (accumulated; caller zeroes it).
 * The value cotangent passes through unchanged. */
int pmx_gather_adj(const pmx_enmesh_spec *spec, const int16_t *pmid,
                   const float *disp, int64_t n, const float *mesh,
                   int64_t channels, const float *val_cot, float *disp_cot,
                   float *mesh_cot, void *stream);

/* --------------------------------------------------------------------------
 * Poisson force (pmwd/gravity.py:47-72) on a persistent workspace
 * ------------------------------------------------------------------------ */

typedef struct pmx_workspace pmx_workspace;

#define PMX_WS_ADJOINT 1   /* also allocate buffers for the force VJP */
#define PMX_WS_CUFFT3D 2   /* use 3-D cuFFT plans even where the fused x pass
                              applies (n0 a power of two in 64..1024);
                              for comparisons and tests */
#define PMX_WS_WINDOW 4    /* deposit through per-warp shared-memory windows
                              flushed with 16-byte vector reductions instead
                              of one global atomic per contribution (opt-in:
                              slower for lattice-ordered particles on GB300) */
#define PMX_WS_PLANE 8     /* with the fused x pass, do the (y, z) plane
                              transforms with the cluster plane kernels
                              instead of slab-wise 2-D cuFFT (square
                              power-of-two planes 64..1024) */
#define PMX_WS_VEC 16      /* deposit z-neighbour pairs that share an aligned
                              group of four floats with one 16-byte vector
                              reduction (n2 % 4 == 0; opt-in: slower on
                              GB300) */
#define PMX_WS_NO_GRAPH 32 /* issue the slab loops of the plane transforms
                              directly instead of replaying captured graphs */
#define PMX_WS_PLANE16 64  /* plane kernels in clusters of 16 CTAs (the
                              non-portable size) instead of 8 */
#define PMX_WS_AGG 128     /* warp-aggregated deposits: lanes whose particles
                              share a cell sum their contributions in shared
                              memory and one lane issues the reductions
                              (helps clustered late-time states) */
#define PMX_WS_TMA 65536   /* forward gathers stage each warp's box of the
                              acceleration meshes in shared memory with one
                              cp.async.bulk.tensor copy (fused x-pass path,
                              n2 % 4 == 0, single-simulation workspaces;
                              opt-in: slower than the global-load gathers on
                              GB300) */
/* Slab-wise plane transforms: number of concurrent chains (1..4; 0 = the
 * default 2) in bits 8..10 and log2 of the x-planes per cuFFT execution
 * (1..15; 0 = the default, the smallest power of two >= 8 reaching 32 MB) in
 * bits 12..15 of the flags.  Results do not depend on either. */
#define PMX_WS_CHAINS_SHIFT 8
#define PMX_WS_SLAB_SHIFT 12
#define PMX_WS_CHAINS(k) (((k) & 7) << PMX_WS_CHAINS_SHIFT)
#define PMX_WS_SLAB_LOG2(s) (((s) & 15) << PMX_WS_SLAB_SHIFT)

/* Device bytes a workspace for this 3-D mesh allocates (meshes, spectra,
 * cuFFT work areas, reduction scratch). */
int pmx_workspace_bytes(const int64_t mesh_shape[3], int32_t flags,
                        size_t *bytes);

/* Creates the workspace on the current device: mesh and spectrum buffers,
 * cuFFT plans (r2c, batched c2r, and for PMX_WS_ADJOINT batched r2c and
 * c2r) with caller-visible work areas.  This is the only call that
 * allocates device memory. */
int pmx_workspace_create(const int64_t mesh_shape[3], int32_t flags,
                         pmx_workspace **ws);
int pmx_workspace_destroy(pmx_workspace *ws);

/* Particle accelerations acc (n, 3), pmwd/gravity.py:47-72: CIC density of
 * mean 1 (val = mesh_size/ptcl_num), overdensity times 1.5*Omega_m, r2c,
 * -1/k^2 (k=0 -> 0), -i k per axis with the Nyquist plane zeroed, c2r with
 * 1/N, CIC gather.  No CIC deconvolution (pmwd applies none).  The spec
 * must be the default enmesh (offset 0, cell_size None), dim 3, and its
 * mesh_shape equal to the workspace's. */
int pmx_force(pmx_workspace *ws, const pmx_enmesh_spec *spec,
              const int16_t *pmid, const float *disp, int64_t n,
              int64_t ptcl_num, double omega_m, float *acc, void *stream);

/* Forward force plus its VJP against acc_cot (n, 3): the
 * ``vjp(gravity, ...)`` of pmwd/nbody.py:108-118.  Writes acc (n, 3),
 * disp_cot (n, 3) and, if omega_m_cot != NULL, the Omega_m cotangent as one
 * double in DEVICE memory.  Needs a PMX_WS_ADJOINT workspace. */
int pmx_force_vjp(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                  const int16_t *pmid, const float *disp, int64_t n,
                  int64_t ptcl_num, double omega_m, const float *acc_cot,
                  float *acc, float *disp_cot, double *omega_m_cot,
                  void *stream);

/* --------------------------------------------------------------------------
 * Leapfrog (pmwd/nbody.py) -- all factors are the float32 casts of the
 * float64 time-step factors the host computes.
 * ------------------------------------------------------------------------ */

/* vel += acc * factor over n3 = 3*n floats, nbody.py:70-77 ``kick``. */
int pmx_kick(float *vel, const float *acc, int64_t n3, float factor,
             void *stream);

/* disp += vel * factor, nbody.py:39-46 ``drift``. */
int pmx_drift(float *disp, const float *vel, int64_t n3, float factor,
              void *stream);

/* nbody.py:80-99 ``kick_adj``: vel += acc*K; disp_cot -= acc_cot*K;
 * dot = sum(vel_cot * acc) written as one double to DEVICE memory (may be
 * NULL).  The sum is deterministic (fixed two-level order). */
int pmx_kick_adj(float *vel, const float *acc, float *disp_cot,
                 const float *acc_cot, const float *vel_cot, int64_t n3,
                 float factor, double *dot, void *stream);

/* nbody.py:49-67 ``drift_adj``: disp += vel*D; vel_cot -= disp_cot*D;
 * dot = sum(disp_cot * vel) (DEVICE double, may be NULL). */
int pmx_drift_adj(float *disp, const float *vel, float *vel_cot,
                  const float *disp_cot, int64_t n3, float factor,
                  double *dot, void *stream);

/* Deterministic float64-accumulated dot product of two float32 arrays;
 * the ``(x * y).sum()`` reductions of nbody.py:67,97. */
int pmx_dot(const float *x, const float *y, int64_t n, double *out,
            void *stream);

/* pmx_dot for callers that cannot let a library allocate device memory
 * (e.g. a JAX process that preallocated most of the GPU, or a framework
 * custom call that must not allocate outside its own allocator).  It has no
 * counterpart in pmwd.  Same result as pmx_dot up to summation order; it
 * calls no cudaMalloc/cudaFree: its partial sums live in a static 64 KiB
 * device array that every GPU loading libpmx holds until the process
 * exits.  n is limited to 2^30 elements (larger n returns PMX_ERR_SHAPE).
 * The first call on a device looks the array up (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  All calls on a device
 * share the one array: calls that overlap on the GPU (e.g. on two streams)
 * race and give wrong sums. */
int pmx_dot_noalloc(const float *x, const float *y, int64_t n, double *out,
                    void *stream);

/* One forward step K(1/2) D F K(1/2) of nbody.py:121-140 (``integrate``
 * with the default symp_splits), fused: factors = {K1, D, K2}. */
int pmx_nbody_step(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                   const int16_t *pmid, float *disp, float *vel, float *acc,
                   int64_t n, int64_t ptcl_num, const float factors[3],
                   double omega_m, void *stream);

/* One reverse step of nbody.py:143-162 (``integrate_adj``): kick_adj(K1),
 * drift_adj(D), force_adj, kick_adj(K2), fused.  acc_cot is pmwd's alpha
 * (``ptcl_cot.acc``).  dots (DEVICE, 4 doubles) receives
 * {sum(vel_cot*acc) at K1, sum(disp_cot*vel) at D, sum(vel_cot*acc_new) at
 * the force and K2, Omega_m cotangent of the new force}. */
int pmx_nbody_adj_step(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                       const int16_t *pmid, float *disp, float *vel,
                       float *acc, float *disp_cot, float *vel_cot,
                       float *acc_cot, int64_t n, int64_t ptcl_num,
                       const float factors[3], double omega_m, double *dots,
                       void *stream);

/* pmx_nbody_step / pmx_nbody_adj_step with Kahan-compensated float32 updates
 * of disp and vel: disp_comp and vel_comp (n, 3) carry the running
 * compensation terms across steps (zero them at the start of a run).  pmwd
 * has no counterpart (its updates are plain float32, nbody.py:44,75); this
 * keeps the rounding of the position/velocity sums from accumulating so the
 * reverse-time reconstruction of the adjoint returns closer to the initial
 * state. */
int pmx_nbody_step_kahan(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                         const int16_t *pmid, float *disp, float *vel, float *acc,
                         float *disp_comp, float *vel_comp, int64_t n,
                         int64_t ptcl_num, const float factors[3], double omega_m,
                         void *stream);
int pmx_nbody_adj_step_kahan(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                             const int16_t *pmid, float *disp, float *vel, float *acc,
                             float *disp_cot, float *vel_cot, float *acc_cot,
                             float *disp_comp, float *vel_comp, int64_t n,
                             int64_t ptcl_num, const float factors[3],
                             double omega_m, double *dots, void *stream);

/* nsteps consecutive forward steps (pmwd/nbody.py:193-223, default splits)
 * in one call; factors (nsteps, 3) as pmx_nbody_step, host memory.  The
 * gather + kick of step i and the kick + drift + deposit of step i+1 run as
 * one particle pass with the same float32 updates in the same order, so the
 * result equals nsteps calls of pmx_nbody_step up to the order of atomic
 * adds. */
int pmx_nbody_steps(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                    const int16_t *pmid, float *disp, float *vel, float *acc,
                    int64_t n, int64_t ptcl_num, int32_t nsteps,
                    const float *factors, double omega_m, void *stream);

/* nsteps consecutive reverse steps with the adjoint (pmwd/nbody.py:226-260)
 * in one call; factors (nsteps, 3) as pmx_nbody_adj_step, host memory; dots
 * (nsteps, 4) in DEVICE memory, row i as the dots of pmx_nbody_adj_step for
 * step i.  The scatter VJP + kick_adj of step i and the kick_adj + drift_adj
 * + deposit of step i+1 run as one particle pass. */
int pmx_nbody_adj_steps(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                        const int16_t *pmid, float *disp, float *vel,
                        float *acc, float *disp_cot, float *vel_cot,
                        float *acc_cot, int64_t n, int64_t ptcl_num,
                        int32_t nsteps, const float *factors, double omega_m,
                        double *dots, void *stream);

/* --------------------------------------------------------------------------
 * Batched simulations: several independent runs that share a mesh shape and
 * cell size advance in one call (pmwd runs one simulation per call,
 * nbody.py:215-276; this is the serving form).  Each simulation occupies one
 * slot of a batched workspace: every particle kernel launch serves all of
 * them (one block row per simulation), and each plane transform runs over
 * all their planes at once.  A simulation's arithmetic is the one of the
 * single-simulation entry points, so its result is the same alone and in a
 * batch up to the order of float32 atomic adds.
 * ------------------------------------------------------------------------ */

/* One simulation of a batched call.  Particle and cotangent arrays are
 * DEVICE memory (n, 3); factors is HOST memory, (nsteps, 3) as for
 * pmx_nbody_steps / pmx_nbody_adj_steps; dots is DEVICE memory, (nsteps + 1,
 * 4), used by the adjoint call only. */
typedef struct pmx_sim {
    const int16_t *pmid;
    float *disp, *vel, *acc;
    float *disp_cot, *vel_cot, *acc_cot;
    int64_t n, ptcl_num;
    double omega_m;
    const float *factors;
    double *dots;
} pmx_sim;

/* A workspace whose buffers hold `slots` simulations (1..16) of the same
 * mesh shape; pmx_workspace_create is the case slots = 1.  Batched calls
 * need the fused x-pass path (n0 a power of two in 64..1024) and the plain
 * deposits (no PMX_WS_WINDOW). */
int pmx_workspace_create_batch(const int64_t mesh_shape[3], int32_t flags,
                               int32_t slots, pmx_workspace **ws);
int pmx_workspace_slots(const pmx_workspace *ws, int32_t *slots);

/* *gave_up = 1 if a TMA-staged gather of this workspace ever stopped waiting
 * for its copy (it then read global memory; results stay correct).  Waits
 * for the device. */
int pmx_workspace_tma_status(pmx_workspace *ws, int32_t *gave_up);

/* For each of the nsim simulations (nsim <= slots): with init_force, first
 * acc = F(disp) as pmx_force; then nsteps steps as pmx_nbody_steps. */
int pmx_nbody_steps_batch(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                          int32_t nsim, const pmx_sim *sims, int32_t init_force,
                          int32_t nsteps, void *stream);

/* For each of the nsim simulations: with init_vjp, first the force VJP at
 * the current positions with acc_cot = vel_cot, as pmx_force_vjp (acc,
 * acc_cot written; the Omega_m term into dots[4 nsteps + 3]); then nsteps
 * reverse steps as pmx_nbody_adj_steps (dots rows 0..nsteps-1). */
int pmx_nbody_adj_steps_batch(pmx_workspace *ws, const pmx_enmesh_spec *spec,
                              int32_t nsim, const pmx_sim *sims, int32_t init_vjp,
                              int32_t nsteps, void *stream);

/* --------------------------------------------------------------------------
 * Power spectrum (pmwd/spec_util.py:50-147)
 * ------------------------------------------------------------------------ */

/* Bins the half spectra F (and G for a cross spectrum; NULL for auto) of a
 * real grid of grid_shape: nbatch consecutive complex64 arrays of shape
 * (n0, n1, n2/2+1) each, summed over the batch (the reference sums leading
 * channel axes).  kx, ky, kz: float64 wavenumbers in cycles per sample
 * (fftfreq, fftfreq, rfftfreq).  For every complex cell: k = |k|, bin =
 * numpy.digitize(k, edges[0:nedges], right), kept when bin < nbin;
 * multiplicity N = 1 on the z = 0 plane and (even n2) the z Nyquist plane,
 * else 2; P = |F|^2 in float64, or F conj(G) in complex64 widened to
 * float64 (re, im); times prod_axes sinc(k_axis)^-deconv when deconv != 0.
 * Accumulates ksum[b] += k N, psum[2b], psum[2b+1] += P N, nsum[b] += N into
 * caller-zeroed float64 device arrays.  ksum and nsum depend on the grid and
 * bins only: for power-of-two grids up to 2048 both may be NULL (then only
 * psum is accumulated, with float32 per-cell products and float64 sums).
 * Replaces the digitize/bincount of spec_util.py:105-140. */
int pmx_powspec_bin(const float *F, const float *G, int64_t nbatch,
                    const int64_t grid_shape[3], const double *kx,
                    const double *ky, const double *kz, const double *edges,
                    int32_t nedges, int32_t right, int32_t nbin, double deconv,
                    double *ksum, double *psum, double *nsum, void *stream);

/* pmx_powspec_bin for spectra stored half-axis major, (n2/2+1, n0, n1) per
 * batch element with the y axis contiguous -- the layout torch's CUDA rfftn
 * returns for (n0, n1, n2/2+1) -- read in place instead of transposed.
 * Power-of-two grids up to 2048 only. */
int pmx_powspec_bin_zmajor(const float *F, const float *G, int64_t nbatch,
                           const int64_t grid_shape[3], const double *kx,
                           const double *ky, const double *kz, const double *edges,
                           int32_t nedges, int32_t right, int32_t nbin, double deconv,
                           double *ksum, double *psum, double *nsum, void *stream);

/* --------------------------------------------------------------------------
 * White noise (pmwd/modes.py:12-49 ``white_noise``)
 * ------------------------------------------------------------------------ */

/* Counter layouts of JAX's Threefry-2x32 bits: ORIGINAL is JAX's
 * jax_threefry_partitionable=False (its default before JAX 0.5, the one
 * pmwd's published outputs were drawn with); PARTITIONABLE is JAX's default
 * since 0.5. */
#define PMX_PRNG_ORIGINAL       0
#define PMX_PRNG_PARTITIONABLE  1

/* out[0..n) = jax.random.bits(key, (n,), uint32) for the Threefry key
 * (k0, k1) -- jax.random.PRNGKey(seed) is (seed >> 32, seed & 0xffffffff).
 * The original layout covers n <= 2^32 - 2. */
int pmx_random_bits(uint32_t k0, uint32_t k1, int64_t n, int layout, uint32_t *out,
                    void *stream);

/* out[0..n) = jax.random.normal(key, (n,), float32), the draw of
 * modes.py:33-36: sqrt(2) erfinv(u) of a uniform u in [nextafter(-1, 0), 1)
 * built from the bits above, erfinv by Giles' single-precision
 * approximation. */
int pmx_normal(uint32_t k0, uint32_t k1, int64_t n, int layout, float *out, void *stream);

/* --------------------------------------------------------------------------
 * Growth functions (host)
 * ------------------------------------------------------------------------ */

/* Integrates the growth ODEs of boltzmann.py:196-203 (replaces the odeint
 * call of growth_integ, boltzmann.py:163-229) on the host with an adaptive
 * Dormand-Prince 5(4) method, for nparam parameter sets params[4 p + (0..3)]
 * = (Omega_m, Omega_k, w_0, w_a), from lna[0] (initial state G1 = 1,
 * G1' = 0, G2 = 3/7, G2' = 0) through the increasing points lna[0..num).
 * Writes y[(s nparam + p) 4 + i] = (G1, dG1/dlna, G2, dG2/dlna) at lna[s]
 * and dy, its derivative with respect to lna there.  Host memory only; no
 * GPU is needed. */
int pmx_growth_ode(const double *params, int64_t nparam, const double *lna,
                   int64_t num, double rtol, double atol, double *y, double *dy);

/* --------------------------------------------------------------------------
 * Stage profiler (no counterpart in pmwd, which only times whole jitted
 * calls with timeit): CUDA events around each stage of the force and step
 * entry points of one workspace.
 * ------------------------------------------------------------------------ */

#define PMX_PROF_STAGES 15

/* Starts (on != 0) or stops recording stage events on this workspace. */
int pmx_profile_enable(pmx_workspace *ws, int on);

/* Waits for the recorded events, writes per stage the summed milliseconds
 * and number of executions (arrays of PMX_PROF_STAGES), and the number of
 * libpmx kernel launches since the last read (cuFFT's own kernels are not
 * counted); then clears the records.  Any pointer may be NULL. */
int pmx_profile_read(pmx_workspace *ws, double *ms, int64_t *calls, int64_t *launches);

/* Name of stage i, or NULL when out of range. */
const char *pmx_profile_stage_name(int i);

#ifdef __cplusplus
}
#endif

#endif /* PMX_H */
