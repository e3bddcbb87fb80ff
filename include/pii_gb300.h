/*
 * pii_gb300.h -- C ABI of the GB300 (sm_103a) fast-spectral inelastic
 * collision operator Q(f,f) and the projective / telescopic time steps that
 * call it.
 *
 * Plain pointers and sizes only.  Every array argument named f, q, df, out is
 * DEVICE memory (cudaMalloc'd or a torch CUDA tensor's data_ptr), row-major,
 * FP64, layout (cells, n, n, n) with the last axis fastest; the first velocity
 * axis is the advection speed v1 (the reference's f layout, src/state.py:64-69,
 * src/solution.py:53-55).  Host arrays (quadrature nodes, integrator
 * parameters) are plain C arrays read during the call.
 *
 * Ownership: the caller owns every array it passes; the library owns the plan,
 * its device tables and its workspace (allocated once in pii_plan_create).
 * Calls are stream-ordered on the given cudaStream_t (NULL = legacy default
 * stream) and are not re-entrant for one plan: one plan, one stream at a time.
 *
 * Errors: every entry point returns PII_OK (0) or a negative status; the
 * message of the last failure on the calling thread is pii_last_error().
 * The Python wrapper raises ValueError / RuntimeError from these codes, the
 * exceptions the reference raises (src/collision/inelastic_collisions.py:47,
 * src/collision/spectral_mesh.py:23, src/solver.py:126-128).
 */
#ifndef PII_GB300_H
#define PII_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PII_OK 0
#define PII_ERR_ARG (-1)      /* invalid argument (ValueError in Python)   */
#define PII_ERR_CUDA (-2)     /* CUDA runtime error                        */
#define PII_ERR_SIZE (-3)     /* batch / size beyond the plan's capacity   */
#define PII_ERR_NONFINITE (-4) /* NaN/Inf guard tripped on FP64 moments   */
#define PII_ERR_STALL (-5)    /* a tensor-core DFT launch of an earlier call on the plan gave up waiting */

#define PII_PREC_FP32 0 /* FP32 FFTs and quadrature sums, FP64 state and islands */
#define PII_PREC_FP64 1 /* everything in FP64 (the parity path)                  */

#define PII_BC_EXTRAP 1   /* src/solver.py:8-9, BC.extrap   */
#define PII_BC_PERIODIC 2 /* src/solver.py:8-10, BC.periodic */

#define PII_INT_EULER 0 /* src/boltzmann.py:82-84   */
#define PII_INT_PFE 1   /* src/boltzmann.py:120-128 */
#define PII_INT_TPI2 2  /* src/boltzmann.py:130-140 */
#define PII_INT_TPI3 3  /* src/boltzmann.py:142-158 */
#define PII_INT_CONSP 4   /* src/boltzmann.py:86-94   */
#define PII_INT_CONSP_M 5 /* src/boltzmann.py:96-118 (3D-velocity form) */

typedef struct pii_plan pii_plan;

/* Message of the last error on this thread ("" if none). */
const char* pii_last_error(void);

/* Library version string. */
const char* pii_version(void);

/*
 * Build an operator plan: quadrature, kernel tables and workspace for up to
 * batch_max cells of n^3 velocity points.  Replaces the construction of
 * FSInelasticVHSCollision(config, SpectralMesh(config))
 * (src/collision/base.py:7-30, src/collision/inelastic_collisions.py:30-137,
 * src/collision/spectral_mesh.py:8-66).
 *   r, w_r       : n_r Gauss-Legendre nodes / weights on [0, R]
 *   sigma        : n_sigma x 3 unit vectors (spherical design), w_sigma weight
 *   L, R         : velocity half-width and collision radius (L = (3+sqrt2)S/2, R = 2S)
 *   e, e0, gamma : restitution law e(r) = (e0-e)/2 tanh(r - R/2) + (e0+e)/2,
 *                  VHS exponent (0 Maxwell molecules, 1 hard spheres)
 * n must be one of 8, 16, 24, 32, 48, 64.
 */
int pii_plan_create(pii_plan** out, int n, int n_r, int n_sigma, const double* r, const double* w_r,
                    const double* sigma, double w_sigma, double L, double R, double e, double e0,
                    double gamma, int precision, int64_t batch_max, int device);

/*
 * The same for velocity dimension dim = 2 or 3 (config["collision-model"]["dim"],
 * src/collision/spectral_mesh.py:17-23, inelastic_collisions.py:42-52).  In 2D
 * the grid is n^2 per cell, sigma holds n_sigma x 2 circle directions
 * (cos phi, sin phi) with weight w_sigma = 2 pi / n_phi
 * (src/collision/spectral_mesh.py:51-56,94-97), the radial kernel is J_0 and
 * the circle constant 2 pi.  pii_plan_create is the dim = 3 case;
 * pii_plan_dim returns a plan's dimension (-1 for NULL).
 */
int pii_plan_create_nd(pii_plan** out, int dim, int n, int n_r, int n_sigma, const double* r, const double* w_r,
                       const double* sigma, double w_sigma, double L, double R, double e, double e0, double gamma,
                       int precision, int64_t batch_max, int device);
int pii_plan_dim(const pii_plan* plan);

/*
 * Per-cell restitution (generalises the operator-wide e, e0 of
 * load_parameters, src/collision/inelastic_collisions.py:30-52,77-80, to an
 * ensemble of independent problems in one plan): cell c of every later call
 * uses (e[c], e0[c]) for its gain tables, c < count <= batch_max; calls with
 * more than `count` cells return PII_ERR_SIZE.  count = 0 restores the plan's
 * own (e, e0) for every cell.  3D-velocity plans; the cluster gain kernel
 * (gain path 1) is then unavailable.  Synchronises the device and drops
 * captured step graphs.  e, e0: host arrays.
 */
int pii_plan_set_restitution(pii_plan* plan, const double* e, const double* e0, int64_t count);

/* Free the plan, its tables and workspace (no reference counterpart: the
 * reference's numpy/cupy arrays are garbage collected). */
int pii_plan_destroy(pii_plan* plan);

/* Bytes of device memory the plan holds. */
int64_t pii_plan_workspace_bytes(const pii_plan* plan);

/*
 * Kernel choice for the gain term of 3D plans (tuning knob, no reference
 * counterpart).  FP32, n = 32: 3 = the fused a-parity kernel on antipodal
 * direction pairs (sigma, -sigma packed into one real-phase pass) plus the
 * exact Nyquist-plane correction (the default where the design is
 * antipodally symmetric), 2 = the fused a-parity kernel with its accumulator
 * in tensor memory, 1 = the fused 2-CTA-cluster kernel.  FP32, n = 16, 24,
 * 48, 64: 4 = the fused kernel (one work item per CTA, or per cluster of
 * 6 / 16 CTAs at n = 48 / 64, exchanging through distributed shared memory,
 * the gain sum in tensor memory; packed with the Nyquist correction where the
 * design is antipodally symmetric; the default at n = 16, 24, 48), 3 = the
 * packed column / plane pipeline.  FP64, every n: 3 = the packed pipeline
 * with the FP64 quadratic-form Nyquist correction (the default on an
 * antipodally symmetric design where that correction fits the memory
 * budget).  0 = the column / plane pipeline on (cell, pair) items, every size
 * and precision.  All compute the same operator.
 */
int pii_plan_set_gain_path(pii_plan* plan, int path);

/*
 * Autotuner (no reference counterpart): times, for `cells` cells, every
 * candidate of the plan's kernel choices -- gain path (a-parity / cluster /
 * pipeline), work items per resident cluster or CTA (2, 4, 6, 8), pipeline
 * chunk size (64K to 512K velocity points), column-transform path (n = 64
 * FP32: CUDA-core FFT or tensor-core DFT) -- on scratch inputs it allocates and frees itself,
 * keeps the fastest and drops captured step graphs.  best_ms (may be NULL)
 * receives the best time of one Q evaluation.  Synchronises the stream.
 * pii_plan_get_tuning reads the current choices.
 */
int pii_plan_autotune(pii_plan* plan, int64_t cells, double* best_ms, void* stream);

/*
 * First-axis column transforms of the n = 64 FP32 pipeline (no reference
 * counterpart; the reference calls FFTW / cuFFT for the whole 3D transform,
 * src/collision/inelastic_collisions.py:212-214): 0 = in-register CUDA-core
 * FFT, 1 = 64-point DFT on the tensor cores (tcgen05.mma, column-scaled split-FP16
 * operands hi + lo, FP32 accumulation in tensor memory).  Path 1 exists for
 * n = 64, FP32, 3D plans only; the autotuner times both.  Every wait of the
 * tensor-core kernel is bounded: a CTA that gives up first waits (bounded)
 * for its copies and MMAs in flight, then frees its tensor memory, and the
 * launch writes a stall word in mapped host memory.  The next pii_collide /
 * pii_step / pii_step_splitting / pii_state_check on the plan returns
 * PII_ERR_STALL (RuntimeError in Python) and clears the word.  get: `stalled`
 * (may be NULL) receives the word without clearing it (1: gave up, 2: and
 * could not drain); reading it synchronises the device.
 */
int pii_plan_set_dft_path(pii_plan* plan, int path);
int pii_plan_get_dft_path(const pii_plan* plan, int* path, int* stalled);
/*
 * Split of the fused gain path (gain path 4; no reference counterpart): the
 * last round(fraction x cells) cells of a call (at most cells - 1) go to the
 * packed column / plane pipeline on a stream of the plan's own, forked from
 * and joined back into the caller's stream, while the fused kernel takes the
 * rest.  At n = 48 and 64 the fused kernel's clusters leave SMs idle (one CTA
 * of a cluster per SM, whole clusters per GPC), and the pipeline's kernels
 * run there.  Needs an antipodally symmetric design; 0 (the default) turns
 * it off.  The autotuner times shares around the idle SMs' share.  set drops
 * captured step graphs; get returns -1 for NULL.
 */
int pii_plan_set_fused_split(pii_plan* plan, double fraction);
double pii_plan_get_fused_split(const pii_plan* plan);
/*
 * Nyquist-plane correction of the packed gain paths (no reference
 * counterpart: the packing is this library's): 0 = the quadratic form
 * C(k) = sum_q A(k, q) f^(q) f^(k - q) - B(k, q) conj f^(q) f^(k + q) with the
 * kernels A, B (N x N real, N = 3 n^2 - 3 n + 1 Nyquist points) precomputed
 * once per plan and restitution set, 1 = the direct per-pass kernels (FP32
 * only).  3D plans on an antipodally symmetric design, n a multiple of 8 up
 * to 64, A and B in the plan's precision; the default is 0 where A, B
 * (2 x 3 N n^2 values per set) fit the memory budget, else 1 (FP64: the
 * unpacked pipeline instead).  set drops captured step graphs (path 0 builds
 * A, B on request); get returns the path in use (-1 for NULL).
 */
int pii_plan_set_nyquist_path(pii_plan* plan, int path);
int pii_plan_get_nyquist_path(const pii_plan* plan);
/* Test hooks of the bounded mbarrier waits of the tensor-core column kernel
 * and the fused cluster kernel (no reference counterpart): wait_limit = polls
 * before a wait gives up (default 4194304); withhold = 1 makes the
 * tensor-core kernel's TMA thread issue no copies and the fused kernel's CTAs
 * issue no exchange stores, so the waits run out on barriers that nothing
 * completes, with no copy, MMA or remote store in flight.  Drops captured
 * step graphs. */
int pii_plan_dft_test_hooks(pii_plan* plan, uint32_t wait_limit, int withhold);
int pii_plan_get_tuning(const pii_plan* plan, int* gain_path, int* items_per_cluster, int64_t* chunk_points);
/* Restores choices read by pii_plan_get_tuning (e.g. saved from an earlier
 * autotune); drops captured step graphs.  items_per_cluster in [1, 64]. */
int pii_plan_set_tuning(pii_plan* plan, int gain_path, int items_per_cluster, int64_t chunk_points);

/*
 * q = Q+(f,f) [- Q-(f,f) if with_loss] [+ heat_bath * Lap_v f], per cell.
 * Replaces BaseCollision.__call__ (src/collision/base.py:32-58) and
 * FSInelasticVHSCollision.collide / laplacian
 * (src/collision/inelastic_collisions.py:208-230).  f and q: cells x n^3 FP64
 * device arrays (may not alias).  mass_fix != 0 subtracts the per-cell mean of
 * q in FP64 (the k = 0 mass-mode correction; not in the reference).
 */
int pii_collide(pii_plan* plan, const double* f, double* q, int64_t cells, int with_loss,
                double heat_bath, int mass_fix, void* stream);

/*
 * out = Lap_v f per cell, the spectral Laplacian Re IFFT(-pi^2 |k|^2 / L^2 FFT(f))
 * of FSInelasticVHSCollision.laplacian (src/collision/inelastic_collisions.py:
 * 229-230, the table of :69), with the transforms of pii_collide in the plan's
 * working precision (FP64 plans: FP64).  pii_collide adds heat_bath times the
 * same term inside its own final transform.  f and out: cells x n^dim FP64
 * device arrays (may not alias).
 */
int pii_laplacian(pii_plan* plan, const double* f, double* out, int64_t cells, void* stream);

/*
 * Transport increment of the second-order upwind + minmod TVD scheme in x,
 * df = -dt/dx (A-dq + A+dq) - dt/dx (F_{i+1/2} - F_{i-1/2}), two ghost cells.
 * Replaces BoltzmannSolver1D.df_advection (src/boltzmann.py:177-205) with the
 * ghost fill of Solver._apply_bcs (src/solver.py:59-105), advection_1D
 * (src/riemann/advection_1D.py:4-21) and tvd.limit / minmod
 * (src/limiters/tvd.py:6-40).  v1: n first-axis velocity centres (host).
 */
int pii_transport_df(pii_plan* plan, const double* f, double* df, int64_t nx, double dt, double dx,
                     const double* v1, int bc_lower, int bc_upper, void* stream);

/*
 * df = transport(f, dt) + dt * Q(f) / kn   (nx == 0: homogeneous, no transport).
 * Replaces BoltzmannSolver.df (src/boltzmann.py:160-164).
 */
int pii_boltzmann_df(pii_plan* plan, const double* f, double* df, int64_t nx, double dt, double dx,
                     const double* v1, int bc_lower, int bc_upper, double kn, int with_loss,
                     int mass_fix, void* stream);

/*
 * One macro-step of size dt of the chosen integrator, updating f in place
 * (FP64).  Replaces BoltzmannSolver.step and its euler_step /
 * proj_euler_step / tel_proj_step2 / tel_proj_step3 (src/boltzmann.py:46-158).
 * inner_steps / inner_dt: host arrays of length levels (1 for PFE, 2 for
 * TPI2, 3 for TPI3; ignored for Euler).  use_graph != 0 captures the whole
 * macro-step into a CUDA graph on first use and replays it on later calls
 * with the same arguments.
 */
int pii_step(pii_plan* plan, int integrator, double* f, int64_t nx, double dt, const int* inner_steps,
             const double* inner_dt, int levels, double dx, const double* v1, int bc_lower, int bc_upper,
             double kn, int with_loss, int mass_fix, int use_graph, void* stream);

/*
 * One convex-splitting step of size dt, updating f in place (FP64):
 *   CONSP   (src/boltzmann.py:86-94):  f += dt / (kn + P dt) Q(f);  f += transport(f, dt)
 *   CONSP_M (src/boltzmann.py:96-118): as CONSP plus the penalised Maxwellian
 *           term P dt / (kn + P dt) (M[rho, u1, T_new] - M[rho, u1, T]) with
 *           T_new = (T - 8 tau / (1 - e^2)) exp(-(1 - e^2) rho dt / (4 kn)) + 8 tau / (1 - e^2),
 *           rho, u1 (first velocity component) and T from the FP64 moments of f.
 *           2D plans: the reference's form (2D Maxwellian, T = E / rho - |u|^2 / 2);
 *           3D plans: its 3D-velocity form (Maxwellian in 3D, bulk velocity
 *           (u1, 0, 0), T = (2/3)(E / rho - |u|^2 / 2)).
 * penalty: P; e, tau: CONSP_M only.  dx <= 0: no transport (homogeneous cells).
 */
int pii_step_splitting(pii_plan* plan, int integrator, double* f, int64_t nx, double dt, double dx,
                       const double* v1, int bc_lower, int bc_upper, double kn, double penalty, double e,
                       double tau, int with_loss, int mass_fix, int use_graph, void* stream);

/*
 * FP64 guard on the state (no reference counterpart; the reference has no
 * failure detection): computes the per-cell moments of f into out[cells * 5]
 * (device, as pii_moments) and checks every value of f for NaN / Inf.
 * Synchronises the stream.  Returns PII_ERR_NONFINITE if any value is not
 * finite, PII_OK otherwise.
 */
int pii_state_check(pii_plan* plan, const double* f, double* out, int64_t cells, const double* v, double delta,
                    void* stream);

/*
 * FP64 moments per cell: out[c*5 + {0,1,2,3,4}] = sum f, sum f v1, sum f v2,
 * sum f v3, sum f |v|^2 / 2, each times delta^dim (State.rho / u / T,
 * src/state.py:31-52,91-92; 2D plans: the reference's form, v3 term 0).
 * v: n velocity centres (host).
 * out is a device array of cells*5 doubles.
 */
int pii_moments(pii_plan* plan, const double* f, double* out, int64_t cells, const double* v, double delta,
                void* stream);

/*
 * One iteration of BoltzmannFastSweep.step (src/iter_solver.py:38-62), FP64, in
 * place on the device state f (nx cells): with q = the collision term of the
 * current f (device, as the operator's __call__ returns it) and rho the
 * cells' densities, a Gauss-Seidel upwind sweep in x
 *   v1 > 0: f[i] = (nu q[i] + (v1/dx) f[i-1]) / (nu rho[i] + v1/dx),  i = 1 .. nx-2
 *   v1 < 0: f[i] = (nu q[i] - (v1/dx) f[i+1]) / (nu rho[i] - v1/dx),  i = nx-2 .. 1
 * with nu = 1 / sqrt(pi/2) / kn.  *err (host) receives max |f_new - f_old|.
 * v1: n first-axis velocity centres (host).  The reference writes the sweep for
 * 2D velocity; 3D plans sweep every (v2, v3) the same way.  Synchronises the stream.
 */
int pii_fast_sweep(pii_plan* plan, double* f, const double* q, int64_t nx, double dx, double kn, const double* v1,
                   double* err, void* stream);

/* f[i] += a * (b * d[i]) for i < count, FP64 (the projective extrapolation
 * f += M_l * df_l, src/boltzmann.py:128,138-140,154-158). */
int pii_axpby(double* f, const double* d, double a, double b, int64_t count, void* stream);

/*
 * Q(f,f) without any allocation.  No counterpart in the reference.  For
 * callers that may not call cudaMalloc where they need Q: a host framework
 * that hands out device memory only through its own pool, a time loop with a
 * fixed memory budget set at start-up, or code that must not stall the device
 * (cudaMalloc / cudaFree may synchronise it); pii_plan_create allocates, so
 * they cannot use it.  Same result as pii_collide in PII_PREC_FP32
 * (heat_bath = 0, mass_fix = 0), but the tables and workspace live in one
 * static device array of 2.5 MiB that the library image reserves on every
 * GPU that loads it.  Limits: n in {8, 16}, cells <= 8, n_r <= 32,
 * n_sigma <= 192, n_r * n_sigma <= 1024; larger requests return
 * PII_ERR_SIZE.  All calls on a device share the array, which keeps the last
 * call's contents: calls whose GPU work overlaps race.  The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress) with that
 * device current; cudaDeviceReset between calls is not supported.  f, q:
 * device arrays of cells x n^3 FP64; r, w_r, sigma: host arrays as for
 * pii_plan_create, read during the call and passed to the GPU by value (no
 * host-to-device copy).
 */
int pii_collide_noalloc(const double* f, double* q, int64_t cells, int n, int n_r, int n_sigma, const double* r,
                        const double* w_r, const double* sigma, double w_sigma, double L, double R, double e,
                        double e0, double gamma, int with_loss, void* stream);

/*
 * Instrumentation (no reference counterpart).
 * pii_kernel_launches: number of kernels this library has enqueued in the
 * process (eager launches, plus the kernel nodes of every CUDA-graph replay).
 * pii_plan_profile(plan, 1) starts per-stage CUDA-event timing of the plan's
 * eager launches (graph capture is bypassed while it is on);
 * pii_plan_profile_read fills ms[PII_NSTAGES] (summed device time) and
 * launches[PII_NSTAGES] after synchronising, and resets the counters.
 */
#define PII_NSTAGES 15
/* stage order: fwd_plane, col_fwd, col_pstart, pair_plane, col_pend, reduce,
 * col_iprep, finish, df, axpy, massfix, gain_cluster, gain_parity, nyq_corr,
 * gain_fused */
int64_t pii_kernel_launches(void);
/* instantiated macro-step graphs held by the plan (at most 8: pii_step and
 * pii_step_splitting evict the least recently replayed one) */
int64_t pii_plan_graph_count(const pii_plan* plan);
int pii_plan_profile(pii_plan* plan, int enable);
int pii_plan_profile_read(pii_plan* plan, double* ms, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* PII_GB300_H */
