// Internal declarations shared by the translation units of libpii_gb300.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/pii_gb300.h"

namespace pii {

void set_error(const char* fmt, ...);

// kernels enqueued by the library (eager launches + kernel nodes of graph replays)
extern std::atomic<int64_t> g_launches;

// Once per device: kernel attributes (cudaFuncSetAttribute) belong to the
// current device, so a process with plans on several GPUs sets them on each.
// 16-byte global -> shared copy that completes asynchronously (cp.async); the
// issuing thread's cp_async_wait_all and a barrier make it visible to the CTA
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
// the same for 8 bytes (both addresses 8-byte aligned)
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
// the same for one 4-byte word (both addresses 4-byte aligned)
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// close the current group of cp.async copies; wait until at most N groups are pending
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

struct PerDeviceOnce {
  std::atomic<uint64_t> mask{0};
  bool done() const {
    int d = 0;
    return cudaGetDevice(&d) == cudaSuccess && d >= 0 && d < 64 && (mask.load() >> d & 1u);
  }
  void set() {
    int d = 0;
    if (cudaGetDevice(&d) == cudaSuccess && d >= 0 && d < 64) mask.fetch_or(uint64_t(1) << d);
  }
};

// modes of the first-axis column pass (collide_kernels.cuh, col_tc.cu)
// column passes along the first velocity axis; the _PK modes take antipodal
// passes (cell, antipodal pair) instead of (cell, pair) items
enum ColMode { COL_FWD = 0, COL_PSTART = 1, COL_PEND = 2, COL_IPREP = 3, COL_PSTART_PK = 4, COL_PEND_PK = 5 };

enum Stage {
  ST_FWD_PLANE = 0, ST_COL_FWD, ST_COL_PSTART, ST_PAIR_PLANE, ST_COL_PEND, ST_REDUCE,
  ST_COL_IPREP, ST_FINISH, ST_DF, ST_AXPY, ST_MASSFIX, ST_GAIN_CLUSTER, ST_GAIN_PARITY, ST_NYQ, ST_GAIN_FUSED, ST_COUNT
};

#define PII_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) {                                                              \
      ::pii::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
      return PII_ERR_CUDA;                                                                \
    }                                                                                     \
  } while (0)

#define PII_CHECK_LAUNCH()                                                                 \
  do {                                                                                     \
    ::pii::g_launches.fetch_add(1, std::memory_order_relaxed);                             \
    cudaError_t _e = cudaGetLastError();                                                   \
    if (_e != cudaSuccess) {                                                               \
      ::pii::set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return PII_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

#define PII_TRY(expr)          \
  do {                         \
    int _s = (expr);           \
    if (_s != PII_OK) return _s; \
  } while (0)

// Device tables, all in the plan's working precision (float or double).
//   ephase [Q][3][n] complex : exp(-i pi r sigma_d k / L); the d = 0 row also
//                              carries the 1/n^dim of the first inverse FFT
//   gphase [Q][3][n] complex : exp(+i a(r) r sigma_d k)
//   gsinc  [n_r][M+1] real   : r^{gamma+dim-1} w_r w_sigma K(a(r) r sqrt(m))
//                              (the sphere constant cancels the 1/(4 pi) or
//                              1/(2 pi) of collide)
//   lossk  [M+1] real        : sum_r S r^{gamma+dim-1} w_r K(pi r sqrt(m) / L)
//   lapl   [M+1] real        : -pi^2 m / L^2
// with k the signed spectral index of the storage position, m = |k|^2 <= M =
// dim (n/2)^2, K = sinc and S = 4 pi in 3D, K = J_0 and S = 2 pi in 2D (the
// third row of the per-axis tables is unused in 2D).
// For n = 32 in FP32 the a-parity kernel also keeps, per pair and parity p
// (W = exp(-2 pi i / 32), e_a / g_a the d = 0 rows above):
//   epar [Q][2][32] complex  : W^{-p k} e_a[k] (k < 16), (-1)^p W^{-p k} e_a[k + 16]
//   gpar [Q][2][32] complex  : W^{p k} g_a[k]
//   gsx  [n_r][513][20] real : gsinc[r][m_bc + q^2] for q = |k_a| <= 16 (0-padded),
//                              m_bc = k_b^2 + k_c^2: one 80-byte row per column
//   gsxc [n_r][153][17] real : the same rows by (|k_b|, |k_c|) pair u <= v, index
//                              v (v + 1) / 2 + u (one radial node: 10.4 KB)
struct Tables {
  void* ephase = nullptr;
  void* gphase = nullptr;
  void* epar = nullptr;
  void* gpar = nullptr;
  void* gsx = nullptr;
  void* gsxc = nullptr;
  void* gsinc = nullptr;
  void* lossk = nullptr;
  void* lapl = nullptr;
  int M = 0;
  // restitution sets of the gain tables (gphase, gsinc, gpar, gsx, gsxc): with
  // more than one, cell c of a call uses set c and each stride is the elements
  // (complex ones for the phase rows) per set; with one, the strides are 0
  int64_t nsets = 1;
  int64_t gph_stride = 0, gs_stride = 0, gpar_stride = 0, gsx_stride = 0, gsxc_stride = 0;
};

struct GraphKey {
  int integrator;
  double* f;
  int64_t nx;
  double dt, dx, kn;
  int bc_lo, bc_hi, with_loss, mass_fix, levels;
  int K[3];
  double h[3];
  void* stream;
  bool operator<(const GraphKey& o) const;
};

struct GraphEntry {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;  // recorded after each replay: eviction waits for the last one
  int64_t kernels = 0;         // kernel launches captured into the graph
  uint64_t last_use = 0;       // plan-local replay counter at the last replay (LRU eviction)
};

// instantiated macro-step graphs kept per plan; the least recently replayed
// one is destroyed when a new key would exceed this
constexpr size_t kMaxGraphs = 8;

struct ProfEvent {
  int stage;
  cudaEvent_t a, b;
};

}  // namespace pii

struct pii_plan {
  int dim = 3;  // velocity dimension (2: J_0 kernel on a circle, 3: sinc on a sphere)
  int n = 0, nr = 0, ns = 0, Q = 0;
  int64_t N = 0;
  int precision = 0;
  int device = 0;
  double L = 0, R = 0, e = 0, e0 = 0, gamma = 0, wsigma = 0;
  int64_t batch_max = 0;
  std::vector<double> r, wr, sigma;
  pii::Tables tab;
  // workspace (precision-typed unless noted)
  void* fhat = nullptr;  // batch_max * N complex
  void* fT = nullptr;    // batch_max * N real
  void* G = nullptr;     // batch_max * N complex
  void* buf = nullptr;   // chunk_items * N complex
  int64_t chunk_items = 0;
  double* q = nullptr;    // batch_max * N, FP64 collide output inside the solver
  double* d0 = nullptr;   // batch_max * N, FP64 level increments
  double* d1 = nullptr;
  double* d2 = nullptr;
  double* v1dev = nullptr;  // n first-axis velocities (device)
  double* mom = nullptr;    // batch_max * 5 FP64 moment sums (CONSP_M)
  int* flag = nullptr;      // 16 device bytes: pii_state_check flag (0), pii_fast_sweep error word (8)
  double delta3 = 0;        // velocity cell volume of the last splitting step
  // gain kernel for n = 32, FP32: 0 = column/plane pipeline, 1 = fused
  // 2-CTA-cluster kernel, 2 = fused a-parity kernel (tensor-memory accumulator),
  // 3 = a-parity kernel on antipodal pairs + Nyquist correction; for other n
  // (FP32, antipodally symmetric design): 0 = pipeline on (cell, pair) items,
  // 3 = pipeline on antipodal passes + the general Nyquist correction
  int gain_path = 0;
  // tunables (pii_plan_autotune): work items per resident cluster, and the
  // points per chunk of the pipeline path (cells per chunk = this / n^3)
  int gc_items_per_cluster = 6;
  int64_t chunk_points = 131072;
  int gc_clusters = 0;
  int64_t gc_max_items = 0;
  void* gc_maps = nullptr;   // int2 thread -> columns [512], column -> slot [1024]
  void* gc_hpart = nullptr;  // per-part Hermitian slots
  int gp_ctas = 0;           // resident CTAs of the a-parity kernel
  int64_t gp_max_items = 0;
  void* gp_hpart = nullptr;  // its per-item Hermitian slots
  int* ap_reps = nullptr;    // device: representative pair of each antipodal pair (0 if the design is not symmetric)
  int ap_count = 0;
  void* nq_part = nullptr;   // Nyquist-correction accumulators [CTAs][3][n^2]
  int64_t nq_ctas = 0;       // their capacity in CTAs (the general kernel, n != 32)
  // quadratic-form Nyquist correction (nyq_quad.cu): paired kernels A~, B~
  // [sets][3 output planes][input-point slots][n^2 output points], f^ transposed
  // within each a-plane, the partial sums of the input-point ranges;
  // nyq_path 0 uses it where built, 1 the direct kernels
  void* nq_A = nullptr;
  void* nq_B = nullptr;
  void* nq_fhT = nullptr;
  void* nq_qpart = nullptr;
  int64_t nq_qpart_units = 0;  // capacity of nq_qpart in (range, cell) units of 3 n^2 points
  void* nq_segs = nullptr;     // segments of the kernel slots: int4 (slice, kind, i1, steps) [nseg], then int j0 [nseg]
  int nq_nseg = 0;
  int nq_npts = 0;
  int nq_slots = 0;            // resident CTAs of the correction kernel on the device
  int64_t nq_quad_bytes = 0;
  int nyq_path = 0;
  // fused gain kernel (gain_fused.cu, n = 16, 24, 48, 64): per-(cluster, cell)
  // segment sums [clusters + batch_max][n^3] and the clusters resident at once
  void* fz_part = nullptr;
  int fz_clusters = 0;
  int fz_sms = 0;           // SMs the resident clusters fill (clusters x CTAs per cluster, one CTA per SM)
  // share of a call's cells that the packed pipeline takes on a side stream
  // while the fused kernel fills its SMs (pii_plan_set_fused_split; 0: none)
  double fz_split = 0.0;
  cudaStream_t side = nullptr;                    // created on first use
  cudaEvent_t side_fork = nullptr, side_join = nullptr;
  void* nq_ft2 = nullptr;    // general kernel: f transposed within each a-plane [batch_max][n^3] (FP32)
  void* nq_fhn = nullptr;    // general kernel: f^ at the Nyquist-plane points [batch_max][3 n^2]
  // first-axis column transforms of the n = 64 FP32 pipeline: 0 = CUDA-core
  // FFT (k_col), 1 = tensor-core split-FP16 DFT (k_col_tc)
  int dft_path = 0;
  void* dft_img = nullptr;  // DFT matrix images (A_hi | A_lo) for DIR = +1 and -1
  int* dft_err = nullptr;   // device address of dft_err_host
  int* dft_err_host = nullptr;  // mapped host word: 1 if a k_col_tc CTA gave up waiting (2: and could not drain; 3: a k_gain_fused exchange)
  uint32_t dft_wait_limit = 1u << 22;  // mbarrier polls before a k_col_tc role gives up
  int dft_withhold = 0;     // test hook: k_col_tc's TMA thread issues no copies
  int dft_ctas = 0;         // resident CTAs of k_col_tc (one per SM)
  void* dft_gs = nullptr;   // gsinc by (set, r, |k_b|, |k_c|, |k_a|) slices (TMA sources)
  int64_t dft_gs_bytes = 0, dft_gs_stride = 0;  // its size, and floats per restitution set (0: one set)
  void* dft_colb = nullptr; // [batch_max][n^2] column bounds max_a |f^|_1 (k_col_bound)
  // TMA tensor maps (CUtensorMap, 128 bytes each) of f^ and of the chunk buffer
  // as 2D FP32 arrays [rows of 64 (a) per grid][8192 floats per row]
  alignas(128) unsigned char dft_tmap[2][128] = {};
  int64_t bytes = 0;
  std::map<pii::GraphKey, pii::GraphEntry> graphs;
  uint64_t graph_tick = 0;
  std::vector<double> v1host;  // the first-axis velocities last uploaded to v1dev
  // per-stage CUDA-event profiling (pii_plan_profile)
  bool prof = false;
  std::vector<pii::ProfEvent> prof_events;
  std::vector<cudaEvent_t> prof_pool;
  double prof_ms[pii::ST_COUNT] = {0};
  int64_t prof_n[pii::ST_COUNT] = {0};
};

namespace pii {
// RAII: records a begin / end event pair around one launch when profiling is on
struct StageTimer {
  pii_plan* p;
  int stage;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  StageTimer(pii_plan* p_, int stage_, cudaStream_t s_);
  ~StageTimer();
};
}  // namespace pii

namespace pii {

// collide.cu
int collide_impl(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb,
                 int mass_fix, cudaStream_t s);
int prepare_impl(pii_plan* p);
// gain_cluster.cu
int gain_cluster_prepare(pii_plan* p);
int gain_cluster_run(pii_plan* p, int64_t cells, cudaStream_t s);
// collide2d_f32.cu / collide2d_f64.cu: the 2D-velocity operator
int collide2d_f32(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb, cudaStream_t s);
int collide2d_f64(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb, cudaStream_t s);
int laplacian2d_f32(pii_plan* p, const double* f, double* out, int64_t cells, cudaStream_t s);
int laplacian2d_f64(pii_plan* p, const double* f, double* out, int64_t cells, cudaStream_t s);
// gain_parity.cu
int gain_parity_prepare(pii_plan* p);
int gain_parity_run(pii_plan* p, int64_t cells, cudaStream_t s, bool packed);
// nyq_corr.cu
int nyq_corr_prepare(pii_plan* p);
int nyq_corr_run(pii_plan* p, int64_t cells, cudaStream_t s);
// col_tc.cu: tensor-core first-axis DFT of the n = 64 FP32 pipeline
int col_tc_prepare(pii_plan* p);
int col_tc_run(pii_plan* p, int mode, int64_t items, int64_t c0, int64_t p0, int64_t np, cudaStream_t s);
int col_tc_bounds(pii_plan* p, int64_t cells, cudaStream_t s);
int col_tc_gain_tables(pii_plan* p);  // (re)builds the sinc slices of every restitution set
// nyq_gen.cu: Nyquist-plane correction of the packed pipeline (n != 32, FP32)
int nyq_gen_prepare(pii_plan* p);
int nyq_gen_run(pii_plan* p, int64_t cells, cudaStream_t s);
// nyq_quad.cu: the same correction as a quadratic form in f^ with precomputed kernels
int nyq_quad_prepare(pii_plan* p);
int gain_fused_prepare(pii_plan* p);
int gain_fused_ensure(pii_plan* p);
int gain_fused_run(pii_plan* p, int64_t cells, cudaStream_t s);
void nyq_quad_release(pii_plan* p);
int nyq_quad_run(pii_plan* p, int64_t cells, cudaStream_t s);
// partial sums on s; if partial_done, s_add waits for it; the sum into G on s_add
int nyq_quad_run2(pii_plan* p, int64_t cells, cudaStream_t s, cudaStream_t s_add, cudaEvent_t partial_done);
// the Nyquist correction of the packed paths: the quadratic form where it was
// built and chosen, else the direct kernel of the plan's n
inline bool nyq_use_quad(const pii_plan* p) { return p->nyq_path == 0 && p->nq_A != nullptr; }
// the packed column / plane pipeline with its Nyquist correction: FP32 (n !=
// 32) with the direct kernels' buffers, FP64 with the quadratic form built
inline bool packed_pipeline_ok(const pii_plan* p) {
  if (p->ap_count <= 0 || p->dim != 3) return false;
  return p->precision == PII_PREC_FP32 ? p->n != 32 && p->nq_part != nullptr : p->nq_A != nullptr;
}
// col_tc.cu: PII_ERR_STALL if a tensor-core DFT launch of an earlier call gave
// up waiting (read from mapped host memory without a synchronisation; cleared
// once reported)
int dft_stall_check(pii_plan* p);
// transport.cu
int transport_impl(pii_plan* p, const double* f, const double* q, double* df, int64_t nx, double dt,
                   double dx, int bc_lo, int bc_hi, double qscale, cudaStream_t s);
int mass_fix_impl(pii_plan* p, double* q, int64_t cells, int64_t N, cudaStream_t s);
int axpy3_impl(pii_plan* p, double* f, const double* d, double s0, double s1, double s2, int64_t count,
               cudaStream_t s);
int upload_v1(pii_plan* p, const double* v1, cudaStream_t s);
// plan.cu: the macro-step graph cache
void graphs_clear(pii_plan* p);
void graph_entry_destroy(GraphEntry& g);
int consp_m_impl(pii_plan* p, double* f, const double* q, int64_t cells, double c, double c2, double dt, double kn,
                 double e, double tau, cudaStream_t s);
int axpy3_impl(pii_plan* p, double* f, const double* d, double s0, double s1, double s2, int64_t count,
               cudaStream_t s);

// per-precision, per-size kernels (collide_kernels_*.cu)
template <typename T, int NV>
struct CollideKernels {
  static int prepare();
  static int fwd(pii_plan* p, const double* f, int64_t c0, int64_t cells, cudaStream_t s);
  // items (cell, pair) for pairs [p0, p0 + np); packed: antipodal passes [p0, p0 + np) of p->ap_reps
  static int pairs(pii_plan* p, int64_t c0, int64_t cells, int64_t p0, int64_t np, bool first,
                   cudaStream_t s, bool packed = false);
  static int finish(pii_plan* p, const double* f, double* q, int64_t c0, int64_t cells, int with_loss,
                    double hb, cudaStream_t s);
};

}  // namespace pii
