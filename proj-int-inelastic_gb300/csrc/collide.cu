// Orchestration of one batched Q(f,f) evaluation (pii_collide) and dispatch on
// (precision, n) to the templated kernels.
#include <cmath>
#include <type_traits>
#include <vector>

#include "pii_internal.cuh"

namespace pii {

template <typename T, int NV>
static int finish_all(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb,
                      cudaStream_t s) {
  const int64_t Fc = std::max<int64_t>(1, p->chunk_items / 2);
  for (int64_t c0 = 0; c0 < cells; c0 += Fc) {
    const int64_t cc = std::min(Fc, cells - c0);
    PII_TRY((CollideKernels<T, NV>::finish(p, f, q, c0, cc, with_loss, hb, s)));
  }
  return PII_OK;
}

// the pipeline's gain sums G of cells [c_lo, c_hi): (cell, pair) items, or
// (cell, antipodal pass) items where packed; a chunk holds Cc cells x Pc of
// them in the L2-resident buffer
template <typename T, int NV>
static int pipeline_gain(pii_plan* p, int64_t c_lo, int64_t c_hi, bool packed, cudaStream_t s) {
  using K = CollideKernels<T, NV>;
  const int64_t N = p->N, cells = c_hi - c_lo;
  const int64_t QQ = packed ? p->ap_count : p->Q;
  int64_t Cc = std::max<int64_t>(1, (p->chunk_points + N - 1) / N);
  Cc = std::min<int64_t>(Cc, std::min<int64_t>(cells, p->chunk_items));
  const int64_t Pc = std::max<int64_t>(1, std::min<int64_t>(QQ, p->chunk_items / Cc));
  for (int64_t c0 = c_lo; c0 < c_hi; c0 += Cc) {
    const int64_t cc = std::min(Cc, c_hi - c0);
    for (int64_t p0 = 0; p0 < QQ; p0 += Pc) {
      const int64_t np = std::min(Pc, QQ - p0);
      PII_TRY(K::pairs(p, c0, cc, p0, np, p0 == 0, s, packed));
    }
  }
  return PII_OK;
}

// the side stream of the fused path's split, with its fork / join events
static int side_ready(pii_plan* p) {
  if (p->side) return PII_OK;
  PII_CUDA(cudaEventCreateWithFlags(&p->side_fork, cudaEventDisableTiming));
  PII_CUDA(cudaEventCreateWithFlags(&p->side_join, cudaEventDisableTiming));
  PII_CUDA(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
  return PII_OK;
}

template <typename T, int NV>
static int collide_t(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb,
                     cudaStream_t s) {
  using K = CollideKernels<T, NV>;
  PII_TRY(K::fwd(p, f, 0, cells, s));
  if constexpr (std::is_same<T, float>::value && NV == 64) {
    if (p->dft_path == 1) PII_TRY(col_tc_bounds(p, cells, s));  // per-column scale bounds of f^
  }
  if constexpr (std::is_same<T, float>::value && NV == 32) {
    if (p->gain_path >= 1 && p->gain_path <= 3) {
      if (p->gain_path == 1) {
        PII_TRY(gain_cluster_run(p, cells, s));
      } else {
        PII_TRY(gain_parity_run(p, cells, s, p->gain_path == 3));
        if (p->gain_path == 3) PII_TRY(nyq_use_quad(p) ? nyq_quad_run(p, cells, s) : nyq_corr_run(p, cells, s));
      }
      return finish_all<T, NV>(p, f, q, cells, with_loss, hb, s);
    }
  }
  if constexpr (std::is_same<T, float>::value && NV != 32) {
    if (p->gain_path == 4) {  // the fused kernel: every item on chip, packed where the design allows
      // Where the fused kernel's clusters leave SMs idle (n = 48, 64), a side
      // stream runs there: the packed pipeline on the last cp cells (the
      // split) and the partial sums of the quadratic-form Nyquist correction,
      // which read f^ only; their sum into G follows the join.  The fused
      // kernel is launched first so that its clusters are placed first.
      const bool pack_pipe = p->ap_count > 0 && p->nq_part;
      const int64_t cp = pack_pipe && p->fz_split > 0 ? std::min<int64_t>(cells - 1, llround(p->fz_split * cells)) : 0;
      const bool quad = p->ap_count > 0 && nyq_use_quad(p);
      const bool beside = cp > 0 || (quad && p->fz_sms > 0);
      if (beside) {
        PII_TRY(side_ready(p));
        PII_CUDA(cudaEventRecord(p->side_fork, s));  // f^ and f of every cell are ready
        PII_CUDA(cudaStreamWaitEvent(p->side, p->side_fork, 0));
      }
      PII_TRY(gain_fused_run(p, cells - cp, s));
      if (cp > 0) PII_TRY((pipeline_gain<T, NV>(p, cells - cp, cells, true, p->side)));
      if (quad) {
        PII_TRY(beside ? nyq_quad_run2(p, cells, p->side, s, p->side_join) : nyq_quad_run(p, cells, s));
      } else {
        if (beside) {
          PII_CUDA(cudaEventRecord(p->side_join, p->side));
          PII_CUDA(cudaStreamWaitEvent(s, p->side_join, 0));
        }
        if (p->ap_count > 0) PII_TRY(nyq_gen_run(p, cells, s));
      }
      return finish_all<T, NV>(p, f, q, cells, with_loss, hb, s);
    }
  }
  // the packed pipeline: FP32 for n != 32 (n = 32 has the a-parity kernel),
  // FP64 for every n, where the quadratic-form correction is built
  bool packed = false;
  if constexpr (!std::is_same<T, float>::value || NV != 32) packed = p->gain_path == 3 && p->ap_count > 0;
  PII_TRY((pipeline_gain<T, NV>(p, 0, cells, packed, s)));
  // what the packed passes leave out, on the Nyquist planes
  if (packed) {
    if constexpr (std::is_same<T, float>::value)
      PII_TRY(nyq_use_quad(p) ? nyq_quad_run(p, cells, s) : nyq_gen_run(p, cells, s));
    else
      PII_TRY(nyq_quad_run(p, cells, s));  // FP64: the quadratic form only
  }
  return finish_all<T, NV>(p, f, q, cells, with_loss, hb, s);
}

template <typename T>
static int collide_n(pii_plan* p, const double* f, double* q, int64_t cells, int wl, double hb, cudaStream_t s) {
  switch (p->n) {
    case 8: return collide_t<T, 8>(p, f, q, cells, wl, hb, s);
    case 16: return collide_t<T, 16>(p, f, q, cells, wl, hb, s);
    case 24: return collide_t<T, 24>(p, f, q, cells, wl, hb, s);
    case 32: return collide_t<T, 32>(p, f, q, cells, wl, hb, s);
    case 48: return collide_t<T, 48>(p, f, q, cells, wl, hb, s);
    case 64: return collide_t<T, 64>(p, f, q, cells, wl, hb, s);
    default: set_error("collide: unsupported n = %d", p->n); return PII_ERR_ARG;
  }
}

// Lap_v f alone: the forward transform, a zero gain sum and the finishing
// inverse transform with heat_bath = 1 and no loss term
template <typename T, int NV>
static int laplacian_t(pii_plan* p, const double* f, double* out, int64_t cells, cudaStream_t s) {
  PII_TRY((CollideKernels<T, NV>::fwd(p, f, 0, cells, s)));
  PII_CUDA(cudaMemsetAsync(p->G, 0, size_t(cells) * size_t(p->N) * 2 * sizeof(T), s));
  return finish_all<T, NV>(p, f, out, cells, 0, 1.0, s);
}

template <typename T>
static int laplacian_n(pii_plan* p, const double* f, double* out, int64_t cells, cudaStream_t s) {
  switch (p->n) {
    case 8: return laplacian_t<T, 8>(p, f, out, cells, s);
    case 16: return laplacian_t<T, 16>(p, f, out, cells, s);
    case 24: return laplacian_t<T, 24>(p, f, out, cells, s);
    case 32: return laplacian_t<T, 32>(p, f, out, cells, s);
    case 48: return laplacian_t<T, 48>(p, f, out, cells, s);
    case 64: return laplacian_t<T, 64>(p, f, out, cells, s);
    default: set_error("laplacian: unsupported n = %d", p->n); return PII_ERR_ARG;
  }
}

int prepare_impl(pii_plan* p) {
  if (p->dim == 2) return PII_OK;  // the 2D kernels set their attributes on first use
  const bool f32 = p->precision == PII_PREC_FP32;
  switch (p->n) {
    case 8: return f32 ? CollideKernels<float, 8>::prepare() : CollideKernels<double, 8>::prepare();
    case 16: return f32 ? CollideKernels<float, 16>::prepare() : CollideKernels<double, 16>::prepare();
    case 24: return f32 ? CollideKernels<float, 24>::prepare() : CollideKernels<double, 24>::prepare();
    case 32: return f32 ? CollideKernels<float, 32>::prepare() : CollideKernels<double, 32>::prepare();
    case 48: return f32 ? CollideKernels<float, 48>::prepare() : CollideKernels<double, 48>::prepare();
    case 64: return f32 ? CollideKernels<float, 64>::prepare() : CollideKernels<double, 64>::prepare();
    default: set_error("unsupported n = %d", p->n); return PII_ERR_ARG;
  }
}

int collide_impl(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb, int mass_fix,
                 cudaStream_t s) {
  if (!p || !f || !q) {
    set_error("pii_collide: NULL argument");
    return PII_ERR_ARG;
  }
  if (cells <= 0 || cells > p->batch_max) {
    set_error("pii_collide: cells = %lld outside [1, batch_max = %lld]", (long long)cells,
              (long long)p->batch_max);
    return PII_ERR_SIZE;
  }
  if (f == q) {
    set_error("pii_collide: f and q must not alias");
    return PII_ERR_ARG;
  }
  if (p->tab.nsets > 1 && cells > p->tab.nsets) {
    set_error("pii_collide: cells = %lld beyond the plan's %lld per-cell restitution sets", (long long)cells,
              (long long)p->tab.nsets);
    return PII_ERR_SIZE;
  }
  PII_TRY(dft_stall_check(p));  // a stall of an earlier launch on this plan
  int st = PII_OK;
  if (p->dim == 2)
    st = p->precision == PII_PREC_FP32 ? collide2d_f32(p, f, q, cells, with_loss, hb, s)
                                       : collide2d_f64(p, f, q, cells, with_loss, hb, s);
  else
    st = p->precision == PII_PREC_FP32 ? collide_n<float>(p, f, q, cells, with_loss, hb, s)
                                       : collide_n<double>(p, f, q, cells, with_loss, hb, s);
  if (st != PII_OK) return st;
  if (mass_fix) PII_TRY(mass_fix_impl(p, q, cells, p->N, s));
  return PII_OK;
}

}  // namespace pii

// Autotuner: time the candidate kernel choices for `cells` cells on scratch
// inputs and keep the fastest.  Candidates: gain path (a-parity / cluster /
// pipeline, where the fused kernels exist), work items per resident cluster or
// CTA, pipeline chunk size, and for n = 64 FP32 plans the column-transform
// path (CUDA-core FFT or tensor-core DFT).
extern "C" int pii_plan_autotune(pii_plan* plan, int64_t cells, double* best_ms, void* stream) {
  using namespace pii;
  if (!plan || cells <= 0 || cells > plan->batch_max) {
    set_error("pii_plan_autotune: cells outside [1, batch_max]");
    return PII_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  double* f = nullptr;
  double* q = nullptr;
  const size_t bytes = size_t(cells) * plan->N * sizeof(double);
  PII_CUDA(cudaMalloc(&f, bytes));
  if (cudaMalloc(&q, bytes) != cudaSuccess) {
    cudaFree(f);
    set_error("pii_plan_autotune: out of memory");
    return PII_ERR_CUDA;
  }
  // zeros: no kernel branches on the values (a zero column of the tensor-core
  // DFT takes scale 1 and the same MMAs), so they do not change the timing
  cudaMemsetAsync(f, 0, bytes, s);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  struct Cand {
    int path, items;
    int64_t points;
    int dft;
    double split;  // fused path: share of the cells for the packed pipeline on the idle SMs
  };
  std::vector<Cand> cands;
  const bool cluster_ok = plan->gc_clusters > 0;
  const bool cluster_path_ok = cluster_ok && plan->tab.nsets == 1;  // the cluster kernel takes one table set
  if (cluster_ok) {
    if (cluster_path_ok)
      for (int items : {2, 4, 6, 8}) cands.push_back({1, items, plan->chunk_points, 0, 0.0});
    cands.push_back({2, plan->gc_items_per_cluster, plan->chunk_points, 0, 0.0});  // even split: no item knob
    if (plan->ap_count > 0) cands.push_back({3, plan->gc_items_per_cluster, plan->chunk_points, 0, 0.0});
  }
  // the pipeline on (cell, pair) items, and on antipodal passes where it is
  // packed (FP32: n != 32; FP64: where the quadratic-form correction is built)
  const bool pack_pipe = pii::packed_pipeline_ok(plan);
  for (int path : {0, 3}) {
    if (path == 3 && !pack_pipe) continue;
    for (int dft = 0; dft <= (plan->dft_img ? 1 : 0); ++dft)
      for (int64_t pts : {int64_t(65536), int64_t(131072), int64_t(262144), int64_t(524288)})
        cands.push_back({path, plan->gc_items_per_cluster, pts, dft, 0.0});
  }
  if (plan->fz_clusters > 0 && pii::gain_fused_ensure(plan) == PII_OK) {
    cands.push_back({4, plan->gc_items_per_cluster, plan->chunk_points, 0, 0.0});
    // where the fused kernel's clusters leave SMs idle (n = 48, 64), shares of
    // the cells for the packed pipeline around the idle SMs' share
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, plan->device);
    if (pack_pipe && plan->fz_sms > 0 && plan->fz_sms < sms) {
      const double idle = double(sms - plan->fz_sms) / double(sms);
      for (double m : {0.5, 0.75, 1.0, 1.25})
        for (int dft = 0; dft <= (plan->dft_img ? 1 : 0); ++dft)
          cands.push_back({4, plan->gc_items_per_cluster, 65536, dft, idle * m});
    }
  }
  const int saved_path = plan->gain_path;
  const int saved_items = plan->gc_items_per_cluster;
  const int64_t saved_points = plan->chunk_points;
  const int saved_dft = plan->dft_path;
  const double saved_split = plan->fz_split;
  float best = 1e30f;
  Cand pick{saved_path, saved_items, saved_points, saved_dft, saved_split};
  int st = PII_OK;
  for (const Cand& c : cands) {
    plan->gain_path = c.path;
    plan->gc_items_per_cluster = c.items;
    plan->chunk_points = c.points;
    plan->dft_path = c.dft;
    plan->fz_split = c.split;
    st = collide_impl(plan, f, q, cells, 1, 0.0, 0, s);  // warm-up
    if (st != PII_OK) break;
    cudaEventRecord(e0, s);
    st = collide_impl(plan, f, q, cells, 1, 0.0, 0, s);
    cudaEventRecord(e1, s);
    if (st != PII_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      st = PII_ERR_CUDA;
      set_error("pii_plan_autotune: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(f);
  cudaFree(q);
  plan->gain_path = st == PII_OK ? pick.path : saved_path;
  plan->gc_items_per_cluster = st == PII_OK ? pick.items : saved_items;
  plan->chunk_points = st == PII_OK ? pick.points : saved_points;
  plan->dft_path = st == PII_OK ? pick.dft : saved_dft;
  plan->fz_split = st == PII_OK ? pick.split : saved_split;
  pii::graphs_clear(plan);  // captured graphs baked the old choices in
  if (best_ms) *best_ms = best;
  return st;
}

extern "C" int pii_plan_get_tuning(const pii_plan* plan, int* gain_path, int* items_per_cluster,
                                   int64_t* chunk_points) {
  if (!plan || !gain_path || !items_per_cluster || !chunk_points) {
    pii::set_error("pii_plan_get_tuning: NULL argument");
    return PII_ERR_ARG;
  }
  *gain_path = plan->gain_path;
  *items_per_cluster = plan->gc_items_per_cluster;
  *chunk_points = plan->chunk_points;
  return PII_OK;
}

extern "C" int pii_plan_set_tuning(pii_plan* plan, int gain_path, int items_per_cluster, int64_t chunk_points) {
  if (!plan || items_per_cluster < 1 || items_per_cluster > 64 || chunk_points < 1) {
    pii::set_error("pii_plan_set_tuning: items_per_cluster must be in [1, 64] and chunk_points positive");
    return PII_ERR_ARG;
  }
  const int st = pii_plan_set_gain_path(plan, gain_path);
  if (st != PII_OK) return st;
  plan->gc_items_per_cluster = items_per_cluster;
  plan->chunk_points = chunk_points;
  pii::graphs_clear(plan);  // captured graphs baked the old choices in
  return PII_OK;
}

extern "C" int pii_plan_set_gain_path(pii_plan* plan, int path) {
  if (!plan || path < 0 || path > 4) {
    pii::set_error(
        "pii_plan_set_gain_path: path must be 0 (pipeline), 1 (cluster), 2 (a-parity), 3 (packed) or 4 (fused)");
    return PII_ERR_ARG;
  }
  if (path == 4 && plan->fz_clusters <= 0) {
    pii::set_error("pii_plan_set_gain_path: the fused kernel exists for n = 16, 24, 48, 64, FP32 3D plans only");
    return PII_ERR_ARG;
  }
  if (path == 4) PII_TRY(pii::gain_fused_ensure(plan));
  if (path == 3 && !(plan->n == 32 && plan->precision == PII_PREC_FP32 ? plan->ap_count > 0 && plan->nq_part
                                                                          : pii::packed_pipeline_ok(plan))) {
    pii::set_error(
        "pii_plan_set_gain_path: the packed path needs a 3D plan on an antipodally symmetric design (FP64: with "
        "the quadratic-form Nyquist correction within the memory budget)");
    return PII_ERR_ARG;
  }
  if ((path == 1 || path == 2) && (plan->gc_clusters <= 0 || plan->gp_ctas <= 0)) {
    pii::set_error("pii_plan_set_gain_path: the fused kernels exist for n = 32, FP32 plans only");
    return PII_ERR_ARG;
  }
  if (path == 1 && plan->tab.nsets > 1) {
    pii::set_error("pii_plan_set_gain_path: the cluster kernel takes one restitution set, not one per cell");
    return PII_ERR_ARG;
  }
  plan->gain_path = path;
  return PII_OK;
}

extern "C" int pii_plan_set_fused_split(pii_plan* plan, double fraction) {
  if (!plan || !(fraction >= 0.0 && fraction < 1.0)) {
    pii::set_error("pii_plan_set_fused_split: fraction must be in [0, 1)");
    return PII_ERR_ARG;
  }
  plan->fz_split = fraction;
  pii::graphs_clear(plan);  // captured graphs baked the old choice in
  return PII_OK;
}

extern "C" double pii_plan_get_fused_split(const pii_plan* plan) { return plan ? plan->fz_split : -1.0; }

extern "C" int pii_plan_set_dft_path(pii_plan* plan, int path) {
  if (!plan || path < 0 || path > 1) {
    pii::set_error("pii_plan_set_dft_path: path must be 0 (CUDA-core FFT) or 1 (tensor-core split-FP16 DFT)");
    return PII_ERR_ARG;
  }
  if (path == 1 && !plan->dft_img) {
    pii::set_error("pii_plan_set_dft_path: the tensor-core DFT exists for n = 64, FP32, 3D plans only");
    return PII_ERR_ARG;
  }
  plan->dft_path = path;
  pii::graphs_clear(plan);  // captured graphs baked the old choice in
  return PII_OK;
}

extern "C" int pii_plan_get_dft_path(const pii_plan* plan, int* path, int* stalled) {
  if (!plan || !path) {
    pii::set_error("pii_plan_get_dft_path: NULL argument");
    return PII_ERR_ARG;
  }
  *path = plan->dft_path;
  if (stalled) {
    *stalled = 0;
    if (plan->dft_err_host) {
      PII_CUDA(cudaSetDevice(plan->device));
      PII_CUDA(cudaDeviceSynchronize());
      *stalled = *reinterpret_cast<volatile int*>(plan->dft_err_host);
    }
  }
  return PII_OK;
}

extern "C" int pii_plan_dft_test_hooks(pii_plan* plan, uint32_t wait_limit, int withhold) {
  if (!plan || wait_limit < 1) {
    pii::set_error("pii_plan_dft_test_hooks: wait_limit must be >= 1");
    return PII_ERR_ARG;
  }
  plan->dft_wait_limit = wait_limit;
  plan->dft_withhold = withhold ? 1 : 0;
  pii::graphs_clear(plan);  // captured graphs baked the old arguments in
  return PII_OK;
}

extern "C" int pii_plan_set_nyquist_path(pii_plan* plan, int path) {
  if (!plan || path < 0 || path > 1) {
    pii::set_error("pii_plan_set_nyquist_path: path must be 0 (quadratic form) or 1 (direct kernels)");
    return PII_ERR_ARG;
  }
  if (path == 1 && plan->precision != PII_PREC_FP32) {
    pii::set_error("pii_plan_set_nyquist_path: the direct kernels are FP32; FP64 plans use the quadratic form");
    return PII_ERR_ARG;
  }
  if (path == 0 && !plan->nq_A) {
    PII_CUDA(cudaSetDevice(plan->device));
    PII_TRY(pii::nyq_quad_prepare(plan));  // built on request
    if (!plan->nq_A) {
      pii::set_error("pii_plan_set_nyquist_path: no quadratic-form kernels for this plan (not a 3D plan on an "
                     "antipodally symmetric design, or beyond the memory budget)");
      return PII_ERR_ARG;
    }
  }
  plan->nyq_path = path;
  pii::graphs_clear(plan);  // captured graphs baked the old choice in
  return PII_OK;
}

extern "C" int pii_plan_get_nyquist_path(const pii_plan* plan) {
  if (!plan) return -1;
  return pii::nyq_use_quad(plan) ? 0 : 1;
}

extern "C" int pii_laplacian(pii_plan* plan, const double* f, double* out, int64_t cells, void* stream) {
  using namespace pii;
  if (!plan || !f || !out) {
    set_error("pii_laplacian: NULL argument");
    return PII_ERR_ARG;
  }
  if (cells <= 0 || cells > plan->batch_max) {
    set_error("pii_laplacian: cells = %lld outside [1, batch_max = %lld]", (long long)cells,
              (long long)plan->batch_max);
    return PII_ERR_SIZE;
  }
  if (f == out) {
    set_error("pii_laplacian: f and out must not alias");
    return PII_ERR_ARG;
  }
  PII_CUDA(cudaSetDevice(plan->device));
  cudaStream_t s = (cudaStream_t)stream;
  const bool f32 = plan->precision == PII_PREC_FP32;
  if (plan->dim == 2)
    return f32 ? laplacian2d_f32(plan, f, out, cells, s) : laplacian2d_f64(plan, f, out, cells, s);
  return f32 ? laplacian_n<float>(plan, f, out, cells, s) : laplacian_n<double>(plan, f, out, cells, s);
}

extern "C" int pii_collide(pii_plan* plan, const double* f, double* q, int64_t cells, int with_loss,
                           double heat_bath, int mass_fix, void* stream) {
  if (plan) {
    cudaError_t e = cudaSetDevice(plan->device);
    if (e != cudaSuccess) {
      pii::set_error("cudaSetDevice: %s", cudaGetErrorString(e));
      return PII_ERR_CUDA;
    }
  }
  return pii::collide_impl(plan, f, q, cells, with_loss, heat_bath, mass_fix, (cudaStream_t)stream);
}
