// Time integrators on the device: forward Euler, projective forward Euler and
// the 2- / 3-level telescopic projective steps (src/boltzmann.py:46-164).
//
// The state f and the level increments are FP64.  The reference keeps the
// increment of the last inner step and adds M_l times it
// (d_{l+1} = M_l d_l, src/boltzmann.py:138,154-158); with one FP64 buffer d0
// every extrapolation f += M_l * ... * M_0 * d0 is applied as
// f += s2 * (s1 * (s0 * d0)), which rounds exactly like the reference's
// chained products.  A whole macro-step can be captured into a CUDA graph and
// replayed.
#include <cmath>

#include "pii_internal.cuh"

namespace pii {

int check_bcs(int lo, int hi);

struct StepCtx {
  pii_plan* p;
  double* f;
  int64_t nx;
  double dx, kn;
  int bc_lo, bc_hi, with_loss, mass_fix;
  cudaStream_t s;
};

// d0 = transport(f, h) + h Q(f) / kn   (BoltzmannSolver.df, src/boltzmann.py:160-164)
static int df_into_d0(const StepCtx& c, double h) {
  PII_TRY(collide_impl(c.p, c.f, c.p->q, c.nx, c.with_loss, 0.0, c.mass_fix, c.s));
  return transport_impl(c.p, c.f, c.p->q, c.p->d0, c.nx, h, c.dx, c.bc_lo, c.bc_hi, c.kn, c.s);
}

static int add(const StepCtx& c, double s0, double s1, double s2) {
  return axpy3_impl(c.p, c.f, c.p->d0, s0, s1, s2, c.nx * c.p->N, c.s);
}

static int step_body(const StepCtx& c, int integrator, double dt, const int* K, const double* h) {
  switch (integrator) {
    case PII_INT_EULER:  // f += df(dt)
      PII_TRY(df_into_d0(c, dt));
      return add(c, 1, 1, 1);
    case PII_INT_PFE: {
      const double M = dt / h[0] - K[0];
      for (int i = 0; i < K[0]; ++i) {
        PII_TRY(df_into_d0(c, h[0]));
        PII_TRY(add(c, 1, 1, 1));
      }
      return add(c, M, 1, 1);
    }
    case PII_INT_TPI2: {
      const double M1 = dt / h[1] - K[1];
      const double M0 = h[1] / h[0] - K[0];
      for (int j = 0; j < K[1]; ++j) {
        for (int i = 0; i < K[0]; ++i) {
          PII_TRY(df_into_d0(c, h[0]));
          PII_TRY(add(c, 1, 1, 1));
        }
        PII_TRY(add(c, M0, 1, 1));  // df1 = M0 df0; f += df1
      }
      return add(c, M0, M1, 1);  // f += M1 df1
    }
    case PII_INT_TPI3: {
      const double M2 = dt / h[2] - K[2];
      const double M1 = h[2] / h[1] - K[1];
      const double M0 = h[1] / h[0] - K[0];
      for (int k = 0; k < K[2]; ++k) {
        for (int j = 0; j < K[1]; ++j) {
          for (int i = 0; i < K[0]; ++i) {
            PII_TRY(df_into_d0(c, h[0]));
            PII_TRY(add(c, 1, 1, 1));
          }
          PII_TRY(add(c, M0, 1, 1));  // df1 = M0 df0
        }
        PII_TRY(add(c, M0, M1, 1));  // df2 = M1 df1
      }
      return add(c, M0, M1, M2);  // f += M2 df2
    }
    default:
      set_error("This time integrator is not implemented.");
      return PII_ERR_ARG;
  }
}

static int validate(pii_plan* p, int integrator, double* f, int64_t nx, const int* K, const double* h,
                    int levels) {
  if (!p || !f || nx <= 0) {
    set_error("pii_step: invalid arguments");
    return PII_ERR_ARG;
  }
  if (nx > p->batch_max) {
    set_error("pii_step: nx = %lld beyond batch_max = %lld", (long long)nx, (long long)p->batch_max);
    return PII_ERR_SIZE;
  }
  const int need = integrator == PII_INT_PFE ? 1 : integrator == PII_INT_TPI2 ? 2 : integrator == PII_INT_TPI3 ? 3 : 0;
  if (integrator < PII_INT_EULER || integrator > PII_INT_TPI3) {
    set_error("This time integrator is not implemented.");
    return PII_ERR_ARG;
  }
  if (need > 0) {
    if (!K || !h || levels < need) {
      set_error("pii_step: integrator needs %d inner levels", need);
      return PII_ERR_ARG;
    }
    for (int l = 0; l < need; ++l)
      if (K[l] < 1 || !(h[l] > 0)) {
        set_error("pii_step: inner_steps must be >= 1 and inner_dt > 0");
        return PII_ERR_ARG;
      }
  }
  return PII_OK;
}

// CONSP / CONSP_M (src/boltzmann.py:86-118): collision update, then transport of the updated f
static int splitting_body(const StepCtx& c, int integrator, double dt, double penalty, double e, double tau) {
  PII_TRY(collide_impl(c.p, c.f, c.p->q, c.nx, c.with_loss, 0.0, c.mass_fix, c.s));
  const double cq = dt / (c.kn + penalty * dt);
  if (integrator == PII_INT_CONSP) {
    PII_TRY(axpy3_impl(c.p, c.f, c.p->q, cq, 1, 1, c.nx * c.p->N, c.s));
  } else {
    const double cm = penalty * dt / (c.kn + penalty * dt);
    PII_TRY(consp_m_impl(c.p, c.f, c.p->q, c.nx, cq, cm, dt, c.kn, e, tau, c.s));
  }
  if (c.dx > 0) {
    PII_TRY(transport_impl(c.p, c.f, nullptr, c.p->d0, c.nx, dt, c.dx, c.bc_lo, c.bc_hi, 1.0, c.s));
    PII_TRY(add(c, 1, 1, 1));
  }
  return PII_OK;
}

// Replays the cached graph of `key`, capturing `body` into a new one first if
// there is none.  At most kMaxGraphs graphs are kept per plan: a new key
// evicts the least recently replayed graph (after its last replay finished),
// so callers that vary dt or rotate state buffers do not accumulate graphs.
template <typename Body>
static int replay_cached(pii_plan* plan, const GraphKey& key, cudaStream_t s, Body body) {
  auto it = plan->graphs.find(key);
  if (it == plan->graphs.end()) {
    while (plan->graphs.size() >= kMaxGraphs) {
      auto lru = plan->graphs.begin();
      for (auto j = plan->graphs.begin(); j != plan->graphs.end(); ++j)
        if (j->second.last_use < lru->second.last_use) lru = j;
      graph_entry_destroy(lru->second);
      plan->graphs.erase(lru);
    }
    PII_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int64_t before = g_launches.load();
    int st = body();
    const int64_t captured = g_launches.load() - before;
    g_launches.fetch_sub(captured);  // captured, not executed
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != PII_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) {
      set_error("graph capture: %s", cudaGetErrorString(e));
      return PII_ERR_CUDA;
    }
    GraphEntry ge;
    ge.graph = g;
    ge.kernels = captured;
    e = cudaGraphInstantiate(&ge.exec, g, 0);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ge.done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      graph_entry_destroy(ge);
      set_error("graph instantiate: %s", cudaGetErrorString(e));
      return PII_ERR_CUDA;
    }
    it = plan->graphs.emplace(key, ge).first;
  }
  it->second.last_use = ++plan->graph_tick;
  PII_CUDA(cudaGraphLaunch(it->second.exec, s));
  PII_CUDA(cudaEventRecord(it->second.done, s));
  g_launches.fetch_add(it->second.kernels);
  return PII_OK;
}

}  // namespace pii

extern "C" {

int pii_step_splitting(pii_plan* plan, int integrator, double* f, int64_t nx, double dt, double dx,
                       const double* v1, int bc_lower, int bc_upper, double kn, double penalty, double e,
                       double tau, int with_loss, int mass_fix, int use_graph, void* stream) {
  if (!plan || !f || nx <= 0 || !v1 || !(kn > 0) || !(dt > 0)) {
    pii::set_error("pii_step_splitting: invalid arguments");
    return PII_ERR_ARG;
  }
  if (integrator != PII_INT_CONSP && integrator != PII_INT_CONSP_M) {
    pii::set_error("This time integrator is not implemented.");
    return PII_ERR_ARG;
  }
  if (!penalty) {
    pii::set_error("The penalty parameter is not given. Please specify it!");
    return PII_ERR_ARG;
  }
  if (integrator == PII_INT_CONSP_M && (!e || !(e * e < 1.0))) {
    pii::set_error("The penalty parameter, e or tau are not given. Please specify it!");
    return PII_ERR_ARG;
  }
  if (nx > plan->batch_max) {
    pii::set_error("pii_step_splitting: nx beyond batch_max");
    return PII_ERR_SIZE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  if (dx > 0) PII_TRY(pii::check_bcs(bc_lower, bc_upper));
  PII_TRY(pii::upload_v1(plan, v1, s));
  const double delta = v1[1] - v1[0];
  plan->delta3 = plan->dim == 3 ? delta * delta * delta : delta * delta;  // velocity cell volume
  PII_TRY(pii::dft_stall_check(plan));  // a stall of an earlier launch on this plan
  pii::StepCtx c{plan, f, nx, dx, kn, bc_lower, bc_upper, with_loss, mass_fix, s};
  if (!use_graph || s == nullptr || plan->prof) return pii::splitting_body(c, integrator, dt, penalty, e, tau);
  pii::GraphKey key{integrator, f, nx, dt, dx, kn, bc_lower, bc_upper, with_loss, mass_fix, 0,
                    {0, 0, 0}, {penalty, e, tau}, stream};
  return pii::replay_cached(plan, key, s, [&] { return pii::splitting_body(c, integrator, dt, penalty, e, tau); });
}


int pii_boltzmann_df(pii_plan* plan, const double* f, double* df, int64_t nx, double dt, double dx,
                     const double* v1, int bc_lower, int bc_upper, double kn, int with_loss, int mass_fix,
                     void* stream) {
  if (!plan || !f || !df || nx <= 0 || !(kn > 0)) {
    pii::set_error("pii_boltzmann_df: invalid arguments");
    return PII_ERR_ARG;
  }
  if (nx > plan->batch_max) {
    pii::set_error("pii_boltzmann_df: nx beyond batch_max");
    return PII_ERR_SIZE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  if (dx > 0) {
    PII_TRY(pii::check_bcs(bc_lower, bc_upper));
    PII_TRY(pii::upload_v1(plan, v1, s));
  }
  PII_TRY(pii::collide_impl(plan, f, plan->q, nx, with_loss, 0.0, mass_fix, s));
  return pii::transport_impl(plan, f, plan->q, df, nx, dt, dx, bc_lower, bc_upper, kn, s);
}

int pii_step(pii_plan* plan, int integrator, double* f, int64_t nx, double dt, const int* inner_steps,
             const double* inner_dt, int levels, double dx, const double* v1, int bc_lower, int bc_upper,
             double kn, int with_loss, int mass_fix, int use_graph, void* stream) {
  PII_TRY(pii::validate(plan, integrator, f, nx, inner_steps, inner_dt, levels));
  if (!(kn > 0) || !(dt > 0)) {
    pii::set_error("pii_step: dt and kn must be > 0");
    return PII_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  if (dx > 0) {
    PII_TRY(pii::check_bcs(bc_lower, bc_upper));
    PII_TRY(pii::upload_v1(plan, v1, s));
  }
  pii::StepCtx c{plan, f, nx, dx, kn, bc_lower, bc_upper, with_loss, mass_fix, s};
  int K[3] = {0, 0, 0};
  double h[3] = {0, 0, 0};
  const int need = integrator == PII_INT_PFE ? 1 : integrator == PII_INT_TPI2 ? 2 : integrator == PII_INT_TPI3 ? 3 : 0;
  for (int l = 0; l < need; ++l) {
    K[l] = inner_steps[l];
    h[l] = inner_dt[l];
  }
  PII_TRY(pii::dft_stall_check(plan));  // a stall of an earlier launch on this plan
  if (!use_graph || s == nullptr || plan->prof) return pii::step_body(c, integrator, dt, K, h);

  pii::GraphKey key{integrator, f, nx, dt, dx, kn, bc_lower, bc_upper, with_loss, mass_fix, need,
                    {K[0], K[1], K[2]}, {h[0], h[1], h[2]}, stream};
  return pii::replay_cached(plan, key, s, [&] { return pii::step_body(c, integrator, dt, K, h); });
}

int64_t pii_plan_graph_count(const pii_plan* plan) { return plan ? int64_t(plan->graphs.size()) : -1; }

}  // extern "C"
