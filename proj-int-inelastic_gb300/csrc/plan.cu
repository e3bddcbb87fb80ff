// Plan construction: quadrature tables in FP64 on the host, uploaded once in
// the working precision; workspace sized for batch_max cells.
//
// Tables follow FSInelasticVHSCollision.perform_precomputation
// (src/collision/inelastic_collisions.py:57-137), factored so that nothing of
// size n_r * n_sigma * n^3 is stored:
//   exp(-i pi r k.sigma / L) = prod_d exp(-i pi r sigma_d k_d / L)   (per-axis rows)
//   exp(+i a(r) r k.sigma)    = prod_d exp(+i a(r) r sigma_d k_d)    (per-axis rows)
//   sinc(a(r) r |k|), sinc(pi r |k| / L) depend on |k|^2 = m only  (tables over m)
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include <utility>

#include "pii_internal.cuh"

namespace pii {

static_assert(ST_COUNT == PII_NSTAGES, "profiling stages out of step with the C ABI");

static thread_local char g_err[1024] = "";
std::atomic<int64_t> g_launches{0};

StageTimer::StageTimer(pii_plan* p_, int stage_, cudaStream_t s_) : p(p_), stage(stage_), s(s_) {
  if (!p || !p->prof) return;
  if (p->prof_pool.size() < 2) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) == cudaSuccess) p->prof_pool.push_back(e);
    }
    if (p->prof_pool.size() < 2) return;
  }
  a = p->prof_pool.back();
  p->prof_pool.pop_back();
  b = p->prof_pool.back();
  p->prof_pool.pop_back();
  cudaEventRecord(a, s);
}

StageTimer::~StageTimer() {
  if (!a) return;
  cudaEventRecord(b, s);
  p->prof_events.push_back(ProfEvent{stage, a, b});
}

static void prof_resolve(pii_plan* p) {
  if (p->prof_events.empty()) return;
  cudaDeviceSynchronize();
  for (auto& e : p->prof_events) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
      p->prof_ms[e.stage] += ms;
      p->prof_n[e.stage] += 1;
    }
    p->prof_pool.push_back(e.a);
    p->prof_pool.push_back(e.b);
  }
  p->prof_events.clear();
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

bool GraphKey::operator<(const GraphKey& o) const {
  return std::tie(integrator, f, nx, dt, dx, kn, bc_lo, bc_hi, with_loss, mass_fix, levels, K[0], K[1], K[2],
                  h[0], h[1], h[2], stream) <
         std::tie(o.integrator, o.f, o.nx, o.dt, o.dx, o.kn, o.bc_lo, o.bc_hi, o.with_loss, o.mass_fix,
                  o.levels, o.K[0], o.K[1], o.K[2], o.h[0], o.h[1], o.h[2], o.stream);
}

void graph_entry_destroy(GraphEntry& g) {
  if (g.done) {
    cudaEventSynchronize(g.done);  // its last replay has finished
    cudaEventDestroy(g.done);
  }
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g = GraphEntry{};
}

void graphs_clear(pii_plan* p) {
  for (auto& kv : p->graphs) graph_entry_destroy(kv.second);
  p->graphs.clear();
}

static double sinc(double x) { return x == 0.0 ? 1.0 : std::sin(x) / x; }

// J_0(x) = (1/pi) int_0^pi cos(x sin t) dt by the trapezoidal rule, which
// converges geometrically for this periodic integrand once the node count
// exceeds ~x (64 + 2 ceil|x| nodes: |error| < 3e-15 up to x = 200 against
// scipy.special.jv(0, x), the reference's kernel, inelastic_collisions.py:42-43)
static double bessel_j0(double x) {
  const double pi = 3.141592653589793238462643383279502884;
  x = std::fabs(x);
  const int nodes = 64 + 2 * int(std::ceil(x));
  const double h = pi / nodes;
  double s = 1.0;  // (f(0) + f(pi)) / 2, f(0) = f(pi) = 1
  for (int k = 1; k < nodes; ++k) s += std::cos(x * std::sin(k * h));
  return s / nodes;
}

// Tables that do not depend on the restitution law: the phase rows of the
// reference's exp table, the a-parity phase rows, the loss and Laplacian
// factors (src/collision/inelastic_collisions.py:62-69,105-114)
template <typename T>
static int upload_shared_tables(pii_plan* p) {
  const int n = p->n, nr = p->nr, ns = p->ns, Q = p->Q, dim = p->dim;
  const int M = dim * (n / 2) * (n / 2);
  p->tab.M = M;
  const double pi = 3.141592653589793238462643383279502884;
  // per-axis rows: always 3 per pair (the 2D operator leaves the third unused)
  std::vector<T> eph(size_t(Q) * 3 * n * 2, T(0));
  std::vector<T> lk(M + 1), lp(M + 1);
  const double invN = 1.0 / double(p->N);
  // sphere (circle) constant 2 pi^{d/2} / Gamma(d/2): 4 pi in 3D, 2 pi in 2D (:50-52)
  const double sphr = dim == 3 ? 4.0 * pi : 2.0 * pi;
  // radial kernel sp_func: sin(x)/x in 3D, J_0 in 2D (:42-45)
  auto kern = [dim](double x) { return dim == 3 ? sinc(x) : bessel_j0(x); };
  std::vector<double> lk_d(M + 1, 0.0);
  for (int ir = 0; ir < nr; ++ir) {
    const double r = p->r[ir], wr = p->wr[ir];
    const double rg = std::pow(r, p->gamma + dim - 1.0);  // pre_fac(r) / sphr  (:54-55)
    for (int m = 0; m <= M; ++m) lk_d[m] += sphr * rg * wr * kern(pi * r * std::sqrt(double(m)) / p->L);  // loss
    for (int is = 0; is < ns; ++is) {
      const int pair = ir * ns + is;
      for (int d = 0; d < dim; ++d) {
        const double sd = p->sigma[size_t(is) * dim + d];
        for (int i = 0; i < n; ++i) {
          const int k = i < n / 2 ? i : i - n;
          const double th_e = -pi * r * sd * double(k) / p->L;
          const double sc = (d == 0) ? invN : 1.0;
          const size_t o = ((size_t(pair) * 3 + d) * n + i) * 2;
          eph[o] = T(sc * std::cos(th_e));
          eph[o + 1] = T(sc * std::sin(th_e));
        }
      }
    }
  }
  auto up = [&](void** dst, const void* src, size_t bytes) -> int {
    PII_CUDA(cudaMalloc(dst, bytes));
    PII_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    p->bytes += int64_t(bytes);
    return PII_OK;
  };
  if (std::is_same<T, float>::value && n == 32 && dim == 3) {
    // a-parity phase rows: the first-axis rows with the radix-2 twiddles of the
    // parity split folded in, evaluated in FP64 (angles reduced exactly)
    std::vector<T> ep2(size_t(Q) * 2 * 32 * 2);
    for (int ir = 0; ir < nr; ++ir) {
      const double r = p->r[ir];
      for (int is = 0; is < ns; ++is) {
        const int pair = ir * ns + is;
        const double sd = p->sigma[size_t(is) * 3];
        for (int par = 0; par < 2; ++par)
          for (int k = 0; k < 32; ++k) {
            const size_t o = ((size_t(pair) * 2 + par) * 32 + k) * 2;
            // epar: k < 16 pairs e_a[k], k >= 16 pairs e_a[k] with the sign (-1)^p
            const int kk = k & 15;
            const int ks = k < 16 ? k : k - 32;
            const double th_e = -pi * r * sd * double(ks) / p->L + 2.0 * pi * double(par * kk) / 32.0 +
                                (k >= 16 && par ? pi : 0.0);
            ep2[o] = T(invN * std::cos(th_e));
            ep2[o + 1] = T(invN * std::sin(th_e));
          }
      }
    }
    PII_TRY(up(&p->tab.epar, ep2.data(), ep2.size() * sizeof(T)));
  }
  for (int m = 0; m <= M; ++m) {
    lk[m] = T(lk_d[m]);
    lp[m] = T(-pi * pi / (p->L * p->L) * double(m));  // (:69)
  }
  PII_TRY(up(&p->tab.ephase, eph.data(), eph.size() * sizeof(T)));
  PII_TRY(up(&p->tab.lossk, lk.data(), lk.size() * sizeof(T)));
  PII_TRY(up(&p->tab.lapl, lp.data(), lp.size() * sizeof(T)));
  return PII_OK;
}

// Tables of the gain that depend on the restitution law through
// a(r) = pi (1 + e(r)) / (4 L), e(r) = (e0 - e) tanh(r - R / 2) / 2 + (e0 + e) / 2
// (src/collision/inelastic_collisions.py:77-103): the gain phase rows, the
// radial sinc table and, for the fused n = 32 kernels, their derived forms.
// One set per (e, e0) of `sets`, stored set after set; the strides are the
// elements per set when there is more than one set (cell c then uses set c)
// and 0 otherwise.
template <typename T>
static int upload_gain_tables(pii_plan* p, const std::vector<std::pair<double, double>>& sets) {
  const int n = p->n, nr = p->nr, ns = p->ns, Q = p->Q, dim = p->dim;
  const int M = dim * (n / 2) * (n / 2);
  const size_t S = sets.size();
  const double pi = 3.141592653589793238462643383279502884;
  auto kern = [dim](double x) { return dim == 3 ? sinc(x) : bessel_j0(x); };
  const size_t gph_set = size_t(Q) * 3 * n, gs_set = size_t(nr) * (M + 1);
  std::vector<T> gph(S * gph_set * 2, T(0)), gs(S * gs_set);
  const bool fused = std::is_same<T, float>::value && n == 32 && dim == 3;
  const size_t gp2_set = size_t(Q) * 2 * 32, gsx_set = size_t(nr) * 513 * 20, gsxc_set = size_t(nr) * 153 * 17;
  std::vector<T> gp2, gsx, gsxc;
  if (p->tab.gphase) {  // replacing earlier sets: their bytes leave the plan's count
    const size_t old = size_t(p->tab.nsets) * (gph_set * 2 + gs_set + (fused ? gp2_set * 2 + gsx_set + gsxc_set : 0));
    p->bytes -= int64_t(old * sizeof(T));
  }
  if (fused) {
    gp2.assign(S * gp2_set * 2, T(0));
    gsx.assign(S * gsx_set, T(0));
    gsxc.assign(S * gsxc_set, T(0));
  }
  for (size_t st = 0; st < S; ++st) {
    const double e = sets[st].first, e0 = sets[st].second;
    T* gphs = gph.data() + st * gph_set * 2;
    T* gss = gs.data() + st * gs_set;
    for (int ir = 0; ir < nr; ++ir) {
      const double r = p->r[ir], wr = p->wr[ir];
      // restitution law and exponential factor (inelastic_collisions.py:77-80)
      const double er = 0.5 * (e0 - e) * std::tanh(r - 0.5 * p->R) + 0.5 * (e0 + e);
      const double afac = 0.25 * pi * (1.0 + er) / p->L;
      const double rg = std::pow(r, p->gamma + dim - 1.0);  // pre_fac(r) / sphr  (:54-55)
      for (int m = 0; m <= M; ++m)
        gss[size_t(ir) * (M + 1) + m] = T(rg * wr * p->wsigma * kern(afac * r * std::sqrt(double(m))));
      for (int is = 0; is < ns; ++is) {
        const int pair = ir * ns + is;
        for (int d = 0; d < dim; ++d) {
          const double sd = p->sigma[size_t(is) * dim + d];
          for (int i = 0; i < n; ++i) {
            const int k = i < n / 2 ? i : i - n;
            const double th_g = afac * r * sd * double(k);
            const size_t o = ((size_t(pair) * 3 + d) * n + i) * 2;
            gphs[o] = T(std::cos(th_g));
            gphs[o + 1] = T(std::sin(th_g));
          }
        }
        if (fused) {
          // a-parity gain rows (the radix-2 twiddles of the parity split folded in)
          const double sd = p->sigma[size_t(is) * 3];
          T* g2 = gp2.data() + st * gp2_set * 2;
          for (int par = 0; par < 2; ++par)
            for (int k = 0; k < 32; ++k) {
              const size_t o = ((size_t(pair) * 2 + par) * 32 + k) * 2;
              const int ks = k < 16 ? k : k - 32;
              const double th_g = afac * r * sd * double(ks) - 2.0 * pi * double(par * k) / 32.0;
              g2[o] = T(std::cos(th_g));
              g2[o + 1] = T(std::sin(th_g));
            }
        }
      }
    }
    if (fused) {
      // per-column rows of the radial sinc table: gsinc[r][m_bc + q^2], q = |k_a| <= 16
      T* gx = gsx.data() + st * gsx_set;
      for (int ir = 0; ir < nr; ++ir)
        for (int mbc = 0; mbc <= 512; ++mbc)
          for (int q = 0; q <= 16 && mbc + q * q <= M; ++q)
            gx[(size_t(ir) * 513 + mbc) * 20 + q] = gss[size_t(ir) * (M + 1) + mbc + q * q];
      // the same by (|k_b|, |k_c|) pair, u = min <= v = max (index v (v + 1) / 2 + u, 153
      // pairs), 17 values q = 0..16: one radial node's slab is 10.4 KB (shared memory)
      T* gc = gsxc.data() + st * gsxc_set;
      for (int ir = 0; ir < nr; ++ir)
        for (int v = 0; v <= 16; ++v)
          for (int u = 0; u <= v; ++u)
            for (int q = 0; q <= 16; ++q)
              gc[(size_t(ir) * 153 + v * (v + 1) / 2 + u) * 17 + q] = gss[size_t(ir) * (M + 1) + u * u + v * v + q * q];
    }
  }
  auto up = [&](void** dst, const void* src, size_t bytes) -> int {
    if (*dst) {
      cudaFree(*dst);
      *dst = nullptr;
    }
    PII_CUDA(cudaMalloc(dst, bytes));
    PII_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    p->bytes += int64_t(bytes);
    return PII_OK;
  };
  PII_TRY(up(&p->tab.gphase, gph.data(), gph.size() * sizeof(T)));
  PII_TRY(up(&p->tab.gsinc, gs.data(), gs.size() * sizeof(T)));
  if (fused) {
    PII_TRY(up(&p->tab.gpar, gp2.data(), gp2.size() * sizeof(T)));
    PII_TRY(up(&p->tab.gsx, gsx.data(), gsx.size() * sizeof(T)));
    PII_TRY(up(&p->tab.gsxc, gsxc.data(), gsxc.size() * sizeof(T)));
  }
  const bool per_cell = S > 1;
  p->tab.nsets = int64_t(S);
  p->tab.gph_stride = per_cell ? int64_t(gph_set) : 0;
  p->tab.gs_stride = per_cell ? int64_t(gs_set) : 0;
  p->tab.gpar_stride = per_cell && fused ? int64_t(gp2_set) : 0;
  p->tab.gsx_stride = per_cell && fused ? int64_t(gsx_set) : 0;
  p->tab.gsxc_stride = per_cell && fused ? int64_t(gsxc_set) : 0;
  return PII_OK;
}

template <typename T>
static int upload_tables(pii_plan* p) {
  PII_TRY(upload_shared_tables<T>(p));
  return upload_gain_tables<T>(p, {{p->e, p->e0}});
}

// Antipodal passes: the symmetric designs list every direction with its
// negative, whose phase and gain tables are the conjugates
// (src/collision/inelastic_collisions.py:86-105: k . sigma changes sign).  One
// representative pair (ir, i < mate(i)) per antipodal pair and radial node, in
// radial-node order; none when the design is not antipodally symmetric.
static int antipodal_setup(pii_plan* p) {
  const int ns = p->ns;
  std::vector<int> mate(ns, -1);
  bool sym = p->dim == 3 && ns % 2 == 0;
  for (int i = 0; i < ns && sym; ++i) {
    for (int j = 0; j < ns; ++j) {
      double d = 0;
      for (int k = 0; k < 3; ++k) d = std::max(d, std::fabs(p->sigma[3 * i + k] + p->sigma[3 * j + k]));
      if (d < 1e-12) {
        mate[i] = j;
        break;
      }
    }
    sym = mate[i] >= 0 && mate[i] != i;
  }
  if (!sym) return PII_OK;
  std::vector<int> reps;
  for (int ir = 0; ir < p->nr; ++ir)
    for (int i = 0; i < ns; ++i)
      if (i < mate[i]) reps.push_back(ir * ns + i);
  if (int(reps.size()) * 2 != p->Q) return PII_OK;
  PII_CUDA(cudaMalloc(&p->ap_reps, reps.size() * sizeof(int)));
  PII_CUDA(cudaMemcpy(p->ap_reps, reps.data(), reps.size() * sizeof(int), cudaMemcpyHostToDevice));
  p->bytes += int64_t(reps.size() * sizeof(int));
  p->ap_count = int(reps.size());
  return PII_OK;
}

static int alloc(pii_plan* p, void** dst, size_t bytes) {
  PII_CUDA(cudaMalloc(dst, bytes));
  p->bytes += int64_t(bytes);
  return PII_OK;
}

static void free_plan(pii_plan* p) {
  if (!p) return;
  prof_resolve(p);
  for (cudaEvent_t e : p->prof_pool) cudaEventDestroy(e);
  graphs_clear(p);
  void* ptrs[] = {p->tab.ephase, p->tab.gphase, p->tab.epar, p->tab.gpar, p->tab.gsx, p->tab.gsxc, p->tab.gsinc, p->tab.lossk, p->tab.lapl, p->fhat, p->fT,
                  p->G,          p->buf,        p->q,         p->d0,        p->d1,       p->d2,  p->v1dev,
                  p->gc_maps,    p->gc_hpart,   p->gp_hpart,  p->ap_reps,   p->nq_part,  p->mom,       p->flag,
                  p->dft_img,    p->dft_gs,     p->dft_colb,  p->nq_ft2,    p->nq_fhn,
                  p->nq_A,       p->nq_B,       p->nq_fhT,    p->nq_qpart,  p->fz_part};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (p->dft_err_host) cudaFreeHost(p->dft_err_host);
  if (p->side_fork) cudaEventDestroy(p->side_fork);
  if (p->side_join) cudaEventDestroy(p->side_join);
  if (p->side) cudaStreamDestroy(p->side);
  delete p;
}

static int create(pii_plan** out, int dim, int n, int nr, int ns, const double* r, const double* wr,
                  const double* sigma, double wsigma, double L, double R, double e, double e0, double gamma,
                  int precision, int64_t batch_max, int device) {
  if (!out) {
    set_error("pii_plan_create: out is NULL");
    return PII_ERR_ARG;
  }
  *out = nullptr;
  if (dim != 2 && dim != 3) {
    set_error("pii_plan_create: Dimension must be 2 or 3.");
    return PII_ERR_ARG;
  }
  if (!(n == 8 || n == 16 || n == 24 || n == 32 || n == 48 || n == 64)) {
    set_error("pii_plan_create: n = %d unsupported (8, 16, 24, 32, 48, 64)", n);
    return PII_ERR_ARG;
  }
  if (nr <= 0 || ns <= 0 || !r || !wr || !sigma || batch_max <= 0 || !(L > 0) || !(R > 0)) {
    set_error("pii_plan_create: invalid quadrature / domain arguments");
    return PII_ERR_ARG;
  }
  if (precision != PII_PREC_FP32 && precision != PII_PREC_FP64) {
    set_error("pii_plan_create: precision must be PII_PREC_FP32 or PII_PREC_FP64");
    return PII_ERR_ARG;
  }
  PII_CUDA(cudaSetDevice(device));
  pii_plan* p = new pii_plan();
  p->n = n;
  p->nr = nr;
  p->ns = ns;
  p->Q = nr * ns;
  p->dim = dim;
  p->N = dim == 3 ? int64_t(n) * n * n : int64_t(n) * n;
  p->precision = precision;
  p->device = device;
  p->L = L;
  p->R = R;
  p->e = e;
  p->e0 = e0;
  p->gamma = gamma;
  p->wsigma = wsigma;
  p->batch_max = batch_max;
  p->r.assign(r, r + nr);
  p->wr.assign(wr, wr + nr);
  p->sigma.assign(sigma, sigma + size_t(ns) * dim);
  int st = precision == PII_PREC_FP32 ? upload_tables<float>(p) : upload_tables<double>(p);
  if (st != PII_OK) {
    free_plan(p);
    return st;
  }
  const size_t rs = precision == PII_PREC_FP32 ? 4 : 8;
  const size_t cs = 2 * rs;
  const size_t N = size_t(p->N);
  // L2-resident chunk of (cell, pair) items: ~48 MB, at least 2 items; 76 MB
  // (38 items) for the n = 64 FP32 plans, whose tensor-core column pass then
  // gives each of 152 SMs 8 whole tiles per launch (measured: 48 MB -> 91.1,
  // 80 MB -> 94.1, 96 MB -> 81.4 cell-evals/s; beyond ~80 MB the chunk no
  // longer stays in the 126 MB L2 next to f^, f and G)
  const size_t target = size_t(n == 64 && precision == PII_PREC_FP32 && dim == 3 ? 76 : 48) << 20;
  p->chunk_items = std::max<int64_t>(2, int64_t(target / (N * cs)));
  int s2 = PII_OK;
  if ((s2 = alloc(p, &p->fhat, size_t(batch_max) * N * cs)) != PII_OK ||
      (s2 = alloc(p, &p->fT, size_t(batch_max) * N * rs)) != PII_OK ||
      (s2 = alloc(p, &p->G, size_t(batch_max) * N * cs)) != PII_OK ||
      (s2 = alloc(p, &p->buf, size_t(p->chunk_items) * N * cs)) != PII_OK ||
      (s2 = alloc(p, (void**)&p->q, size_t(batch_max) * N * 8)) != PII_OK ||
      (s2 = alloc(p, (void**)&p->d0, size_t(batch_max) * N * 8)) != PII_OK ||
      (s2 = alloc(p, (void**)&p->v1dev, size_t(n) * 8)) != PII_OK ||
      (s2 = alloc(p, (void**)&p->mom, size_t(batch_max) * 5 * 8)) != PII_OK ||
      (s2 = alloc(p, (void**)&p->flag, 16)) != PII_OK) {  // guard flag + sweep error word
    free_plan(p);
    return s2;
  }
  if ((s2 = prepare_impl(p)) != PII_OK || (s2 = antipodal_setup(p)) != PII_OK) {
    free_plan(p);
    return s2;
  }
  if (n == 32 && precision == PII_PREC_FP32 && dim == 3) {
    if ((s2 = gain_cluster_prepare(p)) != PII_OK || (s2 = gain_parity_prepare(p)) != PII_OK) {
      free_plan(p);
      return s2;
    }
    p->gain_path = p->ap_count > 0 ? 3 : 2;
  }
  if (n == 64 && precision == PII_PREC_FP32 && dim == 3 && (s2 = col_tc_prepare(p)) != PII_OK) {
    free_plan(p);
    return s2;
  }
  if (n != 32 && precision == PII_PREC_FP32 && dim == 3 && p->ap_count > 0) {
    // the packed pipeline: antipodal passes (half the items) plus the general Nyquist correction
    if ((s2 = nyq_gen_prepare(p)) != PII_OK) {
      free_plan(p);
      return s2;
    }
    p->gain_path = 3;
  }
  // the fused gain kernel (one cluster of CTAs per work item) for n = 16, 24, 48, 64
  if ((s2 = gain_fused_prepare(p)) != PII_OK) {
    free_plan(p);
    return s2;
  }
  if (p->fz_clusters > 0 && n != 64) {  // at n = 64 the packed pipeline is faster
    if ((s2 = gain_fused_ensure(p)) != PII_OK) {
      free_plan(p);
      return s2;
    }
    p->gain_path = 4;
  }
  // the Nyquist correction: the quadratic form wherever its kernels fit the
  // memory budget (3.4x to 9x faster than the direct kernels), else the direct
  // kernels
  p->nyq_path = 1;
  if (dim == 3 && p->ap_count > 0) {
    if ((s2 = nyq_quad_prepare(p)) != PII_OK) {
      free_plan(p);
      return s2;
    }
    if (p->nq_A) p->nyq_path = 0;
    // FP64: the packed pipeline (half the passes) wherever its correction is built
    if (precision != PII_PREC_FP32 && p->nq_A) p->gain_path = 3;
  }
  *out = p;
  return PII_OK;
}

}  // namespace pii

extern "C" {

const char* pii_last_error(void) { return pii::g_err; }

const char* pii_version(void) { return "pii_gb300 0.1 (sm_103a)"; }

int pii_plan_create(pii_plan** out, int n, int n_r, int n_sigma, const double* r, const double* w_r,
                    const double* sigma, double w_sigma, double L, double R, double e, double e0,
                    double gamma, int precision, int64_t batch_max, int device) {
  return pii::create(out, 3, n, n_r, n_sigma, r, w_r, sigma, w_sigma, L, R, e, e0, gamma, precision, batch_max,
                     device);
}

int pii_plan_create_nd(pii_plan** out, int dim, int n, int n_r, int n_sigma, const double* r, const double* w_r,
                       const double* sigma, double w_sigma, double L, double R, double e, double e0, double gamma,
                       int precision, int64_t batch_max, int device) {
  return pii::create(out, dim, n, n_r, n_sigma, r, w_r, sigma, w_sigma, L, R, e, e0, gamma, precision,
                     batch_max, device);
}

int pii_plan_set_restitution(pii_plan* plan, const double* e, const double* e0, int64_t count) {
  using namespace pii;
  if (!plan || count < 0 || (count > 0 && (!e || !e0))) {
    set_error("pii_plan_set_restitution: invalid arguments");
    return PII_ERR_ARG;
  }
  if (count > plan->batch_max) {
    set_error("pii_plan_set_restitution: %lld restitution sets for a plan of batch_max = %lld", (long long)count,
              (long long)plan->batch_max);
    return PII_ERR_SIZE;
  }
  if (count > 1 && plan->dim != 3) {
    set_error("pii_plan_set_restitution: per-cell restitution exists for 3D-velocity plans only");
    return PII_ERR_ARG;
  }
  PII_CUDA(cudaSetDevice(plan->device));
  PII_CUDA(cudaDeviceSynchronize());  // launches in flight may still read the old tables
  std::vector<std::pair<double, double>> sets;
  if (count == 0)
    sets.push_back({plan->e, plan->e0});
  else
    for (int64_t c = 0; c < count; ++c) sets.push_back({e[c], e0[c]});
  int st = plan->precision == PII_PREC_FP32 ? upload_gain_tables<float>(plan, sets)
                                            : upload_gain_tables<double>(plan, sets);
  if (st != PII_OK) return st;
  if (plan->tab.nsets > 1 && plan->gain_path == 1) plan->gain_path = plan->ap_count > 0 ? 3 : 2;
  if (plan->dft_img) PII_TRY(col_tc_gain_tables(plan));  // the tensor-core path's sinc slices
  if (plan->nq_A) {  // A, B per set, rebuilt for the new sets (or dropped beyond the budget)
    PII_TRY(nyq_quad_prepare(plan));
    if (!plan->nq_A) {
      plan->nyq_path = 1;
      // FP64 has no direct correction: back to the unpacked pipeline
      if (plan->precision != PII_PREC_FP32 && plan->gain_path == 3) plan->gain_path = 0;
    }
  }
  graphs_clear(plan);  // captured graphs baked the old tables in
  return PII_OK;
}

int pii_plan_dim(const pii_plan* plan) { return plan ? plan->dim : -1; }

int pii_plan_destroy(pii_plan* plan) {
  if (!plan) {
    pii::set_error("pii_plan_destroy: NULL plan");
    return PII_ERR_ARG;
  }
  cudaSetDevice(plan->device);
  pii::free_plan(plan);
  return PII_OK;
}

int64_t pii_plan_workspace_bytes(const pii_plan* plan) { return plan ? plan->bytes : -1; }

int64_t pii_kernel_launches(void) { return pii::g_launches.load(); }

int pii_plan_profile(pii_plan* plan, int enable) {
  if (!plan) {
    pii::set_error("pii_plan_profile: NULL plan");
    return PII_ERR_ARG;
  }
  if (!enable) pii::prof_resolve(plan);
  plan->prof = enable != 0;
  return PII_OK;
}

int pii_plan_profile_read(pii_plan* plan, double* ms, int64_t* launches) {
  if (!plan || !ms || !launches) {
    pii::set_error("pii_plan_profile_read: NULL argument");
    return PII_ERR_ARG;
  }
  pii::prof_resolve(plan);
  for (int i = 0; i < pii::ST_COUNT; ++i) {
    ms[i] = plan->prof_ms[i];
    launches[i] = plan->prof_n[i];
    plan->prof_ms[i] = 0;
    plan->prof_n[i] = 0;
  }
  return PII_OK;
}

}  // extern "C"
