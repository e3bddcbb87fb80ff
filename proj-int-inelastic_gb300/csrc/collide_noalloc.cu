// pii_collide_noalloc: Q(f,f) for small velocity grids without allocating.
//
// Who needs it: callers that may not call cudaMalloc at the point where they
// want a collision evaluation.  Examples: a host framework that hands out
// device memory only through its own pool and forbids raw cudaMalloc (its
// pool already holds the memory, so a raw allocation can fail or fragment
// it); an embedded time loop with a fixed memory budget decided at start-up;
// code that must not stall the device, since cudaMalloc and cudaFree may
// synchronise it.  pii_plan_create allocates its tables and workspace with
// cudaMalloc, so those callers cannot use it.
//
// What it does instead: the tables, spectra and the chunk buffer of the
// operator live in one file-scope device array (g_noalloc_scratch below) that
// is part of the library image.  Every GPU that loads the library reserves it
// (PII_NOALLOC_SCRATCH_BYTES) until the process exits.  The caller passes f
// and q; nothing else is allocated, on the device or on the host.  The
// quadrature (r, w_r, sigma) travels by value in the table kernel's launch
// parameters, so a call makes no host-to-device copy either.
//
// Limits (checked, PII_ERR_SIZE otherwise): n in {8, 16}, cells <= 8,
// n_r <= 32, n_sigma <= 192, n_r * n_sigma <= 1024.  FP32 arithmetic (the
// mixed-precision path), no heat bath, no mass fix.
//
// Shared state: all calls on one device share the array and it keeps the
// previous call's contents.  Every region is completely written by a call
// before that call reads it (tables, f^, f, the chunk items, and G, which the
// first chunk assigns rather than accumulates), so nothing has to start at
// zero.  Calls whose GPU work overlaps -- on two streams, or from two host
// threads -- race on the array and give wrong results; serialise them.
//
// Set-up: the first call on a device (with that device current) resolves the
// device address of the array with cudaGetSymbolAddress; the host-side name of
// a __device__ array is not a device address and must never be passed to a
// kernel.  The address is kept per device ordinal for the life of the
// process: cudaDeviceReset between calls is not supported (the module is
// reloaded and the kept address may no longer be valid).
#include <algorithm>
#include <cmath>
#include <mutex>

#include "pii_internal.cuh"

namespace pii {

#define PII_NOALLOC_SCRATCH_BYTES (size_t(5) << 19)  // 2.5 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[PII_NOALLOC_SCRATCH_BYTES];

static constexpr int kNoallocMaxDevices = 64;
static void* g_noalloc_ptr[kNoallocMaxDevices] = {nullptr};
static std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device (resolved once).
static int noalloc_scratch(void** out) {
  int dev = 0;
  PII_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    set_error("pii_collide_noalloc: device ordinal %d beyond %d", dev, kNoallocMaxDevices);
    return PII_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    PII_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return PII_OK;
}

// The quadrature at its largest (n_r <= 32, n_sigma <= 192): 5 KB, passed by
// value as a launch parameter (within the 32 KB parameter limit of sm_70+).
struct NoallocQuad {
  double r[32];
  double wr[32];
  double sigma[192 * 3];
};

// Tables of the plan (same definitions as pii_plan_create), evaluated in FP64
// on the device and rounded to FP32.
__global__ void k_noalloc_tables(const NoallocQuad quad, int nr, int ns, int n, double L, double R, double e,
                                 double e0, double gamma, double wsigma, float2* eph, float2* gph, float* gs,
                                 float* lk, float* lp) {
  const double* r = quad.r;
  const double* wr = quad.wr;
  const double* sigma = quad.sigma;
  const double pi = 3.141592653589793238462643383279502884;
  const int M = 3 * (n / 2) * (n / 2);
  const int64_t nphase = int64_t(nr) * ns * 3 * n;
  const int64_t nsinc = int64_t(nr) * (M + 1);
  const int64_t total = nphase + nsinc + (M + 1);
  const double invN = 1.0 / (double(n) * n * n);
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    if (t < nphase) {
      const int i = int(t % n);
      const int d = int((t / n) % 3);
      const int64_t pair = t / (3 * n);
      const int ir = int(pair / ns), is = int(pair % ns);
      const double rr = r[ir];
      const double er = 0.5 * (e0 - e) * tanh(rr - 0.5 * R) + 0.5 * (e0 + e);
      const double afac = 0.25 * pi * (1.0 + er) / L;
      const int k = i < n / 2 ? i : i - n;
      const double sd = sigma[is * 3 + d];
      double s1, c1, s2, c2;
      sincos(-pi * rr * sd * double(k) / L, &s1, &c1);
      sincos(afac * rr * sd * double(k), &s2, &c2);
      const double sc = d == 0 ? invN : 1.0;
      eph[t] = make_float2(float(sc * c1), float(sc * s1));
      gph[t] = make_float2(float(c2), float(s2));
    } else if (t < nphase + nsinc) {
      const int64_t u = t - nphase;
      const int ir = int(u / (M + 1)), m = int(u % (M + 1));
      const double rr = r[ir];
      const double er = 0.5 * (e0 - e) * tanh(rr - 0.5 * R) + 0.5 * (e0 + e);
      const double afac = 0.25 * pi * (1.0 + er) / L;
      const double x = afac * rr * sqrt(double(m));
      gs[u] = float(pow(rr, gamma + 2.0) * wr[ir] * wsigma * (x == 0.0 ? 1.0 : sin(x) / x));
    } else {
      const int m = int(t - nphase - nsinc);
      double acc = 0.0;
      for (int ir = 0; ir < nr; ++ir) {
        const double rr = r[ir];
        const double x = pi * rr * sqrt(double(m)) / L;
        acc += 4.0 * pi * pow(rr, gamma + 2.0) * wr[ir] * (x == 0.0 ? 1.0 : sin(x) / x);
      }
      lk[m] = float(acc);
      lp[m] = float(-pi * pi / (L * L) * double(m));
    }
  }
}

template <int NV>
static int noalloc_run(unsigned char* base, const double* f, double* q, int64_t cells, int nr, int ns,
                       const double* r, const double* wr, const double* sigma, double wsigma, double L, double R,
                       double e, double e0, double gamma, int with_loss, cudaStream_t s) {
  constexpr int64_t N = int64_t(NV) * NV * NV;
  constexpr int M = 3 * (NV / 2) * (NV / 2);
  const int Q = nr * ns;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  float2* eph = reinterpret_cast<float2*>(carve(size_t(Q) * 3 * NV * sizeof(float2)));
  float2* gph = reinterpret_cast<float2*>(carve(size_t(Q) * 3 * NV * sizeof(float2)));
  float* gs = reinterpret_cast<float*>(carve(size_t(nr) * (M + 1) * 4));
  float* lk = reinterpret_cast<float*>(carve(size_t(M + 1) * 4));
  float* lp = reinterpret_cast<float*>(carve(size_t(M + 1) * 4));
  float2* fhat = reinterpret_cast<float2*>(carve(size_t(cells) * N * sizeof(float2)));
  float* fT = reinterpret_cast<float*>(carve(size_t(cells) * N * 4));
  float2* G = reinterpret_cast<float2*>(carve(size_t(cells) * N * sizeof(float2)));
  // the rest of the array is the chunk buffer of (cell, pair) items
  if (off >= PII_NOALLOC_SCRATCH_BYTES) {
    set_error("pii_collide_noalloc: request needs more than the %zu-byte scratch", PII_NOALLOC_SCRATCH_BYTES);
    return PII_ERR_SIZE;
  }
  const int64_t items = int64_t((PII_NOALLOC_SCRATCH_BYTES - off) / (size_t(N) * sizeof(float2)));
  if (items < 2 * cells) {
    set_error("pii_collide_noalloc: scratch too small for %lld cells of n = %d", (long long)cells, NV);
    return PII_ERR_SIZE;
  }
  float2* buf = reinterpret_cast<float2*>(carve(0));

  NoallocQuad quad{};
  std::copy(r, r + nr, quad.r);
  std::copy(wr, wr + nr, quad.wr);
  std::copy(sigma, sigma + size_t(ns) * 3, quad.sigma);
  k_noalloc_tables<<<64, 256, 0, s>>>(quad, nr, ns, NV, L, R, e, e0, gamma, wsigma, eph, gph, gs, lk, lp);
  PII_CHECK_LAUNCH();

  // a plan view onto the scratch: no allocation, no ownership
  pii_plan view;
  view.n = NV;
  view.nr = nr;
  view.ns = ns;
  view.Q = Q;
  view.N = N;
  view.precision = PII_PREC_FP32;
  view.L = L;
  view.R = R;
  view.batch_max = cells;
  view.tab.ephase = eph;
  view.tab.gphase = gph;
  view.tab.gsinc = gs;
  view.tab.lossk = lk;
  view.tab.lapl = lp;
  view.tab.M = M;
  view.fhat = fhat;
  view.fT = fT;
  view.G = G;
  view.buf = buf;
  view.chunk_items = items;
  using K = CollideKernels<float, NV>;
  int st = K::fwd(&view, f, 0, cells, s);
  const int64_t Pc = std::max<int64_t>(1, std::min<int64_t>(Q, items / cells));
  for (int64_t p0 = 0; st == PII_OK && p0 < Q; p0 += Pc)
    st = K::pairs(&view, 0, cells, p0, std::min<int64_t>(Pc, Q - p0), p0 == 0, s);
  if (st == PII_OK) st = K::finish(&view, f, q, 0, cells, with_loss, 0.0, s);
  view.tab = Tables{};  // the view owns nothing
  view.fhat = view.fT = view.G = view.buf = nullptr;
  return st;
}

}  // namespace pii

extern "C" int pii_collide_noalloc(const double* f, double* q, int64_t cells, int n, int n_r, int n_sigma,
                                   const double* r, const double* w_r, const double* sigma, double w_sigma,
                                   double L, double R, double e, double e0, double gamma, int with_loss,
                                   void* stream) {
  using namespace pii;
  if (!f || !q || !r || !w_r || !sigma || f == q || !(L > 0) || !(R > 0)) {
    set_error("pii_collide_noalloc: invalid arguments");
    return PII_ERR_ARG;
  }
  if (!(n == 8 || n == 16) || cells < 1 || cells > 8 || n_r < 1 || n_r > 32 || n_sigma < 1 || n_sigma > 192 ||
      n_r * n_sigma > 1024) {
    set_error(
        "pii_collide_noalloc: n = %d, cells = %lld, n_r = %d, n_sigma = %d outside the static-scratch limits "
        "(n in {8, 16}, cells <= 8, n_r <= 32, n_sigma <= 192, n_r * n_sigma <= 1024); use pii_plan_create",
        n, (long long)cells, n_r, n_sigma);
    return PII_ERR_SIZE;
  }
  void* base = nullptr;
  PII_TRY(noalloc_scratch(&base));
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* b = static_cast<unsigned char*>(base);
  if (n == 8)
    return noalloc_run<8>(b, f, q, cells, n_r, n_sigma, r, w_r, sigma, w_sigma, L, R, e, e0, gamma, with_loss, s);
  return noalloc_run<16>(b, f, q, cells, n_r, n_sigma, r, w_r, sigma, w_sigma, L, R, e, e0, gamma, with_loss, s);
}
