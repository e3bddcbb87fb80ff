// FP64 islands and the transport step:
//   * k_df        : second-order upwind + minmod TVD increment in x, fused with
//                   the collision term  df = transport(f, dt) + dt * Q / kn
//                   (src/boltzmann.py:160-205, src/solver.py:59-105,
//                    src/riemann/advection_1D.py:4-21, src/limiters/tvd.py:6-40)
//   * k_axpy3     : f += s2 * (s1 * (s0 * d))  -- the projective extrapolations
//                   with the reference's rounding order (src/boltzmann.py:120-158)
//   * k_massfix   : per-cell FP64 mean removal of Q (k = 0 mode; not in the reference)
//   * k_moments   : per-cell FP64 sums of f, f v, f |v|^2 / 2
// The state f and every increment are FP64 in every precision mode.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "pii_internal.cuh"

namespace pii {

struct DfArgs {
  const double* f;
  const double* q;  // may be NULL (transport only)
  double* df;
  const double* v1;  // n first-axis velocities
  int64_t nx, N, N2;
  double dt, dtdx, kn;
  int bc_lo, bc_hi, transport;
};

// tvd.limit (src/limiters/tvd.py:6-40): r = (upwind wave u * w) / w^2 (0 where
// w^2 == 0), minmod phi = max(0, min(1, r)), limited wave phi * w.  Written
// without the division (FP64 divisions are software sequences and FP64
// throughput bounds the transport kernel on this part): phi * w is 0 where u
// and w differ in sign (r <= 0), w where |u| >= |w| (r >= 1), else u (r w =
// u up to the rounding of r) -- within 2 ulp of the divided form.  A NaN wave
// gives w, as the divided form does (fmin(1, NaN) = 1).
__device__ __forceinline__ double limited_wave(double w, double wl, double wr, double s) {
  const double u = s > 0.0 ? wl : wr;
  if (w == 0.0 || u * w <= 0.0) return (w == 0.0) ? w : 0.0;
  return fabs(u) < fabs(w) ? u : w;
}

// ghost cell index: extrapolation copies the edge cell, periodic wraps (any nx >= 1)
__device__ __forceinline__ int64_t ghost_cell(int64_t ci, int64_t nx, int bc_lo, int bc_hi) {
  if (ci < 0) {
    if (bc_lo != PII_BC_PERIODIC) return 0;
    while (ci < 0) ci += nx;
  }
  if (ci >= nx) {
    if (bc_hi != PII_BC_PERIODIC) return nx - 1;
    while (ci >= nx) ci -= nx;
  }
  return ci;
}

// One thread per velocity point walks the cells in x with a 5-cell window: each
// f value is loaded once and each interface flux F_{i+1/2} is computed once
// (cell i's right flux is cell i + 1's left flux; the same expressions, so the
// values are those of a per-cell evaluation).  FP64 throughput bounds this
// kernel on this part, so per-point work is what counts.
__global__ void __launch_bounds__(128) k_df(DfArgs a) {
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;  // velocity point
  if (j >= a.N) return;
  const int64_t nx = a.nx, N = a.N;
  if (!a.transport) {
    for (int64_t c = 0; c < nx; ++c) {
      const int64_t gid = c * N + j;
      a.df[gid] = a.q ? a.q[gid] * (a.dt / a.kn) : 0.0;
    }
    return;
  }
  const double s = a.v1[j / a.N2];
  const double dtdx = a.dtdx;
  const double qs = a.dt / a.kn;  // dt Q / kn as Q (dt / kn): a multiply per point, not a division
  const double sabs = fabs(s);
  const double om = 1.0 - sabs * dtdx;
  const double cf = 0.5 * sabs * om;
  const double* fj = a.f + j;
  auto fat = [&](int64_t ci) { return fj[ghost_cell(ci, nx, a.bc_lo, a.bc_hi) * N]; };
  const double fm2 = fat(-2), fm1 = fat(-1), f0 = fj[0];
  double fp1 = fat(1), fp2 = fat(2);
  double wm2 = fm1 - fm2, wm1 = f0 - fm1, w0 = fp1 - f0, wp1 = fp2 - fp1;
  double Fl = cf * limited_wave(wm1, wm2, w0, s);
  for (int64_t c = 0; c < nx; ++c) {
    const int64_t gid = c * N + j;
    double d = -dtdx * (fmin(s, 0.0) * w0 + fmax(s, 0.0) * wm1);
    const double Fr = cf * limited_wave(w0, wm1, wp1, s);
    d -= dtdx * (Fr - Fl);
    if (a.q) d += a.q[gid] * qs;
    a.df[gid] = d;
    if (c + 1 < nx) {  // slide: the waves of cell c + 1 (differences of the same values)
      fp1 = fp2;
      fp2 = fat(c + 3);
      wm2 = wm1;
      wm1 = w0;
      w0 = wp1;
      wp1 = fp2 - fp1;
      Fl = Fr;
    }
  }
}

__global__ void __launch_bounds__(256) k_axpy3(double* f, const double* d, double s0, double s1, double s2,
                                                int64_t count) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double t = s0 * d[i];
  t = s1 * t;
  t = s2 * t;
  f[i] += t;
}

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < NT / 32) r = sh[threadIdx.x];
  if (w == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

__global__ void __launch_bounds__(256) k_massfix(double* q, int64_t N) {
  __shared__ double sh[8];
  __shared__ double mean;
  double* qc = q + int64_t(blockIdx.x) * N;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) s += qc[i];
  s = block_sum<256>(s, sh);
  if (threadIdx.x == 0) mean = s / double(N);
  __syncthreads();
  const double m = mean;
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) qc[i] -= m;
}

// per-cell sums of f, f v1, f v2, f v3 (0 in 2D), f |v|^2 / 2, times dv
__global__ void __launch_bounds__(256) k_moments(const double* f, double* out, const double* v, int n, int dim,
                                                  double dv) {
  __shared__ double sh[8];
  const int64_t N = dim == 3 ? int64_t(n) * n * n : int64_t(n) * n;
  const int64_t slab = N / n;  // points per first-axis index
  const double* fc = f + int64_t(blockIdx.x) * N;
  double m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0;
  for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
    const int a = int(i / slab);
    const int b = dim == 3 ? int((i / n) % n) : int(i % n);
    const double x = fc[i];
    const double va = v[a], vb = v[b], vc = dim == 3 ? v[i % n] : 0.0;
    m0 += x;
    m1 += x * va;
    m2 += x * vb;
    m3 += x * vc;
    m4 += x * (va * va + vb * vb + vc * vc);
  }
  double r[5] = {m0, m1, m2, m3, m4};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double t = block_sum<256>(r[k], sh);
    if (threadIdx.x == 0) out[int64_t(blockIdx.x) * 5 + k] = (k == 4 ? 0.5 * t : t) * dv;
  }
}

// CONSP_M update: f += c Q + c2 (M[rho, u1, T_new] - M[rho, u1, T]) per cell,
// moments from mom.  dim = 2 is the reference's form (src/boltzmann.py:9-13,96-118,
// T = E / rho - |u|^2 / 2 of src/state.py:45-52); dim = 3 its 3D generalisation.
__global__ void __launch_bounds__(256) k_consp_m(double* f, const double* q, const double* mom, const double* v, int n,
                                                  int dim, int64_t count, double c, double c2, double dt, double kn,
                                                  double e, double tau) {
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= count) return;
  const int64_t N = dim == 3 ? int64_t(n) * n * n : int64_t(n) * n;
  const int64_t cell = gid / N;
  const int64_t j = gid - cell * N;
  const double* m = mom + cell * 5;
  const double rho = m[0];
  const double u = m[1] / rho;
  const double ux = m[1] / rho, uy = m[2] / rho, uz = m[3] / rho;
  const double T = (2.0 / dim) * (m[4] / rho - 0.5 * (ux * ux + uy * uy + uz * uz));
  const double ee = 1.0 - e * e;
  const double Tinf = 8.0 * tau / ee;
  const double Tn = (T - Tinf) * exp(-ee / kn / 4.0 * rho * dt) + Tinf;
  const int64_t slab = N / n;
  const double v1 = v[j / slab], v2 = dim == 3 ? v[(j / n) % n] : v[j % n], v3 = dim == 3 ? v[j % n] : 0.0;
  const double d2 = (v1 - u) * (v1 - u) + v2 * v2 + v3 * v3;
  const double pi = 3.141592653589793238462643383279502884;
  const double Mn = dim == 3 ? rho / pow(2.0 * pi * Tn, 1.5) * exp(-d2 / (2.0 * Tn))
                             : rho / (2.0 * pi * Tn) * exp(-d2 / (2.0 * Tn));
  const double Mo = dim == 3 ? rho / pow(2.0 * pi * T, 1.5) * exp(-d2 / (2.0 * T))
                             : rho / (2.0 * pi * T) * exp(-d2 / (2.0 * T));
  f[gid] += c * q[gid] + c2 * (Mn - Mo);
}

// One Gauss-Seidel upwind sweep of BoltzmannFastSweep.step (src/iter_solver.py:38-62)
// for every velocity point j: v1 > 0 runs i = 1 .. nx-2 left to right,
//   f[i] = (nu g[i] + (v1/dx) f[i-1]) / (nu rho[i] + v1/dx),
// v1 < 0 runs i = nx-2 .. 1 right to left with f[i+1] and the signs flipped;
// cells 0 and nx-1 and v1 = 0 points stay.  rho[i] = mom[5 i] (old f), g = the
// collision term of the old f.  max |f_new - f_old| is folded into *errbits
// (the bits of a non-negative double order like the value).
__global__ void __launch_bounds__(256) k_sweep(double* f, const double* g, const double* mom, const double* v1,
                                                int64_t nx, int64_t N, int64_t slab, double dx, double nu,
                                                unsigned long long* errbits) {
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double err = 0.0;
  if (j < N && nx > 2) {
    const double v = v1[j / slab];
    const double vdx = v / dx;
    if (v > 0.0) {
      double prev = f[j];
      for (int64_t i = 1; i < nx - 1; ++i) {
        const double old = f[i * N + j];
        const double nw = (nu * g[i * N + j] + vdx * prev) / (nu * mom[i * 5] + vdx);
        f[i * N + j] = nw;
        err = fmax(err, fabs(nw - old));
        prev = nw;
      }
    } else if (v < 0.0) {
      double prev = f[(nx - 1) * N + j];
      for (int64_t i = nx - 2; i >= 1; --i) {
        const double old = f[i * N + j];
        const double nw = (nu * g[i * N + j] - vdx * prev) / (nu * mom[i * 5] - vdx);
        f[i * N + j] = nw;
        err = fmax(err, fabs(nw - old));
        prev = nw;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_down_sync(0xffffffffu, err, o));
  if ((threadIdx.x & 31) == 0 && err > 0.0) atomicMax(errbits, static_cast<unsigned long long>(__double_as_longlong(err)));
}

__global__ void __launch_bounds__(256) k_nonfinite(const double* f, int64_t count, int* flag) {
  int bad = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
    bad |= !isfinite(f[i]);
  bad = __syncthreads_or(bad);
  if (bad && threadIdx.x == 0) atomicOr(flag, 1);
}

int consp_m_impl(pii_plan* p, double* f, const double* q, int64_t cells, double c, double c2, double dt, double kn,
                 double e, double tau, cudaStream_t s) {
  const int64_t count = cells * p->N;
  {
    StageTimer st(p, ST_AXPY, s);
    k_moments<<<unsigned(cells), 256, 0, s>>>(f, p->mom, p->v1dev, p->n, p->dim, p->delta3);
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_AXPY, s);
    k_consp_m<<<unsigned((count + 255) / 256), 256, 0, s>>>(f, q, p->mom, p->v1dev, p->n, p->dim, count, c, c2, dt,
                                                            kn, e, tau);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int transport_impl(pii_plan* p, const double* f, const double* q, double* df, int64_t nx, double dt, double dx,
                   int bc_lo, int bc_hi, double kn, cudaStream_t s) {
  DfArgs a{};
  a.f = f;
  a.q = q;
  a.df = df;
  a.v1 = p->v1dev;
  a.nx = nx;
  a.N = p->N;
  a.N2 = p->N / p->n;  // points per first-axis velocity index
  a.dt = dt;
  a.kn = kn;
  a.transport = dx > 0.0 ? 1 : 0;
  a.dtdx = dx > 0.0 ? dt / dx : 0.0;
  a.bc_lo = bc_lo;
  a.bc_hi = bc_hi;
  {
    StageTimer st(p, ST_DF, s);
    k_df<<<unsigned((p->N + 127) / 128), 128, 0, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int mass_fix_impl(pii_plan* p, double* q, int64_t cells, int64_t N, cudaStream_t s) {
  {
    StageTimer st(p, ST_MASSFIX, s);
    k_massfix<<<unsigned(cells), 256, 0, s>>>(q, N);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int axpy3_impl(pii_plan* p, double* f, const double* d, double s0, double s1, double s2, int64_t count,
               cudaStream_t s) {
  if (count <= 0) return PII_OK;
  {
    StageTimer st(p, ST_AXPY, s);
    k_axpy3<<<unsigned((count + 255) / 256), 256, 0, s>>>(f, d, s0, s1, s2, count);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int upload_v1(pii_plan* p, const double* v1, cudaStream_t s) {
  if (!v1) {
    set_error("v1 velocity array is NULL");
    return PII_ERR_ARG;
  }
  // uploaded only when it changed (a solver passes the same grid every macro-step)
  if (p->v1host.size() == size_t(p->n) && std::equal(v1, v1 + p->n, p->v1host.begin())) return PII_OK;
  PII_CUDA(cudaMemcpyAsync(p->v1dev, v1, size_t(p->n) * sizeof(double), cudaMemcpyHostToDevice, s));
  p->v1host.assign(v1, v1 + p->n);
  return PII_OK;
}

int check_bcs(int lo, int hi) {
  if ((lo != PII_BC_EXTRAP && lo != PII_BC_PERIODIC) || (hi != PII_BC_EXTRAP && hi != PII_BC_PERIODIC)) {
    set_error("Boundary condition (%d, %d) not implemented", lo, hi);
    return PII_ERR_ARG;
  }
  return PII_OK;
}

}  // namespace pii

extern "C" {

int pii_transport_df(pii_plan* plan, const double* f, double* df, int64_t nx, double dt, double dx,
                     const double* v1, int bc_lower, int bc_upper, void* stream) {
  if (!plan || !f || !df || nx <= 0 || !(dx > 0)) {
    pii::set_error("pii_transport_df: invalid arguments");
    return PII_ERR_ARG;
  }
  if (nx > plan->batch_max) {
    pii::set_error("pii_transport_df: nx beyond batch_max");
    return PII_ERR_SIZE;
  }
  PII_TRY(pii::check_bcs(bc_lower, bc_upper));
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  PII_TRY(pii::upload_v1(plan, v1, s));
  return pii::transport_impl(plan, f, nullptr, df, nx, dt, dx, bc_lower, bc_upper, 1.0, s);
}

int pii_moments(pii_plan* plan, const double* f, double* out, int64_t cells, const double* v, double delta,
                void* stream) {
  if (!plan || !f || !out || !v || cells <= 0) {
    pii::set_error("pii_moments: invalid arguments");
    return PII_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  PII_TRY(pii::upload_v1(plan, v, s));
  pii::k_moments<<<unsigned(cells), 256, 0, s>>>(f, out, plan->v1dev, plan->n, plan->dim,
                                                  plan->dim == 3 ? delta * delta * delta : delta * delta);
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int pii_state_check(pii_plan* plan, const double* f, double* out, int64_t cells, const double* v, double delta,
                    void* stream) {
  if (!plan || !f || !out || !v || cells <= 0) {
    pii::set_error("pii_state_check: invalid arguments");
    return PII_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  PII_TRY(pii::upload_v1(plan, v, s));
  pii::k_moments<<<unsigned(cells), 256, 0, s>>>(f, out, plan->v1dev, plan->n, plan->dim,
                                                  plan->dim == 3 ? delta * delta * delta : delta * delta);
  PII_CHECK_LAUNCH();
  PII_CUDA(cudaMemsetAsync(plan->flag, 0, sizeof(int), s));
  const int64_t count = cells * plan->N;
  const int64_t blocks = std::min<int64_t>((count + 255) / 256, 4096);
  pii::k_nonfinite<<<unsigned(blocks), 256, 0, s>>>(f, count, plan->flag);
  PII_CHECK_LAUNCH();
  int h = 0;
  PII_CUDA(cudaMemcpyAsync(&h, plan->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  PII_CUDA(cudaStreamSynchronize(s));
  PII_TRY(pii::dft_stall_check(plan));  // the state may come from a stalled launch
  if (h) {
    pii::set_error("pii_state_check: f holds NaN or Inf values");
    return PII_ERR_NONFINITE;
  }
  return PII_OK;
}

int pii_fast_sweep(pii_plan* plan, double* f, const double* q, int64_t nx, double dx, double kn, const double* v1,
                   double* err, void* stream) {
  if (!plan || !f || !q || !v1 || !err || nx <= 0 || !(dx > 0) || !(kn > 0)) {
    pii::set_error("pii_fast_sweep: invalid arguments");
    return PII_ERR_ARG;
  }
  if (nx > plan->batch_max) {
    pii::set_error("pii_fast_sweep: nx beyond batch_max");
    return PII_ERR_SIZE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PII_CUDA(cudaSetDevice(plan->device));
  PII_TRY(pii::upload_v1(plan, v1, s));
  const double delta = v1[1] - v1[0];
  const double dv = plan->dim == 3 ? delta * delta * delta : delta * delta;
  pii::k_moments<<<unsigned(nx), 256, 0, s>>>(f, plan->mom, plan->v1dev, plan->n, plan->dim, dv);
  PII_CHECK_LAUNCH();
  // the plan's 16-byte flag block: int guard flag at 0, the sweep's error word at 8
  auto* word = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(plan->flag) + 8);
  PII_CUDA(cudaMemsetAsync(word, 0, sizeof(unsigned long long), s));
  const double pi = 3.141592653589793238462643383279502884;
  const double nu = 1.0 / std::sqrt(pi / 2.0) / kn;  // (src/iter_solver.py:46)
  const int64_t N = plan->N;
  pii::k_sweep<<<unsigned((N + 255) / 256), 256, 0, s>>>(f, q, plan->mom, plan->v1dev, nx, N, N / plan->n, dx, nu,
                                                           word);
  PII_CHECK_LAUNCH();
  unsigned long long h = 0;
  PII_CUDA(cudaMemcpyAsync(&h, word, sizeof(h), cudaMemcpyDeviceToHost, s));
  PII_CUDA(cudaStreamSynchronize(s));
  std::memcpy(err, &h, sizeof(double));
  return PII_OK;
}

int pii_axpby(double* f, const double* d, double a, double b, int64_t count, void* stream) {
  if (!f || !d || count < 0) {
    pii::set_error("pii_axpby: invalid arguments");
    return PII_ERR_ARG;
  }
  return pii::axpy3_impl(nullptr, f, d, b, 1.0, a, count, (cudaStream_t)stream);
}

}  // extern "C"
