// Nyquist-plane correction of the packed gain paths as a quadratic form in f^
// (FP32, every n; the default for n = 64, where it beats the direct kernels,
// built on request for other n).
//
// Per antipodal pass p the packed evaluation leaves out, on the Nyquist planes
// only (nyq_corr.cu / nyq_gen.cu state it in full),
//   C_p(k) = (w.x - w.y) U_p(k) - (w.x + w.y) conj U_p(-k),  w = g-_p(k) gsinc(r_p, |k|^2),
//   U_p(k) = sum_x e^{-i k x} f(x) IFFT3(f^ t-_p)(x) = sum_q t-_p(q) f^(q) f^(k - q)
// with the sum over the Nyquist points q (where t-_p = Re E-_p + Im E-_p
// lives; the 1/n^3 rides on the first-axis phase row) and f^ the unnormalised
// FFT of the real f, so that conj U_p(-k) = sum_q t-_p(q) conj f^(q) f^(k + q).
// Summed over the passes, with REAL kernels that depend on the tables only,
//   C(k) = sum_q A(k, q) f^(q) f^(k - q) - B(k, q) conj f^(q) f^(k + q),
//   A(k, q) = sum_p (w_p.x - w_p.y)(k) t-_p(q),   B(k, q) = sum_p (w_p.x + w_p.y)(k) t-_p(q).
// A and B (Nq x Nq, Nq = 3 n^2 - 3 n + 1 Nyquist points) are built once per
// plan and restitution set: k_quad_coef evaluates t-, w.x - w.y and w.x + w.y
// from the plan's FP32 rows (as the direct kernels do), k_quad_gemm contracts
// them over the passes.  Per call k_quad_prep lays out f^ at the Nyquist
// points and f^ transposed within each a-plane, and k_nyq_quad forms C(k) for
// a tile of output points and a group of cells per CTA: A and B are read
// coalesced ([q][k]) once per group, f^(k -+ q) gathered coalesced along each
// output row (from the transposed copy for the plane k_c = n/2).
#include <algorithm>
#include <vector>

#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {

namespace nqq {
constexpr int THREADS = 256;  // output points per CTA
constexpr int GMAX = 8;       // cells per CTA when every cell shares the kernels
constexpr int TM = 64, TK = 16;  // GEMM tiles: 64 x 64 outputs, 16 passes per step
}  // namespace nqq

__device__ __forceinline__ float2 qq_conj(float2 v) { return make_float2(v.x, -v.y); }

// (X(k) - X~(k)) / 2 for the per-axis rows x (~ conjugates the factor of a
// component equal to the Nyquist index h)
__device__ __forceinline__ float2 qq_minus(const float2* rows, int n, int ka, int kb, int kc) {
  const int h = n / 2;
  const float2 xa = rows[ka], xb = rows[n + kb], xc = rows[2 * n + kc];
  const float2 p = cmul(cmul(xa, xb), xc);
  const float2 q = cmul(cmul(ka == h ? qq_conj(xa) : xa, kb == h ? qq_conj(xb) : xb), kc == h ? qq_conj(xc) : xc);
  return make_float2(0.5f * (p.x - q.x), 0.5f * (p.y - q.y));
}

// T[p][i] = Re E-_p + Im E-_p at Nyquist point i; Al / Be[s][p][i] = w.x -+ ... for set s
__global__ void __launch_bounds__(256) k_quad_coef(const int* pts, int npts, int n, const int* reps, int QP,
                                                    int ns, int M, const float2* ephase, const float2* gphase,
                                                    const float* gsinc, int64_t gph_set, int64_t gs_set, int sets,
                                                    float* T, float* Al, float* Be) {
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t per = int64_t(QP) * npts;
  if (gid >= per * (sets + 1)) return;
  const int64_t s1 = gid / per;  // 0: T, s1 >= 1: set s1 - 1
  const int64_t r = gid - s1 * per;
  const int p = int(r / npts), i = int(r - int64_t(p) * npts);
  const int code = pts[i], n2 = n * n;
  const int ka = code / n2, kb = (code / n) % n, kc = code % n;
  const int pair = reps[p];
  if (s1 == 0) {
    const float2 em = qq_minus(ephase + int64_t(pair) * 3 * n, n, ka, kb, kc);
    T[r] = em.x + em.y;
  } else {
    const int64_t s = s1 - 1;
    const float2 gm = qq_minus(gphase + s * gph_set + int64_t(pair) * 3 * n, n, ka, kb, kc);
    const int kk = kval(ka, n) * kval(ka, n) + kval(kb, n) * kval(kb, n) + kval(kc, n) * kval(kc, n);
    const float g = gsinc[s * gs_set + int64_t(pair / ns) * (M + 1) + kk];
    const float wx = g * gm.x, wy = g * gm.y;
    Al[s * per + r] = wx - wy;
    Be[s * per + r] = wx + wy;
  }
}

// C[q][k] = sum_p T[p][q] X[p][k]  (npts x npts, K = QP; both operands pass-major)
__global__ void __launch_bounds__(256) k_quad_gemm(const float* T, const float* X, float* C, int npts, int QP) {
  using namespace nqq;
  __shared__ float ta[TK][TM], tb[TK][TM];
  const int q0 = blockIdx.y * TM, k0 = blockIdx.x * TM;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 4 x 4 outputs each
  float acc[4][4] = {};
  for (int p0 = 0; p0 < QP; p0 += TK) {
    for (int e = threadIdx.x; e < TK * TM; e += 256) {
      const int pp = e / TM, c = e - pp * TM;
      const bool okp = p0 + pp < QP;
      ta[pp][c] = okp && q0 + c < npts ? T[int64_t(p0 + pp) * npts + q0 + c] : 0.f;
      tb[pp][c] = okp && k0 + c < npts ? X[int64_t(p0 + pp) * npts + k0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int pp = 0; pp < TK; ++pp) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = ta[pp][ty * 4 + i], b[i] = tb[pp][tx * 4 + i];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int q = q0 + ty * 4 + i, k = k0 + tx * 4 + j;
      if (q < npts && k < npts) C[int64_t(q) * npts + k] = acc[i][j];
    }
}

// f^ at the Nyquist points, compact, and f^ transposed within each a-plane
// (fhT[cell][a][c][b] = f^[cell][a][b][c], 32 x 32 tiles through shared memory)
__global__ void __launch_bounds__(256) k_quad_prep(const float2* fhat, float2* fhn, float2* fhT, const int* pts,
                                                    int npts, int n, int64_t cells) {
  __shared__ float2 tile[32][33];
  const int tb_n = (n + 31) / 32;
  const int64_t n2 = int64_t(n) * n, n3 = n2 * n;
  const int64_t bid = blockIdx.x;
  const int64_t tiles = cells * n * tb_n * tb_n;
  if (bid < tiles) {
    const int64_t cp = bid / (tb_n * tb_n);  // (cell, a)
    const int tt = int(bid - cp * tb_n * tb_n), tb = tt / tb_n, tc = tt - tb * tb_n;
    const float2* src = fhat + cp * n2;
    float2* dst = fhT + cp * n2;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int j = ty; j < 32; j += 8) {
      const int b = tb * 32 + j, c = tc * 32 + tx;
      if (b < n && c < n) tile[j][tx] = src[b * n + c];
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
      const int c = tc * 32 + j, b = tb * 32 + tx;
      if (b < n && c < n) dst[c * n + b] = tile[tx][j];
    }
  } else {
    const int64_t gid = (bid - tiles) * 256 + threadIdx.x;
    if (gid >= cells * npts) return;
    const int64_t cell = gid / npts;
    fhn[gid] = fhat[cell * n3 + pts[gid - cell * npts]];
  }
}

// G[cell][k] += sum_q A(k, q) f^(q) f^(k - q) - B(k, q) conj f^(q) f^(k + q)
// for the output points k of this CTA's tile and the NC cells of its group
// (sets > 1: one cell per group, the cell's own kernels)
template <int NC>
__global__ void __launch_bounds__(nqq::THREADS) k_nyq_quad(const float* A, const float* B, const int* pts, int npts,
                                                            int n, const float2* fhat, const float2* fhT,
                                                            const float2* fhn, float2* G, int64_t cells,
                                                            int64_t set_stride) {
  using namespace nqq;
  __shared__ int qs[THREADS];
  __shared__ float2 fq[NC][THREADS];
  const int K = blockIdx.x * THREADS + threadIdx.x;
  const int64_t c0 = int64_t(blockIdx.y) * NC;
  const bool on = K < npts;
  const int n2 = n * n, h = n / 2;
  const int64_t n3 = int64_t(n2) * n;
  const int code = on ? pts[K] : 0;
  const int ka = code / n2, kb = (code / n) % n, kc = code % n;
  // the plane k_c = h (outside k_a = h, k_b = h) runs along k_b: gather from the transposed copy
  const bool pl2 = kc == h && ka != h && kb != h;
  const float2* src[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int64_t cell = min(c0 + c, cells - 1);
    src[c] = (pl2 ? fhT : fhat) + cell * n3;
  }
  const float* Ak = A + (set_stride ? c0 * set_stride : 0) + K;
  const float* Bk = B + (set_stride ? c0 * set_stride : 0) + K;
  float2 acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = make_float2(0.f, 0.f);
  for (int j0 = 0; j0 < npts; j0 += THREADS) {
    // a chunk of the input points and their f^ values into shared memory
    __syncthreads();
    const int jj = j0 + threadIdx.x;
    qs[threadIdx.x] = jj < npts ? pts[jj] : 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const int64_t cell = min(c0 + c, cells - 1);
      fq[c][threadIdx.x] = jj < npts ? fhn[cell * npts + jj] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int jn = min(THREADS, npts - j0);
    if (on) {
#pragma unroll 2
      for (int j = 0; j < jn; ++j) {
        const int qc = qs[j];
        const int qa = qc / n2, qb = (qc / n) % n, qq = qc % n;
        int ma = ka - qa, mb = kb - qb, mc = kc - qq;
        ma += ma < 0 ? n : 0, mb += mb < 0 ? n : 0, mc += mc < 0 ? n : 0;
        int pa = ka + qa, pb = kb + qb, pc = kc + qq;
        pa -= pa >= n ? n : 0, pb -= pb >= n ? n : 0, pc -= pc >= n ? n : 0;
        const int im = pl2 ? ma * n2 + mc * n + mb : ma * n2 + mb * n + mc;
        const int ip = pl2 ? pa * n2 + pc * n + pb : pa * n2 + pb * n + pc;
        const float a = __ldg(Ak + int64_t(j0 + j) * npts), b = __ldg(Bk + int64_t(j0 + j) * npts);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const float2 f0 = fq[c][j];
          const float2 gm = __ldg(src[c] + im), gp = __ldg(src[c] + ip);
          // a f0 gm - b conj(f0) gp
          const float2 u = make_float2(f0.x * gm.x - f0.y * gm.y, f0.x * gm.y + f0.y * gm.x);
          const float2 w = make_float2(f0.x * gp.x + f0.y * gp.y, f0.x * gp.y - f0.y * gp.x);
          acc[c].x += a * u.x - b * w.x;
          acc[c].y += a * u.y - b * w.y;
        }
      }
    }
  }
  if (!on) return;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    if (c0 + c >= cells) break;
    float2* g = G + (c0 + c) * n3 + code;
    g->x += acc[c].x;
    g->y += acc[c].y;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static void free_quad(pii_plan* p) {
  for (void** q : {&p->nq_A, &p->nq_B, &p->nq_pts, &p->nq_fhT, &p->nq_fhq})
    if (*q) {
      cudaFree(*q);
      *q = nullptr;
    }
  p->bytes -= p->nq_quad_bytes;
  p->nq_quad_bytes = 0;
  p->nq_npts = 0;
}

// (Re)builds A and B for the plan's restitution sets; leaves the plan without
// them (the direct correction kernels) when they exceed the memory budget
int nyq_quad_prepare(pii_plan* p) {
  using namespace nqq;
  free_quad(p);
  if (p->ap_count <= 0 || p->precision != PII_PREC_FP32 || p->dim != 3) return PII_OK;
  const int n = p->n, h = n / 2, n2 = n * n;
  std::vector<int> pts;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) pts.push_back(h * n2 + r * n + c);  // k_a = h
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if (r != h) pts.push_back(r * n2 + h * n + c);  // k_b = h, k_a != h
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if (r != h && c != h) pts.push_back(r * n2 + c * n + h);  // k_c = h, k_a, k_b != h
  const int64_t npts = int64_t(pts.size()), sets = p->tab.nsets, QP = p->ap_count;
  const size_t kern = size_t(npts) * npts * sizeof(float) * 2 * size_t(sets);
  const size_t fh = size_t(p->batch_max) * (size_t(n2) * n + size_t(npts)) * sizeof(float2);
  size_t free_b = 0, total_b = 0;
  PII_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const size_t budget = std::min<size_t>(size_t(16) << 30, free_b / 4);
  if (kern + fh > budget) return PII_OK;  // the direct kernels stay in use
  float *T = nullptr, *Al = nullptr, *Be = nullptr;
  const size_t coef = size_t(QP) * npts * sizeof(float);
  int st = PII_OK;
  auto al = [&](void** d, size_t b) {
    if (st == PII_OK && cudaMalloc(d, b) != cudaSuccess) {
      set_error("nyq_quad_prepare: out of memory");
      st = PII_ERR_CUDA;
    }
  };
  al(&p->nq_pts, pts.size() * sizeof(int));
  al(&p->nq_A, kern / 2);
  al(&p->nq_B, kern / 2);
  al(&p->nq_fhT, size_t(p->batch_max) * n2 * n * sizeof(float2));
  al(&p->nq_fhq, size_t(p->batch_max) * npts * sizeof(float2));
  al((void**)&T, coef);
  al((void**)&Al, coef * sets);
  al((void**)&Be, coef * sets);
  if (st == PII_OK) {
    PII_CUDA(cudaMemcpy(p->nq_pts, pts.data(), pts.size() * sizeof(int), cudaMemcpyHostToDevice));
    const int64_t work = QP * npts * (sets + 1);
    k_quad_coef<<<unsigned((work + 255) / 256), 256>>>(
        static_cast<const int*>(p->nq_pts), int(npts), n, p->ap_reps, int(QP), p->ns, p->tab.M,
        static_cast<const float2*>(p->tab.ephase), static_cast<const float2*>(p->tab.gphase),
        static_cast<const float*>(p->tab.gsinc), p->tab.gph_stride, p->tab.gs_stride, int(sets), T, Al, Be);
    const dim3 grid(unsigned((npts + TM - 1) / TM), unsigned((npts + TM - 1) / TM));
    for (int64_t s = 0; s < sets; ++s) {
      k_quad_gemm<<<grid, 256>>>(T, Al + s * QP * npts, static_cast<float*>(p->nq_A) + s * npts * npts, int(npts),
                                 int(QP));
      k_quad_gemm<<<grid, 256>>>(T, Be + s * QP * npts, static_cast<float*>(p->nq_B) + s * npts * npts, int(npts),
                                 int(QP));
    }
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      set_error("nyq_quad_prepare: %s", cudaGetErrorString(e));
      st = PII_ERR_CUDA;
    }
  }
  cudaFree(T);
  cudaFree(Al);
  cudaFree(Be);
  if (st != PII_OK) {
    free_quad(p);
    return st;
  }
  p->nq_npts = int(npts);
  p->nq_quad_bytes = int64_t(kern + fh + pts.size() * sizeof(int));
  p->bytes += p->nq_quad_bytes;
  return PII_OK;
}

void nyq_quad_release(pii_plan* p) { free_quad(p); }

int nyq_quad_run(pii_plan* p, int64_t cells, cudaStream_t s) {
  using namespace nqq;
  if (!p->nq_A || p->nq_npts <= 0) {
    set_error("nyq_quad_run: the plan has no quadratic-form kernels");
    return PII_ERR_ARG;
  }
  const int n = p->n, npts = p->nq_npts;
  const int tb = (n + 31) / 32;
  {
    StageTimer st(p, ST_NYQ, s);
    const int64_t tiles = cells * n * tb * tb, pb = (cells * npts + 255) / 256;
    k_quad_prep<<<unsigned(tiles + pb), 256, 0, s>>>(static_cast<const float2*>(p->fhat),
                                                      static_cast<float2*>(p->nq_fhq),
                                                      static_cast<float2*>(p->nq_fhT),
                                                      static_cast<const int*>(p->nq_pts), npts, n, cells);
  }
  PII_CHECK_LAUNCH();
  const unsigned kt = unsigned((npts + THREADS - 1) / THREADS);
  const float* A = static_cast<const float*>(p->nq_A);
  const float* B = static_cast<const float*>(p->nq_B);
  const int* pts = static_cast<const int*>(p->nq_pts);
  const float2* fh = static_cast<const float2*>(p->fhat);
  const float2* fhT = static_cast<const float2*>(p->nq_fhT);
  const float2* fhq = static_cast<const float2*>(p->nq_fhq);
  float2* G = static_cast<float2*>(p->G);
  {
    StageTimer st(p, ST_NYQ, s);
    if (p->tab.nsets > 1) {  // every cell its own kernels
      const int64_t stride = int64_t(npts) * npts;
      k_nyq_quad<1><<<dim3(kt, unsigned(cells)), THREADS, 0, s>>>(A, B, pts, npts, n, fh, fhT, fhq, G, cells, stride);
    } else {
      k_nyq_quad<GMAX><<<dim3(kt, unsigned((cells + GMAX - 1) / GMAX)), THREADS, 0, s>>>(A, B, pts, npts, n, fh, fhT,
                                                                                       fhq, G, cells, 0);
    }
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
