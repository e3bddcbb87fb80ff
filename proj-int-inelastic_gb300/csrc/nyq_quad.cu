// Nyquist-plane correction of the packed gain paths as a quadratic form in f^
// (FP32, n a multiple of 8 up to 64; the default wherever its kernels fit the
// memory budget, the direct kernels of nyq_corr.cu / nyq_gen.cu otherwise).
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
// them over the passes, storing them in the order the correction kernel reads.
//
// Blocking.  The output points form three planes, one per orientation d
// (k_a = h, k_b = h, k_c = h with h = n / 2; points of an earlier plane are
// skipped), each indexed by its in-plane coordinates (k1, k2).  Seen from
// orientation d, the input points q group into n slices by their coordinate
// s along d: slice s != h is the row i1 = h plus the column i2 = h of the
// plane at s, slice h the whole plane at h.  For k on the plane at h and q in
// slice s, k - q lies in the plane at h - s and k + q in the plane at h + s
// (the same plane, h - s = -(h + s) mod n), at in-plane offsets
// (k1 -+ i1, k2 -+ i2).  k_nyq_quad stages those two planes of f^ for a group
// of cells in shared memory once per slice (plane 0 and the input plane h for
// s = h) and walks the slice's input points by segment (a row of n points,
// or the column of n - 1); each thread owns R consecutive k2 of one k1, and
// along a row it keeps the f^(k -+ q) it needs in a sliding window of
// registers, one new value per step and plane.  A and B are laid out
// [d][q in slice order][k2 / R][k1][k2 % R], so a warp reads them as one
// coalesced 16-byte vector per lane and step, once per group of cells.  The
// input points of an orientation are split into ranges across CTAs; each
// range writes its partial sums and k_quad_add adds them into G.
//
// Pairing.  f is real, so f^(-q) = conj f^(q), and the terms of q and -q
// (both Nyquist points) combine into one:
//   A~(k, q) f^(q) f^(k - q) - B~(k, q) conj f^(q) f^(k + q),
//   A~ = w (A(k, q) - B(k, -q)),  B~ = w (B(k, q) - A(k, -q)),
// with w = 1/2 where q = -q.  The kernel walks one of each pair: slices
// 1 .. h - 1 whole (their partners are slices n - 1 .. h + 1) and half of the
// self-paired slices 0 and h (their rows i1 = 0, h up to i2 = h, padded to a
// multiple of R with zero kernels, and slice 0's column up to i1 < h): the
// same two planes per slice, about half the input points.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {

namespace nqq {
constexpr int R = 4;             // consecutive k2 per thread (every supported n / 2 is a multiple)
constexpr int SPLIT_MAX = 8;     // input-point ranges per orientation
constexpr int TM = 64, TK = 16;  // GEMM tiles: 64 x 64 outputs, 16 passes per step
}  // namespace nqq

// the FP32 and FP64 plans run the same kernels in their own arithmetic
template <typename V>
__device__ __forceinline__ V qq_conj(V v) {
  return mk<V>(v.x, -v.y);
}

// (X(k) - X~(k)) / 2 for the per-axis rows x (~ conjugates the factor of a
// component equal to the Nyquist index h)
template <typename V>
__device__ __forceinline__ V qq_minus(const V* rows, int n, int ka, int kb, int kc) {
  using S = decltype(V::x);
  const int h = n / 2;
  const V xa = rows[ka], xb = rows[n + kb], xc = rows[2 * n + kc];
  const V p = cmul(cmul(xa, xb), xc);
  const V q = cmul(cmul(ka == h ? qq_conj(xa) : xa, kb == h ? qq_conj(xb) : xb), kc == h ? qq_conj(xc) : xc);
  return mk<V>(S(0.5) * (p.x - q.x), S(0.5) * (p.y - q.y));
}

// T[p][i] = Re E-_p + Im E-_p at Nyquist point i; Al / Be[s][p][i] = w.x -+ ... for set s
template <typename S>
__global__ void __launch_bounds__(256) k_quad_coef(const int* pts, int npts, int n, const int* reps, int QP,
                                                    int ns, int M, const c2<S>* ephase, const c2<S>* gphase,
                                                    const S* gsinc, int64_t gph_set, int64_t gs_set, int sets,
                                                    S* T, S* Al, S* Be) {
  using V = c2<S>;
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
    const V em = qq_minus(ephase + int64_t(pair) * 3 * n, n, ka, kb, kc);
    T[r] = em.x + em.y;
  } else {
    const int64_t s = s1 - 1;
    const V gm = qq_minus(gphase + s * gph_set + int64_t(pair) * 3 * n, n, ka, kb, kc);
    const int kk = kval(ka, n) * kval(ka, n) + kval(kb, n) * kval(kb, n) + kval(kc, n) * kval(kc, n);
    const S g = gsinc[s * gs_set + int64_t(pair / ns) * (M + 1) + kk];
    const S wx = g * gm.x, wy = g * gm.y;
    Al[s * per + r] = wx - wy;
    Be[s * per + r] = wx + wy;
  }
}

// C[j][kk] = w_j sum_p (T[p][q1_j] X1[p][ki[kk]] - T[p][q2_j] X2[p][ki[kk]]):
// the paired kernel of slot j (q1 its input point, q2 = -q1; q1 < 0 marks a
// padding slot, zero) at the output points ki (ki < 0: skipped, zero); T, X1
// and X2 rows hold npts entries in point order
template <typename S>
__global__ void __launch_bounds__(256) k_quad_gemm(const S* T, const S* X1, const S* X2, const int* q1,
                                                    const int* q2, const S* w, const int* ki, S* C, int M,
                                                    int Ncol, int QP, int npts) {
  using namespace nqq;
  __shared__ S ta[TK][TM], tb[TK][TM];
  const int q0 = blockIdx.y * TM, k0 = blockIdx.x * TM;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 4 x 4 outputs each
  S acc[4][4] = {};
  for (int p0 = 0; p0 < 2 * QP; p0 += TK) {  // the passes twice: + T(q) X1, - T(-q) X2
    for (int e = threadIdx.x; e < TK * TM; e += 256) {
      const int pp = e / TM, c = e - pp * TM;
      const int pg = p0 + pp, second = pg >= QP ? 1 : 0, p = pg - second * QP;
      const bool okp = pg < 2 * QP;
      const int kidx = okp && k0 + c < Ncol ? ki[k0 + c] : -1;
      S tv = S(0);
      if (okp && q0 + c < M && q1[q0 + c] >= 0) {
        const int qq = second ? q2[q0 + c] : q1[q0 + c];
        tv = (second ? -w[q0 + c] : w[q0 + c]) * T[int64_t(p) * npts + qq];
      }
      ta[pp][c] = tv;
      tb[pp][c] = kidx >= 0 ? (second ? X2 : X1)[int64_t(p) * npts + kidx] : S(0);
    }
    __syncthreads();
#pragma unroll
    for (int pp = 0; pp < TK; ++pp) {
      S a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = ta[pp][ty * 4 + i], b[i] = tb[pp][tx * 4 + i];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int q = q0 + ty * 4 + i, k = k0 + tx * 4 + j;
      if (q < M && k < Ncol) C[int64_t(q) * Ncol + k] = acc[i][j];
    }
}

// f^ transposed within each a-plane: fhT[cell][a][c][b] = f^[cell][a][b][c]
// (32 x 32 tiles through shared memory)
template <typename V>
__global__ void __launch_bounds__(256) k_quad_prep(const V* fhat, V* fhT, int n, int64_t cells) {
  __shared__ V tile[32][33];
  const int tb_n = (n + 31) / 32;
  const int64_t n2 = int64_t(n) * n;
  const int64_t bid = blockIdx.x;
  const int64_t cp = bid / (tb_n * tb_n);  // (cell, a)
  if (cp >= cells * n) return;
  const int tt = int(bid - cp * tb_n * tb_n), tb = tt / tb_n, tc = tt - tb * tb_n;
  const V* src = fhat + cp * n2;
  V* dst = fhT + cp * n2;
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
}

template <typename S>
struct QuadArgs {
  using V = c2<S>;
  const S* A;
  const S* B;
  const V* fhat;
  const V* fhT;
  V* part;             // [split][cells][3][n][n]
  const int4* segs;    // segments of the kernel slots: (slice, 0 row / 1 column, row i1, steps)
  const int* seg_j0;   // first kernel slot of each segment
  int nseg;
  int64_t cells;
  int64_t set_stride;  // entries between consecutive cells' kernels (0: one set for every cell)
  int n, npts, W, split;  // npts: kernel slots per orientation
};

template <typename S, typename V>
__device__ __forceinline__ void qq_term(V& acc, S a, S b, V f0, V gm, V gp) {
  // acc += a f0 gm - b conj(f0) gp
  const S x1 = fma(a, gm.x, -b * gp.x), x2 = fma(a, gm.y, b * gp.y);
  const S x3 = fma(a, gm.y, -b * gp.y), x4 = fma(a, gm.x, b * gp.x);
  acc.x = fma(f0.x, x1, fma(-f0.y, x2, acc.x));
  acc.y = fma(f0.x, x3, fma(f0.y, x4, acc.y));
}

// R = 4 consecutive kernel entries (16 bytes FP32, 2 x 16 bytes FP64)
__device__ __forceinline__ void qq_ld4(const float* p, float (&o)[4]) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
__device__ __forceinline__ void qq_ld4(const double* p, double (&o)[4]) {
  const double2 v0 = __ldg(reinterpret_cast<const double2*>(p)), v1 = __ldg(reinterpret_cast<const double2*>(p) + 1);
  o[0] = v0.x, o[1] = v0.y, o[2] = v1.x, o[3] = v1.y;
}
// one complex element into shared memory
__device__ __forceinline__ void qq_cp(float2* d, const float2* s) { cp_async8(d, s); }
__device__ __forceinline__ void qq_cp(double2* d, const double2* s) { cp_async16(d, s); }

// partial C over one range of one orientation's input points, for R output
// points per thread and NC cells per CTA (NC = 1 when every cell has its own
// kernels); grid (n / W, cell groups, 3 x split), n W / R threads
template <typename S, int NC, int MAXT>
__global__ void __launch_bounds__(MAXT) k_nyq_quad(QuadArgs<S> a) {
  using V = c2<S>;
  constexpr int R = nqq::R;
  extern __shared__ __align__(16) unsigned char qsm_raw[];
  V* qsm = reinterpret_cast<V*>(qsm_raw);
  const int n = a.n, h = n >> 1, n2 = n * n, LD = n + 1;
  const int64_t n3 = int64_t(n2) * n;
  const int d = blockIdx.z / a.split, range = blockIdx.z - d * a.split;
  const int tid = threadIdx.x, rows_step = blockDim.x / n;
  const int k1 = tid % n, kb = tid / n;
  const int k20 = blockIdx.x * a.W + kb * R;
  const int64_t c0 = int64_t(blockIdx.y) * NC;
  const int per_cell = 2 * n * LD + 2 * n;  // P1 [n][LD], P2 [n][LD], QR [n], QC [n]
  const V* src[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int64_t cell = min(c0 + c, a.cells - 1);
    src[c] = (d == 2 ? a.fhT : a.fhat) + cell * n3;
  }
  // plane v of orientation d, element (i1, i2): off(v) + i1 * s1 + i2 (the
  // plane k_c = v comes from the transposed copy)
  const int s1 = d == 0 ? n : n2, vstride = d == 0 ? n2 : n;
  const int64_t kset = a.set_stride ? c0 * a.set_stride : 0;
  const int64_t kofs = kset + int64_t(d) * a.npts * n2 + (int64_t(k20 / R) * n + k1) * R;
  const S* Ab = a.A + kofs;
  const S* Bb = a.B + kofs;
  V acc[NC][R];
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int r = 0; r < R; ++r) acc[c][r] = mk<V>(S(0), S(0));

  const int nseg = a.nseg;
  const int g0 = range * nseg / a.split, g1 = (range + 1) * nseg / a.split;
  int cur = -1;
  for (int g = g0; g < g1; ++g) {
    const int4 sg = __ldg(a.segs + g);
    const int s = sg.x, kind = sg.y, i1f = sg.z, len = sg.w, j0 = __ldg(a.seg_j0 + g);
    if (s != cur) {  // stage the slice's planes for the group's cells
      __syncthreads();
      const int vm = (h - s + n) % n, vp = (n - vm) % n, v2 = s == h ? h : vp;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        V* P1 = qsm + c * per_cell;
        V* P2 = P1 + n * LD;
        const V* sm_ = src[c] + int64_t(vm) * vstride;
        const V* s2_ = src[c] + int64_t(v2) * vstride;
        for (int i1 = kb; i1 < n; i1 += rows_step) {
          qq_cp(P1 + i1 * LD + k1, sm_ + int64_t(i1) * s1 + k1);
          qq_cp(P2 + i1 * LD + k1, s2_ + int64_t(i1) * s1 + k1);
        }
        if (s != h && kb < 2) {  // QR: row h of the plane at s; QC: its column h
          const V* ss = src[c] + int64_t(s) * vstride;
          V* Q = P2 + n * LD + kb * n;
          qq_cp(Q + k1, kb == 0 ? ss + int64_t(h) * s1 + k1 : ss + int64_t(k1) * s1 + h);
        }
      }
      cp_async_commit();
      cp_async_wait_group<0>();
      __syncthreads();
      cur = s;
    }
    if (kind == 0) {  // a row of input points: i1 = i1f, i2 = 0 .. len - 1 (len a multiple of R)
      int rm = k1 - i1f, rp = k1 + i1f;
      rm += rm < 0 ? n : 0;
      rp -= rp >= n ? n : 0;
      const V* pm[NC];
      const V* pp[NC];
      const V* qrow[NC];
      V wm[NC][R], wp[NC][R];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const V* P1 = qsm + c * per_cell;
        const V* P2 = P1 + n * LD;
        pm[c] = P1 + rm * LD;
        pp[c] = (s == h ? P1 : P2) + rp * LD;
        qrow[c] = s == h ? P2 + i1f * LD : P2 + n * LD;
#pragma unroll
        for (int r = 1; r < R; ++r) wm[c][r] = pm[c][k20 + r];
#pragma unroll
        for (int r = 0; r < R - 1; ++r) wp[c][r] = pp[c][k20 + r];
      }
      const S* Aj = Ab + int64_t(j0) * n2;
      const S* Bj = Bb + int64_t(j0) * n2;
      S an[R][R], bn[R][R];  // the kernels of the next R input points, loaded one block ahead
#pragma unroll
      for (int t = 0; t < R; ++t) {
        qq_ld4(Aj + int64_t(t) * n2, an[t]);
        qq_ld4(Bj + int64_t(t) * n2, bn[t]);
      }
      for (int i20 = 0; i20 < len; i20 += R) {
        S ac[R][R], bc[R][R];
#pragma unroll
        for (int t = 0; t < R; ++t)
#pragma unroll
          for (int r = 0; r < R; ++r) ac[t][r] = an[t][r], bc[t][r] = bn[t][r];
        if (i20 + R < len) {
#pragma unroll
          for (int t = 0; t < R; ++t) {
            qq_ld4(Aj + int64_t(i20 + R + t) * n2, an[t]);
            qq_ld4(Bj + int64_t(i20 + R + t) * n2, bn[t]);
          }
        }
#pragma unroll
        for (int t = 0; t < R; ++t) {
          const int i2 = i20 + t;
          int um = k20 - i2, up = k20 + R - 1 + i2;
          um += um < 0 ? n : 0;
          up -= up >= n ? n : 0;
          const S(&al)[R] = ac[t];
          const S(&be)[R] = bc[t];
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            wm[c][(R - t) % R] = pm[c][um];
            wp[c][(R - 1 + t) % R] = pp[c][up];
            const V f0 = qrow[c][i2];
#pragma unroll
            for (int r = 0; r < R; ++r) qq_term(acc[c][r], al[r], be[r], f0, wm[c][(r - t + R) % R], wp[c][(r + t) % R]);
          }
        }
      }
    } else {  // the column i2 = h of slice s != h: i1 = m (m < h), m + 1 (m >= h), m < len
      const int cm = (k20 + h) % n;  // k2 -+ h for the thread's first k2 (no wrap within the R)
      // the column's input points are consecutive in the kernels: j0 + m
      S an[R], bn[R];
      qq_ld4(Ab + int64_t(j0) * n2, an);
      qq_ld4(Bb + int64_t(j0) * n2, bn);
      for (int m = 0; m < len; ++m) {
        const int i1 = m < h ? m : m + 1;
        int rm = k1 - i1, rp = k1 + i1;
        rm += rm < 0 ? n : 0;
        rp -= rp >= n ? n : 0;
        S al[R], be[R];
#pragma unroll
        for (int r = 0; r < R; ++r) al[r] = an[r], be[r] = bn[r];
        if (m + 1 < len) {
          qq_ld4(Ab + int64_t(j0 + m + 1) * n2, an);
          qq_ld4(Bb + int64_t(j0 + m + 1) * n2, bn);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const V* P1 = qsm + c * per_cell;
          const V* P2 = P1 + n * LD;
          const V* gmr = P1 + rm * LD + cm;
          const V* gpr = P2 + rp * LD + cm;
          const V f0 = P2[n * LD + n + i1];
#pragma unroll
          for (int r = 0; r < R; ++r) qq_term(acc[c][r], al[r], be[r], f0, gmr[r], gpr[r]);
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int64_t cell = c0 + c;
    if (cell >= a.cells) break;
    V* o = a.part + ((int64_t(range) * a.cells + cell) * 3 + d) * n2 + int64_t(k1) * n + k20;
#pragma unroll
    for (int r = 0; r < R; ++r) o[r] = acc[c][r];
  }
}

// G[cell][k] += the partial sums of every range, for the output points of the
// three planes (points of an earlier plane skipped)
template <typename V>
__global__ void __launch_bounds__(256) k_quad_add(const V* part, V* G, int n, int64_t cells, int split) {
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int n2 = n * n, h = n >> 1;
  if (gid >= cells * 3 * n2) return;
  const int64_t cd = gid / n2;  // (cell, d)
  const int e = int(gid - cd * n2), k1 = e / n, k2 = e - k1 * n;
  const int d = int(cd % 3);
  if ((d == 1 && k1 == h) || (d == 2 && (k1 == h || k2 == h))) return;
  const int64_t cell = cd / 3;
  V sum = mk<V>(0, 0);
  for (int r = 0; r < split; ++r) {
    const V v = part[(int64_t(r) * cells * 3 + cd) * n2 + e];
    sum.x += v.x, sum.y += v.y;
  }
  const int code = d == 0 ? h * n2 + k1 * n + k2 : d == 1 ? k1 * n2 + h * n + k2 : k1 * n2 + k2 * n + h;
  V* g = G + cell * int64_t(n2) * n + code;
  g->x += sum.x;
  g->y += sum.y;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct QuadCfg {
  int nc, W, threads;
  size_t smem;
};

// FP32: 2 cells per CTA (4 at n = 32 hold 253 registers, 8 warps per SM:
// 0.948 against 0.906 ms per 128-cell step); FP64 (twice the shared memory
// and registers per value): 2 up to n = 48, else 1; one with a set per cell
template <typename S>
static QuadCfg quad_cfg(int n, int nsets) {
  constexpr bool f64 = std::is_same<S, double>::value;
  QuadCfg c{};
  c.nc = nsets > 1 ? 1 : f64 ? (n <= 48 ? 2 : 1) : 2;
  c.W = n == 32 || n == 48 ? 16 : n;
  if (n == 64) c.W = c.nc == 1 ? 16 : 32;  // 256 or 512 threads
  c.threads = n * c.W / nqq::R;
  c.smem = size_t(c.nc) * size_t(2 * n * (n + 1) + 2 * n) * sizeof(c2<S>);
  return c;
}

template <typename S, int NC, int MAXT>
static int quad_occupancy(const QuadCfg& c, int* per_sm) {
  PII_CUDA(cudaFuncSetAttribute(k_nyq_quad<S, NC, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(c.smem)));
  PII_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_nyq_quad<S, NC, MAXT>, c.threads, c.smem));
  return PII_OK;
}

template <typename S>
static int quad_kernel_setup(const QuadCfg& c, int* per_sm) {
  if constexpr (std::is_same<S, float>::value) {
    if (c.nc == 2) return quad_occupancy<S, 2, 512>(c, per_sm);
    return quad_occupancy<S, 1, 256>(c, per_sm);
  } else {
    if (c.nc == 2) return quad_occupancy<S, 2, 256>(c, per_sm);
    return quad_occupancy<S, 1, 256>(c, per_sm);
  }
}

// input-point ranges per orientation for `cells` cells: about two waves of CTAs
static int quad_split(const pii_plan* p, const QuadCfg& c, int64_t cells) {
  const int64_t base = int64_t(p->n / c.W) * ((cells + c.nc - 1) / c.nc) * 3;
  const int64_t want = (2 * int64_t(p->nq_slots) + base - 1) / base;
  return int(std::max<int64_t>(1, std::min<int64_t>(want, std::min(nqq::SPLIT_MAX, std::max(1, p->nq_nseg)))));
}

static void free_quad(pii_plan* p) {
  for (void** q : {&p->nq_A, &p->nq_B, &p->nq_fhT, &p->nq_qpart, &p->nq_segs})
    if (*q) {
      cudaFree(*q);
      *q = nullptr;
    }
  p->bytes -= p->nq_quad_bytes;
  p->nq_quad_bytes = 0;
  p->nq_npts = 0;
  p->nq_nseg = 0;
  p->nq_qpart_units = 0;
}

// (Re)builds A and B for the plan's restitution sets; leaves the plan without
// them (FP32: the direct correction kernels; FP64: the unpacked pipeline)
// when they exceed the memory budget
template <typename S>
static int quad_prepare_t(pii_plan* p) {
  using namespace nqq;
  const int n = p->n, h = n / 2, n2 = n * n;
  if (n % 8 != 0 || n > 64) return PII_OK;  // R | h and the launch shapes below
  std::vector<int> pts;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) pts.push_back(h * n2 + r * n + c);  // k_a = h
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if (r != h) pts.push_back(r * n2 + h * n + c);  // k_b = h, k_a != h
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if (r != h && c != h) pts.push_back(r * n2 + c * n + h);  // k_c = h, k_a, k_b != h
  const int npts = int(pts.size());
  std::vector<int> pidx(size_t(n2) * n, -1);
  for (int i = 0; i < npts; ++i) pidx[pts[i]] = i;
  auto code = [&](int d, int v, int i1, int i2) {
    return d == 0 ? v * n2 + i1 * n + i2 : d == 1 ? i1 * n2 + v * n + i2 : i1 * n2 + i2 * n + v;
  };
  // the kernel slots: one input point of each pair {q, -q}, by segment (the
  // same index pattern for every orientation); rows padded to a multiple of R
  std::vector<int4> segs;
  std::vector<int> seg_j0;
  std::vector<char> seg_half;
  int NJ = 0;
  auto addseg = [&](int s, int kind, int i1, int len, bool half) {
    segs.push_back(make_int4(s, kind, i1, len));
    seg_j0.push_back(NJ);
    seg_half.push_back(half ? 1 : 0);
    NJ += len;
  };
  for (int s = 0; s <= h; ++s) {
    if (s == 0) {
      addseg(0, 0, h, h + R, true);  // the row of slice 0 up to i2 = h
      addseg(0, 1, h, h, false);     // its column up to i1 < h
    } else if (s < h) {
      addseg(s, 0, h, n, false);
      addseg(s, 1, h, n - 1, false);
    } else {
      for (int i1 = 0; i1 <= h; ++i1) addseg(h, 0, i1, i1 == 0 || i1 == h ? h + R : n, i1 == 0 || i1 == h);
    }
  }
  const int nseg = int(segs.size());
  auto negc = [&](int c) {
    const int a = c / n2, b = (c / n) % n, cc = c % n;
    return ((n - a) % n) * n2 + ((n - b) % n) * n + (n - cc) % n;
  };
  // per orientation and slot: the point q, its negative, the pair weight;
  // output points in the kernels' layout
  std::vector<int> q1, q2, ki;
  std::vector<S> wq;
  for (int d = 0; d < 3; ++d) {
    for (int g = 0; g < nseg; ++g) {
      const int4 sg = segs[g];
      for (int m = 0; m < sg.w; ++m) {
        int c = -1;
        if (sg.y == 0) {
          if (!(seg_half[g] && m > h)) c = code(d, sg.x, sg.z, m);
        } else {
          c = code(d, sg.x, m < h ? m : m + 1, h);
        }
        if (c < 0) {
          q1.push_back(-1), q2.push_back(0), wq.push_back(S(0));
          continue;
        }
        const int cn = negc(c);
        if (pidx[c] < 0 || pidx[cn] < 0) {
          set_error("nyq_quad_prepare: internal error in the input-point order");
          return PII_ERR_ARG;
        }
        q1.push_back(pidx[c]), q2.push_back(pidx[cn]), wq.push_back(c == cn ? S(0.5) : S(1));
      }
    }
    for (int kbg = 0; kbg < n / R; ++kbg)
      for (int k1 = 0; k1 < n; ++k1)
        for (int r = 0; r < R; ++r) {
          const int k2 = kbg * R + r;
          const bool skip = (d == 1 && k1 == h) || (d == 2 && (k1 == h || k2 == h));
          ki.push_back(skip ? -1 : pidx[code(d, h, k1, k2)]);
        }
  }
  p->nq_nseg = nseg;
  const int64_t sets = p->tab.nsets, QP = p->ap_count;
  const QuadCfg cfg = quad_cfg<S>(n, int(sets));
  int per_sm = 0, sms = 0;
  PII_TRY(quad_kernel_setup<S>(cfg, &per_sm));
  PII_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  if (per_sm < 1) return PII_OK;  // the launch shape does not fit: the direct kernels stay in use
  p->nq_slots = per_sm * sms;
  int64_t units = 0;  // (range, cell) units of the partial sums at the largest use
  for (int64_t c = 1; c <= p->batch_max; ++c) units = std::max(units, int64_t(quad_split(p, cfg, c)) * c);
  const size_t kern = size_t(sets) * 3 * size_t(NJ) * n2 * sizeof(S);  // each of A, B
  const size_t fhT = size_t(p->batch_max) * size_t(n2) * n * sizeof(c2<S>);
  const size_t part = size_t(units) * 3 * n2 * sizeof(c2<S>);
  size_t free_b = 0, total_b = 0;
  PII_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const size_t budget = std::min<size_t>(size_t(16) << 30, free_b / 4);
  const size_t segb = size_t(nseg) * (sizeof(int4) + sizeof(int));
  if (2 * kern + fhT + part + segb > budget) {  // the direct kernels stay in use
    p->nq_nseg = 0;
    return PII_OK;
  }
  S *T = nullptr, *Al = nullptr, *Be = nullptr, *dw = nullptr;
  int *dpts = nullptr, *dq1 = nullptr, *dq2 = nullptr, *dki = nullptr;
  const size_t coef = size_t(QP) * npts * sizeof(S);
  int st = PII_OK;
  auto al = [&](void** dst, size_t b) {
    if (st == PII_OK && cudaMalloc(dst, b) != cudaSuccess) {
      set_error("nyq_quad_prepare: out of memory");
      st = PII_ERR_CUDA;
    }
  };
  al(&p->nq_A, kern);
  al(&p->nq_B, kern);
  al(&p->nq_fhT, fhT);
  al(&p->nq_qpart, part);
  al(&p->nq_segs, segb);
  al((void**)&T, coef);
  al((void**)&Al, coef * sets);
  al((void**)&Be, coef * sets);
  al((void**)&dpts, pts.size() * sizeof(int));
  al((void**)&dq1, q1.size() * sizeof(int));
  al((void**)&dq2, q2.size() * sizeof(int));
  al((void**)&dw, wq.size() * sizeof(S));
  al((void**)&dki, ki.size() * sizeof(int));
  if (st == PII_OK) {
    PII_CUDA(cudaMemcpy(dpts, pts.data(), pts.size() * sizeof(int), cudaMemcpyHostToDevice));
    PII_CUDA(cudaMemcpy(dq1, q1.data(), q1.size() * sizeof(int), cudaMemcpyHostToDevice));
    PII_CUDA(cudaMemcpy(dq2, q2.data(), q2.size() * sizeof(int), cudaMemcpyHostToDevice));
    PII_CUDA(cudaMemcpy(dw, wq.data(), wq.size() * sizeof(S), cudaMemcpyHostToDevice));
    PII_CUDA(cudaMemcpy(dki, ki.data(), ki.size() * sizeof(int), cudaMemcpyHostToDevice));
    PII_CUDA(cudaMemcpy(p->nq_segs, segs.data(), size_t(nseg) * sizeof(int4), cudaMemcpyHostToDevice));
    PII_CUDA(cudaMemcpy(static_cast<char*>(p->nq_segs) + size_t(nseg) * sizeof(int4), seg_j0.data(),
                        size_t(nseg) * sizeof(int), cudaMemcpyHostToDevice));
    const int64_t work = QP * npts * (sets + 1);
    k_quad_coef<S><<<unsigned((work + 255) / 256), 256>>>(
        dpts, npts, n, p->ap_reps, int(QP), p->ns, p->tab.M, static_cast<const c2<S>*>(p->tab.ephase),
        static_cast<const c2<S>*>(p->tab.gphase), static_cast<const S*>(p->tab.gsinc), p->tab.gph_stride,
        p->tab.gs_stride, int(sets), T, Al, Be);
    const dim3 grid(unsigned((n2 + TM - 1) / TM), unsigned((NJ + TM - 1) / TM));
    for (int64_t s = 0; s < sets; ++s)
      for (int d = 0; d < 3; ++d) {
        const int64_t o = (s * 3 + d) * int64_t(NJ) * n2;
        const S *al_s = Al + s * QP * npts, *be_s = Be + s * QP * npts;
        const int *q1d = dq1 + d * NJ, *q2d = dq2 + d * NJ;
        const S* wd = dw + d * NJ;
        // A~ = w (A(k, q) - B(k, -q)),  B~ = w (B(k, q) - A(k, -q))
        k_quad_gemm<S><<<grid, 256>>>(T, al_s, be_s, q1d, q2d, wd, dki + d * n2, static_cast<S*>(p->nq_A) + o, NJ,
                                      n2, int(QP), npts);
        k_quad_gemm<S><<<grid, 256>>>(T, be_s, al_s, q1d, q2d, wd, dki + d * n2, static_cast<S*>(p->nq_B) + o, NJ,
                                      n2, int(QP), npts);
      }
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      set_error("nyq_quad_prepare: %s", cudaGetErrorString(e));
      st = PII_ERR_CUDA;
    }
  }
  for (void* q : {(void*)T, (void*)Al, (void*)Be, (void*)dw, (void*)dpts, (void*)dq1, (void*)dq2, (void*)dki})
    cudaFree(q);
  if (st != PII_OK) {
    free_quad(p);
    return st;
  }
  p->nq_npts = NJ;
  p->nq_qpart_units = units;
  p->nq_quad_bytes = int64_t(2 * kern + fhT + part + segb);
  p->bytes += p->nq_quad_bytes;
  return PII_OK;
}

int nyq_quad_prepare(pii_plan* p) {
  free_quad(p);
  if (p->ap_count <= 0 || p->dim != 3) return PII_OK;
  return p->precision == PII_PREC_FP32 ? quad_prepare_t<float>(p) : quad_prepare_t<double>(p);
}

void nyq_quad_release(pii_plan* p) { free_quad(p); }

// the correction's partial sums (f^ only: it may run beside the gain kernels)
// on stream s, then their sum into G on stream s_add (the caller orders s_add
// after s and after the gain sums' writes of G)
int nyq_quad_run(pii_plan* p, int64_t cells, cudaStream_t s) { return nyq_quad_run2(p, cells, s, s, nullptr); }

template <typename S>
static int quad_run_t(pii_plan* p, int64_t cells, cudaStream_t s, cudaStream_t s_add, cudaEvent_t partial_done) {
  using namespace nqq;
  using V = c2<S>;
  const int n = p->n, n2 = n * n;
  const QuadCfg cfg = quad_cfg<S>(n, int(p->tab.nsets));
  int split = quad_split(p, cfg, cells);
  split = int(std::min<int64_t>(split, p->nq_qpart_units / std::max<int64_t>(cells, 1)));
  if (split < 1) {
    set_error("nyq_quad_run: %lld cells exceed the partial-sum buffer", (long long)cells);
    return PII_ERR_SIZE;
  }
  QuadArgs<S> a{};
  a.A = static_cast<const S*>(p->nq_A);
  a.B = static_cast<const S*>(p->nq_B);
  a.fhat = static_cast<const V*>(p->fhat);
  a.fhT = static_cast<const V*>(p->nq_fhT);
  a.part = static_cast<V*>(p->nq_qpart);
  a.cells = cells;
  a.set_stride = p->tab.nsets > 1 ? int64_t(3) * p->nq_npts * n2 : 0;
  a.segs = static_cast<const int4*>(p->nq_segs);
  a.seg_j0 = reinterpret_cast<const int*>(static_cast<const char*>(p->nq_segs) + size_t(p->nq_nseg) * sizeof(int4));
  a.nseg = p->nq_nseg;
  a.n = n, a.npts = p->nq_npts, a.W = cfg.W, a.split = split;
  {
    StageTimer st(p, ST_NYQ, s);
    const int tb = (n + 31) / 32;
    k_quad_prep<V><<<unsigned(cells * n * tb * tb), 256, 0, s>>>(a.fhat, static_cast<V*>(p->nq_fhT), n, cells);
    PII_CHECK_LAUNCH();
    const dim3 grid(unsigned(n / cfg.W), unsigned((cells + cfg.nc - 1) / cfg.nc), unsigned(3 * split));
    if constexpr (std::is_same<S, float>::value) {
      if (cfg.nc == 2)
        k_nyq_quad<S, 2, 512><<<grid, cfg.threads, cfg.smem, s>>>(a);
      else
        k_nyq_quad<S, 1, 256><<<grid, cfg.threads, cfg.smem, s>>>(a);
    } else {
      if (cfg.nc == 2)
        k_nyq_quad<S, 2, 256><<<grid, cfg.threads, cfg.smem, s>>>(a);
      else
        k_nyq_quad<S, 1, 256><<<grid, cfg.threads, cfg.smem, s>>>(a);
    }
    PII_CHECK_LAUNCH();
  }
  if (partial_done) {
    PII_CUDA(cudaEventRecord(partial_done, s));
    PII_CUDA(cudaStreamWaitEvent(s_add, partial_done, 0));
  }
  StageTimer st(p, ST_NYQ, s_add);
  const int64_t tot = cells * 3 * n2;
  k_quad_add<V><<<unsigned((tot + 255) / 256), 256, 0, s_add>>>(a.part, static_cast<V*>(p->G), n, cells, split);
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int nyq_quad_run2(pii_plan* p, int64_t cells, cudaStream_t s, cudaStream_t s_add, cudaEvent_t partial_done) {
  if (!p->nq_A || p->nq_npts <= 0) {
    set_error("nyq_quad_run: the plan has no quadratic-form kernels");
    return PII_ERR_ARG;
  }
  return p->precision == PII_PREC_FP32 ? quad_run_t<float>(p, cells, s, s_add, partial_done)
                                       : quad_run_t<double>(p, cells, s, s_add, partial_done);
}

}  // namespace pii
