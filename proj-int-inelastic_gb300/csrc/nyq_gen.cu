// Nyquist-plane correction of the packed pipeline, FP32, any even n other than
// 32 (n = 32 has its own shared-memory kernel, nyq_corr.cu).
//
// The packed column passes (COL_PSTART_PK / COL_PEND_PK) evaluate the
// Hermitian parts E+, g+ of each antipodal pair's phase and gain tables
// exactly; what the rest, E- = E - E+ and g- = g - g+, contributes lives on the
// three Nyquist planes of k (a component equal to the storage index h = n / 2,
// its own negative on the grid fftshift(arange(-n/2, n/2)) of
// src/collision/inelastic_collisions.py:62).  Per antipodal pair, on those
// planes only,
//   C(k) = (w.x - w.y) U(k) - (w.x + w.y) conj U(-k),   w = g-_p(k),
//   U    = FFT3(V f),   V = IFFT3(f^ t-),   t- = Re E-_p + Im E-_p.
// t- lives on the Nyquist planes, so with the point sets A = {k_a = h},
// B = {k_b = h, k_a != h}, C = {k_c = h, k_a != h, k_b != h} and P_x the
// unnormalised 2D inverse transform of f^ t- on set x (the 1/n^3 rides on the
// first-axis phase row),
//   V(a, b, c) = (-1)^a P_a(b, c) + (-1)^b P_b(a, c) + (-1)^c P_c(a, b),
// and U on the plane k_a = h is the 2D forward transform of
//   R_a(b, c) = P_a F_a + (-1)^b sum_a (-1)^a P_b(a, c) f + (-1)^c sum_a (-1)^a P_c(a, b) f
// (F_a = sum_a f; likewise R_b, R_c).  A CTA owns one cell and a range of its
// antipodal passes, PB at a time: f^ t- onto the planes, their 2D inverse
// transforms (two threads per line), the three reductions, the 2D forward
// transforms, then C(k) into the CTA's accumulator; k_nyq_gen_add sums the
// CTAs' accumulators into G.  f reaches the reductions a few planes at a time
// (perpendicular to the summed axis), staged in shared memory by cp.async one
// step ahead; k_nyq_gen_prep lays out what the kernel reads: f transposed
// within each a-plane (so that the planes c = const are made of rows too) and
// f^ on the Nyquist planes, compact.
#include <algorithm>

#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {

namespace nqg {
template <int NV>
struct Geo {
  static constexpr int H = NV / 2, N2 = NV * NV, N3 = NV * N2;
  static constexpr int LD = NV + 1, PL = NV * LD;  // padded plane rows
  static constexpr int PB = NV >= 48 ? 1 : 2;     // antipodal pairs per batch
  static constexpr int XS = NV >= 48 ? 2 : 1;     // f planes per staging step of the reductions
  static constexpr int THREADS = 512;
  static constexpr int NPTS = 3 * N2;              // points of the three planes (shared ones counted once each)
  // reductions: thread t owns column t % n, rows t / n + k RG (k < KR)
  static constexpr int RG = THREADS / NV;
  static constexpr int KR = (NV + RG - 1) / RG;
  // shared memory: the planes P[PB][3] (padded), the batch's phase and gain rows
  // [PB][2][3 NV], their Nyquist row factors [PB][2][6 NV], and two buffers of
  // XS f planes [2][XS][n^2] (the reductions' operand, one step ahead)
  static constexpr size_t OFF_ROWS = size_t(PB) * 3 * PL * sizeof(float2);
  static constexpr size_t OFF_FAC = OFF_ROWS + size_t(PB) * 2 * 3 * NV * sizeof(float2);
  static constexpr size_t OFF_FP = OFF_FAC + size_t(PB) * 2 * 6 * NV * sizeof(float2);
  static constexpr size_t SMEM = OFF_FP + size_t(2) * XS * N2 * sizeof(float);
  static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
  static_assert(NV % 4 == 0 && NV % XS == 0, "16-byte plane pieces, whole staging steps");
};
}  // namespace nqg

struct NyqGenArgs {
  const float2* fhn;     // [cells][3 n^2] f^ at the Nyquist-plane points (k_nyq_gen_prep)
  const float* fT;       // [cells][N3] f
  const float* fT2;      // [cells][a][c][b] f transposed within each a-plane (k_nyq_gen_prep)
  const float2* ephase;  // [Q][3][NV]
  const float2* gphase;  // [sets][Q][3][NV]
  const float* gsinc;    // [sets][n_r][M + 1]
  const int* reps;       // [QP] representative pair of each antipodal pass
  int64_t gph_stride, gs_stride;  // elements per restitution set (0: one set)
  int M, ns, QP;
  int64_t cells;
  int blocks;            // CTAs per cell
  float2* part;          // [cells][blocks][3][N2] accumulators
};

__device__ __forceinline__ float2 ng_conj(float2 v) { return make_float2(v.x, -v.y); }

// Row factors of (X(k) - X~(k)) / 2 on the three planes for one table X with
// per-axis rows xa, xb, xc (~ conjugates the factor of a Nyquist component):
//   plane 0, k = (h, r, c): (A0[r] xc(c) - A1[r] xc~(c)) / 2, A0 = xa(h) xb(r), A1 = conj xa(h) xb~(r)
//   plane 1, k = (r, h, c): (B0[r] xc(c) - B1[r] xc~(c)) / 2, B0 = xa(r) xb(h), B1 = xa~(r) conj xb(h)
//   plane 2, k = (r, c, h): (xa(r) C0[c] - xa~(r) C1[c]) / 2, C0 = xb(c) xc(h), C1 = xb~(c) conj xc(h)
// fac = [A0, A1, B0, B1, C0, C1] x NV
template <int NV>
__device__ __forceinline__ float2 ng_row_factor(const float2* rows, int i) {
  constexpr int H = NV / 2;
  const int which = i / NV, r = i - which * NV;
  const float2* xa = rows;
  const float2* xb = rows + NV;
  const float2* xc = rows + 2 * NV;
  auto tl = [](float2 v, int k) { return k == H ? ng_conj(v) : v; };
  switch (which) {
    case 0: return cmul(xa[H], xb[r]);
    case 1: return cmul(ng_conj(xa[H]), tl(xb[r], r));
    case 2: return cmul(xa[r], xb[H]);
    case 3: return cmul(tl(xa[r], r), ng_conj(xb[H]));
    case 4: return cmul(xb[r], xc[H]);
    default: return cmul(tl(xb[r], r), ng_conj(xc[H]));
  }
}
template <int NV>
__device__ __forceinline__ float2 ng_minus(const float2* rows, const float2* fac, int plane, int r, int c) {
  constexpr int H = NV / 2;
  float2 p, q;
  if (plane == 2) {
    const float2 x = rows[r];
    p = cmul(x, fac[4 * NV + c]);
    q = cmul(r == H ? ng_conj(x) : x, fac[5 * NV + c]);
  } else {
    const float2 x = rows[2 * NV + c];
    p = cmul(fac[2 * NV * plane + r], x);
    q = cmul(fac[2 * NV * plane + NV + r], c == H ? ng_conj(x) : x);
  }
  return make_float2(0.5f * (p.x - q.x), 0.5f * (p.y - q.y));
}

// Nyquist point i in [0, 3 n^2): plane 0: k = (h, r, c), plane 1: (r, h, c),
// plane 2: (r, c, h) (storage indices); false where an earlier plane holds it
template <int NV>
__device__ __forceinline__ bool ng_point(int i, int& plane, int& r, int& c, int& ka, int& kb, int& kc) {
  constexpr int H = NV / 2, N2 = NV * NV;
  plane = i / N2;
  const int e = i - plane * N2;
  r = e / NV;
  c = e - r * NV;
  if (plane == 0) {
    ka = H, kb = r, kc = c;
    return true;
  }
  if (plane == 1) {
    ka = r, kb = H, kc = c;
    return r != H;
  }
  ka = r, kb = c, kc = H;
  return r != H && c != H;
}

// unnormalised 2D transforms of `np` padded planes in place: rows, then
// columns, two threads per line split by output parity (decimation in
// frequency: the even outputs are the half-length transform of x_j + x_{j+n/2},
// the odd ones of (x_j - x_{j+n/2}) w^j), so a thread holds half a line.  The
// tasks run in rounds of one per thread; both threads of a line are in the same
// round and read it before the barrier that precedes their writes.  Every
// thread of the CTA calls it (unconditional barriers).
template <int NV, int DIR>
__device__ __forceinline__ void ng_planes_fft2(float2* P, int np) {
  using G = nqg::Geo<NV>;
  constexpr int HN = NV / 2;
  static_assert(G::THREADS % 2 == 0, "the two halves of a line share a round");
  float2 y[HN];
  const int tasks = np * NV * 2;
#pragma unroll 1
  for (int pass = 0; pass < 2; ++pass) {
    const int stride = pass == 0 ? 1 : G::LD;
#pragma unroll 1
    for (int r0 = 0; r0 < tasks; r0 += G::THREADS) {
      const int task = r0 + int(threadIdx.x);
      const bool on = task < tasks;
      const int par = task & 1, l = task >> 1;
      const int pl = l / NV, line = l - pl * NV;
      float2* L = P + pl * G::PL + (pass == 0 ? line * G::LD : line);
      if (on) {
        if (par == 0) {
#pragma unroll
          for (int j = 0; j < HN; ++j) y[j] = cadd(L[j * stride], L[(j + HN) * stride]);
        } else {
          static_for<0, HN>([&](auto ji) {
            constexpr int j = decltype(ji)::value;
            y[j] = twiddle<j, NV, DIR>(csub(L[j * stride], L[(j + HN) * stride]));
          });
        }
        fft_line<HN, DIR>(y);
      }
      __syncthreads();  // both halves of every line of the round have been read
      if (on) {
        static_for<0, HN>([&](auto mi) {
          constexpr int m = decltype(mi)::value;
          L[(2 * m + par) * stride] = y[pos(HN, m)];
        });
      }
      __syncthreads();
    }
  }
}

// f^ at the Nyquist-plane points, compact, and f transposed within each
// a-plane: fT2[cell][a][c][b] = f[cell][a][b][c] (32 x 32 tiles through shared memory)
template <int NV>
__global__ void __launch_bounds__(256) k_nyq_gen_prep(const float2* fhat, const float* fT, float2* fhn, float* fT2,
                                                       int64_t cells) {
  using G = nqg::Geo<NV>;
  __shared__ float tile[32][33];
  constexpr int TB = (NV + 31) / 32;  // 32 x 32 tiles per plane side
  const int64_t bid = blockIdx.x;
  const int64_t tiles = cells * NV * TB * TB;
  if (bid < tiles) {
    const int64_t cp = bid / (TB * TB);  // (cell, a)
    const int tt = int(bid - cp * TB * TB), tb = tt / TB, tc = tt - tb * TB;
    const float* src = fT + cp * G::N2;
    float* dst = fT2 + cp * G::N2;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int j = ty; j < 32; j += 8) {
      const int b = tb * 32 + j, c = tc * 32 + tx;
      if (b < NV && c < NV) tile[j][tx] = src[b * NV + c];
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
      const int c = tc * 32 + j, b = tb * 32 + tx;
      if (b < NV && c < NV) dst[c * NV + b] = tile[tx][j];
    }
  } else {
    const int64_t gid = (bid - tiles) * 256 + threadIdx.x;
    if (gid >= cells * G::NPTS) return;
    const int64_t cell = gid / G::NPTS;
    const int i = int(gid - cell * G::NPTS);
    int plane, r, c, ka, kb, kc;
    ng_point<NV>(i, plane, r, c, ka, kb, kc);
    fhn[gid] = fhat[cell * G::N3 + int64_t(ka) * G::N2 + kb * NV + kc];
  }
}

template <int NV>
__global__ void __launch_bounds__(nqg::Geo<NV>::THREADS, 1) k_nyq_gen(NyqGenArgs a) {
  using G = nqg::Geo<NV>;
  constexpr int N2 = G::N2, N3 = G::N3, PB = G::PB, LD = G::LD, PL = G::PL, XS = G::XS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* P = reinterpret_cast<float2*>(smem_raw);                 // [PB][3][PL]
  float2* Rows = reinterpret_cast<float2*>(smem_raw + G::OFF_ROWS);  // [PB][2][3 NV]: phase, gain
  float2* Fac = reinterpret_cast<float2*>(smem_raw + G::OFF_FAC);    // [PB][2][6 NV]
  float* Fp = reinterpret_cast<float*>(smem_raw + G::OFF_FP);        // [2][XS][n^2]: f planes
  const int t = threadIdx.x;
  const int64_t cell = blockIdx.x / a.blocks;
  const int blk = int(blockIdx.x - cell * a.blocks);
  const int per = (a.QP + a.blocks - 1) / a.blocks;
  const int i0 = blk * per, i1 = min(a.QP, i0 + per);
  const float2* fhn = a.fhn + cell * G::NPTS;
  const float* fr = a.fT + cell * N3;
  const float* fr2 = a.fT2 + cell * N3;
  const float2* gph = a.gphase + cell * a.gph_stride;
  const float* gsn = a.gsinc + cell * a.gs_stride;
  float2* acc = a.part + (cell * a.blocks + blk) * int64_t(G::NPTS);  // this CTA's accumulator
  for (int i = t; i < G::NPTS; i += G::THREADS) acc[i] = make_float2(0.f, 0.f);
  // planes x .. x + XS - 1 of f along the summed axis of reduction `lay`, each as
  // [u][v] (the outputs' row and column), into buffer buf: lay 0: f[x][u][v];
  // lay 1: f[u][x][v]; lay 2: f(u, v, x) = fT2[u][x][v].  One cp.async group.
  auto stage_planes = [&](int lay, int x, int buf) {
    for (int q = t; q < XS * N2 / 4; q += G::THREADS) {
      const int xi = (4 * q) / N2, e = 4 * q - xi * N2;
      const int u = e / NV, v = e - u * NV;
      const float* src = lay == 0 ? fr + int64_t(x + xi) * N2 + e
                                  : (lay == 1 ? fr : fr2) + int64_t(u) * N2 + (x + xi) * NV + v;
      cp_async16(Fp + (buf * XS + xi) * N2 + e, src);
    }
    cp_async_commit();
  };

  for (int ib = i0; ib < i1; ib += PB) {
    const int nb = min(PB, i1 - ib);
    stage_planes(0, 0, 0);  // the first reduction's first planes, in flight from here
    // ---- 0. the batch's phase and gain rows, then their row factors
    for (int i = t; i < PB * 2 * 3 * NV; i += G::THREADS) {
      const int s = i / (6 * NV), w = (i / (3 * NV)) & 1, e = i % (3 * NV);
      float2 v = make_float2(0.f, 0.f);
      if (s < nb) {
        const int64_t pair = a.reps[ib + s];
        v = (w == 0 ? a.ephase : gph)[pair * 3 * NV + e];
      }
      Rows[i] = v;
    }
    __syncthreads();
    for (int i = t; i < PB * 2 * 6 * NV; i += G::THREADS) {
      const int sw = i / (6 * NV);  // (pair, table) = (sw / 2, sw % 2)
      Fac[i] = ng_row_factor<NV>(Rows + sw * 3 * NV, i - sw * 6 * NV);
    }
    __syncthreads();
    // ---- 1. f^ t- on the three point sets (0 elsewhere on the planes)
    for (int i = t; i < PB * G::NPTS; i += G::THREADS) {
      const int s = i / G::NPTS, ii = i - s * G::NPTS;
      int plane, r, c, ka, kb, kc;
      const bool on = ng_point<NV>(ii, plane, r, c, ka, kb, kc) && s < nb;
      float2 y = make_float2(0.f, 0.f);
      if (on) {
        const float2 em = ng_minus<NV>(Rows + s * 6 * NV, Fac + s * 12 * NV, plane, r, c);
        const float tm = em.x + em.y;
        const float2 fv = fhn[ii];
        y = make_float2(fv.x * tm, fv.y * tm);
      }
      P[(s * 3 + plane) * PL + r * LD + c] = y;
    }
    __syncthreads();
    // ---- 2. P = unnormalised 2D inverse transforms
    ng_planes_fft2<NV, +1>(P, 3 * PB);
    // ---- 3. reductions R_a (plane 0: outputs (b, c)), R_b (1: (a, c)), R_c (2: (a, b)),
    // kept in registers until every plane has been read.  Thread t owns the
    // outputs (u, v) of column v = t % n and rows u = t / n + k RG: the plane
    // value indexed by v (ps) is loaded once per x for all of its rows.  The f
    // planes of each step are in shared memory; the next step's are copied meanwhile.
    float2 R[3][G::KR][PB];
    const bool act = t < G::RG * NV;
    const int v = t % NV, r0 = t / NV;
#pragma unroll
    for (int lay = 0; lay < 3; ++lay) {
      float2 sh[G::KR][PB], un[G::KR][PB];
      float F[G::KR];
#pragma unroll
      for (int k = 0; k < G::KR; ++k) {
        F[k] = 0.f;
#pragma unroll
        for (int s = 0; s < PB; ++s) sh[k][s] = un[k][s] = make_float2(0.f, 0.f);
      }
#pragma unroll 1
      for (int x0 = 0; x0 < NV; x0 += XS) {
        const int buf = ((lay * NV + x0) / XS) & 1;
        // the next step's planes (of this reduction, or the next one's first) into the other buffer
        const bool next = x0 + XS < NV || lay < 2;
        if (x0 + XS < NV)
          stage_planes(lay, x0 + XS, buf ^ 1);
        else if (lay < 2)
          stage_planes(lay + 1, 0, buf ^ 1);
        // this step's planes have landed: only the group just issued may still be pending
        if (next)
          cp_async_wait_group<1>();
        else
          cp_async_wait_group<0>();
        __syncthreads();
        if (act) {
#pragma unroll
          for (int xi = 0; xi < XS; ++xi) {
            const int x = x0 + xi;
            const float* fp = Fp + (buf * XS + xi) * N2;
            const float sx = (x & 1) ? -1.f : 1.f;
#pragma unroll
            for (int s = 0; s < PB; ++s) {
              const float2* Pa = P + (s * 3 + 0) * PL;
              const float2* Pb = P + (s * 3 + 1) * PL;
              const float2* Pc = P + (s * 3 + 2) * PL;
              // the shared term: P_b(a = x, c = v), P_a(b = x, c = v), P_a(b = v, c = x)
              const float2 ps = lay == 0 ? Pb[x * LD + v] : lay == 1 ? Pa[x * LD + v] : Pa[v * LD + x];
#pragma unroll
              for (int k = 0; k < G::KR; ++k) {
                const int u = r0 + k * G::RG;
                if (u >= NV) break;
                // the row term: P_c(a = x, b = u), P_c(a = u, b = x), P_b(a = u, c = x)
                const float2 pu = lay == 0 ? Pc[x * LD + u] : lay == 1 ? Pc[u * LD + x] : Pb[u * LD + x];
                const float g0 = fp[u * NV + v];
                if (s == 0) F[k] += g0;
                const float g = sx * g0;
                sh[k][s].x = fmaf(ps.x, g, sh[k][s].x), sh[k][s].y = fmaf(ps.y, g, sh[k][s].y);
                un[k][s].x = fmaf(pu.x, g, un[k][s].x), un[k][s].y = fmaf(pu.y, g, un[k][s].y);
              }
            }
          }
        }
        __syncthreads();  // the buffer is rewritten two steps on
      }
      // R_a = P_a F + (-1)^b sh + (-1)^c un;  R_b = (-1)^a sh + P_b F + (-1)^c un;
      // R_c = (-1)^a sh + (-1)^b un + P_c F  (the own plane is plane `lay`):
      // sh takes (-1)^u, un (-1)^v
      const float sv = (v & 1) ? -1.f : 1.f;
#pragma unroll
      for (int k = 0; k < G::KR; ++k) {
        const int u = r0 + k * G::RG;
        const float su = (u & 1) ? -1.f : 1.f;
#pragma unroll
        for (int s = 0; s < PB; ++s) {
          const float2 own = act && u < NV ? P[(s * 3 + lay) * PL + u * LD + v] : make_float2(0.f, 0.f);
          R[lay][k][s] = make_float2(own.x * F[k] + su * sh[k][s].x + sv * un[k][s].x,
                                     own.y * F[k] + su * sh[k][s].y + sv * un[k][s].y);
        }
      }
    }
    // (the last barrier of the loop above: every plane of P has been read)
    if (act) {
#pragma unroll
      for (int lay = 0; lay < 3; ++lay)
#pragma unroll
        for (int k = 0; k < G::KR; ++k) {
          const int u = r0 + k * G::RG;
          if (u >= NV) break;
#pragma unroll
          for (int s = 0; s < PB; ++s) P[(s * 3 + lay) * PL + u * LD + v] = R[lay][k][s];
        }
    }
    __syncthreads();
    // ---- 4. U = unnormalised 2D forward transforms of R
    ng_planes_fft2<NV, -1>(P, 3 * PB);
    // ---- 5. C(k) = (w.x - w.y) U(k) - (w.x + w.y) conj U(-k), w = g-_p(k) gsinc, accumulated
    for (int i = t; i < G::NPTS; i += G::THREADS) {
      int plane, r, c, ka, kb, kc;
      if (!ng_point<NV>(i, plane, r, c, ka, kb, kc)) continue;
      const int nr = (NV - r) % NV, nc = (NV - c) % NV;
      const int kk = kval(ka, NV) * kval(ka, NV) + kval(kb, NV) * kval(kb, NV) + kval(kc, NV) * kval(kc, NV);
      float2 av = acc[i];
#pragma unroll
      for (int s = 0; s < PB; ++s) {
        if (s >= nb) break;
        const int p = a.reps[ib + s];
        const float gsv = gsn[int64_t(p / a.ns) * (a.M + 1) + kk];
        const float2 gm = ng_minus<NV>(Rows + s * 6 * NV + 3 * NV, Fac + s * 12 * NV + 6 * NV, plane, r, c);
        const float wx = gsv * gm.x, wy = gsv * gm.y;
        const float2 uu = P[(s * 3 + plane) * PL + r * LD + c];
        const float2 um = P[(s * 3 + plane) * PL + nr * LD + nc];
        const float cp = wx - wy, cm = wx + wy;
        av.x += cp * uu.x - cm * um.x;
        av.y += cp * uu.y + cm * um.y;
      }
      acc[i] = av;  // each thread owns the same points in every batch
    }
    __syncthreads();  // the planes and rows are rewritten by the next batch
  }
}

// G[cell][k] += sum over the cell's CTAs of the correction at the Nyquist points
template <int NV>
__global__ void __launch_bounds__(256) k_nyq_gen_add(float2* Gsum, const float2* part, int64_t cells, int blocks) {
  using G = nqg::Geo<NV>;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * G::NPTS) return;
  const int64_t cell = gid / G::NPTS;
  const int i = int(gid - cell * G::NPTS);
  int plane, r, c, ka, kb, kc;
  if (!ng_point<NV>(i, plane, r, c, ka, kb, kc)) return;
  float2 s = make_float2(0.f, 0.f);
  for (int b = 0; b < blocks; ++b) {
    const float2 v = part[(cell * blocks + b) * int64_t(G::NPTS) + i];
    s.x += v.x;
    s.y += v.y;
  }
  float2* g = Gsum + cell * G::N3 + int64_t(ka) * G::N2 + kb * NV + kc;
  g->x += s.x;
  g->y += s.y;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int NV>
static int nyq_gen_prepare_t(pii_plan* p) {
  using G = nqg::Geo<NV>;
  PII_CUDA(cudaFuncSetAttribute(k_nyq_gen<NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(G::SMEM)));
  int sms = 0;
  PII_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  // accumulators of at most 4 waves of CTAs or one CTA per cell
  const size_t ctas = std::max<size_t>(size_t(4) * sms, size_t(p->batch_max));
  const size_t bytes = ctas * size_t(G::NPTS) * sizeof(float2);
  PII_CUDA(cudaMalloc(&p->nq_part, bytes));
  p->bytes += int64_t(bytes);
  p->nq_ctas = int64_t(ctas);
  // the transposed f and the compact Nyquist-plane spectra of every cell
  const size_t b2 = size_t(p->batch_max) * G::N3 * sizeof(float), b3 = size_t(p->batch_max) * G::NPTS * sizeof(float2);
  PII_CUDA(cudaMalloc(&p->nq_ft2, b2));
  PII_CUDA(cudaMalloc(&p->nq_fhn, b3));
  p->bytes += int64_t(b2 + b3);
  return PII_OK;
}

int nyq_gen_prepare(pii_plan* p) {
  switch (p->n) {
    case 8: return nyq_gen_prepare_t<8>(p);
    case 16: return nyq_gen_prepare_t<16>(p);
    case 24: return nyq_gen_prepare_t<24>(p);
    case 48: return nyq_gen_prepare_t<48>(p);
    case 64: return nyq_gen_prepare_t<64>(p);
    default: set_error("nyq_gen_prepare: n = %d has no general Nyquist correction", p->n); return PII_ERR_ARG;
  }
}

template <int NV>
static int nyq_gen_run_t(pii_plan* p, int64_t cells, cudaStream_t s) {
  using G = nqg::Geo<NV>;
  NyqGenArgs a{};
  a.fhn = static_cast<const float2*>(p->nq_fhn);
  a.fT = static_cast<const float*>(p->fT);
  a.fT2 = static_cast<const float*>(p->nq_ft2);
  a.ephase = static_cast<const float2*>(p->tab.ephase);
  a.gphase = static_cast<const float2*>(p->tab.gphase);
  a.gsinc = static_cast<const float*>(p->tab.gsinc);
  a.reps = p->ap_reps;
  a.gph_stride = p->tab.gph_stride;
  a.gs_stride = p->tab.gs_stride;
  a.M = p->tab.M;
  a.ns = p->ns;
  a.QP = p->ap_count;
  a.cells = cells;
  int sms = 0;
  PII_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  // CTAs per cell: about 4 waves over the whole batch, each with at least 4
  // antipodal passes, within the accumulator buffer
  const int64_t bmax = std::max<int64_t>(1, std::min<int64_t>(a.QP / 4, p->nq_ctas / cells));
  a.blocks = int(std::min<int64_t>(bmax, std::max<int64_t>(1, (4 * int64_t(sms) + cells - 1) / cells)));
  a.part = static_cast<float2*>(p->nq_part);
  {
    StageTimer st(p, ST_NYQ, s);
    constexpr int TB = (NV + 31) / 32;
    const int64_t tiles = cells * NV * TB * TB, pts = (cells * G::NPTS + 255) / 256;
    k_nyq_gen_prep<NV><<<unsigned(tiles + pts), 256, 0, s>>>(static_cast<const float2*>(p->fhat),
                                                             static_cast<const float*>(p->fT),
                                                             static_cast<float2*>(p->nq_fhn),
                                                             static_cast<float*>(p->nq_ft2), cells);
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_NYQ, s);
    k_nyq_gen<NV><<<unsigned(cells * a.blocks), G::THREADS, G::SMEM, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_NYQ, s);
    k_nyq_gen_add<NV><<<unsigned((cells * G::NPTS + 255) / 256), 256, 0, s>>>(static_cast<float2*>(p->G), a.part,
                                                                             cells, a.blocks);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int nyq_gen_run(pii_plan* p, int64_t cells, cudaStream_t s) {
  if (!p->nq_part || p->ap_count <= 0) {
    set_error("nyq_gen_run: the plan has no antipodal passes or correction buffer");
    return PII_ERR_ARG;
  }
  switch (p->n) {
    case 8: return nyq_gen_run_t<8>(p, cells, s);
    case 16: return nyq_gen_run_t<16>(p, cells, s);
    case 24: return nyq_gen_run_t<24>(p, cells, s);
    case 48: return nyq_gen_run_t<48>(p, cells, s);
    case 64: return nyq_gen_run_t<64>(p, cells, s);
    default: set_error("nyq_gen_run: n = %d has no general Nyquist correction", p->n); return PII_ERR_ARG;
  }
}

}  // namespace pii
