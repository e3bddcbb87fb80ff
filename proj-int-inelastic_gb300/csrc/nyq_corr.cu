// Nyquist-plane correction of the packed (antipodal) gain kernel, n = 32, FP32.
//
// For a pair p with phase E (src/collision/inelastic_collisions.py:91-105) split
// as E = E+ + E- (E+ Hermitian, E- = (E(k) - conj E(-k)) / 2, non-zero only where
// a component of k is the Nyquist index 16) and gain g = g+ + g-, the packed
// kernel adds g+ B_R exactly; what it leaves out is, per antipodal pair
// (p, q = -sigma_p), on the three Nyquist planes of k only,
//   C(k) = (w.x - w.y) U(k) - (w.x + w.y) conj U(-k),   w = g-_p(k),
//   U    = FFT3(V f),   V = IFFT3(f^ t-),   t- = Re E-_p + Im E-_p.
// t- lives on the Nyquist planes of k, so V is a sum of three lifted 2D
// transforms: with the point sets A = {k_a = 16}, B = {k_b = 16, k_a != 16},
// C = {k_c = 16, k_a != 16, k_b != 16},
//   V(a,b,c) = (-1)^a P_a(b,c) + (-1)^b P_b(a,c) + (-1)^c P_c(a,b),
// P_x the unnormalised 2D inverse transform of f^ t- on set x (the 1/n^3 rides
// on the first-axis phase row).  U on plane k_a = 16 is the 2D forward
// transform of R_a(b,c) = sum_a (-1)^a V f (and likewise R_b, R_c), and
//   R_a = P_a F_a + (-1)^b sum_a (-1)^a P_b(a,c) f + (-1)^c sum_a (-1)^a P_c(a,b) f,
//   R_b = (-1)^a sum_b (-1)^b P_a(b,c) f + P_b F_b + (-1)^c sum_b (-1)^b P_c(a,b) f,
//   R_c = (-1)^a sum_c (-1)^c P_a(b,c) f + (-1)^b sum_c (-1)^c P_b(a,c) f + P_c F_c,
// with F_a = sum_a f etc.  A CTA owns one cell and a range of antipodal pairs,
// two at a time: build f^ t- on the three sets, six 2D inverse transforms, the
// reductions with f resident in shared memory (three thread layouts: (b,c),
// (a,c), (a,b) columns), six 2D forward transforms, then C(k) into per-thread
// accumulators.  k_nyq_add sums the CTAs' accumulators into G.
#include <algorithm>

#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {

namespace nq {
constexpr int N2 = 1024, N3 = 32768;
constexpr int THREADS = 512;
constexpr int PB = 2;        // antipodal pairs per batch
constexpr int PL = 32 * 33;  // plane footprint: rows padded to 33 (row and column access conflict-free)
// shared memory: f of the cell [a][b][c ^ b] (float), f^ on the three Nyquist
// planes [3][N2] (float2), P[PB][3] planes (float2), the phase / gain rows of
// two batches [2][PB][2][96] (the next batch's copied by cp.async while this
// one runs), the batch's row factors [PB][2][6 x 32] (float2) and the radial
// sinc values of two batches [2][PB][GSN] (staged like the rows); the
// correction accumulator lives in registers (each thread owns the same points
// in every batch)
constexpr size_t OFF_P = size_t(N3) * sizeof(float) + size_t(3 * N2) * sizeof(float2);
// radial sinc values gsinc[r][m] of a pair's radial node on the Nyquist planes:
// m = |k|^2 in [256, 768], 513 of them (padded to 516)
constexpr int GSN = 516;
constexpr size_t OFF_GS = OFF_P + size_t(3 * PB) * PL * sizeof(float2) + size_t(2 * PB) * 2 * 96 * sizeof(float2) +
                          size_t(PB) * 2 * 6 * 32 * sizeof(float2);
constexpr size_t SMEM = OFF_GS + size_t(2 * PB) * GSN * sizeof(float);
static_assert(SMEM <= 232448, "shared memory per CTA");
static_assert((OFF_P + size_t(3 * PB) * PL * sizeof(float2)) % 16 == 0, "cp.async destinations are 16-byte aligned");
constexpr int PTS = 3 * N2 / THREADS;  // Nyquist points per thread
__device__ __forceinline__ int sw(int r, int c) { return r * 33 + c; }
__device__ __forceinline__ int fidx(int a, int b, int c) { return a * N2 + b * 32 + (c ^ b); }
}  // namespace nq

struct NyqArgs {
  const float2* fhat;    // [cells][N3]
  const float* fT;       // [cells][N3]
  const float2* ephase;  // [Q][3][32]
  const float2* gphase;  // [Q][3][32]
  const float* gsinc;    // [n_r][M + 1]
  const int* reps;       // [QP] representative pair of each antipodal pass
  int64_t gph_stride;    // complex elements of gphase per restitution set (0: one set)
  int64_t gs_stride;     // floats of gsinc per restitution set (0: one set)
  int M, ns, QP;
  int64_t cells;
  int blocks;            // CTAs per cell
  float2* part;          // [cells][blocks][3][N2]
};

__device__ __forceinline__ float2 nq_conj(float2 v) { return make_float2(v.x, -v.y); }

// 2D transform of padded 32 x 32 planes in place, two warps per plane: lane =
// line, warp parity = parity of the outputs the warp produces (decimation in
// frequency: even outputs are the 16-point transform of x_j + x_{j+16}, odd
// ones of (x_j - x_{j+16}) w^j).  Every thread of the CTA calls it: its
// barriers are unconditional; only warps with a plane compute.
template <int DIR, int PAR>
__device__ __forceinline__ void split_half(const float2* L, int stride, float2 (&y)[16]) {
  float2 x[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) x[j] = L[j * stride];
  static_for<0, 16>([&](auto ji) {
    constexpr int j = decltype(ji)::value;
    y[j] = PAR == 0 ? cadd(x[j], x[j + 16]) : twiddle<j, 32, DIR>(csub(x[j], x[j + 16]));
  });
  fft_line<16, DIR>(y);
}

template <int PAR>
__device__ __forceinline__ void split_store(float2* L, int stride, const float2 (&y)[16]) {
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    L[(2 * m + PAR) * stride] = y[pos(16, m)];
  });
}

template <int DIR>
__device__ __forceinline__ void planes_fft2(float2* base, int nplanes, int warp, int lane) {
  using namespace nq;
  const int plane = warp >> 1, par = warp & 1;
  const bool active = plane < nplanes;
  float2* P = base + (active ? plane : 0) * PL;
  float2 y[16];
#pragma unroll 1
  for (int pass = 0; pass < 2; ++pass) {
    // pass 0: line = row `lane` (elements along the row); pass 1: column `lane`
    float2* L = pass == 0 ? P + lane * 33 : P + lane;
    const int stride = pass == 0 ? 1 : 33;
    if (active) {
      if (par == 0)
        split_half<DIR, 0>(L, stride, y);
      else
        split_half<DIR, 1>(L, stride, y);
    }
    __syncthreads();  // both halves of every line have been read
    if (active) {
      if (par == 0)
        split_store<0>(L, stride, y);
      else
        split_store<1>(L, stride, y);
    }
    __syncthreads();
  }
}

// (E(k) - E~(k)) / 2 and (g(k) - g~(k)) / 2 for k = (ka, kb, kc): ~ conjugates
// the factor of every Nyquist component
__device__ __forceinline__ float2 minus_part(const float2* rows, int ka, int kb, int kc) {
  const float2 xa = rows[ka], xb = rows[32 + kb], xc = rows[64 + kc];
  const float2 p = cmul(cmul(xa, xb), xc);
  const float2 q = cmul(cmul(ka == 16 ? nq_conj(xa) : xa, kb == 16 ? nq_conj(xb) : xb), kc == 16 ? nq_conj(xc) : xc);
  return make_float2(0.5f * (p.x - q.x), 0.5f * (p.y - q.y));
}

// Row factors of (X(k) - X~(k)) / 2 on the three planes for one table X (the
// per-axis rows xa, xb, xc; ~ conjugates the factor of a Nyquist component):
//   plane 0, k = (16, r, c): (A0[r] xc(c) - A1[r] xc~(c)) / 2, A0 = xa(16) xb(r), A1 = conj xa(16) xb~(r)
//   plane 1, k = (r, 16, c): (B0[r] xc(c) - B1[r] xc~(c)) / 2, B0 = xa(r) xb(16), B1 = xa~(r) conj xb(16)
//   plane 2, k = (r, c, 16): (xa(r) C0[c] - xa~(r) C1[c]) / 2, C0 = xb(c) xc(16), C1 = xb~(c) conj xc(16)
// fac = [A0, A1, B0, B1, C0, C1] x 32
__device__ __forceinline__ void row_factors(const float2* rows, float2* fac, int i) {
  const int which = i >> 5, r = i & 31;
  const float2* xa = rows;
  const float2* xb = rows + 32;
  const float2* xc = rows + 64;
  auto tl = [](float2 v, int k) { return k == 16 ? nq_conj(v) : v; };
  float2 v;
  switch (which) {
    case 0: v = cmul(xa[16], xb[r]); break;
    case 1: v = cmul(nq_conj(xa[16]), tl(xb[r], r)); break;
    case 2: v = cmul(xa[r], xb[16]); break;
    case 3: v = cmul(tl(xa[r], r), nq_conj(xb[16])); break;
    case 4: v = cmul(xb[r], xc[16]); break;
    default: v = cmul(tl(xb[r], r), nq_conj(xc[16])); break;
  }
  fac[i] = v;
}
__device__ __forceinline__ float2 minus_from(const float2* rows, const float2* fac, int plane, int r, int c) {
  float2 p, q;
  if (plane == 2) {
    const float2 x = rows[r];
    p = cmul(x, fac[128 + c]);
    q = cmul(r == 16 ? nq_conj(x) : x, fac[160 + c]);
  } else {
    const float2 x = rows[64 + c];
    p = cmul(fac[64 * plane + r], x);
    q = cmul(fac[64 * plane + 32 + r], c == 16 ? nq_conj(x) : x);
  }
  return make_float2(0.5f * (p.x - q.x), 0.5f * (p.y - q.y));
}

// set / in-plane index of Nyquist point i in [0, 3 N2): plane 0: k = (16, r, c),
// plane 1: (r, 16, c), plane 2: (r, c, 16); a point belongs to the first plane holding it
__device__ __forceinline__ bool nyq_point(int i, int& plane, int& r, int& c, int& ka, int& kb, int& kc) {
  plane = i >> 10;
  r = (i >> 5) & 31;
  c = i & 31;
  if (plane == 0) {
    ka = 16, kb = r, kc = c;
    return true;
  }
  if (plane == 1) {
    ka = r, kb = 16, kc = c;
    return r != 16;
  }
  ka = r, kb = c, kc = 16;
  return r != 16 && c != 16;
}

__global__ void __launch_bounds__(nq::THREADS, 1) k_nyq_corr(NyqArgs a) {
  using namespace nq;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* fS = reinterpret_cast<float*>(smem_raw);  // f(a, b, c) at fidx(a, b, c)
  float2* Fh = reinterpret_cast<float2*>(fS + N3);  // [3][N2]: f^(16,r,c), f^(r,16,c), f^(r,c,16)
  float2* P = reinterpret_cast<float2*>(smem_raw + OFF_P);  // [PB][3] planes: P, then R, then U
  float2* RowsBuf = P + PB * 3 * PL;                         // [2][PB][2][96]: phase rows, gain rows
  float2* Fac = RowsBuf + 2 * PB * 2 * 96;                   // [PB][2][6 x 32] row factors
  float* GsBuf = reinterpret_cast<float*>(smem_raw + OFF_GS);  // [2][PB][GSN] radial sinc values
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int64_t cell = blockIdx.x / a.blocks;
  const int blk = int(blockIdx.x - cell * a.blocks);
  const int per = (a.QP + a.blocks - 1) / a.blocks;
  const int i0 = blk * per, i1 = min(a.QP, i0 + per);
  const float2* fh = a.fhat + cell * N3;
  const float* fr = a.fT + cell * N3;

  for (int i = t; i < N3; i += THREADS) fS[fidx(i >> 10, (i >> 5) & 31, i & 31)] = fr[i];
  for (int i = t; i < 3 * N2; i += THREADS) {
    const int plane = i >> 10, r = (i >> 5) & 31, c = i & 31;
    Fh[i] = fh[plane == 0 ? (16 * N2 + r * 32 + c) : plane == 1 ? (r * N2 + 16 * 32 + c) : (r * N2 + c * 32 + 16)];
  }
  // rows of the nbn pairs from jb into buffer b: 16-byte copies (a row is 48),
  // zeros for absent pairs; and their radial sinc values gsinc[r][256 ..] (4-byte copies)
  const float* gsn = a.gsinc + cell * a.gs_stride;
  auto stage_rows = [&](int jb, int nbn, int b) {
    float2* dst = RowsBuf + b * PB * 192;
    for (int i = t; i < PB * 2 * 48; i += THREADS) {
      const int sidx = i / 96, w = (i / 48) & 1, e = 2 * (i % 48);
      float2* d = dst + sidx * 192 + w * 96 + e;
      if (sidx < nbn) {
        cp_async16(d, (w == 0 ? a.ephase : a.gphase + cell * a.gph_stride) + int64_t(a.reps[jb + sidx]) * 96 + e);
      } else {
        d[0] = make_float2(0.f, 0.f);
        d[1] = make_float2(0.f, 0.f);
      }
    }
    float* gdst = GsBuf + b * PB * GSN;
    for (int i = t; i < PB * 513; i += THREADS) {
      const int sidx = i / 513, m = i - sidx * 513;
      if (sidx < nbn) cp_async4(gdst + sidx * GSN + m, gsn + int64_t(a.reps[jb + sidx] / a.ns) * (a.M + 1) + 256 + m);
    }
  };
  if (i0 < i1) stage_rows(i0, min(PB, i1 - i0), 0);
  cp_async_wait_all();
  float2 acc[PTS];
#pragma unroll
  for (int k = 0; k < PTS; ++k) acc[k] = make_float2(0.f, 0.f);
  __syncthreads();

  for (int ib = i0, bp = 0; ib < i1; ib += PB, bp ^= 1) {
    const int nb = min(PB, i1 - ib);
    const float2* Rows = RowsBuf + bp * PB * 192;  // this batch's rows (staged during the previous batch)
    const float* Gs = GsBuf + bp * PB * GSN;       // and their radial sinc values
    // the next batch's rows into the other buffer, last read before the previous batch's final barrier
    if (ib + PB < i1) stage_rows(ib + PB, min(PB, i1 - ib - PB), bp ^ 1);
    for (int i = t; i < PB * 2 * 192; i += THREADS) row_factors(Rows + (i / 192) * 96, Fac + (i / 192) * 192, i % 192);
    __syncthreads();
    // ---- 1. f^ t- on the three point sets (0 elsewhere on the planes)
#pragma unroll 4
    for (int it = 0; it < PB * 3 * N2 / THREADS; ++it) {  // fixed trip count: loads of several points in flight
      const int i = t + it * THREADS;
      const int s = i / (3 * N2);
      const int ii = i - s * 3 * N2;
      int plane, r, c, ka, kb, kc;
      const bool on = nyq_point(ii, plane, r, c, ka, kb, kc) && s < nb;
      float2 y = make_float2(0.f, 0.f);
      if (on) {
        const float2 em = minus_from(Rows + s * 192, Fac + s * 384, plane, r, c);
        const float tm = em.x + em.y;
        const float2 fv = Fh[ii];
        y = make_float2(fv.x * tm, fv.y * tm);
      }
      P[(s * 3 + plane) * PL + sw(r, c)] = y;
    }
    __syncthreads();
    // ---- 2. P = unnormalised 2D inverse transforms (two warps per plane)
    planes_fft2<+1>(P, 3 * nb, warp, lane);
    // ---- 3. reductions R_a (lay 0), R_b (1), R_c (2) for both pairs of the
    // batch; outputs (row w and w + 16, column lane) of the layout's plane;
    // results stay in registers until every layout has read the P planes
    float2 Rr[3][2][PB];
#pragma unroll
    for (int lay = 0; lay < 3; ++lay) {
      const int o0 = warp, o1 = warp + 16;
      float2 sh[2][PB], un[2][PB];
#pragma unroll
      for (int s = 0; s < PB; ++s) sh[0][s] = sh[1][s] = un[0][s] = un[1][s] = make_float2(0.f, 0.f);
      float F0 = 0.f, F1 = 0.f;  // sums of f along the axis (the own-plane term)
#pragma unroll 8
      for (int x = 0; x < 32; ++x) {
        // f along the summed axis for the two outputs, signed by (-1)^x
        float g0, g1;
        if (lay == 0) {  // outputs (b, c): f(x, b, c)
          g0 = fS[fidx(x, o0, lane)], g1 = fS[fidx(x, o1, lane)];
        } else if (lay == 1) {  // outputs (a, c): f(a, x, c)
          g0 = fS[fidx(o0, x, lane)], g1 = fS[fidx(o1, x, lane)];
        } else {  // outputs (a, b): f(a, b, x)
          g0 = fS[fidx(o0, lane, x)], g1 = fS[fidx(o1, lane, x)];
        }
        F0 += g0, F1 += g1;
        if (x & 1) g0 = -g0, g1 = -g1;
#pragma unroll
        for (int s = 0; s < PB; ++s) {
          const float2* Pa = P + (s * 3 + 0) * PL;
          const float2* Pb = P + (s * 3 + 1) * PL;
          const float2* Pc = P + (s * 3 + 2) * PL;
          // "shared" plane value (both outputs) and the two "uniform" ones
          float2 ps, pu0, pu1;
          if (lay == 0) {  // sum over a: P_b(a, c) shared, P_c(a, b) uniform
            ps = Pb[sw(x, lane)], pu0 = Pc[sw(x, o0)], pu1 = Pc[sw(x, o1)];
          } else if (lay == 1) {  // sum over b: P_a(b, c) shared, P_c(a, b) uniform
            ps = Pa[sw(x, lane)], pu0 = Pc[sw(o0, x)], pu1 = Pc[sw(o1, x)];
          } else {  // sum over c: P_a(b, c) shared (b = lane), P_b(a, c) uniform
            ps = Pa[sw(lane, x)], pu0 = Pb[sw(o0, x)], pu1 = Pb[sw(o1, x)];
          }
          sh[0][s].x = fmaf(ps.x, g0, sh[0][s].x), sh[0][s].y = fmaf(ps.y, g0, sh[0][s].y);
          sh[1][s].x = fmaf(ps.x, g1, sh[1][s].x), sh[1][s].y = fmaf(ps.y, g1, sh[1][s].y);
          un[0][s].x = fmaf(pu0.x, g0, un[0][s].x), un[0][s].y = fmaf(pu0.y, g0, un[0][s].y);
          un[1][s].x = fmaf(pu1.x, g1, un[1][s].x), un[1][s].y = fmaf(pu1.y, g1, un[1][s].y);
        }
      }
      // own-plane term and the signs of the output indices
      const float so0 = (o0 & 1) ? -1.f : 1.f, so1 = (o1 & 1) ? -1.f : 1.f;
      const float sl = (lane & 1) ? -1.f : 1.f;
#pragma unroll
      for (int s = 0; s < PB; ++s) {
        const float2 p0 = P[(s * 3 + lay) * PL + sw(o0, lane)], p1 = P[(s * 3 + lay) * PL + sw(o1, lane)];
        // R_a = P_a F_a + (-1)^b sh + (-1)^c un;  R_b = (-1)^a sh + P_b F_b + (-1)^c un;
        // R_c = (-1)^a sh + (-1)^b un + P_c F_c  (sh / un as assigned above)
        const float a0 = sl, b0 = so0, b1 = so1;
        Rr[lay][0][s] = make_float2(p0.x * F0 + b0 * sh[0][s].x + a0 * un[0][s].x,
                                    p0.y * F0 + b0 * sh[0][s].y + a0 * un[0][s].y);
        Rr[lay][1][s] = make_float2(p1.x * F1 + b1 * sh[1][s].x + a0 * un[1][s].x,
                                    p1.y * F1 + b1 * sh[1][s].y + a0 * un[1][s].y);
      }
    }
    __syncthreads();  // every layout has read P
#pragma unroll
    for (int lay = 0; lay < 3; ++lay)
#pragma unroll
      for (int s = 0; s < PB; ++s) {
        P[(s * 3 + lay) * PL + sw(warp, lane)] = Rr[lay][0][s];
        P[(s * 3 + lay) * PL + sw(warp + 16, lane)] = Rr[lay][1][s];
      }
    __syncthreads();
    // ---- 4. U = unnormalised 2D forward transforms of R
    planes_fft2<-1>(P, 3 * nb, warp, lane);
    // ---- 5. C(k) = (w.x - w.y) U(k) - (w.x + w.y) conj U(-k), w = g-_p(k), accumulated
#pragma unroll
    for (int it = 0; it < PTS; ++it) {
      const int i = t + it * THREADS;
      int plane, r, c, ka, kb, kc;
      if (!nyq_point(i, plane, r, c, ka, kb, kc)) continue;
      const int nr = (32 - r) & 31, nc = (32 - c) & 31;
      const int kk = kval(ka, 32) * kval(ka, 32) + kval(kb, 32) * kval(kb, 32) + kval(kc, 32) * kval(kc, 32);
#pragma unroll
      for (int s = 0; s < PB; ++s) {
        if (s >= nb) break;
        const float gsv = Gs[s * GSN + kk - 256];  // kk >= 256: one component is the Nyquist index
        const float2 gm = minus_from(Rows + s * 192 + 96, Fac + s * 384 + 192, plane, r, c);
        const float wx = gsv * gm.x, wy = gsv * gm.y;
        const float2 u = P[(s * 3 + plane) * PL + sw(r, c)];
        const float2 um = P[(s * 3 + plane) * PL + sw(nr, nc)];
        const float cp = wx - wy, cm = wx + wy;
        acc[it].x += cp * u.x - cm * um.x;
        acc[it].y += cp * u.y + cm * um.y;
      }
    }
    cp_async_wait_all();  // the next batch's rows have landed before the barrier
    __syncthreads();
  }
  float2* out = a.part + (cell * a.blocks + blk) * 3 * N2;
#pragma unroll
  for (int it = 0; it < PTS; ++it) out[t + it * THREADS] = acc[it];
}

// G[cell][k] += sum over the cell's CTAs of the correction at the Nyquist points
__global__ void __launch_bounds__(256) k_nyq_add(float2* G, const float2* part, int64_t cells, int blocks) {
  using namespace nq;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * 3 * N2) return;
  const int64_t cell = gid / (3 * N2);
  const int i = int(gid - cell * 3 * N2);
  int plane, r, c, ka, kb, kc;
  if (!nyq_point(i, plane, r, c, ka, kb, kc)) return;
  float2 s = make_float2(0.f, 0.f);
  for (int b = 0; b < blocks; ++b) {
    const float2 v = part[(cell * blocks + b) * 3 * N2 + i];
    s.x += v.x;
    s.y += v.y;
  }
  float2* g = G + cell * N3 + ka * N2 + kb * 32 + kc;
  g->x += s.x;
  g->y += s.y;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int nyq_corr_prepare(pii_plan* p) {
  using namespace nq;
  PII_CUDA(cudaFuncSetAttribute(k_nyq_corr, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM)));
  return PII_OK;
}

int nyq_corr_run(pii_plan* p, int64_t cells, cudaStream_t s) {
  using namespace nq;
  NyqArgs a{};
  a.fhat = static_cast<const float2*>(p->fhat);
  a.fT = static_cast<const float*>(p->fT);
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
  // 8 to 16 waves of CTAs (one per SM), each with at least 16 antipodal pairs so
  // that loading the cell's f into shared memory stays a small share; among
  // those, the CTA count per cell whose last wave is fullest (128 cells on 152
  // SMs: 19 per cell, 16 whole waves, instead of 10 and a 42 % last wave)
  const int64_t bmax = std::max(1, a.QP / 16);
  const int64_t blo = std::min<int64_t>(bmax, std::max<int64_t>(1, (8 * int64_t(sms) + cells - 1) / cells));
  const int64_t bhi = std::min<int64_t>(bmax, std::max<int64_t>(blo, (16 * int64_t(sms) + cells - 1) / cells));
  int64_t best = blo;
  double best_idle = 2.0;
  for (int64_t b = blo; b <= bhi; ++b) {
    const int64_t ctas = cells * b, tail = ctas % sms;
    const double idle = tail == 0 ? 0.0 : double(sms - tail) / double(ctas + sms - tail);
    if (idle < best_idle - 1e-9) {
      best_idle = idle;
      best = b;
    }
  }
  a.blocks = int(best);
  a.part = static_cast<float2*>(p->nq_part);
  {
    StageTimer st(p, ST_NYQ, s);
    k_nyq_corr<<<unsigned(cells * a.blocks), THREADS, SMEM, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_NYQ, s);
    k_nyq_add<<<unsigned((cells * 3 * N2 + 255) / 256), 256, 0, s>>>(static_cast<float2*>(p->G), a.part, cells,
                                                                      a.blocks);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
