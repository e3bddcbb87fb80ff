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
// reductions with f held in registers (three thread layouts: (b,c), (a,c),
// (a,b) columns), six 2D forward transforms, then C(k) into a per-CTA
// accumulator.  k_nyq_add sums the CTAs' accumulators into G.
#include <algorithm>

#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {

namespace nq {
constexpr int NV = 32, N2 = 1024, N3 = 32768;
constexpr int THREADS = 512;
constexpr int PB = 2;  // antipodal pairs per batch
// shared memory: Fh[3][N2] + P[PB][3][N2] + R[PB][3][N2] + Acc[3][N2], all float2
constexpr size_t SMEM = size_t(3 + 6 * PB + 3) * N2 * sizeof(float2);
__device__ __forceinline__ int sw(int r, int c) { return r * 32 + (c ^ r); }  // swizzled plane element
}  // namespace nq

struct NyqArgs {
  const float2* fhat;    // [cells][N3]
  const float* fT;       // [cells][N3]
  const float2* ephase;  // [Q][3][32]
  const float2* gphase;  // [Q][3][32]
  const float* gsinc;    // [n_r][M + 1]
  const int* reps;       // [QP] representative pair of each antipodal pass
  int M, ns, QP;
  int64_t cells;
  int blocks;            // CTAs per cell
  float2* part;          // [cells][blocks][3][N2]
};

__device__ __forceinline__ float2 nq_conj(float2 v) { return make_float2(v.x, -v.y); }

// one warp transforms one swizzled 32 x 32 plane in place: rows then columns
template <int DIR>
__device__ __forceinline__ void plane_fft2(float2* P, int lane) {
  using namespace nq;
  float2 x[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) x[c] = P[sw(lane, c)];
  fft_line<32, DIR>(x);
  static_for<0, 32>([&](auto ci) {
    constexpr int c = decltype(ci)::value;
    P[sw(lane, c)] = x[pos(32, c)];
  });
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 32; ++r) x[r] = P[sw(r, lane)];
  fft_line<32, DIR>(x);
  static_for<0, 32>([&](auto ri) {
    constexpr int r = decltype(ri)::value;
    P[sw(r, lane)] = x[pos(32, r)];
  });
}

// (E(k) - E~(k)) / 2 and (g(k) - g~(k)) / 2 for k = (ka, kb, kc): ~ conjugates
// the factor of every Nyquist component
__device__ __forceinline__ float2 minus_part(const float2* rows, int ka, int kb, int kc) {
  const float2 xa = rows[ka], xb = rows[32 + kb], xc = rows[64 + kc];
  const float2 p = cmul(cmul(xa, xb), xc);
  const float2 q = cmul(cmul(ka == 16 ? nq_conj(xa) : xa, kb == 16 ? nq_conj(xb) : xb), kc == 16 ? nq_conj(xc) : xc);
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
  float2* Fh = reinterpret_cast<float2*>(smem_raw);  // [3][N2] f^ on the planes, swizzled
  float2* P = Fh + 3 * N2;                           // [PB][3][N2]
  float2* R = P + PB * 3 * N2;                       // [PB][3][N2]
  float2* Acc = R + PB * 3 * N2;                     // [3][N2]
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int64_t cell = blockIdx.x / a.blocks;
  const int blk = int(blockIdx.x - cell * a.blocks);
  const int per = (a.QP + a.blocks - 1) / a.blocks;
  const int i0 = blk * per, i1 = min(a.QP, i0 + per);
  const float2* fh = a.fhat + cell * N3;
  const float* fr = a.fT + cell * N3;

  for (int i = t; i < 3 * N2; i += THREADS) {
    const int plane = i >> 10, r = (i >> 5) & 31, c = i & 31;
    const int e = plane == 0 ? (16 * N2 + r * 32 + c) : plane == 1 ? (r * N2 + 16 * 32 + c) : (r * N2 + c * 32 + 16);
    Fh[plane * N2 + sw(r, c)] = fh[e];
    Acc[plane * N2 + sw(r, c)] = make_float2(0.f, 0.f);
  }
  __syncthreads();

  for (int ib = i0; ib < i1; ib += PB) {
    const int nb = min(PB, i1 - ib);
    // ---- 1. f^ t- on the three point sets (0 elsewhere on the planes)
    for (int i = t; i < PB * 3 * N2; i += THREADS) {
      const int s = i / (3 * N2);
      const int ii = i - s * 3 * N2;
      int plane, r, c, ka, kb, kc;
      const bool on = nyq_point(ii, plane, r, c, ka, kb, kc) && s < nb;
      float2 y = make_float2(0.f, 0.f);
      if (on) {
        const int p = a.reps[ib + s];
        const float2 em = minus_part(a.ephase + int64_t(p) * 96, ka, kb, kc);
        const float tm = em.x + em.y;
        const float2 fv = Fh[plane * N2 + sw(r, c)];
        y = make_float2(fv.x * tm, fv.y * tm);
      }
      P[(s * 3 + plane) * N2 + sw(r, c)] = y;
    }
    __syncthreads();
    // ---- 2. P = unnormalised 2D inverse transforms (one warp per plane)
    if (warp < PB * 3) plane_fft2<+1>(P + warp * N2, lane);
    __syncthreads();
    // ---- 3. reductions R_a, R_b, R_c; thread layouts: rows w and w + 16, lane = column
#pragma unroll 1
    for (int lay = 0; lay < 3; ++lay) {
      // f along the summed axis for the thread's two outputs
      float f0[32], f1[32];
      if (lay == 0) {  // outputs (b, c) = (w, lane), (w + 16, lane): f(., b, c)
#pragma unroll
        for (int x = 0; x < 32; ++x) {
          f0[x] = fr[x * N2 + warp * 32 + lane];
          f1[x] = fr[x * N2 + (warp + 16) * 32 + lane];
        }
      } else if (lay == 1) {  // outputs (a, c): f(a, ., c)
#pragma unroll
        for (int x = 0; x < 32; ++x) {
          f0[x] = fr[warp * N2 + x * 32 + lane];
          f1[x] = fr[(warp + 16) * N2 + x * 32 + lane];
        }
      } else {  // outputs (a, b) = (w, lane), (w + 16, lane): f(a, b, .)
        const float4* q0 = reinterpret_cast<const float4*>(fr + warp * N2 + lane * 32);
        const float4* q1 = reinterpret_cast<const float4*>(fr + (warp + 16) * N2 + lane * 32);
#pragma unroll
        for (int x = 0; x < 8; ++x) {
          const float4 v0 = q0[x], v1 = q1[x];
          f0[4 * x] = v0.x, f0[4 * x + 1] = v0.y, f0[4 * x + 2] = v0.z, f0[4 * x + 3] = v0.w;
          f1[4 * x] = v1.x, f1[4 * x + 1] = v1.y, f1[4 * x + 2] = v1.z, f1[4 * x + 3] = v1.w;
        }
      }
      float F0 = 0.f, F1 = 0.f;
#pragma unroll
      for (int x = 0; x < 32; ++x) {
        F0 += f0[x];
        F1 += f1[x];
      }
      for (int s = 0; s < nb; ++s) {
        const float2* Pa = P + (s * 3 + 0) * N2;
        const float2* Pb = P + (s * 3 + 1) * N2;
        const float2* Pc = P + (s * 3 + 2) * N2;
        // "shared" plane value (same for both outputs) and the two "uniform" ones
        float2 sh0 = make_float2(0.f, 0.f), sh1 = sh0, un0 = sh0, un1 = sh0;
#pragma unroll
        for (int x = 0; x < 32; ++x) {
          float2 ps, pu0, pu1;
          if (lay == 0) {  // sum over a: P_b(a, c) shared, P_c(a, b) uniform
            ps = Pb[sw(x, lane)];
            pu0 = Pc[sw(x, warp)];
            pu1 = Pc[sw(x, warp + 16)];
          } else if (lay == 1) {  // sum over b: P_a(b, c) shared, P_c(a, b) uniform
            ps = Pa[sw(x, lane)];
            pu0 = Pc[sw(warp, x)];
            pu1 = Pc[sw(warp + 16, x)];
          } else {  // sum over c: P_a(b, c) shared (b = lane), P_b(a, c) uniform
            ps = Pa[sw(lane, x)];
            pu0 = Pb[sw(warp, x)];
            pu1 = Pb[sw(warp + 16, x)];
          }
          const float g0 = (x & 1) ? -f0[x] : f0[x], g1 = (x & 1) ? -f1[x] : f1[x];
          sh0.x = fmaf(ps.x, g0, sh0.x), sh0.y = fmaf(ps.y, g0, sh0.y);
          sh1.x = fmaf(ps.x, g1, sh1.x), sh1.y = fmaf(ps.y, g1, sh1.y);
          un0.x = fmaf(pu0.x, g0, un0.x), un0.y = fmaf(pu0.y, g0, un0.y);
          un1.x = fmaf(pu1.x, g1, un1.x), un1.y = fmaf(pu1.y, g1, un1.y);
        }
        // combine with the own-plane term and the signs of the output indices
        float2 r0, r1;
        const int o0 = warp, o1 = warp + 16;  // first output index of each row
        const float so0 = (o0 & 1) ? -1.f : 1.f, so1 = (o1 & 1) ? -1.f : 1.f;
        const float sl = (lane & 1) ? -1.f : 1.f;
        if (lay == 0) {  // R_a(b,c) = P_a F_a + (-1)^b sh + (-1)^c un
          const float2 p0 = Pa[sw(o0, lane)], p1 = Pa[sw(o1, lane)];
          r0 = make_float2(p0.x * F0 + so0 * sh0.x + sl * un0.x, p0.y * F0 + so0 * sh0.y + sl * un0.y);
          r1 = make_float2(p1.x * F1 + so1 * sh1.x + sl * un1.x, p1.y * F1 + so1 * sh1.y + sl * un1.y);
        } else if (lay == 1) {  // R_b(a,c) = (-1)^a sh + P_b F_b + (-1)^c un
          const float2 p0 = Pb[sw(o0, lane)], p1 = Pb[sw(o1, lane)];
          r0 = make_float2(so0 * sh0.x + p0.x * F0 + sl * un0.x, so0 * sh0.y + p0.y * F0 + sl * un0.y);
          r1 = make_float2(so1 * sh1.x + p1.x * F1 + sl * un1.x, so1 * sh1.y + p1.y * F1 + sl * un1.y);
        } else {  // R_c(a,b) = (-1)^a sh + (-1)^b un + P_c F_c
          const float2 p0 = Pc[sw(o0, lane)], p1 = Pc[sw(o1, lane)];
          r0 = make_float2(so0 * sh0.x + sl * un0.x + p0.x * F0, so0 * sh0.y + sl * un0.y + p0.y * F0);
          r1 = make_float2(so1 * sh1.x + sl * un1.x + p1.x * F1, so1 * sh1.y + sl * un1.y + p1.y * F1);
        }
        R[(s * 3 + lay) * N2 + sw(o0, lane)] = r0;
        R[(s * 3 + lay) * N2 + sw(o1, lane)] = r1;
      }
    }
    __syncthreads();
    // ---- 4. U = unnormalised 2D forward transforms of R
    if (warp < PB * 3) plane_fft2<-1>(R + warp * N2, lane);
    __syncthreads();
    // ---- 5. C(k) = (w.x - w.y) U(k) - (w.x + w.y) conj U(-k), w = g-_p(k), into Acc
    for (int i = t; i < 3 * N2; i += THREADS) {
      int plane, r, c, ka, kb, kc;
      if (!nyq_point(i, plane, r, c, ka, kb, kc)) continue;
      const int nr = (32 - r) & 31, nc = (32 - c) & 31;
      const int kk = kval(ka, 32) * kval(ka, 32) + kval(kb, 32) * kval(kb, 32) + kval(kc, 32) * kval(kc, 32);
      float2 acc = Acc[plane * N2 + sw(r, c)];
      for (int s = 0; s < nb; ++s) {
        const int p = a.reps[ib + s];
        const float gsv = a.gsinc[int64_t(p / a.ns) * (a.M + 1) + kk];
        const float2 gm = minus_part(a.gphase + int64_t(p) * 96, ka, kb, kc);
        const float wx = gsv * gm.x, wy = gsv * gm.y;
        const float2 u = R[(s * 3 + plane) * N2 + sw(r, c)];
        const float2 um = R[(s * 3 + plane) * N2 + sw(nr, nc)];
        const float cp = wx - wy, cm = wx + wy;
        acc.x += cp * u.x - cm * um.x;
        acc.y += cp * u.y + cm * um.y;
      }
      Acc[plane * N2 + sw(r, c)] = acc;
    }
    __syncthreads();
  }
  float2* out = a.part + (cell * a.blocks + blk) * 3 * N2;
  for (int i = t; i < 3 * N2; i += THREADS) {
    const int plane = i >> 10, r = (i >> 5) & 31, c = i & 31;
    out[i] = Acc[plane * N2 + sw(r, c)];
  }
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
  a.M = p->tab.M;
  a.ns = p->ns;
  a.QP = p->ap_count;
  a.cells = cells;
  int sms = 0;
  PII_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  a.blocks = int(std::max<int64_t>(1, std::min<int64_t>(16, (2 * int64_t(sms) + cells - 1) / cells)));
  a.blocks = std::min(a.blocks, std::max(1, a.QP / PB));
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
