// Fused gain term of Q(f,f) for n = 32 in FP32, split by the parity of the
// first velocity axis: two independent CTAs per (cell, range of quadrature
// pairs), no cluster and no exchange between them.
//
// CTA p (p = 0, 1) owns the a-planes a = 2 m + p (m < 16) of the 32^3 work
// grid in 132 KB of shared memory (rows padded as in the cluster kernel).  Per
// pair (src/collision/inelastic_collisions.py:212-217):
//   A  inverse transform along a, decimated in frequency: the parity-p outputs
//      of a 32-point inverse DFT are the 16-point inverse DFT of
//      W^{-p k} (Y[k] + (-1)^p Y[k + 16]), k < 16, with Y = exp_rs(k) f^(k)
//      (the twiddles are folded into the per-pair rows `epar`);
//   B  plane pass, one warp per plane: IFFT_c, IFFT_b, * f, FFT_b, FFT_c;
//   C  forward transform along a, decimated in time: the planes of parity p
//      contribute W^{p k} Z_p[k mod 16] to every k_a, with Z_p the 16-point DFT
//      over the CTA's own planes.  Times gain_rs(k) (twiddle folded into
//      `gpar`), accumulated.
// Only Re IFFT3(G) is ever used, so each CTA accumulates the Hermitian part
// H(k) = (G_p(k) + conj G_p(-k)) / 2 of its own contribution G_p on half of
// k-space: thread t owns a column pair {j, -j} (or two self-conjugate columns)
// and all 32 k_a of it.  That accumulator (514 slots x 32 x 8 bytes) lives in
// tensor memory: thread t of warp w uses TMEM lane 32 (w mod 4) + (t mod 32),
// columns [128 (w / 4), 128 (w / 4) + 128); region 0 (first 64 columns) sums
// gain * X over the first column of the pair, region 1 the conjugated
// contributions of the second, and the two are combined once per work item.
// Against the cluster kernel this halves the stage-A transform, removes the
// distributed-shared-memory reads of stage C and the cluster barriers, and
// doubles the gain products of stage C (each CTA forms all 32 k_a).
#include <algorithm>

#include "gain_common.cuh"
#include "tmem.cuh"

namespace pii {
// packed FP32x2 butterflies in the 16-point a-axis transforms of stages A and
// C (16.82 instead of 17.27 ms per 128-cell launch), not in the plane pass's
// 32-point ones (18.09 ms)
constexpr bool PAR_PK_AC = true, PAR_PK_B = false;

namespace gpar {
using namespace gc;
constexpr int TMEM_COLS = 512;
// f of the CTA's 16 planes, transposed per plane to [c][b] with a 36-float row
// pitch: each lane of the plane pass reads its 32 values in 16-byte loads
// without bank conflicts
constexpr int FPITCH = 36;
constexpr size_t FS_OFF = size_t(PLANES) * PSTR * sizeof(float2);
// packed mode: the current radial node's sinc slab gsxc[r] ([153][17] floats, 16-byte padded)
constexpr int GSC = 153 * 17;
constexpr size_t GSC_OFF = FS_OFF + size_t(PLANES) * 32 * FPITCH * sizeof(float);
// packed mode: per-axis phase and gain rows of the pairs, [2 buffers][phase, gain][96]
// (float2), copied one stage ahead of their use with cp.async
constexpr size_t ROW_OFF = GSC_OFF + size_t((GSC + 3) / 4 * 4) * sizeof(float);
constexpr size_t SMEM = ROW_OFF + size_t(2 * 2 * 96) * sizeof(float2) + 16;
static_assert(ROW_OFF % 16 == 0, "cp.async destinations are 16-byte aligned");
}  // namespace gpar

struct GainParityArgs {
  const float2* fhat;    // [cells][N3] spectra of f
  const float* fT;       // [cells][N3] f in FP32
  const float2* ephase;  // [Q][3][32]
  const float2* gphase;  // [Q][3][32]
  const float2* epar;    // [Q][2][32]
  const float2* gpar;    // [Q][2][32]
  const float* gsx;      // [n_r][513][20]
  const float* gsxc;     // [n_r][153][17] (packed mode)
  // elements per restitution set (0: one set for every cell) of gphase
  // (complex), gpar (complex), gsx and gsxc
  int64_t gph_stride, gpar_stride, gsx_stride, gsxc_stride;
  int ns, Q;
  int QP;                // passes per (cell, parity): Q, or the antipodal pairs when packed
  const int* reps;       // [QP] pair index of each packed pass (packed mode)
  int64_t cells;
  float2* hpart;      // [CTAs + 2 cells][32][HSLOTS]
  const int4* ucols;  // [THREADS] (column, column, first slot, 1 if two self-conjugate columns)
};

// stage A, parity-PAR outputs of the inverse transform along a, for the
// thread's column pair (j, -j).  f is real, so f^(k, -j) = conj f^(-k, j): the
// 32 values of column j give both columns (half the bytes of reading both):
//   u_j[k]  = e_bc(j)  (F[k] eA[k] + F[k + 16] eB[k])
//   u_-j[k] = e_bc(-j) (conj F[-k] eA[k] + conj F[-k - 16] eB[k])   (indices mod 32)
// so the loaded pair (F[k], F[k + 16]) also serves u_-j[(16 - k) mod 16].
template <int PAR>
__device__ __forceinline__ void par_stage_a_pair(float2* W, const float2* fh, const float2* ep, const float2* epp,
                                                 int j) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  const int nb = (32 - jb) & 31, nc = (32 - jc) & 31;
  const float2 ebc0 = cmul(ep[32 + jb], ep[64 + jc]), ebc1 = cmul(ep[32 + nb], ep[64 + nc]);
  float2 u0[16], u1[16];
  static_for<0, 16>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    constexpr int k1 = (16 - k) & 15;
    const float2 lo = fh[k * N2 + j], hi = fh[(k + 16) * N2 + j];
    u0[k] = cmul(cfma(hi, epp[16 + k], cmul(lo, epp[k])), ebc0);
    const float2 clo = make_float2(lo.x, -lo.y), chi = make_float2(hi.x, -hi.y);
    if constexpr (k == 0)
      u1[0] = cmul(cfma(chi, epp[16], cmul(clo, epp[0])), ebc1);
    else
      u1[k1] = cmul(cfma(clo, epp[16 + k1], cmul(chi, epp[k1])), ebc1);
  });
  fft_line<16, +1, PAR_PK_AC>(u0);
  fft_line<16, +1, PAR_PK_AC>(u1);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    W[widx(m, jb, jc)] = u0[pos(16, m)];
    W[widx(m, nb, nc)] = u1[pos(16, m)];
  });
}

// stage A for one column j from its own 32 values (the warp holding the
// self-conjugate columns)
template <int PAR>
__device__ __forceinline__ void par_stage_a_col(float2* W, const float2* fh, const float2* ep, const float2* epp,
                                                int j) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  const float2 ebc = cmul(ep[32 + jb], ep[64 + jc]);
  float2 u[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) u[k] = cmul(cfma(fh[(k + 16) * N2 + j], epp[16 + k], cmul(fh[k * N2 + j], epp[k])), ebc);
  fft_line<16, +1, PAR_PK_AC>(u);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    W[widx(m, jb, jc)] = u[pos(16, m)];
  });
}

// stage C for one column of the thread's pair: PASS 0 adds gain * X(k) to
// region 0, PASS 1 adds conj(gain * X(-k)) to region 1, for all 32 k_a.
// gsr = the pair's radial row of gsx: the column's 17 sinc values |k_a| = 0..16
// come in five 16-byte loads instead of 32 scattered ones.
template <int PASS>
__device__ __forceinline__ void par_stage_c(const float2* W, int j, const float2* gp, const float2* gpp,
                                            const float* gsr, uint32_t treg) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  uint32_t r[16];
  tm_ld16(treg, r);  // chunk 0 of the accumulator, in flight during the transform
  float2 z[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) z[m] = W[widx(m, jb, jc)];
  fft_line<16, -1, PAR_PK_AC>(z);
  const int kb = kval(jb, 32), kc = kval(jc, 32);
  const float4* grow = reinterpret_cast<const float4*>(gsr + (kb * kb + kc * kc) * 20);
  float g[20];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const float4 v = grow[i];
    g[4 * i] = v.x;
    g[4 * i + 1] = v.y;
    g[4 * i + 2] = v.z;
    g[4 * i + 3] = v.w;
  }
  const float2 gbc = cmul(gp[32 + jb], gp[64 + jc]);
#pragma unroll
  for (int m = 0; m < 16; ++m) z[m] = cmul(z[m], gbc);
  const float4* gpp4 = reinterpret_cast<const float4*>(gpp);
  static_for<0, 4>([&](auto ci) {
    constexpr int c = decltype(ci)::value;
    if constexpr (c > 0) tm_ld16(treg + 16 * c, r);
    tm_wait_ld(r);
    static_for<0, 8>([&](auto ii) {
      constexpr int i = decltype(ii)::value;
      constexpr int k = 8 * c + i;
      constexpr int src = PASS == 0 ? k : ((32 - k) & 31);
      constexpr int q = kval(src, 32) < 0 ? -kval(src, 32) : kval(src, 32);
      const float4 w4 = gpp4[src >> 1];
      const float2 w = (src & 1) ? make_float2(w4.z, w4.w) : make_float2(w4.x, w4.y);
      const float2 zz = z[pos(16, src & 15)];
      const float re = zz.x * w.x - zz.y * w.y;
      const float im = zz.x * w.y + zz.y * w.x;
      r[2 * i] = __float_as_uint(fmaf(g[q], re, __uint_as_float(r[2 * i])));
      r[2 * i + 1] = __float_as_uint(fmaf(PASS == 0 ? g[q] : -g[q], im, __uint_as_float(r[2 * i + 1])));
    });
    tm_st16(treg + 16 * c, r);
  });
}

// ---------------------------------------------------------------------------
// Packed (antipodal) mode.  The designs are symmetric: pair q = (r, -sigma_p)
// has E_q = conj E_p and gain_q = conj gain_p.  With E+ = (E(k) + conj E(-k))/2
// (the Hermitian part of the phase; it differs from E only where a component of
// k is the Nyquist index 16), the real fields Re A_p = IFFT3(f^ E+_p) and
// Re A_q pack into one complex pipeline whose input is f^ t with the REAL
//   t(k) = Re E+_p(k) + Im E+_p(k)        (E+_p + i E+_q = (1 + i) t),
// and whose output F gives the pairs' Hermitian gain contributions with the
// REAL coefficient 2 s(k), s = Re g+_p - Im g+_p, g+ = (g(k) + conj g(-k))/2.
// The remaining parts of the two pairs (E- = E - E+, g- = g - g+), which live on
// the Nyquist planes only, are added by the Nyquist correction kernel.
// Per column the separable factors give, for k_a != 16,
//   t(k_a, j) = e_a.x (c.x + c.y) + e_a.y (c.x - c.y),  c = (e_bc(j) + e~_bc(j)) / 2,
//   s(k_a, j) = g_a.x (d.x - d.y) - g_a.y (d.x + d.y),  d = (g_bc(j) + g~_bc(j)) / 2,
// where ~ conjugates the factor of a Nyquist component; k_a = 16 takes the
// two-term form directly.
__device__ __forceinline__ float2 cconj(float2 v) { return make_float2(v.x, -v.y); }

struct PackCol {
  float cp, cm, t16;  // t(k_a, j) = e_a.x cp + e_a.y cm (k_a != 16); t(16, j) = t16
};
__device__ __forceinline__ PackCol pack_col_consts(const float2* ep, int jb, int jc) {
  using namespace gc;
  const float2 eb = ep[32 + jb], ec = ep[64 + jc];
  const float2 ebc = cmul(eb, ec);
  const float2 ebct = cmul(jb == 16 ? cconj(eb) : eb, jc == 16 ? cconj(ec) : ec);
  const float2 c = make_float2(0.5f * (ebc.x + ebct.x), 0.5f * (ebc.y + ebct.y));
  const float2 e16 = ep[16];
  const float2 u = cmul(e16, ebc), v = cmul(cconj(e16), ebct);
  PackCol r;
  r.cp = c.x + c.y;
  r.cm = c.x - c.y;
  r.t16 = 0.5f * (u.x + v.x + u.y + v.y);
  return r;
}
__device__ __forceinline__ float pack_t(float2 ea, const PackCol& c) { return fmaf(ea.y, c.cm, ea.x * c.cp); }

// stage A (packed) for the column pair (j, -j), as par_stage_a_pair with the real phase t
template <int PAR>
__device__ __forceinline__ void pack_stage_a_pair(float2* W, const float2* fh, const float2* ep, int j) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  const int nb = (32 - jb) & 31, nc = (32 - jc) & 31;
  const PackCol c0 = pack_col_consts(ep, jb, jc), c1 = pack_col_consts(ep, nb, nc);
  const float4* e4 = reinterpret_cast<const float4*>(ep);
  auto ea = [&](int k) {
    const float4 v = e4[k >> 1];
    return (k & 1) ? make_float2(v.z, v.w) : make_float2(v.x, v.y);
  };
  constexpr float sg = PAR ? -1.f : 1.f;
  float2 u0[16], u1[16];
  static_for<0, 16>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    constexpr int k1 = (16 - k) & 15;
    const float2 lo = fh[k * N2 + j], hi = fh[(k + 16) * N2 + j];
    const float tl = pack_t(ea(k), c0);
    const float th = k == 0 ? c0.t16 : pack_t(ea(k + 16), c0);
    const float2 y0 = make_float2(lo.x * tl + sg * hi.x * th, lo.y * tl + sg * hi.y * th);
    u0[k] = twiddle<PAR * k, 32, +1>(y0);
    const float ta = pack_t(ea(k1), c1);
    const float tb = k1 == 0 ? c1.t16 : pack_t(ea(k1 + 16), c1);
    // column -j: Y[k1] = conj F[-k1] t, Y[k1 + 16] = conj F[-k1 - 16] t (indices mod 32)
    const float2 A = k == 0 ? cconj(lo) : cconj(hi), B = k == 0 ? cconj(hi) : cconj(lo);
    const float2 y1 = make_float2(A.x * ta + sg * B.x * tb, A.y * ta + sg * B.y * tb);
    u1[k1] = twiddle<PAR * k1, 32, +1>(y1);
  });
  fft_line<16, +1, PAR_PK_AC>(u0);
  fft_line<16, +1, PAR_PK_AC>(u1);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    W[widx(m, jb, jc)] = u0[pos(16, m)];
    W[widx(m, nb, nc)] = u1[pos(16, m)];
  });
}

// stage A (packed) for one column j from its own values
template <int PAR>
__device__ __forceinline__ void pack_stage_a_col(float2* W, const float2* fh, const float2* ep, int j) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  const PackCol c0 = pack_col_consts(ep, jb, jc);
  constexpr float sg = PAR ? -1.f : 1.f;
  float2 u[16];
  static_for<0, 16>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    const float2 lo = fh[k * N2 + j], hi = fh[(k + 16) * N2 + j];
    const float tl = pack_t(ep[k], c0);
    const float th = k == 0 ? c0.t16 : pack_t(ep[k + 16], c0);
    u[k] = twiddle<PAR * k, 32, +1>(make_float2(lo.x * tl + sg * hi.x * th, lo.y * tl + sg * hi.y * th));
  });
  fft_line<16, +1, PAR_PK_AC>(u);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    W[widx(m, jb, jc)] = u[pos(16, m)];
  });
}

// the column's 17 sinc values |k_a| = 0..16 from the radial node's slab in shared memory
__device__ __forceinline__ void load_gsc(const float* slab, int j, float (&g)[20]) {
  int u = kval(j >> 5, 32), v = kval(j & 31, 32);
  u = u < 0 ? -u : u;
  v = v < 0 ? -v : v;
  const float* row = slab + ((u < v ? v * (v + 1) / 2 + u : u * (u + 1) / 2 + v) * 17);
#pragma unroll
  for (int q = 0; q < 17; ++q) g[q] = row[q];
}

// the column's 17 sinc values |k_a| = 0..16 (of 20 padded) from its radial row of gsx
__device__ __forceinline__ void load_gsx(const float* gsr, int j, float (&g)[20]) {
  const int kb = kval(j >> 5, 32), kc = kval(j & 31, 32);
  const float4* grow = reinterpret_cast<const float4*>(gsr + (kb * kb + kc * kc) * 20);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const float4 v = grow[i];
    g[4 * i] = v.x;
    g[4 * i + 1] = v.y;
    g[4 * i + 2] = v.z;
    g[4 * i + 3] = v.w;
  }
}

// stage C (packed): X(k) = s(k) F(k) with F(k) = W^{PAR k} Z[k mod 16]; g = the
// column's sinc values (load_gsx; the columns j and -j of a pair share them)
template <int PAR, int PASS>
__device__ __forceinline__ void pack_stage_c(const float2* W, int j, const float2* gp, const float (&g)[20],
                                             uint32_t treg) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  uint32_t r[16];
  tm_ld16(treg, r);  // chunk 0 of the accumulator, in flight during the transform
  float2 z[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) z[m] = W[widx(m, jb, jc)];
  fft_line<16, -1, PAR_PK_AC>(z);
  float2 zw[16];
  static_for<0, 16>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    zw[k] = twiddle<PAR * k, 32, -1>(z[pos(16, k)]);
  });
  // d = (g_bc + g~_bc) / 2; s(k_a) = g_a.x dp - g_a.y dm (k_a != 16), s16 at k_a = 16
  const float2 gb = gp[32 + jb], gc2 = gp[64 + jc];
  const float2 gbc = cmul(gb, gc2);
  const float2 gbct = cmul(jb == 16 ? cconj(gb) : gb, jc == 16 ? cconj(gc2) : gc2);
  const float2 d = make_float2(0.5f * (gbc.x + gbct.x), 0.5f * (gbc.y + gbct.y));
  const float dp = d.x - d.y, dm = d.x + d.y;
  float s16;
  {
    const float2 g16 = gp[16];
    const float2 u = cmul(g16, gbc), v = cmul(cconj(g16), gbct);
    s16 = 0.5f * ((u.x + v.x) - (u.y + v.y));
  }
  const float4* g4 = reinterpret_cast<const float4*>(gp);
  static_for<0, 4>([&](auto ci) {
    constexpr int c = decltype(ci)::value;
    if constexpr (c > 0) tm_ld16(treg + 16 * c, r);
    tm_wait_ld(r);
    static_for<0, 8>([&](auto ii) {
      constexpr int i = decltype(ii)::value;
      constexpr int k = 8 * c + i;
      constexpr int src = PASS == 0 ? k : ((32 - k) & 31);
      constexpr int q = kval(src, 32) < 0 ? -kval(src, 32) : kval(src, 32);
      float sv;
      if constexpr (src == 16) {
        sv = s16;
      } else {
        const float4 w4 = g4[src >> 1];
        const float2 ga = (src & 1) ? make_float2(w4.z, w4.w) : make_float2(w4.x, w4.y);
        sv = fmaf(-ga.y, dm, ga.x * dp);
      }
      const float cf = g[q] * sv;
      const float2 F = src < 16 ? zw[src] : (PAR ? make_float2(-zw[src - 16].x, -zw[src - 16].y) : zw[src - 16]);
      r[2 * i] = __float_as_uint(fmaf(cf, F.x, __uint_as_float(r[2 * i])));
      r[2 * i + 1] = __float_as_uint(fmaf(PASS == 0 ? cf : -cf, F.y, __uint_as_float(r[2 * i + 1])));
    });
    tm_st16(treg + 16 * c, r);
  });
}

template <bool PACK>
__global__ void __launch_bounds__(gc::THREADS, 1) k_gain_parity(GainParityArgs a) {
  using namespace gpar;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* W = reinterpret_cast<float2*>(smem_raw);
  float* fS = reinterpret_cast<float*>(smem_raw + FS_OFF);
  float* gsc = reinterpret_cast<float*>(smem_raw + GSC_OFF);
  // packed mode: phase row of buffer b at rows + 192 b, gain row at rows + 192 b + 96
  float2* rows = reinterpret_cast<float2*>(smem_raw + ROW_OFF);
  int gsc_ir = -1;  // radial node whose slab is in gsc
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + SMEM - 16);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (warp == 0) {
    tm_alloc(tslot, TMEM_COLS);
    tm_relinquish();
  }
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const uint32_t tbase = *tslot;
  // this thread's lane (32 (warp mod 4) + lane) and columns [128 (warp / 4), + 128)
  const uint32_t treg0 = tbase + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(128 * (warp >> 2));

  // Work units = (cell, parity, pair) flattened with the pair fastest; CTA b takes
  // the contiguous range [T b / G, T (b + 1) / G) of the T = 2 cells Q units,
  // split into segments of constant (cell, parity); segment (b, cp) writes
  // Hermitian slot set b + cp.
  const int64_t total = a.cells * 2 * a.QP;
  const int64_t w0 = total * blockIdx.x / gridDim.x, w1 = total * (blockIdx.x + 1) / gridDim.x;

  for (int64_t w = w0; w < w1;) {
    const int64_t cp = w / a.QP;
    const int par = int(cp & 1);
    const int64_t cell = cp >> 1;
    const int p0 = int(w - cp * a.QP);
    const int p1 = int(min(int64_t(a.QP), w1 - cp * a.QP));
    w = cp * a.QP + p1;
    {
      uint32_t zr[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) zr[i] = 0u;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        tm_st16(treg0 + 16 * c, zr);
        tm_st16(treg0 + 64 + 16 * c, zr);
      }
    }
    const float2* fh = a.fhat + cell * N3;
    // the cell's restitution set (the same tables for every cell when there is one)
    const float2* gph_c = a.gphase + cell * a.gph_stride;
    const float2* gpar_c = a.gpar + cell * a.gpar_stride;
    const float* gsx_c = a.gsx + cell * a.gsx_stride;
    const float* gsxc_c = a.gsxc + cell * a.gsxc_stride;
    if (a.gsxc_stride) gsc_ir = -1;  // another cell's slab may be staged
    {
      // fS[m][c][b] = f[cell][2 m + par][b][c] (read before the first plane pass:
      // the stage-A barrier orders it)
      const float* fc = a.fT + cell * N3;
#pragma unroll 4
      for (int i = t; i < PLANES * N2; i += THREADS) {
        const int m = i >> 10, b = (i >> 5) & 31, c = i & 31;
        fS[(m * 32 + c) * FPITCH + b] = fc[(2 * m + par) * N2 + b * 32 + c];
      }
    }
    if constexpr (PACK) {
      // the first pass's phase row (later ones are copied one pass ahead)
      if (t < 48) cp_async16(rows + 192 * (p0 & 1) + 2 * t, a.ephase + int64_t(a.reps[p0]) * 96 + 2 * t);
      cp_async_wait_all();
      __syncthreads();
    }

    for (int ip = p0; ip < p1; ++ip) {
      const int p = PACK ? a.reps[ip] : ip;
      if constexpr (PACK) {
        // the radial node's sinc slab (every 16 passes; ir is the same in every thread):
        // the barrier ends the previous item's stage C reads of the old slab, the
        // stage-A barrier below orders these writes before this item's reads
        const int ir = p / a.ns;
        if (ir != gsc_ir) {
          __syncthreads();
          const float* src = gsxc_c + int64_t(ir) * GSC;
          for (int e = t; e < GSC; e += THREADS) gsc[e] = src[e];
          gsc_ir = ir;
        }
        // this pass's gain row (read in stage C) and the next pass's phase row
        // (its stage A), landing while stages A and B run.  Buffer parity = pass
        // parity: the buffers written here were last read in stage A of the
        // previous pass and stage C of the one before, both behind a barrier
        // already passed (a thread still in the previous stage C reads the other
        // gain buffer).
        if (t >= 48 && t < 96)
          cp_async16(rows + 192 * (ip & 1) + 96 + 2 * (t - 48), gph_c + int64_t(p) * 96 + 2 * (t - 48));
        if (t < 48 && ip + 1 < p1)
          cp_async16(rows + 192 * ((ip + 1) & 1) + 2 * t, a.ephase + int64_t(a.reps[ip + 1]) * 96 + 2 * t);
      }
      // (per-pair pointers are formed inside each stage so that none stays
      // live across the register-heavy plane pass)
      // ---- A: the thread's two columns (those it also takes in stage C)
      {
        const float2* ep = PACK ? rows + 192 * (ip & 1) : a.ephase + int64_t(p) * 96;
        const float2* epp = a.epar + (int64_t(p) * 2 + par) * 32;
        const int4 uc = a.ucols[t];
        if (warp < 15) {  // column pairs {j, -j}: rows 1..15 and 31..17
          if constexpr (PACK) {
            if (par == 0)
              pack_stage_a_pair<0>(W, fh, ep, uc.x);
            else
              pack_stage_a_pair<1>(W, fh, ep, uc.x);
          } else {
            if (par == 0)
              par_stage_a_pair<0>(W, fh, ep, epp, uc.x);
            else
              par_stage_a_pair<1>(W, fh, ep, epp, uc.x);
          }
        } else {  // rows 0 and 16 (with the self-conjugate columns): each column from its own values
#pragma unroll 1
          for (int h = 0; h < 2; ++h) {
            if constexpr (PACK) {
              if (par == 0)
                pack_stage_a_col<0>(W, fh, ep, h ? uc.y : uc.x);
              else
                pack_stage_a_col<1>(W, fh, ep, h ? uc.y : uc.x);
            } else {
              if (par == 0)
                par_stage_a_col<0>(W, fh, ep, epp, h ? uc.y : uc.x);
              else
                par_stage_a_col<1>(W, fh, ep, epp, h ? uc.y : uc.x);
            }
          }
        }
      }
      __syncthreads();
      // ---- B: warp `warp` owns local plane `warp` (a = 2 warp + par)
      plane_pass<true, PAR_PK_B>(W + warp * PSTR, fS + (warp * 32 + lane) * FPITCH, lane);
      if constexpr (PACK) cp_async_wait_all();  // the rows copied at the top of this pass
      __syncthreads();
      // ---- C: the thread's two columns (the previous pair's TMEM stores are complete first)
      {
        const float2* gp = PACK ? rows + 192 * (ip & 1) + 96 : gph_c + int64_t(p) * 96;
        const float2* gpp = gpar_c + (int64_t(p) * 2 + par) * 32;
        const float* gsr = gsx_c + int64_t(p / a.ns) * (513 * 20);
        const int4 uc = a.ucols[t];
        tm_wait_st();
        if constexpr (PACK) {
          // |k_b|^2 + |k_c|^2 is the same for j and -j: one sinc row serves both
          // columns of a pair; only the self-conjugate columns differ
          float g[20];
          load_gsc(gsc, uc.x, g);
          if (par == 0)
            pack_stage_c<0, 0>(W, uc.x, gp, g, treg0);
          else
            pack_stage_c<1, 0>(W, uc.x, gp, g, treg0);
          if (uc.w) load_gsc(gsc, uc.y, g);
          if (par == 0)
            pack_stage_c<0, 1>(W, uc.y, gp, g, treg0 + 64);
          else
            pack_stage_c<1, 1>(W, uc.y, gp, g, treg0 + 64);
        } else {
          par_stage_c<0>(W, uc.x, gp, gpp, gsr, treg0);
          par_stage_c<1>(W, uc.y, gp, gpp, gsr, treg0 + 64);
        }
      }
      // No barrier here: a thread's stage A of the next pair writes exactly the
      // plane entries (its columns j and -j, all 16 planes) that its own stage C
      // has just read, and its accumulator lanes are its own, so threads may run
      // ahead into the next pair's loads; the barrier after stage A orders the
      // planes before the plane pass.
    }
    __syncthreads();  // every stage C has read the planes before they hold the parked slots
    // ---- write the work item's Hermitian slots (x 1/2; packed: x 1, its
    // coefficient is 2 s).  Every thread of a
    // warp issues the same TMEM loads (they are warp-collective); values are
    // parked in the thread's own entries S[k][t] of the (now free) plane buffer.
    tm_wait_st();
    const int4 uc = a.ucols[t];
    float2* out = a.hpart + (int64_t(blockIdx.x) + cp) * 32 * HSLOTS;
    float2* S = W;
    constexpr float sc = PACK ? 1.f : 0.5f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      uint32_t r[16];
      tm_ld16(treg0 + 16 * c, r);
      tm_wait_ld(r);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        S[(8 * c + i) * THREADS + t] = make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
    }
    // self-conjugate column s: H(j_s, k) = region_s(k) + conj region_s(-k)
    auto self_conj = [&](int s) {
#pragma unroll 4
      for (int k = 0; k < 32; ++k) {
        const float2 h = S[k * THREADS + t], g = S[((32 - k) & 31) * THREADS + t];
        out[k * HSLOTS + uc.z + s] = make_float2(sc * (h.x + g.x), sc * (h.y - g.y));
      }
    };
    if (uc.w) self_conj(0);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      uint32_t r[16];
      __syncwarp();  // converged again after the self-conjugate branches
      tm_ld16(treg0 + 64 + 16 * c, r);
      tm_wait_ld(r);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int k = 8 * c + i;
        const float2 v = make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
        if (uc.w == 0) {  // column pair: H(j, k) = region0(k) + region1(k)
          const float2 h = S[k * THREADS + t];
          out[k * HSLOTS + uc.z] = make_float2(sc * (h.x + v.x), sc * (h.y + v.y));
        } else {
          S[k * THREADS + t] = v;
        }
      }
    }
    if (uc.w) self_conj(1);
    __syncthreads();  // the parked slots are read before the next segment's stage A
  }
  // every thread's TMEM traffic is complete before the columns are released
  tm_wait_st();
  tm_fence_before();
  __syncthreads();
  if (warp == 0) {
    tm_fence_after();
    tm_dealloc(tbase, TMEM_COLS);
  }
}

// G[cell][a][j] = sum over the segments of both parities of the Hermitian
// slots, expanded to all k (conjugate-mirrored for the negated partner columns)
__global__ void __launch_bounds__(256) k_herm_expand_par(float2* G, const float2* hpart, const int2* colslot,
                                                          int64_t cells, int Q, int ctas) {
  using namespace gc;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * N3) return;
  const int64_t cell = gid / N3;
  const int e = int(gid - cell * N3);
  const int a = e >> 10, j = e & 1023;
  const int2 cs = colslot[j];  // (slot, kind): 0 representative, 1 negated partner, 2 self-conjugate
  const int aa = cs.y == 1 ? ((32 - a) & 31) : a;
  const int64_t W = cells * 2 * Q;
  float2 s = make_float2(0.f, 0.f);
  for (int par = 0; par < 2; ++par) {
    const int64_t cp = 2 * cell + par, lo = cp * Q, hi = lo + Q;
    for (int64_t b = lo * ctas / W; b < ctas; ++b) {
      const int64_t wb0 = W * b / ctas, wb1 = W * (b + 1) / ctas;
      if (wb0 >= hi) break;
      if (wb1 <= lo) continue;  // this CTA's range ends where the segment starts
      const float2 v = hpart[((b + cp) * 32 + aa) * HSLOTS + cs.x];
      s.x += v.x;
      s.y += v.y;
    }
  }
  if (cs.y == 1) s.y = -s.y;
  G[gid] = s;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int gain_parity_prepare(pii_plan* p) {
  using namespace gpar;
  if (!p->tab.epar || !p->tab.gpar || !p->tab.gsx || !p->tab.gsxc || !p->gc_maps) {
    set_error("gain_parity_prepare: parity tables or column map missing");
    return PII_ERR_ARG;
  }
  PII_CUDA(cudaFuncSetAttribute(k_gain_parity<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM)));
  PII_CUDA(cudaFuncSetAttribute(k_gain_parity<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM)));
  int per_sm = 0, sms = 0;
  PII_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gain_parity<true>, THREADS, SMEM));
  PII_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
  if (per_sm != 1) {
    // every CTA takes all 512 TMEM columns: exactly one may be resident per SM
    set_error("gain_parity_prepare: %d resident CTAs per SM, expected 1", per_sm);
    return PII_ERR_CUDA;
  }
  p->gp_ctas = sms;
  // Hermitian slot sets: one per (CTA, cell-parity) segment, at most CTAs + 2 batch_max
  const int64_t max_items = int64_t(sms) + 2 * p->batch_max;
  const size_t bytes = size_t(max_items) * 32 * HSLOTS * sizeof(float2);
  PII_CUDA(cudaMalloc(&p->gp_hpart, bytes));
  p->bytes += int64_t(bytes);
  p->gp_max_items = max_items;
  // the antipodal passes (representative pair of each (sigma, -sigma) per radial
  // node) are set up with the plan; the packed kernel adds the Nyquist correction
  if (p->ap_count > 0) {
    // Nyquist-correction accumulators: cells x ceil(16 SMs / cells) <= 16 SMs + cells CTAs
    const size_t nq = (size_t(16 * sms) + size_t(p->batch_max)) * 3 * N2 * sizeof(float2);
    PII_CUDA(cudaMalloc(&p->nq_part, nq));
    p->bytes += int64_t(nq);
    PII_TRY(nyq_corr_prepare(p));
  }
  return PII_OK;
}

int gain_parity_run(pii_plan* p, int64_t cells, cudaStream_t s, bool packed) {
  using namespace gpar;
  if (packed && p->ap_count == 0) {
    set_error("gain_parity_run: the packed kernel needs an antipodally symmetric design");
    return PII_ERR_ARG;
  }
  const int QP = packed ? p->ap_count : p->Q;
  // one CTA per SM, each with an equal share of the (cell, parity, pass) work
  const int nct = int(std::min<int64_t>(p->gp_ctas, cells * 2 * QP));
  if (nct + 2 * cells > p->gp_max_items) {
    set_error("gain_parity_run: %lld cells beyond the plan's capacity", (long long)cells);
    return PII_ERR_SIZE;
  }
  GainParityArgs a{};
  a.fhat = static_cast<const float2*>(p->fhat);
  a.fT = static_cast<const float*>(p->fT);
  a.ephase = static_cast<const float2*>(p->tab.ephase);
  a.gphase = static_cast<const float2*>(p->tab.gphase);
  a.epar = static_cast<const float2*>(p->tab.epar);
  a.gpar = static_cast<const float2*>(p->tab.gpar);
  a.gsx = static_cast<const float*>(p->tab.gsx);
  a.gsxc = static_cast<const float*>(p->tab.gsxc);
  a.gph_stride = p->tab.gph_stride;
  a.gpar_stride = p->tab.gpar_stride;
  a.gsx_stride = p->tab.gsx_stride;
  a.gsxc_stride = p->tab.gsxc_stride;
  a.ns = p->ns;
  a.Q = p->Q;
  a.QP = QP;
  a.reps = packed ? p->ap_reps : nullptr;
  a.cells = cells;
  a.hpart = static_cast<float2*>(p->gp_hpart);
  a.ucols = static_cast<const int4*>(p->gc_maps);
  {
    StageTimer st(p, ST_GAIN_PARITY, s);
    if (packed)
      k_gain_parity<true><<<unsigned(nct), THREADS, SMEM, s>>>(a);
    else
      k_gain_parity<false><<<unsigned(nct), THREADS, SMEM, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_REDUCE, s);
    k_herm_expand_par<<<unsigned((cells * N3 + 255) / 256), 256, 0, s>>>(
        static_cast<float2*>(p->G), a.hpart,
        reinterpret_cast<const int2*>(static_cast<const char*>(p->gc_maps) + THREADS * sizeof(int4)), cells, QP,
        nct);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
