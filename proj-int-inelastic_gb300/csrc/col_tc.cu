// Column pass along the first velocity axis of the n = 64 pipeline on the
// tensor cores: the 64-point DFT of every (b, c) column as a dense GEMM with
// split-FP16 operands and FP32 accumulation in tensor memory.
//
// One item (cell, pair) is a 64 x 4096 complex array X[a][j] (j = (b, c)); its
// transform along a, Y[k][j] = sum_a W^{k a} X[a][j] with W = exp(DIR 2 pi i / 64)
// (DIR = +1 for the inverse transform of the first stage, -1 for the forward
// transform of the last), is split once by decimation in frequency,
//   Y[2 k'] = sum_{a' < 32} S[a'] W^{2 k' a'},   Y[2 k' + 1] = sum_{a' < 32} D[a'] W^{(2 k' + 1) a'},
//   S = X[a'] + X[a' + 32],  D = X[a'] - X[a' + 32],
// and each half is, per tile of 128 columns, the real GEMM (g = even, odd)
//   D_g[n][o] = sum_kappa Z_g[n][kappa] F_g[o][kappa],   n < 128 columns,
// kappa = a' (Re Z) or 32 + a' (Im Z), o = 2 k' (Re) or 2 k' + 1 (Im), Z = S or D,
//   F_g[2k'][a'] = C, F_g[2k'][32+a'] = -S, F_g[2k'+1][a'] = S, F_g[2k'+1][32+a'] = C,
//   C + i S = W^{2 k' a'} (even) or W^{(2 k' + 1) a'} (odd)
// (K = 64, N = 64: half the products of the dense 64-point DFT).  Both
// operands are split into FP16 pairs, x = x_hi + x_lo (x_hi = fp16(x),
// x_lo = fp16(x - x_hi): 22 significant bits), and the product is formed as
// Z_hi F_hi + Z_lo F_hi + Z_hi F_lo with FP32 accumulation (the dropped
// Z_lo F_lo and the residual of the split are ~2^-22 of each term).  Each
// column is first scaled by a power of two that brings a bound on its S and D
// components (L1 norms of the inputs and phases, within ~3x of the largest)
// into [1/2, 1) (FP16 range, and x_lo stays a normal number for the column's
// large entries); the epilogue undoes it.  BF16 pairs (16 bits)
// measured 1.3e-5 relative L-inf against FP64 on a peaked cell with a small
// quadrature; FP16 pairs bring the path to the CUDA-core FFT's level.
//
// Kernel: persistent, one CTA per SM, warp-specialised, every stage double-buffered:
//   warp 17     TMA: one 2D tensor-map load of the tile (64 rows a x 128
//               columns, 64 KB) into raw buffer i % 2 (PSTART: f^, plus a bulk
//               copy of the pair's phase rows, src/collision/inelastic_collisions.py:212;
//               PEND: the plane-pass output in the chunk buffer);
//   warps 0-7   converters: lane = column n, warps w and w + 4 take a' in
//               [0, 16) and [16, 32); the two exchange their partial bounds
//               (named barrier 1), multiply by the phase (PSTART), form S and
//               D, scale, split to FP16 hi / lo, tcgen05.st the operands into
//               tensor memory (buffer i % 2: row n = TMEM lane n, K pairs per
//               column) and write the column's scale to scale buffer i % 4;
//   warp 16     issuer (one thread): arrives on sready (the scales of the tile
//               are visible), 2 x 3 x 4 tcgen05.mma (M = 128, N = 64, K = 16,
//               A = Z_g from tensor memory, B = F_g from shared memory) into
//               accumulator i % 2 (D_even | D_odd), then commits to xempty
//               (operand buffer free) and tfull;
//   warps 8-15  epilogue: tcgen05.ld of the accumulator (lane = column n,
//               TMEM column = output o: whole complex outputs per thread),
//               undo the column's scale, arrive on tempty, store Y[k][j]
//               coalesced along j (PEND: times
//               the pair's gain, :213-214: its phase rows and the slices
//               gsinc[r][|k_b|^2 + |k_c|^2 + |k_a|^2] of the tile's two k_b,
//               bulk-copied by the TMA thread into gain buffer i % 2).
// Tensor memory: operand buffers at columns [0, 256) (per buffer: S_hi, D_hi,
// S_lo, D_lo, 32 columns each), accumulators at [256, 512).  The F images
// (F_even hi / lo, F_odd hi / lo in FP16, 32 KB, laid out on the host) are
// bulk-copied once per CTA.  A scale buffer is rewritten four tiles later,
// after the MMAs of tile i + 2 -- issued only once the epilogue of tile i has
// released its accumulator, i.e. after it read the scales.  Every mbarrier wait is bounded; a role that gives up raises a
// shared abort flag that ends the other roles' waits, and the device error
// word is set.  Replaces k_col<float, 64, PSTART / PEND>.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fft_reg.cuh"
#include "pack.cuh"
#include "pii_internal.cuh"
#include "tmem.cuh"
#include "umma.cuh"

namespace pii {

namespace ctc {
constexpr int NV = 64, N2 = NV * NV, N3 = NV * N2;
constexpr int CONVERTERS = 256, EPILOGUE = 256;
// two more warps with one working lane each: the MMA issuer and the TMA thread
// (in separate warps: a lane suspended in an mbarrier wait would hold up the
// other's path; measured 20-25 % slower with the two roles in one warp)
constexpr int ISSUER_WARP = (CONVERTERS + EPILOGUE) / 32, TMA_WARP = ISSUER_WARP + 1;
constexpr int THREADS = CONVERTERS + EPILOGUE + 64;
constexpr int TN = 128;                     // columns per tile (MMA M)
constexpr int TILES_PER_ITEM = N2 / TN;     // 32
constexpr uint32_t SBO = 1024, LBO = 128;   // K = 64 16-bit elements per row: 8 core matrices of 128 B
constexpr int FOP = 64 * 64 * 2;            // bytes of one 64 x 64 FP16 matrix F_g (hi or lo)
constexpr int FIMG = 4 * FOP;               // F_even hi, F_even lo, F_odd hi, F_odd lo
constexpr int RAW = NV * TN * 8;            // one raw tile: 64 rows of 128 complex columns
constexpr int PROW = 3 * NV * 8;            // one pair's phase rows (3 x 64 complex)
constexpr int OFF_F = 0;                    // F_hi, F_lo
constexpr int OFF_R = FIMG;                 // raw tiles 0, 1, then the two phase rows
constexpr int OFF_P = OFF_R + 2 * RAW;
// radial sinc factor of the gain by |k| components: slice [|k_c| < 36 (33 used)][|k_a| pitch 33]
// per (r, |k_b|); odd pitch: lanes with distinct |k_c| read distinct banks
constexpr int KS = NV / 2 + 1, KC_ROWS = 36, KA_PITCH = 33;
constexpr int SLICE = KC_ROWS * KA_PITCH;   // floats (a multiple of 4: 16-byte bulk copies)
constexpr int GROW = 2 * SLICE + 2 * 3 * NV;  // two slices (the tile's two k_b), then the 3 x 64 phases (floats)
constexpr int OFF_G = OFF_P + 2 * PROW;     // gain rows of the epilogue's two accumulators
constexpr int OFF_SC = OFF_G + 2 * GROW * 4;  // column scales [4 tiles][128 columns] (floats)
constexpr int OFF_XB = OFF_SC + 4 * TN * 4;     // partial bounds [2 tiles][2 halves][128 columns]
constexpr int OFF_BAR = OFF_XB + 2 * 2 * TN * 4;
// rfull[2] rempty[2] xfull[2] xempty[2] tfull[2] tempty[2] fbar gfull[2] gempty[2] sready[2] dbar
constexpr int NBAR = 20;
constexpr int SMEM = OFF_BAR + NBAR * 8 + 16;
constexpr uint32_t TMEM_COLS = 512;         // X buffers [0, 256), accumulators [256, 512)
constexpr uint32_t WAIT_LIMIT = 1u << 22;   // default mbarrier polls before a role gives up
static_assert(SMEM <= 232448, "shared memory per CTA");
}  // namespace ctc

struct ColTcArgs {
  const float2* src;    // PSTART: f^ [cells][N3]; PEND: the chunk buffer (in place)
  float2* dst;          // the chunk buffer [items][N3]
  const uint4* fimg;    // DFT matrix images of the direction (F_even hi, lo, F_odd hi, lo)
  const float2* ephase;  // [Q][3][64]
  const float2* gphase;  // [Q][3][64]
  const float* gsk;      // [sets][n_r][|k_b| < 33][SLICE]: gsinc[r][k_b^2 + k_c^2 + k_a^2]
  int64_t gph_stride;    // complex elements of gphase per restitution set (0: one set)
  int64_t gsk_stride;    // floats of gsk per restitution set (0: one set)
  const float* colb;     // PSTART: [cells][N2] max over a of |f^(a, j)|_1 (k_col_bound)
  int ns;
  int64_t items, c0, p0, np;
  const int* reps;      // _PK modes: representative pair of each antipodal pass
  int* err;             // host-mapped word: 1 if a role gave up waiting, 2 if the drain also timed out
  uint32_t wait_limit;  // mbarrier polls before a role gives up
  int withhold;         // test hook: the TMA thread issues no copies, so the other roles' waits run out
};

__device__ __forceinline__ uint32_t h2_bits(__half2 v) { return *reinterpret_cast<uint32_t*>(&v); }

// FP16 hi / lo words of the K pair (x0, x1) (x already scaled into [-1, 1))
__device__ __forceinline__ void split_pair(float x0, float x1, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(x0, x1);
  const float2 hf = __half22float2(h);
  hi = h2_bits(h);
  lo = h2_bits(__floats2half2_rn(x0 - hf.x, x1 - hf.y));
}

// bounded wait that also ends when another role has raised the abort flag
__device__ __forceinline__ bool mbar_wait_role(uint64_t* mbar, uint32_t parity, volatile int* abort,
                                               uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_try_wait(mbar, parity)) return true;
    if (*abort) return false;
  }
  atomicMax(const_cast<int*>(abort), 1);
  return false;
}

// true in every thread of the named barrier `ID` (COUNT threads) if `pred` holds in any of them
template <int ID, int COUNT>
__device__ __forceinline__ bool bar_any(bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"(uint32_t(pred)), "n"(ID), "n"(COUNT)
      : "memory");
  return r != 0;
}

template <int MODE>
__global__ void __launch_bounds__(ctc::THREADS, 1) k_col_tc(const __grid_constant__ CUtensorMap tmap, ColTcArgs a) {
  using namespace ctc;
  // START: the inverse transform of the first stage (PSTART, or PSTART_PK on an
  // antipodal pass with the real phase t); !START: the forward transform of the
  // last stage with the complex gain (PEND) or the real coefficient 2 s (PEND_PK)
  constexpr bool START = MODE == COL_PSTART || MODE == COL_PSTART_PK;
  constexpr bool PACK = MODE == COL_PSTART_PK || MODE == COL_PEND_PK;
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
  uint64_t* rfull = bars;
  uint64_t* rempty = bars + 2;
  uint64_t* xfull = bars + 4;
  uint64_t* xempty = bars + 6;
  uint64_t* tfull = bars + 8;
  uint64_t* tempty = bars + 10;
  uint64_t* fbar = bars + 12;
  uint64_t* gfull = bars + 13;
  uint64_t* gempty = bars + 15;
  uint64_t* sready = bars + 17;
  uint64_t* dbar = bars + 19;  // the issuer's final commit: every MMA it issued has completed
  const uint32_t lim = a.wait_limit;
  bool drained = true;
  float* scl = reinterpret_cast<float*>(sm + OFF_SC);
  volatile int* abort = reinterpret_cast<volatile int*>(bars + NBAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + NBAR) + 1;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

  if (warp == 0) {
    tm_alloc(tslot, TMEM_COLS);
    tm_relinquish();
  }
  if (t == 0) {
    for (int b = 0; b < 2; ++b) {
      mbar_init(rfull + b, 1);
      mbar_init(rempty + b, CONVERTERS);
      mbar_init(xfull + b, CONVERTERS);
      mbar_init(xempty + b, 1);
      mbar_init(tfull + b, 1);
      mbar_init(tempty + b, EPILOGUE);
      mbar_init(gfull + b, 1);
      mbar_init(gempty + b, EPILOGUE);
      mbar_init(sready + b, 1);
    }
    mbar_init(fbar, 1);
    mbar_init(dbar, 1);
    *abort = 0;
  }
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const uint32_t tmem = *tslot;
  const int64_t ntiles = a.items * TILES_PER_ITEM;

  if (warp < CONVERTERS / 32) {
    // ---- converters: warp w -> TMEM lanes 32 (w % 4) + lane (column n), a' in [16 h, 16 h + 16)
    const int qd = warp & 3, h = warp >> 2, n = 32 * qd + lane;
    float* xb = reinterpret_cast<float*>(sm + OFF_XB);
    auto l1 = [](float2 v) { return fabsf(v.x) + fabsf(v.y); };
    int i = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = i & 1;
      const uint32_t u = uint32_t(i >> 1) & 1u;
      // PSTART: the cell's column bound, in flight during the waits below
      float cb = 0.f;
      if constexpr (START)
        cb = a.colb[(a.c0 + (tile / TILES_PER_ITEM) / a.np) * N2 + int(tile % TILES_PER_ITEM) * TN + n];
      // the raw tile is in and operand buffer b is free (MMAs of tile i - 2 done)
      const bool ok = mbar_wait_role(rfull + b, u, abort, lim) && mbar_wait_role(xempty + b, u ^ 1u, abort, lim);
      const float2* raw = reinterpret_cast<const float2*>(sm + OFF_R + b * RAW);
      const float2* ep = reinterpret_cast<const float2*>(sm + OFF_P + b * PROW);
      float2 ebc = make_float2(1.f, 0.f);
      float tcp = 0.f, tcm = 0.f, tth = 0.f;  // PSTART_PK: the real phase's column constants
      if constexpr (MODE == COL_PSTART) {
        const int j = int(tile % TILES_PER_ITEM) * TN + n;
        if (ok) ebc = cmul(ep[NV + (j >> 6)], ep[2 * NV + (j & 63)]);
      }
      if constexpr (MODE == COL_PSTART_PK) {
        const int j = int(tile % TILES_PER_ITEM) * TN + n;
        if (ok) pack_t_consts<float, float2, NV>(ep, j >> 6, j & 63, tcp, tcm, tth);
      }
      float mx = 0.f;
      if constexpr (MODE == COL_PSTART_PK) {
        // |x0 t0 +- x1 t1| <= 2 max_a |f^(a, j)|_1 max_a |t|, |t| <= sqrt 2 |e_0| (|c| <= 1, and
        // the a-row phases share the modulus |e_0|)
        if (!ok) break;  // no barrier in this mode: threads may leave one by one
        mx = 2.f * cb * (1.001f * 1.41422f * sqrtf(ep[0].x * ep[0].x + ep[0].y * ep[0].y));
      } else if constexpr (MODE == COL_PSTART) {
        // the cell's column bound (k_col_bound): |x0 e0 +- x1 e1| <= 2 max_a |f^(a, j)|_1 |e_a| |e_bc|_1;
        // the a-row phases exp(i phi) / n^3 share one modulus, |e_0| (FP32 rounding of the table
        // can leave a bound a few ulp low: the scaled values then exceed 1 by as much, well
        // inside FP16 range)
        if (!ok) break;  // no barrier in this mode: threads may leave one by one
        mx = 2.f * cb * (1.001f * sqrtf(ep[0].x * ep[0].x + ep[0].y * ep[0].y)) * l1(ebc);
      } else {
        if (ok) {
          // pass 1: this half's bound on |x0 +- x1| (L1 norms)
          float mb = 0.f;
#pragma unroll 8
          for (int q = 0; q < 16; ++q) {
            const int ap = 16 * h + q;
            mb = fmaxf(mb, l1(raw[ap * TN + n]) + l1(raw[(ap + 32) * TN + n]));
          }
          xb[((i & 1) * 2 + h) * TN + n] = mb;
        }
        // exchange with the other half of the column; every exit of this loop is
        // voted here, so the barrier never waits for a converter that left
        if (bar_any<1, CONVERTERS>(!ok)) break;
        mx = fmaxf(xb[((i & 1) * 2 + h) * TN + n], xb[((i & 1) * 2 + (h ^ 1)) * TN + n]);
      }
      // power of two bringing the bound into [1/2, 1): exponent arithmetic only
      const int ex = mx > 0.f ? int((__float_as_uint(mx) >> 23) & 0xFF) - 126 : 0;
      const float down = __uint_as_float(uint32_t(127 - ex) << 23), up = __uint_as_float(uint32_t(127 + ex) << 23);
      tm_fence_after();
      // pass 2: operand buffer b (columns 128 b + ...): S_hi [0, 32), D_hi [32, 64),
      // S_lo [64, 96), D_lo [96, 128); K index kappa = a' (re) -> column a' / 2,
      // 32 + a' (im) -> 16 + a' / 2.  Two quarters of 8 a' (4 K pairs each).
      const uint32_t tx = tmem + (uint32_t(32 * qd) << 16) + uint32_t(128 * b);
#pragma unroll
      for (int s4 = 0; s4 < 2; ++s4) {
        uint32_t w[8][4];  // [S re hi, S re lo, S im hi, S im lo, D re hi, D re lo, D im hi, D im lo][pair]
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int a0 = 16 * h + 8 * s4 + 2 * q;
          float2 x0 = raw[a0 * TN + n], x1 = raw[(a0 + 1) * TN + n];
          float2 y0 = raw[(a0 + 32) * TN + n], y1 = raw[(a0 + 33) * TN + n];
          if constexpr (MODE == COL_PSTART) {
            x0 = cmul(x0, cmul(ep[a0], ebc));
            x1 = cmul(x1, cmul(ep[a0 + 1], ebc));
            y0 = cmul(y0, cmul(ep[a0 + 32], ebc));
            y1 = cmul(y1, cmul(ep[a0 + 33], ebc));
          } else if constexpr (MODE == COL_PSTART_PK) {
            auto tt = [&](int aa) { return aa == NV / 2 ? tth : fmaf(ep[aa].y, tcm, ep[aa].x * tcp); };
            x0 = cscale(x0, tt(a0));
            x1 = cscale(x1, tt(a0 + 1));
            y0 = cscale(y0, tt(a0 + 32));
            y1 = cscale(y1, tt(a0 + 33));
          }
          const float2 v[2][2] = {{cadd(x0, y0), cadd(x1, y1)}, {csub(x0, y0), csub(x1, y1)}};
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            split_pair(v[g][0].x * down, v[g][1].x * down, w[4 * g + 0][q], w[4 * g + 1][q]);
            split_pair(v[g][0].y * down, v[g][1].y * down, w[4 * g + 2][q], w[4 * g + 3][q]);
          }
        }
        const uint32_t c = uint32_t(8 * h + 4 * s4);  // column of the first K pair (re)
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          const uint32_t base = tx + uint32_t(32 * g);
          tm_st4(base + c, w[4 * g + 0]);            // re hi
          tm_st4(base + 64 + c, w[4 * g + 1]);       // re lo
          tm_st4(base + 16 + c, w[4 * g + 2]);       // im hi
          tm_st4(base + 64 + 16 + c, w[4 * g + 3]);  // im lo
        }
      }
      // the raw tile has been read
      mbar_arrive(rempty + b);
      if (h == 0) scl[(i & 3) * TN + n] = up;
      tm_wait_st();
      tm_fence_before();
      mbar_arrive(xfull + b);
    }
  } else if (warp < (CONVERTERS + EPILOGUE) / 32) {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) + lane (column n) and
    // accumulator columns [64 h', 64 h' + 64): D_even (h' = 0, outputs k = 2 k')
    // or D_odd (h' = 1, k = 2 k' + 1), k' < 32
    const int ew = warp - CONVERTERS / 32, qd = ew & 3, hh = ew >> 2;
    const int n = 32 * qd + lane;
    int i = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int d = i & 1;
      const int64_t item = tile / TILES_PER_ITEM;
      const int j = int(tile - item * TILES_PER_ITEM) * TN + n;
      float2* out = a.dst + item * N3 + j;
      // PEND: gain(k, j) = g_a[k] g_b[jb] g_c[jc] * gsinc[r][k_b^2 + k_c^2 + k_a^2], from
      // the pair's rows in gain buffer d
      const float* gsl = reinterpret_cast<const float*>(sm + OFF_G) + d * GROW;
      const float2* gpS = reinterpret_cast<const float2*>(gsl + 2 * SLICE);
      const uint32_t u = uint32_t(i >> 1) & 1u;
      if (!mbar_wait_role(tfull + d, u, abort, lim)) break;
      if (!mbar_wait_role(sready + d, u, abort, lim)) break;
      if (!START && !mbar_wait_role(gfull + d, u, abort, lim)) break;
      tm_fence_after();
      const float up = scl[(i & 3) * TN + n];  // the column's scale (S and D alike)
      const uint32_t ta = tmem + (uint32_t(32 * qd) << 16) + uint32_t(256 + 128 * d + 64 * hh);
      float2 gbc = make_float2(1.f, 0.f);
      float sdp = 0.f, sdm = 0.f, ssh = 0.f;  // PEND_PK: the real coefficient's column constants
      const float* grow = gsl;
      if constexpr (!START) {
        const int jb = j >> 6, jc = j & 63;
        if constexpr (PACK)
          pack_s_consts<float, float2, NV>(gpS, jb, jc, sdp, sdm, ssh);
        else
          gbc = cmul(gpS[NV + jb], gpS[2 * NV + jc]);
        const int kc = kval(jc, NV);
        grow = gsl + (n >> 6) * SLICE + (kc < 0 ? -kc : kc) * KA_PITCH;  // slice of this column's k_b, row |k_c|
      }
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        tm_ld16(ta + 16 * c, r);
        tm_wait_ld(r);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = 2 * (8 * c + q) + hh;
          float2 y = make_float2(up * __uint_as_float(r[2 * q]), up * __uint_as_float(r[2 * q + 1]));
          if constexpr (MODE == COL_PEND) {
            const int ka = kval(k, NV);
            y = cmul(y, cscale(cmul(gpS[k], gbc), grow[ka < 0 ? -ka : ka]));
          } else if constexpr (MODE == COL_PEND_PK) {
            const int ka = kval(k, NV);
            const float2 g = gpS[k];
            const float sv = k == NV / 2 ? ssh : fmaf(-g.y, sdm, g.x * sdp);
            y = cscale(y, 2.f * sv * grow[ka < 0 ? -ka : ka]);
          }
          out[int64_t(k) * N2] = y;
        }
      }
      // the accumulator has been read: the issuer may overwrite it
      tm_fence_before();
      mbar_arrive(tempty + d);
      if constexpr (!START) mbar_arrive(gempty + d);  // and the gain rows
    }
  } else if (warp == ISSUER_WARP) {
    if (lane == 0) {
      // ---- issuer
      const uint32_t sf = smem_u32(sm + OFF_F);
      constexpr uint32_t idesc = umma_idesc_f16(TN, 64);
      bool go = mbar_wait_role(fbar, 0, abort, lim);
      bool issued = false;
      int i = 0;
      for (int64_t tile = blockIdx.x; go && tile < ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1;
        const uint32_t u = uint32_t(i >> 1) & 1u;
        if (!mbar_wait_role(xfull + b, u, abort, lim)) break;
        if (!mbar_wait_role(tempty + b, u ^ 1u, abort, lim)) break;
        mbar_arrive(sready + b);  // the converters' scales of this tile are visible from here
        tm_fence_after();
        const uint32_t tx = tmem + uint32_t(128 * b), td = tmem + uint32_t(256 + 128 * b);
#pragma unroll
        for (int g = 0; g < 2; ++g) {  // even outputs from S, odd outputs from D
          const uint32_t zhi = tx + uint32_t(32 * g), zlo = zhi + 64, dg = td + uint32_t(64 * g);
          const uint32_t fh = sf + uint32_t(2 * g * FOP), fl = fh + uint32_t(FOP);
#pragma unroll
          for (int st = 0; st < 4; ++st) {
            const uint32_t ko = 256u * st;  // two core matrices of F_g along K per step
            const uint64_t fhi = umma_sdesc(fh + ko, LBO, SBO), flo = umma_sdesc(fl + ko, LBO, SBO);
            umma_bf16_ts(dg, zhi + uint32_t(8 * st), fhi, idesc, st > 0 ? 1u : 0u);  // Z_hi F_hi
            umma_bf16_ts(dg, zlo + uint32_t(8 * st), fhi, idesc, 1u);                // Z_lo F_hi
            umma_bf16_ts(dg, zhi + uint32_t(8 * st), flo, idesc, 1u);                // Z_hi F_lo
          }
        }
        umma_commit(xempty + b);
        umma_commit(tfull + b);
        issued = true;
      }
      // drain: wait (bounded, not cut short by the abort flag) until every MMA
      // issued here has completed, so no MMA writes tensor memory after it is freed
      if (issued) {
        umma_commit(dbar);
        drained = mbar_wait_bounded(dbar, 0, lim);
      }
    }
  } else if (warp == TMA_WARP) {
    if (lane == 0) {
      // ---- TMA: the F image, then each tile's rows (and the pair's phase rows)
      // rphases[b] / gphases[b]: copies issued into raw / gain buffer b (one
      // barrier phase each; at most one in flight per buffer)
      int rphases[2] = {0, 0}, gphases[2] = {0, 0};
      const bool go = !a.withhold;
      if (go) {
        mbar_arrive_tx(fbar, FIMG);
#pragma unroll 1
        for (int c = 0; c < 4; ++c)
          bulk_g2s(sm + OFF_F + c * FOP, reinterpret_cast<const char*>(a.fimg) + c * FOP, FOP, fbar);
      }
      int i = 0;
      for (int64_t tile = blockIdx.x; go && tile < ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1;
        if (!mbar_wait_role(rempty + b, (uint32_t(i >> 1) & 1u) ^ 1u, abort, lim)) break;
        const int64_t item = tile / TILES_PER_ITEM;
        const int j0 = int(tile - item * TILES_PER_ITEM) * TN;
        const int64_t ci = item / a.np;
        const int64_t pair = PACK ? int64_t(a.reps[a.p0 + (item - ci * a.np)]) : a.p0 + (item - ci * a.np);
        // rows of 64 per grid: f^ of cell c0 + ci, or item `item` of the chunk buffer
        const int y = int(START ? (a.c0 + ci) * NV : item * NV);
        mbar_arrive_tx(rfull + b, RAW + (START ? PROW : 0));
        ++rphases[b];
        tma_load_2d(sm + OFF_R + b * RAW, &tmap, 2 * j0, y, rfull + b);
        if constexpr (START) bulk_g2s(sm + OFF_P + b * PROW, a.ephase + pair * 3 * NV, PROW, rfull + b);
        if constexpr (!START) {
          // the pair's gain rows into gain buffer b once the epilogue of tile i - 2 is done with it
          if (!mbar_wait_role(gempty + b, (uint32_t(i >> 1) & 1u) ^ 1u, abort, lim)) break;
          unsigned char* g = sm + OFF_G + b * GROW * 4;
          mbar_arrive_tx(gfull + b, 2 * SLICE * 4 + PROW);
          ++gphases[b];
          const int64_t cell = a.c0 + ci;  // its restitution set, when the plan has one per cell
          const float* gr = a.gsk + cell * a.gsk_stride + int64_t(pair / a.ns) * KS * SLICE;
          for (int h = 0; h < 2; ++h) {  // columns j0 .. j0 + 127 span k_b rows j0 / 64 and j0 / 64 + 1
            const int kb = kval(j0 / NV + h, NV);
            bulk_g2s(g + h * SLICE * 4, gr + (kb < 0 ? -kb : kb) * SLICE, SLICE * 4, gfull + b);
          }
          bulk_g2s(g + 2 * SLICE * 4, a.gphase + cell * a.gph_stride + pair * 3 * NV, PROW, gfull + b);
        }
      }
      // drain: wait (bounded, not cut short by the abort flag) for the last copy
      // into every buffer, so none lands in shared memory after the CTA is gone
      if (go) drained = mbar_wait_bounded(fbar, 0, lim);
      for (int b = 0; b < 2; ++b) {
        if (rphases[b] > 0) drained &= mbar_wait_bounded(rfull + b, uint32_t(rphases[b] - 1) & 1u, lim);
        if (gphases[b] > 0) drained &= mbar_wait_bounded(gfull + b, uint32_t(gphases[b] - 1) & 1u, lim);
      }
    }
  }
  if (!drained) atomicMax(const_cast<int*>(abort), 2);  // only the issuer and TMA lanes can fail to drain
  __syncthreads();
  if (t == 0 && *abort) {
    // report to the host-mapped word (read by the next call on the plan)
    *reinterpret_cast<volatile int*>(a.err) = *abort == 2 ? 2 : 1;
    __threadfence_system();
  }
  tm_fence_before();
  __syncthreads();
  if (warp == 0) {
    tm_fence_after();
    tm_dealloc(tmem, TMEM_COLS);
  }
}

// colb[cell][j] = max over a of |f^(a, j)|_1: the PSTART column bound (f^ is
// the same for every pair of the cell)
__global__ void __launch_bounds__(256) k_col_bound(const float2* fhat, float* colb, int64_t cells) {
  using namespace ctc;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * N2) return;
  const int64_t cell = gid / N2;
  const int j = int(gid - cell * N2);
  const float2* x = fhat + cell * N3 + j;
  float m = 0.f;
#pragma unroll 8
  for (int a0 = 0; a0 < NV; ++a0) {
    const float2 v = x[a0 * N2];
    m = fmaxf(m, fabsf(v.x) + fabsf(v.y));
  }
  colb[gid] = m;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// IEEE half: round to nearest even, for |x| < 65504 (no overflow handling needed here)
static uint16_t host_f16(double x) {
  const uint16_t sign = x < 0 ? 0x8000 : 0;
  double a = x < 0 ? -x : x;
  if (a == 0.0) return sign;
  int e = 0;
  std::frexp(a, &e);  // a = m 2^e, m in [1/2, 1)
  int E = e - 1;      // a = 1.f x 2^E
  if (E < -14) E = -14;  // subnormal range: fixed spacing 2^-24
  const double q = std::ldexp(a, 10 - E);  // value in units of the last place
  double r = std::nearbyint(q);             // round half to even (default rounding mode)
  if (r >= 2048.0) {                         // carried into the next binade
    r /= 2.0;
    ++E;
  }
  const uint32_t mant = uint32_t(r);
  if (mant < 1024) return uint16_t(sign | mant);  // subnormal (E == -14)
  return uint16_t(sign | (uint32_t(E + 15) << 10) | (mant - 1024));
}
static double host_f16_d(uint16_t h) {
  const int E = (h >> 10) & 0x1F, m = h & 0x3FF;
  const double v = E == 0 ? std::ldexp(double(m), -24) : std::ldexp(double(1024 + m), E - 25);
  return (h & 0x8000) ? -v : v;
}

// F_even hi, lo, F_odd hi, lo images (rows o = 2 k' + part, K index kappa, K-major,
// SBO / LBO as in the kernel) for DIR = +1 (index 0) and -1 (index 1)
static void build_dft_images(std::vector<uint16_t>& img) {
  using namespace ctc;
  constexpr int E = FOP / 2;  // entries per matrix
  img.assign(size_t(2) * 4 * E, 0);
  for (int d = 0; d < 2; ++d) {
    const int dir = d == 0 ? 1 : -1;
    for (int g = 0; g < 2; ++g) {
      uint16_t* hi = img.data() + size_t(d) * 4 * E + size_t(2 * g) * E;
      uint16_t* lo = hi + E;
      for (int o = 0; o < 64; ++o)
        for (int kap = 0; kap < 64; ++kap) {
          const int k = o >> 1, ap = kap & 31;
          const long long m = (long long)(2 * k + g) * ap % NV;  // W^{(2 k' + g) a'}
          const CS w = cs_turn(m, NV);
          const double c = w.c, sn = dir * w.s;
          const double v = (o & 1) == 0 ? (kap < 32 ? c : -sn) : (kap < 32 ? sn : c);
          const uint16_t h = host_f16(v);
          const uint16_t l = host_f16(v - host_f16_d(h));
          const uint32_t off = umma_kmajor_off(o, kap, SBO, LBO) / 2;
          hi[off] = h;
          lo[off] = l;
        }
    }
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// 2D FP32 view [grids x 64 rows][8192 floats] of `base`, box 256 floats x 64 rows (one tile)
static int make_tmap(unsigned char* out, void* base, int64_t grids) {
  using namespace ctc;
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      set_error("col_tc_prepare: cuTensorMapEncodeTiled is not available");
      return PII_ERR_CUDA;
    }
    encode = reinterpret_cast<EncodeTiledFn>(fn);
  }
  CUtensorMap m;
  const cuuint64_t dims[2] = {cuuint64_t(2 * N2), cuuint64_t(grids) * NV};
  const cuuint64_t strides[1] = {cuuint64_t(2 * N2) * 4};
  const cuuint32_t box[2] = {2 * TN, NV};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("col_tc_prepare: cuTensorMapEncodeTiled failed (%d)", int(r));
    return PII_ERR_CUDA;
  }
  static_assert(sizeof(CUtensorMap) == 128, "tensor map size");
  memcpy(out, &m, sizeof(m));
  return PII_OK;
}

int col_tc_prepare(pii_plan* p) {
  using namespace ctc;
  PII_TRY(make_tmap(p->dft_tmap[0], p->fhat, p->batch_max));
  PII_TRY(make_tmap(p->dft_tmap[1], p->buf, p->chunk_items));
  PII_CUDA(cudaFuncSetAttribute(k_col_tc<COL_PSTART>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
  PII_CUDA(cudaFuncSetAttribute(k_col_tc<COL_PEND>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
  PII_CUDA(cudaFuncSetAttribute(k_col_tc<COL_PSTART_PK>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
  PII_CUDA(cudaFuncSetAttribute(k_col_tc<COL_PEND_PK>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
  if (!p->dft_img) {
    std::vector<uint16_t> img;
    build_dft_images(img);
    PII_CUDA(cudaMalloc(&p->dft_img, img.size() * 2));
    PII_CUDA(cudaMemcpy(p->dft_img, img.data(), img.size() * 2, cudaMemcpyHostToDevice));
    // the stall word lives in mapped host memory: the host reads it without a
    // synchronisation at the start of every later call on the plan
    PII_CUDA(cudaHostAlloc(&p->dft_err_host, sizeof(int), cudaHostAllocMapped));
    *p->dft_err_host = 0;
    PII_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&p->dft_err), p->dft_err_host, 0));
    p->bytes += int64_t(img.size() * 2 + sizeof(int));
  }
  if (!p->dft_gs) PII_TRY(col_tc_gain_tables(p));
  if (!p->dft_colb) {
    PII_CUDA(cudaMalloc(&p->dft_colb, size_t(p->batch_max) * N2 * sizeof(float)));
    p->bytes += int64_t(p->batch_max) * N2 * sizeof(float);
  }
  PII_CUDA(cudaDeviceGetAttribute(&p->dft_ctas, cudaDevAttrMultiProcessorCount, p->device));
  return PII_OK;
}

// gsinc[r][k_b^2 + k_c^2 + k_a^2] by (set, r, |k_b|, |k_c|, |k_a|): the bulk-copy
// sources of the PEND epilogue's sinc slices, one block per restitution set
int col_tc_gain_tables(pii_plan* p) {
  using namespace ctc;
  const int M1 = p->tab.M + 1;
  const int64_t sets = p->tab.nsets;
  const size_t per = size_t(p->nr) * KS * SLICE;
  std::vector<float> gs(size_t(sets) * p->nr * M1), gk(size_t(sets) * per, 0.f);
  PII_CUDA(cudaMemcpy(gs.data(), p->tab.gsinc, gs.size() * sizeof(float), cudaMemcpyDeviceToHost));
  for (int64_t st = 0; st < sets; ++st)
    for (int r = 0; r < p->nr; ++r)
      for (int kb = 0; kb < KS; ++kb)
        for (int kc = 0; kc < KS; ++kc)
          for (int ka = 0; ka < KS; ++ka)
            gk[size_t(st) * per + (size_t(r) * KS + kb) * SLICE + kc * KA_PITCH + ka] =
                gs[(size_t(st) * p->nr + r) * M1 + kb * kb + kc * kc + ka * ka];
  if (p->dft_gs) {
    cudaFree(p->dft_gs);
    p->bytes -= p->dft_gs_bytes;
    p->dft_gs = nullptr;
  }
  PII_CUDA(cudaMalloc(&p->dft_gs, gk.size() * sizeof(float)));
  PII_CUDA(cudaMemcpy(p->dft_gs, gk.data(), gk.size() * sizeof(float), cudaMemcpyHostToDevice));
  p->dft_gs_bytes = int64_t(gk.size() * sizeof(float));
  p->bytes += p->dft_gs_bytes;
  p->dft_gs_stride = sets > 1 ? int64_t(per) : 0;
  return PII_OK;
}

int dft_stall_check(pii_plan* p) {
  if (!p || !p->dft_err_host) return PII_OK;
  volatile int* w = p->dft_err_host;
  const int v = *w;
  if (!v) return PII_OK;
  *w = 0;
  set_error(v == 3   ? "fused gain kernel: a CTA gave up waiting for a cluster exchange (bounded mbarrier wait); "
                       "results of that launch are invalid"
            : v == 2 ? "tensor-core DFT: a CTA gave up waiting and could not drain its copies; results of that "
                       "launch are invalid"
                     : "tensor-core DFT: a CTA gave up waiting (bounded mbarrier wait); results of that launch are "
                       "invalid");
  return PII_ERR_STALL;
}

int col_tc_bounds(pii_plan* p, int64_t cells, cudaStream_t s) {
  using namespace ctc;
  {
    StageTimer st(p, ST_COL_FWD, s);
    k_col_bound<<<unsigned((cells * N2 + 255) / 256), 256, 0, s>>>(static_cast<const float2*>(p->fhat),
                                                                     static_cast<float*>(p->dft_colb), cells);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int col_tc_run(pii_plan* p, int mode, int64_t items, int64_t c0, int64_t p0, int64_t np, cudaStream_t s) {
  using namespace ctc;
  if (p->n != NV || p->tab.M != 3 * (NV / 2) * (NV / 2)) {
    set_error("col_tc_run: plan is not an n = 64 3D plan");
    return PII_ERR_ARG;
  }
  const bool start = mode == COL_PSTART || mode == COL_PSTART_PK;
  const bool pack = mode == COL_PSTART_PK || mode == COL_PEND_PK;
  if (mode != COL_PSTART && mode != COL_PEND && !pack) {
    set_error("col_tc_run: unknown column mode %d", mode);
    return PII_ERR_ARG;
  }
  if (pack && !p->ap_reps) {
    set_error("col_tc_run: antipodal passes need an antipodally symmetric design");
    return PII_ERR_ARG;
  }
  ColTcArgs a{};
  a.src = static_cast<const float2*>(start ? p->fhat : p->buf);
  a.reps = p->ap_reps;
  a.dst = static_cast<float2*>(p->buf);
  a.fimg = reinterpret_cast<const uint4*>(static_cast<const char*>(p->dft_img) + (start ? 0 : FIMG));
  a.ephase = static_cast<const float2*>(p->tab.ephase);
  a.gphase = static_cast<const float2*>(p->tab.gphase);
  a.gsk = static_cast<const float*>(p->dft_gs);
  a.gph_stride = p->tab.gph_stride;
  a.gsk_stride = p->dft_gs_stride;
  a.colb = static_cast<const float*>(p->dft_colb);
  a.ns = p->ns;
  a.items = items;
  a.c0 = c0;
  a.p0 = p0;
  a.np = np;
  a.err = p->dft_err;
  a.wait_limit = p->dft_wait_limit;
  a.withhold = p->dft_withhold;
  const int64_t tiles = items * TILES_PER_ITEM;
  const unsigned grid = unsigned(std::min<int64_t>(p->dft_ctas, tiles));
  CUtensorMap tm;
  memcpy(&tm, p->dft_tmap[start ? 0 : 1], sizeof(tm));
  {
    StageTimer st(p, start ? ST_COL_PSTART : ST_COL_PEND, s);
    if (mode == COL_PSTART)
      k_col_tc<COL_PSTART><<<grid, THREADS, SMEM, s>>>(tm, a);
    else if (mode == COL_PEND)
      k_col_tc<COL_PEND><<<grid, THREADS, SMEM, s>>>(tm, a);
    else if (mode == COL_PSTART_PK)
      k_col_tc<COL_PSTART_PK><<<grid, THREADS, SMEM, s>>>(tm, a);
    else
      k_col_tc<COL_PEND_PK><<<grid, THREADS, SMEM, s>>>(tm, a);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
