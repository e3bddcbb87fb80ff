// Column pass along the first velocity axis of the n = 64 pipeline on the
// tensor cores: the 64-point DFT of every (b, c) column as a dense GEMM with
// split-BF16 operands and FP32 accumulation in tensor memory.
//
// One item (cell, pair) is a 64 x 4096 complex array X[a][j] (j = (b, c)); its
// transform along a, Y[k][j] = sum_a W^{k a} X[a][j] with W = exp(DIR 2 pi i / 64)
// (DIR = +1 for the inverse transform of the first stage, -1 for the forward
// transform of the last), is, per tile of 128 columns, the real GEMM
//   D[n][o] = sum_kappa X[n][kappa] F[o][kappa],   n < 128 columns,
// kappa = a (Re X) or 64 + a (Im X), o = 2 k (Re Y[k]) or 2 k + 1 (Im Y[k]),
//   F[2k][a] = C, F[2k][64+a] = -S, F[2k+1][a] = S, F[2k+1][64+a] = C,   C + i S = W^{k a}.
// Both operands are split into BF16 pairs, x = x_hi + x_lo (x_hi = bf16(x),
// x_lo = bf16(x - x_hi): 16 significant bits), and the product is formed as
// X_hi F_hi + X_lo F_hi + X_hi F_lo with FP32 accumulation (the dropped
// X_lo F_lo and the residual of the split are ~2^-17 of each term).
//
// Kernel: persistent, one CTA per SM, warp-specialised, every stage double-buffered:
//   warp 17     TMA: one 2D tensor-map load of the tile (64 rows a x 128
//               columns, 64 KB) into raw buffer i % 2 (PSTART: f^, plus a bulk
//               copy of the pair's phase rows, src/collision/inelastic_collisions.py:212;
//               PEND: the plane-pass output in the chunk buffer);
//   warps 0-7   converters: lane = column n; multiply by the phase (PSTART),
//               split to BF16 hi / lo and tcgen05.st the operand X into tensor
//               memory (X buffer i % 2: row n = TMEM lane n, K pairs per column);
//   warp 16     issuer (one thread): 3 x 8 tcgen05.mma (M = N = 128, K = 16,
//               A = X from tensor memory, B = F from shared memory) into
//               accumulator i % 2, then commits to xempty (X buffer free) and tfull;
//   warps 8-15  epilogue: tcgen05.ld of the accumulator (lane = column n,
//               TMEM column = output o: whole complex outputs per thread),
//               arrive on tempty, store Y[k][j] coalesced along j (PEND: times
//               the pair's gain, :213-214, from its radial sinc row and phase
//               rows, bulk-copied by the TMA thread into gain buffer i % 2).
// Tensor memory: X buffers at columns [0, 256), accumulators at [256, 512).
// The F image (F_hi | F_lo, 64 KB, laid out on the host) is bulk-copied once
// per CTA.  Every mbarrier wait is bounded; a role that gives up raises a
// shared abort flag that ends the other roles' waits, and the device error
// word is set.  Replaces k_col<float, 64, PSTART / PEND>.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "fft_reg.cuh"
#include "pii_internal.cuh"
#include "tmem.cuh"
#include "umma.cuh"

namespace pii {

namespace ctc {
constexpr int NV = 64, N2 = NV * NV, N3 = NV * N2;
constexpr int CONVERTERS = 256, EPILOGUE = 256;
constexpr int ISSUER_WARP = (CONVERTERS + EPILOGUE) / 32, TMA_WARP = ISSUER_WARP + 1;
constexpr int THREADS = CONVERTERS + EPILOGUE + 64;
constexpr int TN = 128;                     // columns per tile (MMA M)
constexpr int TILES_PER_ITEM = N2 / TN;     // 32
constexpr uint32_t SBO = 2048, LBO = 128;   // K = 128 bf16 per row: 16 core matrices of 128 B
constexpr int OPB = 128 * 128 * 2;          // bytes of one 128 x 128 BF16 operand
constexpr int RAW = NV * TN * 8;            // one raw tile: 64 rows of 128 complex columns
constexpr int PROW = 3 * NV * 8;            // one pair's phase rows (3 x 64 complex)
constexpr int OFF_F = 0;                    // F_hi, F_lo
constexpr int OFF_R = 2 * OPB;              // raw tiles 0, 1, then the two phase rows
constexpr int OFF_P = OFF_R + 2 * RAW;
constexpr int GS_MAX = 3 * 32 * 32 + 1;     // gsinc row: |k|^2 <= 3 (n / 2)^2
constexpr int GS_PAD = (GS_MAX + 3) / 4 * 4;   // row pitch of the padded copy (16-byte rows)
constexpr int GROW = GS_PAD + 2 * 3 * NV;   // one pair's gain rows: gsinc row, then the 3 x 64 phases (floats)
constexpr int OFF_G = OFF_P + 2 * PROW;     // gain rows of the epilogue's two accumulators
constexpr int OFF_BAR = OFF_G + 2 * GROW * 4;
constexpr int NBAR = 17;  // rfull[2] rempty[2] xfull[2] xempty[2] tfull[2] tempty[2] fbar gfull[2] gempty[2]
constexpr int SMEM = OFF_BAR + NBAR * 8 + 16;
constexpr uint32_t TMEM_COLS = 512;         // X buffers [0, 256), accumulators [256, 512)
constexpr uint32_t WAIT_LIMIT = 1u << 22;   // mbarrier polls before a role gives up
static_assert(SMEM <= 232448, "shared memory per CTA");
}  // namespace ctc

struct ColTcArgs {
  const float2* src;    // PSTART: f^ [cells][N3]; PEND: the chunk buffer (in place)
  float2* dst;          // the chunk buffer [items][N3]
  const uint4* fimg;    // DFT matrix image of the direction (F_hi | F_lo)
  const float2* ephase;  // [Q][3][64]
  const float2* gphase;  // [Q][3][64]
  const float* gsinc;    // [n_r][GS_PAD]: the radial sinc rows, padded to 16-byte rows
  int ns;
  int64_t items, c0, p0, np;
  int* err;             // set to 1 if a role gave up waiting
};

__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t*>(&v); }

// bounded wait that also ends when another role has raised the abort flag
__device__ __forceinline__ bool mbar_wait_role(uint64_t* mbar, uint32_t parity, volatile int* abort) {
  for (uint32_t i = 0; i < ctc::WAIT_LIMIT; ++i) {
    if (mbar_try_wait(mbar, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}

template <int MODE>
__global__ void __launch_bounds__(ctc::THREADS, 1) k_col_tc(const __grid_constant__ CUtensorMap tmap, ColTcArgs a) {
  using namespace ctc;
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
    }
    mbar_init(fbar, 1);
    *abort = 0;
  }
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const uint32_t tmem = *tslot;
  const int64_t ntiles = a.items * TILES_PER_ITEM;

  if (warp < CONVERTERS / 32) {
    // ---- converters: warp w -> TMEM lanes 32 (w % 4) + lane (column n), a in [32 h, 32 h + 32)
    const int qd = warp & 3, h = warp >> 2, n = 32 * qd + lane;
    int i = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = i & 1;
      const uint32_t u = uint32_t(i >> 1) & 1u;
      if (!mbar_wait_role(rfull + b, u, abort)) break;
      const float2* raw = reinterpret_cast<const float2*>(sm + OFF_R + b * RAW);
      const float2* ep = reinterpret_cast<const float2*>(sm + OFF_P + b * PROW);
      float2 ebc = make_float2(1.f, 0.f);
      if constexpr (MODE == COL_PSTART) {
        const int j = int(tile % TILES_PER_ITEM) * TN + n;
        ebc = cmul(ep[NV + (j >> 6)], ep[2 * NV + (j & 63)]);
      }
      if (!mbar_wait_role(xempty + b, u ^ 1u, abort)) break;
      tm_fence_after();
      // X buffer b: hi at columns 128 b + [0, 64), lo at 128 b + [64, 128); K index
      // kappa = a (re) -> column kappa / 2, 64 + a (im) -> column 32 + a / 2.
      // Two halves of 16 a: 8 K pairs of real parts and 8 of imaginary parts, hi and lo.
      const uint32_t tx = tmem + (uint32_t(32 * qd) << 16) + uint32_t(128 * b);
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        uint32_t w[4][8];  // re hi, re lo, im hi, im lo
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int a0 = 32 * h + 16 * s + 2 * q;
          float2 v0 = raw[a0 * TN + n], v1 = raw[(a0 + 1) * TN + n];
          if constexpr (MODE == COL_PSTART) {
            v0 = cmul(v0, cmul(ep[a0], ebc));
            v1 = cmul(v1, cmul(ep[a0 + 1], ebc));
          }
          const __nv_bfloat162 rh = __floats2bfloat162_rn(v0.x, v1.x), ih = __floats2bfloat162_rn(v0.y, v1.y);
          const float2 rhf = __bfloat1622float2(rh), ihf = __bfloat1622float2(ih);
          w[0][q] = bf2_bits(rh);
          w[1][q] = bf2_bits(__floats2bfloat162_rn(v0.x - rhf.x, v1.x - rhf.y));
          w[2][q] = bf2_bits(ih);
          w[3][q] = bf2_bits(__floats2bfloat162_rn(v0.y - ihf.x, v1.y - ihf.y));
        }
        const uint32_t c = uint32_t(16 * h + 8 * s);
        tm_st8(tx + c, w[0]);
        tm_st8(tx + 64 + c, w[1]);
        tm_st8(tx + 32 + c, w[2]);
        tm_st8(tx + 96 + c, w[3]);
      }
      // the raw tile has been read
      mbar_arrive(rempty + b);
      tm_wait_st();
      tm_fence_before();
      mbar_arrive(xfull + b);
    }
  } else if (warp < (CONVERTERS + EPILOGUE) / 32) {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) + lane (column n) and
    // accumulator columns [64 h', 64 h' + 64) (outputs k = 32 h' .. 32 h' + 31)
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
      const float* gsS = reinterpret_cast<const float*>(sm + OFF_G) + d * GROW;
      const float2* gpS = reinterpret_cast<const float2*>(gsS + GS_PAD);
      const uint32_t u = uint32_t(i >> 1) & 1u;
      if (!mbar_wait_role(tfull + d, u, abort)) break;
      if (MODE == COL_PEND && !mbar_wait_role(gfull + d, u, abort)) break;
      tm_fence_after();
      const uint32_t ta = tmem + (uint32_t(32 * qd) << 16) + uint32_t(256 + 128 * d + 64 * hh);
      float2 gbc = make_float2(1.f, 0.f);
      int mbc = 0;
      if constexpr (MODE == COL_PEND) {
        const int jb = j >> 6, jc = j & 63;
        gbc = cmul(gpS[NV + jb], gpS[2 * NV + jc]);
        const int kb = kval(jb, NV), kc = kval(jc, NV);
        mbc = kb * kb + kc * kc;
      }
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        uint32_t r[16];
        tm_ld16(ta + 16 * c, r);
        tm_wait_ld(r);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = 32 * hh + 8 * c + q;
          float2 y = make_float2(__uint_as_float(r[2 * q]), __uint_as_float(r[2 * q + 1]));
          if constexpr (MODE == COL_PEND) {
            const int ka = kval(k, NV);
            y = cmul(y, cscale(cmul(gpS[k], gbc), gsS[mbc + ka * ka]));
          }
          out[int64_t(k) * N2] = y;
        }
      }
      // the accumulator has been read: the issuer may overwrite it
      tm_fence_before();
      mbar_arrive(tempty + d);
      if constexpr (MODE == COL_PEND) mbar_arrive(gempty + d);  // and the gain rows
    }
  } else if (warp == ISSUER_WARP) {
    if (lane == 0) {
      // ---- issuer
      const uint32_t sf = smem_u32(sm + OFF_F);
      constexpr uint32_t idesc = umma_idesc_bf16(TN, 128);
      bool go = mbar_wait_role(fbar, 0, abort);
      int i = 0;
      for (int64_t tile = blockIdx.x; go && tile < ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1;
        const uint32_t u = uint32_t(i >> 1) & 1u;
        if (!mbar_wait_role(xfull + b, u, abort)) break;
        if (!mbar_wait_role(tempty + b, u ^ 1u, abort)) break;
        tm_fence_after();
        const uint32_t tx = tmem + uint32_t(128 * b), td = tmem + uint32_t(256 + 128 * b);
#pragma unroll
        for (int s = 0; s < 8; ++s) {
          const uint32_t ko = 256u * s;  // two core matrices of F along K per step
          const uint64_t fhi = umma_sdesc(sf + ko, LBO, SBO), flo = umma_sdesc(sf + OPB + ko, LBO, SBO);
          umma_bf16_ts(td, tx + uint32_t(8 * s), fhi, idesc, s > 0 ? 1u : 0u);  // X_hi F_hi
          umma_bf16_ts(td, tx + uint32_t(64 + 8 * s), fhi, idesc, 1u);          // X_lo F_hi
          umma_bf16_ts(td, tx + uint32_t(8 * s), flo, idesc, 1u);               // X_hi F_lo
        }
        umma_commit(xempty + b);
        umma_commit(tfull + b);
      }
    }
  } else if (warp == TMA_WARP && lane == 0) {
    // ---- TMA: the F image, then each tile's rows (and the pair's phase rows)
    mbar_arrive_tx(fbar, 2 * OPB);
#pragma unroll 1
    for (int c = 0; c < 4; ++c)
      bulk_g2s(sm + OFF_F + c * (OPB / 2), reinterpret_cast<const char*>(a.fimg) + c * (OPB / 2), OPB / 2, fbar);
    int i = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = i & 1;
      if (!mbar_wait_role(rempty + b, (uint32_t(i >> 1) & 1u) ^ 1u, abort)) break;
      const int64_t item = tile / TILES_PER_ITEM;
      const int j0 = int(tile - item * TILES_PER_ITEM) * TN;
      const int64_t ci = item / a.np;
      const int64_t pair = a.p0 + (item - ci * a.np);
      // rows of 64 per grid: f^ of cell c0 + ci, or item `item` of the chunk buffer
      const int y = int(MODE == COL_PSTART ? (a.c0 + ci) * NV : item * NV);
      mbar_arrive_tx(rfull + b, RAW + (MODE == COL_PSTART ? PROW : 0));
      tma_load_2d(sm + OFF_R + b * RAW, &tmap, 2 * j0, y, rfull + b);
      if constexpr (MODE == COL_PSTART) bulk_g2s(sm + OFF_P + b * PROW, a.ephase + pair * 3 * NV, PROW, rfull + b);
      if constexpr (MODE == COL_PEND) {
        // the pair's gain rows into gain buffer b once the epilogue of tile i - 2 is done with it
        if (!mbar_wait_role(gempty + b, (uint32_t(i >> 1) & 1u) ^ 1u, abort)) break;
        unsigned char* g = sm + OFF_G + b * GROW * 4;
        mbar_arrive_tx(gfull + b, GS_PAD * 4 + PROW);
        bulk_g2s(g, a.gsinc + int64_t(pair / a.ns) * GS_PAD, GS_PAD * 4, gfull + b);
        bulk_g2s(g + GS_PAD * 4, a.gphase + pair * 3 * NV, PROW, gfull + b);
      }
    }
  }
  __syncthreads();
  if (*abort) {
    if (t == 0) atomicExch(a.err, 1);
  }
  tm_fence_before();
  __syncthreads();
  if (warp == 0) {
    tm_fence_after();
    tm_dealloc(tmem, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static uint16_t host_bf16(float x) {  // round to nearest even (finite inputs)
  uint32_t u;
  memcpy(&u, &x, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}
static float host_bf16_f(uint16_t h) {
  const uint32_t u = uint32_t(h) << 16;
  float x;
  memcpy(&x, &u, 4);
  return x;
}

// F_hi | F_lo images (rows o = 2 k + part, K index kappa) for DIR = +1 (index 0) and -1 (index 1)
static void build_dft_images(std::vector<uint16_t>& img) {
  using namespace ctc;
  img.assign(size_t(4) * OPB / 2, 0);
  for (int d = 0; d < 2; ++d) {
    const int dir = d == 0 ? 1 : -1;
    uint16_t* hi = img.data() + size_t(d) * OPB;  // OPB / 2 entries per operand, two operands
    uint16_t* lo = hi + OPB / 2;
    for (int o = 0; o < 128; ++o)
      for (int kap = 0; kap < 128; ++kap) {
        const int k = o >> 1, aa = kap & 63;
        const CS w = cs_turn((long long)(k * aa) % NV, NV);
        const double c = w.c, s = dir * w.s;
        const double v = (o & 1) == 0 ? (kap < 64 ? c : -s) : (kap < 64 ? s : c);
        const uint16_t h = host_bf16(float(v));
        const uint16_t l = host_bf16(float(v - double(host_bf16_f(h))));
        const uint32_t off = umma_kmajor_off(o, kap, SBO, LBO) / 2;
        hi[off] = h;
        lo[off] = l;
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
  if (!p->dft_img) {
    std::vector<uint16_t> img;
    build_dft_images(img);
    PII_CUDA(cudaMalloc(&p->dft_img, img.size() * 2));
    PII_CUDA(cudaMemcpy(p->dft_img, img.data(), img.size() * 2, cudaMemcpyHostToDevice));
    PII_CUDA(cudaMalloc(&p->dft_err, sizeof(int)));
    PII_CUDA(cudaMemset(p->dft_err, 0, sizeof(int)));
    p->bytes += int64_t(img.size() * 2 + sizeof(int));
  }
  if (!p->dft_gs) {  // the radial sinc rows with a 16-byte row pitch (bulk-copy sources)
    PII_CUDA(cudaMalloc(&p->dft_gs, size_t(p->nr) * GS_PAD * sizeof(float)));
    PII_CUDA(cudaMemset(p->dft_gs, 0, size_t(p->nr) * GS_PAD * sizeof(float)));
    PII_CUDA(cudaMemcpy2D(p->dft_gs, GS_PAD * sizeof(float), p->tab.gsinc, size_t(p->tab.M + 1) * sizeof(float),
                          size_t(p->tab.M + 1) * sizeof(float), size_t(p->nr), cudaMemcpyDeviceToDevice));
    p->bytes += int64_t(p->nr) * GS_PAD * sizeof(float);
  }
  PII_CUDA(cudaDeviceGetAttribute(&p->dft_ctas, cudaDevAttrMultiProcessorCount, p->device));
  return PII_OK;
}

int col_tc_run(pii_plan* p, int mode, int64_t items, int64_t c0, int64_t p0, int64_t np, cudaStream_t s) {
  using namespace ctc;
  if (p->n != NV || p->tab.M + 1 > GS_MAX) {
    set_error("col_tc_run: plan is not an n = 64 3D plan");
    return PII_ERR_ARG;
  }
  ColTcArgs a{};
  a.src = static_cast<const float2*>(mode == COL_PSTART ? p->fhat : p->buf);
  a.dst = static_cast<float2*>(p->buf);
  a.fimg = reinterpret_cast<const uint4*>(static_cast<const char*>(p->dft_img) + (mode == COL_PSTART ? 0 : 2 * OPB));
  a.ephase = static_cast<const float2*>(p->tab.ephase);
  a.gphase = static_cast<const float2*>(p->tab.gphase);
  a.gsinc = static_cast<const float*>(p->dft_gs);
  a.ns = p->ns;
  a.items = items;
  a.c0 = c0;
  a.p0 = p0;
  a.np = np;
  a.err = p->dft_err;
  const int64_t tiles = items * TILES_PER_ITEM;
  const unsigned grid = unsigned(std::min<int64_t>(p->dft_ctas, tiles));
  CUtensorMap tm;
  memcpy(&tm, p->dft_tmap[mode == COL_PSTART ? 0 : 1], sizeof(tm));
  if (mode == COL_PSTART) {
    StageTimer st(p, ST_COL_PSTART, s);
    k_col_tc<COL_PSTART><<<grid, THREADS, SMEM, s>>>(tm, a);
  } else {
    StageTimer st(p, ST_COL_PEND, s);
    k_col_tc<COL_PEND><<<grid, THREADS, SMEM, s>>>(tm, a);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
