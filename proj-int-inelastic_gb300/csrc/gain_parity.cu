// Fused gain term of Q(f,f) for n = 32 in FP32, split by the parity of the
// first velocity axis: two independent CTAs per (cell, range of quadrature
// pairs), no cluster and no exchange between them.
//
// CTA p (p = 0, 1) owns the a-planes a = 2 m + p (m < 16) of the 32^3 work
// grid in 128 KB of shared memory (row-swizzled as in the cluster kernel).  Per
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

namespace pii {

namespace gpar {
using namespace gc;
constexpr int TMEM_COLS = 512;
// f of the CTA's 16 planes, transposed per plane to [c][b] with a 36-float row
// pitch: each lane of the plane pass reads its 32 values in 16-byte loads
// without bank conflicts
constexpr int FPITCH = 36;
constexpr size_t FS_OFF = size_t(PLANES) * N2 * sizeof(float2);
constexpr size_t SMEM = FS_OFF + size_t(PLANES) * 32 * FPITCH * sizeof(float) + 16;
}  // namespace gpar

// ---- tensor-memory access (PTX tcgen05, CTA group 1)
__device__ __forceinline__ void tm_alloc(uint32_t* slot, uint32_t ncols) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(slot));
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(a), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tm_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tm_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tm_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tm_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 16 consecutive 32-bit columns of this thread's lane
__device__ __forceinline__ void tm_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// completes the loads above; the registers are tied to it so that no use is
// scheduled before the wait
__device__ __forceinline__ void tm_wait_ld(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]));
}
__device__ __forceinline__ void tm_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]));
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;"); }

struct GainParityArgs {
  const float2* fhat;    // [cells][N3] spectra of f
  const float* fT;       // [cells][N3] f in FP32
  const float2* ephase;  // [Q][3][32]
  const float2* gphase;  // [Q][3][32]
  const float2* epar;    // [Q][2][32]
  const float2* gpar;    // [Q][2][32]
  const float* gsx;      // [n_r][513][20]
  int ns, Q;
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
  fft_line<16, +1>(u0);
  fft_line<16, +1>(u1);
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
  fft_line<16, +1>(u);
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
  fft_line<16, -1>(z);
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

__global__ void __launch_bounds__(gc::THREADS, 1) k_gain_parity(GainParityArgs a) {
  using namespace gpar;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* W = reinterpret_cast<float2*>(smem_raw);
  float* fS = reinterpret_cast<float*>(smem_raw + FS_OFF);
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
  const int64_t total = a.cells * 2 * a.Q;
  const int64_t w0 = total * blockIdx.x / gridDim.x, w1 = total * (blockIdx.x + 1) / gridDim.x;

  for (int64_t w = w0; w < w1;) {
    const int64_t cp = w / a.Q;
    const int par = int(cp & 1);
    const int64_t cell = cp >> 1;
    const int p0 = int(w - cp * a.Q);
    const int p1 = int(min(int64_t(a.Q), w1 - cp * a.Q));
    w = cp * a.Q + p1;
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

    for (int p = p0; p < p1; ++p) {
      // (per-pair pointers are formed inside each stage so that none stays
      // live across the register-heavy plane pass)
      // ---- A: the thread's two columns (those it also takes in stage C)
      {
        const float2* ep = a.ephase + int64_t(p) * 96;
        const float2* epp = a.epar + (int64_t(p) * 2 + par) * 32;
        const int4 uc = a.ucols[t];
        if (warp < 15) {  // column pairs {j, -j}: rows 1..15 and 31..17
          if (par == 0)
            par_stage_a_pair<0>(W, fh, ep, epp, uc.x);
          else
            par_stage_a_pair<1>(W, fh, ep, epp, uc.x);
        } else {  // rows 0 and 16 (with the self-conjugate columns): each column from its own values
#pragma unroll 1
          for (int h = 0; h < 2; ++h) {
            if (par == 0)
              par_stage_a_col<0>(W, fh, ep, epp, h ? uc.y : uc.x);
            else
              par_stage_a_col<1>(W, fh, ep, epp, h ? uc.y : uc.x);
          }
        }
      }
      __syncthreads();
      // ---- B: warp `warp` owns local plane `warp` (a = 2 warp + par)
      plane_pass<true>(W + warp * N2, fS + (warp * 32 + lane) * FPITCH, lane);
      __syncthreads();
      // ---- C: the thread's two columns (the previous pair's TMEM stores are complete first)
      {
        const float2* gp = a.gphase + int64_t(p) * 96;
        const float2* gpp = a.gpar + (int64_t(p) * 2 + par) * 32;
        const float* gsr = a.gsx + int64_t(p / a.ns) * (513 * 20);
        const int4 uc = a.ucols[t];
        tm_wait_st();
        par_stage_c<0>(W, uc.x, gp, gpp, gsr, treg0);
        par_stage_c<1>(W, uc.y, gp, gpp, gsr, treg0 + 64);
      }
      __syncthreads();  // the next pair's stage A overwrites the planes
    }
    // ---- write the work item's Hermitian slots (x 1/2).  Every thread of a
    // warp issues the same TMEM loads (they are warp-collective); values are
    // parked in the thread's own entries S[k][t] of the (now free) plane buffer.
    tm_wait_st();
    const int4 uc = a.ucols[t];
    float2* out = a.hpart + (int64_t(blockIdx.x) + cp) * 32 * HSLOTS;
    float2* S = W;
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
        out[k * HSLOTS + uc.z + s] = make_float2(0.5f * (h.x + g.x), 0.5f * (h.y - g.y));
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
          out[k * HSLOTS + uc.z] = make_float2(0.5f * (h.x + v.x), 0.5f * (h.y + v.y));
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
  if (!p->tab.epar || !p->tab.gpar || !p->tab.gsx || !p->gc_maps) {
    set_error("gain_parity_prepare: parity tables or column map missing");
    return PII_ERR_ARG;
  }
  PII_CUDA(cudaFuncSetAttribute(k_gain_parity, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM)));
  int per_sm = 0, sms = 0;
  PII_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gain_parity, THREADS, SMEM));
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
  return PII_OK;
}

int gain_parity_run(pii_plan* p, int64_t cells, cudaStream_t s) {
  using namespace gpar;
  // one CTA per SM, each with an equal share of the (cell, parity, pair) work
  const int nct = int(std::min<int64_t>(p->gp_ctas, cells * 2 * p->Q));
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
  a.ns = p->ns;
  a.Q = p->Q;
  a.cells = cells;
  a.hpart = static_cast<float2*>(p->gp_hpart);
  a.ucols = static_cast<const int4*>(p->gc_maps);
  {
    StageTimer st(p, ST_GAIN_PARITY, s);
    k_gain_parity<<<unsigned(nct), THREADS, SMEM, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_REDUCE, s);
    k_herm_expand_par<<<unsigned((cells * N3 + 255) / 256), 256, 0, s>>>(
        static_cast<float2*>(p->G), a.hpart,
        reinterpret_cast<const int2*>(static_cast<const char*>(p->gc_maps) + THREADS * sizeof(int4)), cells, p->Q,
        nct);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
