// Fused gain term of Q(f,f) for the FP32 plans of n in {16, 24, 48, 64}: every
// (cell, pass) work item stays on chip from the phase product to the gain sum.
//
// One work item is the n^3 complex grid of one quadrature pair (or antipodal
// pass) of one cell (src/collision/inelastic_collisions.py:212-217):
//   A  X = phase(k) f^(k), inverse transform along a          (column layout)
//   B  inverse along b, inverse along c, * f, forward along c,
//      forward along b                                         (plane layout)
//   C  forward along a, * gain(k), summed over the cell's items (column layout)
// A cluster of CS CTAs holds the item: CTA r owns the a-planes
// [r NPL, (r + 1) NPL) in stage B and the columns (b, c) with b in the same
// range in stages A and C (NPL = n / CS; n = 16, 24: CS = 1, the item fits one
// CTA; n = 48: CS = 6; n = 64: CS = 16).  Between the layouts each thread
// stores its line straight into the owning CTA's shared memory with st.async,
// which counts the bytes on the receiver's mbarrier: a column's n values go to
// the n / NPL plane owners, a plane column's n values to the column owners,
// 256 contiguous bytes per warp store; the CTA's own share goes by plain
// shared-memory stores (the cluster path runs at ~16 B/clk per SM, and the
// exchanges' stores were a third of the kernel's time at n = 48).  A CTA
// waits (bounded) for its mbarrier to see the other CTAs' bytes of an
// exchange and every own thread's arrival after its plain stores; a cluster barrier
// arrived on right after a buffer's last read (split arrive / wait, so the
// transform that follows hides it) keeps the next exchange from overwriting
// a buffer still being read.  The phase and gain rows of a pass and the sinc
// row of its radial node are copied to shared memory by cp.async one stage
// ahead of their use.
// The gain sum of the CTA's columns, n k_a values each (147 KB per CTA at
// n = 48, 131 KB at n = 64), lives in tensor memory for all the items of a
// cell, next to the columns' spectra f^(a, j), which are the same for every
// pass of the cell (copied there once per cell).  At n = 48 f of the CTA's
// planes takes the rest of tensor memory instead, one row per plane line, so
// that the CTA's shared memory holds only its planes: the spectra of five
// warps are kept in the shared memory left over, the other seven warps read
// theirs from L2 every pass.  At the end of a
// cell's range the CTA writes its sums to a per-part slot, and
// k_fused_expand adds the parts of each cell into G.  Antipodally
// symmetric designs run the packed passes (real phase t, real coefficient
// 2 s; pack.cuh), followed by the Nyquist correction.
#include <algorithm>

#include "fft_reg.cuh"
#include "pack.cuh"
#include "pii_internal.cuh"
#include "tmem.cuh"
#include "umma.cuh"

namespace pii {

namespace gfu {
template <int NV>
struct Cfg;
// CS: CTAs of a cluster; F_TM: f of the CTA's planes in tensor memory (one
// n-column row per plane line) instead of shared memory; PK_AC, PK_B: the line
// transforms' butterflies on the packed FP32x2 pipe in stages A and C, in
// stage B
template <>
struct Cfg<16> {
  static constexpr bool PK_AC = true, PK_B = true;
  static constexpr int CS = 1;
  static constexpr bool F_TM = false;
};
template <>
struct Cfg<24> {  // packed butterflies: 0.538 ms per Q (32 cells) instead of 0.526
  static constexpr bool PK_AC = false, PK_B = false;
  static constexpr int CS = 1;
  static constexpr bool F_TM = false;
};
template <>
struct Cfg<48> {  // 6 CTAs of 12 warps: three 6-CTA clusters per 19-SM GPC; 7.61 -> 7.25 ms per Q (16 cells) packed
  static constexpr bool PK_AC = true, PK_B = true;
  static constexpr int CS = 6;
  static constexpr bool F_TM = true;
};
template <>
struct Cfg<64> {  // packed butterflies: 99.5 -> 88.7 ms per Q on 16 cells (A and C alone: 88.1)
  static constexpr bool PK_AC = true, PK_B = true;
  static constexpr int CS = 16;
  static constexpr bool F_TM = false;
};

template <int NV>
struct Geo {
  static constexpr int CS = Cfg<NV>::CS;
  static constexpr int N2 = NV * NV, N3 = N2 * NV;
  static constexpr int NPL = NV / CS;    // a-planes of a CTA
  static constexpr int NCOL = N2 / CS;   // (b, c) columns of a CTA
  static constexpr int THREADS = NCOL;   // = NPL * NV plane lines
  // padded plane row (complex elements): n + 1, or n + 2 where n is a
  // multiple of 16 (48, 64), so that every row starts on 16 bytes and the row
  // pass moves two elements per 16-byte access (a quarter-warp of 16-byte
  // accesses at row stride 4 mod 32 words is conflict-free; so are the
  // column pass's 8-byte accesses, whose half-warps never straddle planes)
  static constexpr bool ROW16 = NV % 16 == 0;
  static constexpr int LD = NV + (ROW16 ? 2 : 1);
  static constexpr int LDF = NV + 1;  // row of f in shared memory (floats)
  static constexpr int PLANE = NPL * NV * LD;
  static constexpr int COLS = NV * NCOL;
  static constexpr int BUF = PLANE > COLS ? PLANE : COLS;
  static constexpr bool F_TM = Cfg<NV>::F_TM;
  static constexpr bool PK_AC = Cfg<NV>::PK_AC, PK_B = Cfg<NV>::PK_B;
  static constexpr size_t F_OFF = size_t(BUF) * sizeof(float2);
  // f of the CTA's planes, rows padded to LD floats (the row pass reads
  // f[pl][b][c] for one c across lanes of consecutive b), unless in tensor memory
  static constexpr size_t ROW_OFF = F_OFF + (F_TM ? 0 : size_t(NPL) * NV * LDF * sizeof(float));
  // the pass's phase row and gain row (3 n complex each), the radial node's sinc row
  // (n = 48: entry m = |k|^2 at m + m / 32; the lanes of a warp gather at
  // |k|^2 values that differ by squares, which fall into few banks without the
  // pad word: 5.5 wavefronts per gather, 2.3 with it.  At n = 64, 8 and 2.7,
  // but the index arithmetic costs more at 255 registers: 87.6 instead of
  // 86.2 ms per Q on 16 cells)
  static constexpr int M1 = 3 * (NV / 2) * (NV / 2) + 1;
  static constexpr bool SLAB_PAD = NV == 48;
  static constexpr int M1P = SLAB_PAD ? M1 + M1 / 32 + 1 : M1;
  __host__ __device__ static constexpr int slab_at(int m) { return SLAB_PAD ? m + (m >> 5) : m; }
  static constexpr size_t SLAB_OFF = ROW_OFF + size_t(6 * NV) * sizeof(float2);
  static constexpr size_t BAR_OFF = (SLAB_OFF + size_t(M1P) * sizeof(float) + 15) / 16 * 16;
  static constexpr int WARPS = THREADS / 32;
  static constexpr int REGIONS = (WARPS + 3) / 4;  // column groups of 2 n tensor-memory columns
  static constexpr int TCOLS_USED = REGIONS * 2 * NV;
  // then the f rows of the plane lines (F_TM): column FCOL0 + (warp / 4) n
  static constexpr int FCOL0 = TCOLS_USED;
  static constexpr int TCOLS_F = TCOLS_USED + (F_TM ? REGIONS * NV : 0);
  // then (where they fit) each column's spectrum: region (warp / 4) of 2 n columns
  static constexpr int TCOLS_ALL = TCOLS_F + TCOLS_USED;
  static constexpr int TCOLS = TCOLS_ALL <= 32    ? 32
                               : TCOLS_ALL <= 64  ? 64
                               : TCOLS_ALL <= 128 ? 128
                               : TCOLS_ALL <= 256 ? 256
                                                  : 512;
  static constexpr int SCOL0 = TCOLS_F;
  static constexpr int CHUNKS = 2 * NV / 16;  // 16-column tensor-memory chunks of a thread's sum
  // warps from FW0 on find no tensor-memory region for their columns' spectra;
  // the next SMW keep them in shared memory, [a][lane] per warp, as many as
  // fit, and the rest read them from L2 every pass
  static constexpr int FW0_ = (TCOLS - TCOLS_F) / (2 * NV) * 4;
  static constexpr int FW0 = FW0_ < WARPS ? FW0_ : WARPS;
  static constexpr size_t FSM_OFF = BAR_OFF + 16 + 16;  // after two mbarriers and the tensor-memory slot
  static constexpr size_t SMEM_MAX = 227 * 1024;
  static constexpr int SMW_FIT = int((SMEM_MAX - FSM_OFF) / (32 * NV * sizeof(float2)));
  static constexpr int SMW = WARPS - FW0 < SMW_FIT ? WARPS - FW0 : SMW_FIT;
  static constexpr size_t SMEM = FSM_OFF + size_t(SMW) * 32 * NV * sizeof(float2);
  static_assert(THREADS % 32 == 0 && NV % CS == 0 && TCOLS_F <= 512 && (2 * NV) % 16 == 0, "launch shape");
  static_assert(CS == 1 || (NPL % 2 == 0 && LD % 2 == 0 && NCOL % 2 == 0 && NV % 2 == 0), "16-byte exchange pairs");
  static_assert(SMEM <= SMEM_MAX && FSM_OFF <= SMEM_MAX, "shared memory of one CTA");
};
}  // namespace gfu

struct FusedArgs {
  const float2* fhat;    // [cells][N3] spectra of f
  const float* fT;       // [cells][N3] f in FP32
  const float2* ephase;  // [Q][3][n]
  const float2* gphase;  // [sets][Q][3][n]
  const float* gsinc;    // [sets][n_r][M + 1]
  int64_t gph_stride, gs_stride;
  int M, ns, QP;
  const int* reps;  // packed: the representative pair of each pass
  int64_t cells;
  float2* part;  // [clusters + cells][N3]: the gain sums of each (cluster, cell) segment
  int* err;      // mapped stall word: 3 if an exchange wait gave up
  uint32_t wait_limit;
  int withhold;  // test hook: issue no exchange stores and no expected bytes, so every exchange wait runs out
};

__device__ __forceinline__ uint32_t fz_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t fz_map(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void fz_st_async4(uint32_t addr, float4 v, uint32_t mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(addr),
               "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ float2 fz_xor1(float2 v) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, 1), __shfl_xor_sync(0xffffffffu, v.y, 1));
}
// a lane pair (columns c, c + 1 of one line set, c even) turns its values
// a0, a1 of two planes m, m + 1 into one 16-byte pair per lane: the even lane
// returns plane m's elements at columns (c, c + 1), the odd lane plane m + 1's
__device__ __forceinline__ float4 fz_pair(float2 a0, float2 a1, bool odd) {
  const float2 w = fz_xor1(odd ? a0 : a1);
  return odd ? make_float4(w.x, w.y, a1.x, a1.y) : make_float4(a0.x, a0.y, w.x, w.y);
}
// waits (bounded) for phase `parity` of a barrier whose bytes other CTAs deliver
__device__ __forceinline__ bool fz_wait_bar(uint64_t* mbar, uint32_t parity, uint32_t limit) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(mbar));
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void fz_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void fz_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

template <int NV, bool PACK>
__global__ void __launch_bounds__(gfu::Geo<NV>::THREADS, 1) k_gain_fused(FusedArgs a) {
  using G = gfu::Geo<NV>;
  constexpr int CS = G::CS, NPL = G::NPL, NCOL = G::NCOL, LD = G::LD, N2 = G::N2, N3 = G::N3, H = NV / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* buf = reinterpret_cast<float2*>(smem_raw);
  float* fS = reinterpret_cast<float*>(smem_raw + G::F_OFF);
  float2* erow = reinterpret_cast<float2*>(smem_raw + G::ROW_OFF);  // phase row of the current pass
  float2* grow = erow + 3 * NV;                                      // gain row
  float* slab = reinterpret_cast<float*>(smem_raw + G::SLAB_OFF);    // sinc row of the radial node
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + G::BAR_OFF);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + G::BAR_OFF + 16);
  const int t = threadIdx.x, warp = t >> 5;
  const int rank = CS > 1 ? int(fz_rank()) : 0;
  const int cl = int(blockIdx.x) / CS, ncl = int(gridDim.x) / CS;
  if (warp == 0) {
    tm_alloc(tslot, G::TCOLS);
    tm_relinquish();
  }
  if (CS > 1 && t == 0) {
    // an exchange's barrier completes when the other CTAs' bytes have landed
    // (thread 0 arrives with their count) and every thread has arrived after
    // its plain stores into the CTA's own buffer
    mbar_init(&bars[0], G::THREADS + 1);  // stage-A exchange
    mbar_init(&bars[1], G::THREADS + 1);  // stage-B exchange
  }
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t treg = tbase + (uint32_t(32 * (warp & 3)) << 16) + uint32_t((warp >> 2) * 2 * NV);
  // the column's spectrum f^(a, j), a < n, for a cell's whole range of
  // passes: in tensor memory where a region is left for the warp, else in
  // shared memory where room is left, else read from L2 every pass
  const bool f_tm = G::FW0 >= G::WARPS || warp < G::FW0;
  const bool f_sm = !f_tm && (G::FW0 + G::SMW >= G::WARPS || warp < G::FW0 + G::SMW);
  const uint32_t freg = tbase + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(G::SCOL0 + (warp >> 2) * 2 * NV);
  float2* fsm = reinterpret_cast<float2*>(smem_raw + G::FSM_OFF) + (f_sm ? (warp - G::FW0) * 32 * NV : 0) + (t & 31);
  // f of the plane line (pl, l) in tensor memory (F_TM)
  const uint32_t frow = tbase + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(G::FCOL0 + (warp >> 2) * NV);
  // stages A and C: this thread's column (jb, jc), jb in the CTA's rows;
  // stage B: plane pl = t / NV of the CTA, line l = t mod NV (the same numbers)
  const int pl = t / NV, l = t - pl * NV;
  const int jb = rank * NPL + pl, jc = l;
  const int j = jb * NV + jc;
  const int kb = kval(jb, NV), kc = kval(jc, NV);
  const int mbc = kb * kb + kc * kc;
  const uint32_t buf_s = static_cast<uint32_t>(__cvta_generic_to_shared(buf));
  const uint32_t bar_s = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
  // bytes one CTA receives from the other CTAs per exchange (its own share it
  // stores itself)
  constexpr uint32_t XBYTES = uint32_t(N3 / CS) * 8 / CS * (CS - 1);
  uint32_t phase = 0;
  bool gave_up = false;
  // the first wait (before the first exchange) also makes sure that every CTA
  // of the cluster runs, with its barriers initialised, before any shared
  // memory of another is written
  if constexpr (CS > 1) fz_arrive();

  const int64_t total = a.cells * a.QP;
  const int64_t w0 = total * cl / ncl, w1 = total * (cl + 1) / ncl;
  int64_t cur = -1, slab_key = -1;
  if (w0 < w1) {  // the first pass's phase row
    const int p0 = PACK ? a.reps[int(w0 % a.QP)] : int(w0 % a.QP);
    for (int e = t; e < 3 * NV; e += G::THREADS) erow[e] = a.ephase[int64_t(p0) * 3 * NV + e];
    __syncthreads();
  }
  auto flush = [&](int64_t cell) {  // the segment's sums -> part[cl + cell][a][j]
    tm_wait_st();
    float2* out = a.part + (int64_t(cl) + cell) * N3 + j;
#pragma unroll
    for (int c = 0; c < G::CHUNKS; ++c) {
      uint32_t r[16];
      tm_ld16(treg + 16 * c, r);
      tm_wait_ld(r);
#pragma unroll
      for (int i = 0; i < 8; ++i) out[int64_t(8 * c + i) * N2] = make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
    }
  };
  for (int64_t w = w0; w < w1; ++w) {
    const int64_t cell = w / a.QP;
    const int ip = int(w - cell * a.QP);
    if (cell != cur) {
      if (cur >= 0) flush(cur);
      uint32_t z[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) z[i] = 0u;
#pragma unroll
      for (int c = 0; c < G::CHUNKS; ++c) tm_st16(treg + 16 * c, z);
      if (f_tm) {  // the column's spectrum, chunk c = a in [8 c, 8 c + 8)
        const float2* fh = a.fhat + cell * N3 + j;
#pragma unroll
        for (int c = 0; c < G::CHUNKS; ++c) {
          uint32_t r[16];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float2 v = fh[int64_t(8 * c + i) * N2];
            r[2 * i] = __float_as_uint(v.x);
            r[2 * i + 1] = __float_as_uint(v.y);
          }
          tm_st16(freg + 16 * c, r);
        }
        tm_wait_st();
      } else if (f_sm) {  // the thread's own entries of its warp's shared-memory copy
        const float2* fh = a.fhat + cell * N3 + j;
#pragma unroll 4
        for (int q = 0; q < NV; ++q) fsm[q * 32] = fh[int64_t(q) * N2];
      }
      // f of the CTA's planes (read in stage B after the exchange barrier below)
      const float* fc = a.fT + cell * N3 + int64_t(rank * NPL) * N2;
      if constexpr (G::F_TM) {  // the thread's plane line, n / 16 chunks of 16 columns
        const float4* fl = reinterpret_cast<const float4*>(fc + (pl * NV + l) * NV);
#pragma unroll
        for (int c = 0; c < NV / 16; ++c) {
          uint32_t r[16];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float4 v = fl[4 * c + i];
            r[4 * i] = __float_as_uint(v.x), r[4 * i + 1] = __float_as_uint(v.y);
            r[4 * i + 2] = __float_as_uint(v.z), r[4 * i + 3] = __float_as_uint(v.w);
          }
          tm_st16(frow + 16 * c, r);
        }
        tm_wait_st();
      } else {
        for (int e = t; e < NPL * N2; e += G::THREADS) {
          const int p2 = e / N2, rem = e - p2 * N2, b = rem / NV, c = rem - b * NV;
          fS[(p2 * NV + b) * G::LDF + c] = fc[e];
        }
      }
      cur = cell;
    }
    const int pair = PACK ? a.reps[ip] : ip;
    float2 x[NV];
    // ---- A: phase product and inverse transform along a of the column
    {
      if (f_tm) {  // two 16-column chunks in flight at a time (the last alone when their count is odd)
        static_for<0, (G::CHUNKS + 1) / 2>([&](auto ci) {
          constexpr int c = 2 * decltype(ci)::value;
          constexpr bool two = c + 1 < G::CHUNKS;
          uint32_t r0[16], r1[16];
          tm_ld16(freg + 16 * c, r0);
          if constexpr (two) tm_ld16(freg + 16 * c + 16, r1);
          tm_wait_ld(r0);
          if constexpr (two) tm_wait_ld(r1);
          static_for<0, 8>([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            x[8 * c + i] = make_float2(__uint_as_float(r0[2 * i]), __uint_as_float(r0[2 * i + 1]));
            if constexpr (two)
              x[8 * c + 8 + i] = make_float2(__uint_as_float(r1[2 * i]), __uint_as_float(r1[2 * i + 1]));
          });
        });
      } else if (f_sm) {
#pragma unroll
        for (int q = 0; q < NV; ++q) x[q] = fsm[q * 32];
      } else {
        const float2* fh = a.fhat + cur * N3 + j;
#pragma unroll
        for (int q = 0; q < NV; ++q) x[q] = fh[int64_t(q) * N2];
      }
      const float2* ep = erow;
      if constexpr (PACK) {
        float cp, cm, th;
        pack_t_consts<float, float2, NV>(ep, jb, jc, cp, cm, th);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          const float2 e = ep[q];
          x[q] = cscale(x[q], q == H ? th : fmaf(e.y, cm, e.x * cp));
        }
      } else {
        const float2 ebc = cmul(ep[NV + jb], ep[2 * NV + jc]);
#pragma unroll
        for (int q = 0; q < NV; ++q) x[q] = cmul(x[q], cmul(ep[q], ebc));
      }
      fft_line<NV, +1, G::PK_AC>(x);
    }
    if constexpr (CS > 1) {
      fz_wait();  // every buffer of the cluster has been read by the previous item's stage C
      if (t == 0 && !a.withhold) mbar_arrive_tx(&bars[0], XBYTES);
      if (!a.withhold) {
        // 16 bytes per store: lanes of columns (jc, jc + 1) pair up their
        // values of planes (m, m + 1)
        const bool odd = (jc & 1) != 0;
        static_for<0, CS>([&](auto ri) {
          constexpr int r = decltype(ri)::value;
          const uint32_t base = fz_map(buf_s, uint32_t(r)), rb = fz_map(bar_s, uint32_t(r));
          static_for<0, NPL / 2>([&](auto mi) {
            constexpr int m0 = 2 * decltype(mi)::value;
            const float4 v = fz_pair(x[pos(NV, r * NPL + m0)], x[pos(NV, r * NPL + m0 + 1)], odd);
            const int e = ((m0 + (odd ? 1 : 0)) * NV + jb) * LD + (jc & ~1);
            if (r == rank)  // the CTA's own planes: plain stores
              *reinterpret_cast<float4*>(buf + e) = v;
            else
              fz_st_async4(base + uint32_t(e * 8), v, rb);
          });
        });
        mbar_arrive(&bars[0]);  // release: this thread's own-plane stores
      }
      // the planes of the CTA are complete once every CTA's elements have landed
      if (!fz_wait_bar(&bars[0], phase, a.wait_limit)) gave_up = true;
    } else {
      __syncthreads();  // the previous item's stage C has read the buffer
      static_for<0, NV>([&](auto qi) {
        constexpr int q = decltype(qi)::value;
        buf[(q * NV + jb) * LD + jc] = x[pos(NV, q)];
      });
      __syncthreads();
    }
    // every thread of the CTA is past this pass's stage A and the previous
    // pass's stage C: copy this pass's gain row, the next pass's phase row and,
    // on a change of radial node (or cell, with one restitution set per cell),
    // the sinc row; complete before the barriers ahead of stages C and A
    {
      const float2* gsrc = a.gphase + cell * a.gph_stride + int64_t(pair) * 3 * NV;
      for (int e = t; e < 3 * NV; e += G::THREADS) cp_async8(grow + e, gsrc + e);
      if (w + 1 < w1) {
        const int ipn = int((w + 1) % a.QP);
        const int pn = PACK ? a.reps[ipn] : ipn;
        for (int e = t; e < 3 * NV; e += G::THREADS) cp_async8(erow + e, a.ephase + int64_t(pn) * 3 * NV + e);
      }
      const int ir = pair / a.ns;
      const int64_t key = a.gs_stride ? cell * 65536 + ir : ir;
      if (key != slab_key) {
        const float* src = a.gsinc + cell * a.gs_stride + int64_t(ir) * (a.M + 1);
        for (int e = t; e < G::M1; e += G::THREADS) cp_async4(slab + G::slab_at(e), src + e);
        slab_key = key;
      }
      cp_async_commit();
    }
    // ---- B: inverse along b (column (pl, l))
    {
      float2* col = buf + pl * NV * LD + l;
#pragma unroll
      for (int b = 0; b < NV; ++b) x[b] = col[b * LD];
      fft_line<NV, +1, G::PK_B>(x);
      static_for<0, NV>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        col[b * LD] = x[pos(NV, b)];
      });
    }
    cp_async_wait_group<0>();  // the rows and the sinc row (read after the next barrier)
    __syncthreads();
    // inverse along c, * f, forward along c (row (pl, l))
    {
      float2* row = buf + (pl * NV + l) * LD;
      if constexpr (G::ROW16) {
        const float4* r4 = reinterpret_cast<const float4*>(row);
#pragma unroll
        for (int c = 0; c < NV / 2; ++c) {
          const float4 v = r4[c];
          x[2 * c] = make_float2(v.x, v.y);
          x[2 * c + 1] = make_float2(v.z, v.w);
        }
      } else {
#pragma unroll
        for (int c = 0; c < NV; ++c) x[c] = row[c];
      }
      fft_line<NV, +1, G::PK_B>(x);
      float2 y[NV];
      if constexpr (G::F_TM) {
        static_for<0, NV / 16>([&](auto ci) {
          constexpr int c = decltype(ci)::value;
          uint32_t r[16];
          tm_ld16(frow + 16 * c, r);
          tm_wait_ld(r);
          static_for<0, 16>([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            y[16 * c + i] = cscale(x[pos(NV, 16 * c + i)], __uint_as_float(r[i]));
          });
        });
      } else {
        const float* fr = fS + (pl * NV + l) * G::LDF;
        static_for<0, NV>([&](auto ci) {
          constexpr int c = decltype(ci)::value;
          y[c] = cscale(x[pos(NV, c)], fr[c]);
        });
      }
      fft_line<NV, -1, G::PK_B>(y);
      if constexpr (G::ROW16) {
        float4* r4 = reinterpret_cast<float4*>(row);
        static_for<0, NV / 2>([&](auto ci) {
          constexpr int c = decltype(ci)::value;
          const float2 a0 = y[pos(NV, 2 * c)], a1 = y[pos(NV, 2 * c + 1)];
          r4[c] = make_float4(a0.x, a0.y, a1.x, a1.y);
        });
      } else {
        static_for<0, NV>([&](auto ci) {
          constexpr int c = decltype(ci)::value;
          row[c] = y[pos(NV, c)];
        });
      }
    }
    __syncthreads();
    // forward along b (column (pl, l)), then to the column owners
    {
      float2* col = buf + pl * NV * LD + l;
#pragma unroll
      for (int b = 0; b < NV; ++b) x[b] = col[b * LD];
      if constexpr (CS > 1) fz_arrive();  // this thread's reads of its planes are done
      fft_line<NV, -1, G::PK_B>(x);
      if constexpr (CS > 1) {
        const int ag = rank * NPL + pl;  // the plane's a
        fz_wait();                       // every CTA has read its planes
        if (t == 0 && !a.withhold) mbar_arrive_tx(&bars[1], XBYTES);
        if (!a.withhold) {
          const bool odd = (l & 1) != 0;
          static_for<0, CS>([&](auto ri) {
            constexpr int r = decltype(ri)::value;
            const uint32_t base = fz_map(buf_s, uint32_t(r)), rb = fz_map(bar_s + 8, uint32_t(r));
            static_for<0, NPL / 2>([&](auto mi) {
              constexpr int m0 = 2 * decltype(mi)::value;
              const float4 v = fz_pair(x[pos(NV, r * NPL + m0)], x[pos(NV, r * NPL + m0 + 1)], odd);
              const int e = ag * NCOL + (m0 + (odd ? 1 : 0)) * NV + (l & ~1);
              if (r == rank)  // the CTA's own columns: plain stores
                *reinterpret_cast<float4*>(buf + e) = v;
              else
                fz_st_async4(base + uint32_t(e * 8), v, rb);
            });
          });
          mbar_arrive(&bars[1]);  // release: this thread's own-column stores
        }
        if (!fz_wait_bar(&bars[1], phase, a.wait_limit)) gave_up = true;  // the CTA's columns have landed
        phase ^= 1;
      } else {
        static_for<0, NV>([&](auto bi) {
          constexpr int b = decltype(bi)::value;
          col[b * LD] = x[pos(NV, b)];
        });
        __syncthreads();
      }
    }
    // ---- C: forward along a of the column, * gain, summed in tensor memory
    {
      if constexpr (CS > 1) {
#pragma unroll
        for (int q = 0; q < NV; ++q) x[q] = buf[q * NCOL + t];
        fz_arrive();  // read: the next item may overwrite the buffer
      } else {
#pragma unroll
        for (int q = 0; q < NV; ++q) x[q] = buf[(q * NV + jb) * LD + jc];
      }
      fft_line<NV, -1, G::PK_AC>(x);
      const float2* gp = grow;
      auto gs = [&](int kk) {
        return slab[G::slab_at(mbc + kk)];
      };
      float2 v[NV];
      if constexpr (PACK) {
        float dp, dm, sh;
        pack_s_consts<float, float2, NV>(gp, jb, jc, dp, dm, sh);
        static_for<0, NV>([&](auto qi) {
          constexpr int q = decltype(qi)::value;
          constexpr int kq = kval(q, NV);
          const float2 g = gp[q];
          const float sv = q == H ? sh : fmaf(-g.y, dm, g.x * dp);
          v[q] = cscale(x[pos(NV, q)], 2.f * sv * gs(kq * kq));
        });
      } else {
        const float2 gbc = cmul(gp[NV + jb], gp[2 * NV + jc]);
        static_for<0, NV>([&](auto qi) {
          constexpr int q = decltype(qi)::value;
          constexpr int kq = kval(q, NV);
          v[q] = cmul(x[pos(NV, q)], cscale(cmul(gp[q], gbc), gs(kq * kq)));
        });
      }
      tm_wait_st();
      static_for<0, G::CHUNKS>([&](auto ci) {
        constexpr int c = decltype(ci)::value;
        uint32_t r[16];
        tm_ld16(treg + 16 * c, r);
        tm_wait_ld(r);
        static_for<0, 8>([&](auto ii) {
          constexpr int i = decltype(ii)::value;
          r[2 * i] = __float_as_uint(__uint_as_float(r[2 * i]) + v[8 * c + i].x);
          r[2 * i + 1] = __float_as_uint(__uint_as_float(r[2 * i + 1]) + v[8 * c + i].y);
        });
        tm_st16(treg + 16 * c, r);
      });
    }
  }
  if (cur >= 0) flush(cur);
  if constexpr (CS > 1) fz_wait();  // matches the last arrive; no CTA leaves while others may still write to it
  if (gave_up) atomicMax(a.err, 3);
  tm_wait_st();
  tm_fence_before();
  __syncthreads();
  if (warp == 0) {
    tm_fence_after();
    tm_dealloc(tbase, G::TCOLS);
  }
}

// G[cell] = the sum of the parts of the clusters whose ranges meet the cell
__global__ void __launch_bounds__(256) k_fused_expand(float2* G, const float2* part, int64_t cells, int QP, int ncl,
                                                      int64_t N3) {
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * N3) return;
  const int64_t cell = gid / N3, e = gid - cell * N3;
  const int64_t total = cells * QP, lo = cell * QP, hi = lo + QP;
  float2 s = make_float2(0.f, 0.f);
  for (int64_t c = lo * ncl / total; c < ncl; ++c) {
    const int64_t r0 = total * c / ncl, r1 = total * (c + 1) / ncl;
    if (r0 >= hi) break;
    if (r1 <= lo) continue;
    const float2 v = part[(c + cell) * N3 + e];
    s.x += v.x, s.y += v.y;
  }
  G[gid] = s;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int NV, bool PACK>
static int fused_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr, int clusters, cudaStream_t s) {
  using G = gfu::Geo<NV>;
  cfg = {};
  cfg.gridDim = dim3(unsigned(clusters * G::CS), 1, 1);
  cfg.blockDim = dim3(G::THREADS, 1, 1);
  cfg.dynamicSmemBytes = G::SMEM;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G::CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return PII_OK;
}

template <int NV, bool PACK>
static int fused_setup(int* clusters) {
  using G = gfu::Geo<NV>;
  PII_CUDA(cudaFuncSetAttribute(k_gain_fused<NV, PACK>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(G::SMEM)));
  if (G::CS > 8) PII_CUDA(cudaFuncSetAttribute(k_gain_fused<NV, PACK>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if (G::CS == 1) {  // single-CTA items: every resident CTA of every SM
    int per_sm = 0, sms = 0, dev = 0;
    PII_CUDA(cudaGetDevice(&dev));
    PII_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PII_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gain_fused<NV, PACK>, G::THREADS, G::SMEM));
    *clusters = per_sm * sms;
    return PII_OK;
  }
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  fused_config<NV, PACK>(cfg, attr, 1, nullptr);
  PII_CUDA(cudaOccupancyMaxActiveClusters(clusters, k_gain_fused<NV, PACK>, &cfg));
  return PII_OK;
}

template <int NV>
static int fused_prepare_t(pii_plan* p) {
  if (p->tab.M + 1 != gfu::Geo<NV>::M1) return PII_OK;  // the sinc row size the kernel stages
  int c1 = 0, c2 = 0;
  PII_TRY((fused_setup<NV, true>(&c1)));
  PII_TRY((fused_setup<NV, false>(&c2)));
  const int clusters = std::min(c1, c2);
  if (clusters < 1) return PII_OK;  // no cluster of this shape fits: the pipeline stays in use
  p->fz_clusters = clusters;  // the segment sums are allocated when the path is first chosen
  p->fz_sms = clusters * gfu::Geo<NV>::CS * (gfu::Geo<NV>::CS == 1 ? 0 : 1);  // CS = 1: the grid fills every SM
  if (!p->dft_err_host) {  // the mapped stall word (shared with the tensor-core column passes)
    PII_CUDA(cudaHostAlloc(&p->dft_err_host, sizeof(int), cudaHostAllocMapped));
    *p->dft_err_host = 0;
    PII_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&p->dft_err), p->dft_err_host, 0));
  }
  return PII_OK;
}

// the per-(cluster, cell) segment sums of the fused path, allocated on first use
int gain_fused_ensure(pii_plan* p) {
  if (p->fz_part || p->fz_clusters < 1) return PII_OK;
  const size_t bytes = size_t(p->fz_clusters + p->batch_max) * size_t(p->N) * sizeof(float2);
  PII_CUDA(cudaSetDevice(p->device));
  PII_CUDA(cudaMalloc(&p->fz_part, bytes));
  p->bytes += int64_t(bytes);
  return PII_OK;
}

int gain_fused_prepare(pii_plan* p) {
  if (p->precision != PII_PREC_FP32 || p->dim != 3) return PII_OK;
  switch (p->n) {
    case 16: return fused_prepare_t<16>(p);
    case 24: return fused_prepare_t<24>(p);
    case 48: return fused_prepare_t<48>(p);
    case 64: return fused_prepare_t<64>(p);
    default: return PII_OK;
  }
}

template <int NV>
static int fused_run_t(pii_plan* p, int64_t cells, cudaStream_t s) {
  using G = gfu::Geo<NV>;
  const bool packed = p->ap_count > 0;
  FusedArgs a{};
  a.fhat = static_cast<const float2*>(p->fhat);
  a.fT = static_cast<const float*>(p->fT);
  a.ephase = static_cast<const float2*>(p->tab.ephase);
  a.gphase = static_cast<const float2*>(p->tab.gphase);
  a.gsinc = static_cast<const float*>(p->tab.gsinc);
  a.gph_stride = p->tab.gph_stride;
  a.gs_stride = p->tab.gs_stride;
  a.M = p->tab.M;
  a.ns = p->ns;
  a.QP = packed ? p->ap_count : p->Q;
  a.reps = p->ap_reps;
  a.cells = cells;
  a.part = static_cast<float2*>(p->fz_part);
  a.err = p->dft_err;
  a.wait_limit = p->dft_wait_limit;
  a.withhold = p->dft_withhold;
  const int clusters = int(std::min<int64_t>(p->fz_clusters, cells * a.QP));
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  {
    StageTimer st(p, ST_GAIN_FUSED, s);
    cudaError_t e;
    if (packed) {
      fused_config<NV, true>(cfg, attr, clusters, s);
      e = cudaLaunchKernelEx(&cfg, k_gain_fused<NV, true>, a);
    } else {
      fused_config<NV, false>(cfg, attr, clusters, s);
      e = cudaLaunchKernelEx(&cfg, k_gain_fused<NV, false>, a);
    }
    if (e != cudaSuccess) {
      set_error("k_gain_fused launch: %s", cudaGetErrorString(e));
      return PII_ERR_CUDA;
    }
    k_fused_expand<<<unsigned((cells * G::N3 + 255) / 256), 256, 0, s>>>(static_cast<float2*>(p->G), a.part, cells,
                                                                        a.QP, clusters, G::N3);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

int gain_fused_run(pii_plan* p, int64_t cells, cudaStream_t s) {
  if (!p->fz_part || p->fz_clusters < 1) {
    set_error("gain_fused_run: the plan has no fused gain kernel");
    return PII_ERR_ARG;
  }
  switch (p->n) {
    case 16: return fused_run_t<16>(p, cells, s);
    case 24: return fused_run_t<24>(p, cells, s);
    case 48: return fused_run_t<48>(p, cells, s);
    case 64: return fused_run_t<64>(p, cells, s);
    default:
      set_error("gain_fused_run: no fused gain kernel for n = %d", p->n);
      return PII_ERR_ARG;
  }
}

}  // namespace pii
