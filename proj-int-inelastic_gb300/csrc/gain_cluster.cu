// Fused gain term of Q(f,f) for n = 32 in FP32: one kernel, every quadrature
// pair's 3D transforms on chip.
//
// A 2-CTA thread-block cluster owns one (cell, range of quadrature pairs).
// CTA r (r = 0, 1) holds the a-planes [16 r, 16 r + 16) of the 32^3 work grid
// in 132 KB of shared memory (rows padded: element (b, c) of a plane sits at
// b * 33 + c, conflict-free for row and column access).  Per pair
// (src/collision/inelastic_collisions.py:212-217):
//   A  column pass: P = exp_rs(k) f^ (per-axis phase rows), full 32-point
//      inverse transform along a for the CTA's columns; keep the CTA's planes
//      (the transform is duplicated in both CTAs, so no exchange is needed).
//   B  plane pass, one warp per plane: IFFT_c, IFFT_b, * f, FFT_b, FFT_c.
//   C  forward transform along a split radix-2 across the pair: CTA 0 makes
//      the even k_a from M(a) + M(a + 16), CTA 1 the odd k_a from
//      (M(a) - M(a + 16)) W^a, reading the peer's planes through distributed
//      shared memory; then multiply by gain_rs(k) and accumulate.
// Only Re IFFT3(G) is ever used, so the accumulator keeps the Hermitian part
// H(k) = (G(k) + conj G(-k)) / 2 on half of k-space: each thread owns a column
// pair {(b, c), (-b, -c)} (or two self-conjugate columns, handled by the same
// instructions with a 0/1 weight so that no warp diverges), 16 k_a values of
// its CTA's parity -> 514 slots x 16 x 8 bytes = 64 KB of shared memory.
// Measured on GB300 (per-warp clock64 stamps), a pair costs ~37K cycles per
// CTA: stage A ~9.5K, B ~12.7K, C ~8-12K (the distributed-shared-memory loads
// dominate it: ~17 B/clk/SM), the two cluster barriers the rest.  At the
// end of a work item the CTA writes its slots to a per-part buffer; a small
// kernel sums the parts and expands H to the full spectrum G for the existing
// final inverse transform.
#include <cooperative_groups.h>

#include <algorithm>

#include "gain_common.cuh"

namespace cg = cooperative_groups;

namespace pii {

namespace gc {
constexpr size_t SMEM = size_t(PLANES) * PSTR * sizeof(float2) + size_t(16) * HSLOTS * sizeof(float2);
// index of k_a = -(2 m + par) within the parity half
__host__ __device__ constexpr int neg_m(int m, int par) { return par == 0 ? ((16 - m) & 15) : (15 - m); }
}  // namespace gc

struct GainClusterArgs {
  const float2* fhat;    // [cells][N3] spectra of f
  const float* fT;       // [cells][N3] f in FP32
  const float2* ephase;  // [Q][3][32]
  const float2* gphase;  // [Q][3][32]
  const float* gsinc;    // [n_r][M + 1]
  int M, ns, Q;
  int64_t cells;
  int parts;        // work items per cell
  float2* hpart;    // [cells * parts][2][16][HSLOTS]
  const int4* ucols;  // [THREADS] (column, column, first slot, 1 if two self-conjugate columns)
};

// stage A for one column j: full inverse transform along a, keep this CTA's planes
template <int PAR>
__device__ __forceinline__ void stage_a(float2* W, const float2* fh, const float2* ep, int j) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  const float2 ebc = cmul(ep[32 + jb], ep[64 + jc]);
  float2 x[32];
#pragma unroll
  for (int a = 0; a < 32; ++a) x[a] = cmul(fh[a * N2 + j], cmul(ep[a], ebc));
  fft_line<32, +1>(x);
  static_for<0, 16>([&](auto ai) {
    constexpr int a = decltype(ai)::value;
    W[widx(a, jb, jc)] = x[pos(32, a + 16 * PAR)];
  });
}

// stage C for one column: this CTA's 16 k_a of the forward transform along a, times the gain
template <int PAR>
__device__ __forceinline__ void stage_c_col(const float2* W, const float2* Wp, int j, const float2* gp,
                                            const float* gs, float2 (&X)[16]) {
  using namespace gc;
  const int jb = j >> 5, jc = j & 31;
  float2 x[16];
#pragma unroll
  for (int a = 0; a < 16; ++a) {
    const float2 own = W[widx(a, jb, jc)];
    const float2 oth = Wp[widx(a, jb, jc)];
    x[a] = PAR == 0 ? cadd(own, oth) : csub(oth, own);  // CTA 1 holds the upper half
  }
  if constexpr (PAR == 1) {
    static_for<1, 16>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      x[a] = twiddle<a, 32, -1>(x[a]);
    });
  }
  fft_line<16, -1>(x);
  const int kb = kval(jb, 32), kc = kval(jc, 32);
  const int mbc = kb * kb + kc * kc;
  const float2 gbc = cmul(gp[32 + jb], gp[64 + jc]);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    constexpr int a = 2 * m + PAR;  // storage index of k_a
    constexpr int ka = kval(a, 32);
    const float2 g = cscale(cmul(gp[a], gbc), gs[mbc + ka * ka]);
    X[m] = cmul(x[pos(16, m)], g);
  });
}

// Every thread runs the same code: a column pair {j, -j} accumulates
//   H(k_a, j) += X_j(k_a) + conj X_{-j}(-k_a)            (one slot),
// two self-conjugate columns j0, j1 accumulate
//   H(k_a, j_i) += X_{j_i}(k_a) + conj X_{j_i}(-k_a)     (slots z, z + 1),
// selected by the 0 / 1 weight sc without divergence.
template <int PAR>
__device__ __forceinline__ void stage_c(const float2* W, const float2* Wp, float2* H, int4 uc,
                                        const float2* gp, const float* gs) {
  using namespace gc;
  const float sc = float(uc.w);
  const int z0 = uc.z, z1 = uc.z + uc.w;
  float2 X[16];
  stage_c_col<PAR>(W, Wp, uc.x, gp, gs, X);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    constexpr int mm = neg_m(m, PAR);
    float2 h = H[m * HSLOTS + z0];
    h.x += X[m].x + sc * X[mm].x;
    h.y += X[m].y - sc * X[mm].y;
    H[m * HSLOTS + z0] = h;
  });
  stage_c_col<PAR>(W, Wp, uc.y, gp, gs, X);
  static_for<0, 16>([&](auto mi) {
    constexpr int m = decltype(mi)::value;
    constexpr int mm = neg_m(m, PAR);
    float2 h = H[m * HSLOTS + z1];
    h.x += X[mm].x + sc * X[m].x;
    h.y += sc * X[m].y - X[mm].y;
    H[m * HSLOTS + z1] = h;
  });
}

__global__ void __launch_bounds__(gc::THREADS, 1) k_gain_cluster(GainClusterArgs a) {
  using namespace gc;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* W = reinterpret_cast<float2*>(smem_raw);
  float2* H = W + PLANES * PSTR;
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = int(cluster.block_rank());
  const float2* Wp = cluster.map_shared_rank(W, crank ^ 1);
  const int64_t cid = blockIdx.x >> 1;
  const int64_t nclus = gridDim.x >> 1;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int64_t items = a.cells * a.parts;
  const int per_part = (a.Q + a.parts - 1) / a.parts;
  const int4 uc = a.ucols[t];
  const int nslot = 1 + uc.w;
  const int slot0 = uc.z;

  for (int64_t it = cid; it < items; it += nclus) {
    const int64_t cell = it / a.parts;
    const int part = int(it - cell * a.parts);
    const int p0 = part * per_part;
    const int p1 = min(a.Q, p0 + per_part);
#pragma unroll
    for (int m = 0; m < 16; ++m)
      for (int s = 0; s < nslot; ++s) H[m * HSLOTS + slot0 + s] = make_float2(0.f, 0.f);
    const float2* fh = a.fhat + cell * N3;
    const float* fr = a.fT + cell * N3 + int64_t(16 * crank + warp) * N2 + lane;  // f[cell][a][b][c = lane]

    for (int p = p0; p < p1; ++p) {
      const float2* ep = a.ephase + int64_t(p) * 96;
      const float2* gp = a.gphase + int64_t(p) * 96;
      const float* gs = a.gsinc + int64_t(p / a.ns) * (a.M + 1);
      // ---- A: columns t and t + 512
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        if (crank == 0)
          stage_a<0>(W, fh, ep, t + 512 * h);
        else
          stage_a<1>(W, fh, ep, t + 512 * h);
      }
      __syncthreads();
      // ---- B: warp `warp` owns plane `warp`; lane = row / column index
      plane_pass(W + warp * PSTR, fr, lane);
      cluster.sync();  // both CTAs' planes are final for this pair
      // ---- C
      if (crank == 0)
        stage_c<0>(W, Wp, H, uc, gp, gs);
      else
        stage_c<1>(W, Wp, H, uc, gp, gs);
      cluster.sync();  // the peer has finished reading this CTA's planes
    }
    // ---- write this CTA's Hermitian slots (x 1/2) for the work item
    float2* out = a.hpart + ((it * 2 + crank) * 16) * HSLOTS;
#pragma unroll
    for (int m = 0; m < 16; ++m)
      for (int s = 0; s < nslot; ++s) {
        const float2 h = H[m * HSLOTS + slot0 + s];
        out[m * HSLOTS + slot0 + s] = make_float2(0.5f * h.x, 0.5f * h.y);
      }
  }
}

// G[cell][a][j] = sum over parts of the Hermitian slots, expanded to all k
__global__ void __launch_bounds__(256) k_herm_expand(float2* G, const float2* hpart, const int2* colslot,
                                                      int64_t cells, int parts) {
  using namespace gc;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * N3) return;
  const int64_t cell = gid / N3;
  const int e = int(gid - cell * N3);
  const int a = e >> 10, j = e & 1023;
  const int par = a & 1, m = a >> 1;
  const int2 cs = colslot[j];  // (slot, kind): 0 representative, 1 negated partner, 2 self-conjugate
  const int mm = cs.y == 1 ? neg_m(m, par) : m;
  float2 s = make_float2(0.f, 0.f);
  for (int p = 0; p < parts; ++p) {
    const float2 h = hpart[(((cell * parts + p) * 2 + par) * 16 + mm) * HSLOTS + cs.x];
    s.x += h.x;
    s.y += h.y;
  }
  if (cs.y == 1) s.y = -s.y;
  G[gid] = s;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
bool gc::build_column_map(std::vector<int4>& uc, std::vector<int2>& cs) {
  using namespace gc;
  uc.assign(THREADS, make_int4(0, 0, 0, 0));
  cs.assign(N2, make_int2(-1, -1));
  int slot = 0;
  auto pair_unit = [&](int t, int j) {
    const int nj = neg_col(j);
    uc[t] = make_int4(j, nj, slot, 0);
    cs[j] = make_int2(slot, 0);
    cs[nj] = make_int2(slot, 1);
    ++slot;
  };
  for (int t = 0; t < 480; ++t) pair_unit(t, (1 + t / 32) * 32 + (t % 32));
  for (int t = 480; t < 495; ++t) pair_unit(t, 0 * 32 + (t - 479));   // row 0, columns 1..15
  for (int t = 496; t < 511; ++t) pair_unit(t, 16 * 32 + (t - 495));  // row 16, columns 1..15
  const int selfc[4] = {0 * 32 + 0, 0 * 32 + 16, 16 * 32 + 0, 16 * 32 + 16};
  for (int k = 0; k < 2; ++k) {
    const int t = k == 0 ? 495 : 511;
    uc[t] = make_int4(selfc[2 * k], selfc[2 * k + 1], slot, 1);
    cs[selfc[2 * k]] = make_int2(slot, 2);
    cs[selfc[2 * k + 1]] = make_int2(slot + 1, 2);
    slot += 2;
  }
  for (int j = 0; j < N2; ++j)
    if (cs[j].x < 0) return false;
  return slot == HSLOTS;
}

int gain_cluster_prepare(pii_plan* p) {
  using namespace gc;
  PII_CUDA(cudaFuncSetAttribute(k_gain_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM)));
  std::vector<int4> uc;
  std::vector<int2> cs;
  if (!build_column_map(uc, cs)) {
    set_error("gain_cluster_prepare: column map does not cover the %d columns", N2);
    return PII_ERR_ARG;
  }
  void* d = nullptr;
  const size_t maps = THREADS * sizeof(int4) + N2 * sizeof(int2);
  PII_CUDA(cudaMalloc(&d, maps));
  p->bytes += int64_t(maps);
  p->gc_maps = d;
  PII_CUDA(cudaMemcpy(d, uc.data(), THREADS * sizeof(int4), cudaMemcpyHostToDevice));
  PII_CUDA(cudaMemcpy(static_cast<char*>(d) + THREADS * sizeof(int4), cs.data(), N2 * sizeof(int2),
                      cudaMemcpyHostToDevice));
  // clusters that fit at once
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(2, 1, 1);
  cfg.blockDim = dim3(THREADS, 1, 1);
  cfg.dynamicSmemBytes = SMEM;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclus = 0;
  PII_CUDA(cudaOccupancyMaxActiveClusters(&nclus, k_gain_cluster, &cfg));
  if (nclus < 1) {
    set_error("gain_cluster_prepare: no 2-CTA cluster fits (%zu bytes of shared memory)", SMEM);
    return PII_ERR_CUDA;
  }
  p->gc_clusters = nclus;
  // per-part Hermitian slots: at most (8 * clusters + batch_max) work items, and
  // never more than batch_max cells x Q / 8 parts
  const int64_t max_items =
      std::min<int64_t>(int64_t(8) * nclus + p->batch_max, p->batch_max * std::max(1, p->Q / 8));
  PII_CUDA(cudaMalloc(&p->gc_hpart, size_t(max_items) * 2 * 16 * HSLOTS * sizeof(float2)));
  p->bytes += max_items * 2 * 16 * HSLOTS * int64_t(sizeof(float2));
  p->gc_max_items = max_items;
  return PII_OK;
}

int gain_cluster_run(pii_plan* p, int64_t cells, cudaStream_t s) {
  using namespace gc;
  const int nclus = p->gc_clusters;
  int parts = int(std::max<int64_t>(1, (int64_t(p->gc_items_per_cluster) * nclus + cells - 1) / cells));
  parts = std::min(parts, std::max(1, p->Q / 8));
  while (cells * parts > p->gc_max_items && parts > 1) --parts;
  parts = (p->Q + (p->Q + parts - 1) / parts - 1) / ((p->Q + parts - 1) / parts);  // no empty parts
  if (cells * parts > p->gc_max_items) {
    set_error("gain_cluster_run: %lld cells beyond the plan's capacity", (long long)cells);
    return PII_ERR_SIZE;
  }
  GainClusterArgs a{};
  a.fhat = static_cast<const float2*>(p->fhat);
  a.fT = static_cast<const float*>(p->fT);
  a.ephase = static_cast<const float2*>(p->tab.ephase);
  a.gphase = static_cast<const float2*>(p->tab.gphase);
  a.gsinc = static_cast<const float*>(p->tab.gsinc);
  a.M = p->tab.M;
  a.ns = p->ns;
  a.Q = p->Q;
  a.cells = cells;
  a.parts = parts;
  a.hpart = static_cast<float2*>(p->gc_hpart);
  a.ucols = static_cast<const int4*>(p->gc_maps);
  const int64_t items = cells * parts;
  const int64_t grid_clusters = std::min<int64_t>(items, nclus);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(unsigned(2 * grid_clusters), 1, 1);
  cfg.blockDim = dim3(THREADS, 1, 1);
  cfg.dynamicSmemBytes = SMEM;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  {
    StageTimer st(p, ST_GAIN_CLUSTER, s);
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_gain_cluster, a);
    if (e != cudaSuccess) {
      set_error("k_gain_cluster launch: %s", cudaGetErrorString(e));
      return PII_ERR_CUDA;
    }
  }
  PII_CHECK_LAUNCH();
  {
    StageTimer st(p, ST_REDUCE, s);
    k_herm_expand<<<unsigned((cells * N3 + 255) / 256), 256, 0, s>>>(
        static_cast<float2*>(p->G), a.hpart,
        reinterpret_cast<const int2*>(static_cast<const char*>(p->gc_maps) + THREADS * sizeof(int4)), cells, parts);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii
