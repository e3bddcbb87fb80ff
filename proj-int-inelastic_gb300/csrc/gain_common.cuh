// Pieces shared by the two fused n = 32 FP32 gain kernels (gain_cluster.cu,
// gain_parity.cu): the padded plane layout, the per-plane pass and the
// thread -> column-pair map of the Hermitian accumulator.
#pragma once
#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {
namespace gc {
constexpr int NV = 32, N2 = 1024, N3 = 32768;
constexpr int THREADS = 512;
constexpr int PLANES = 16;
constexpr int HSLOTS = 514;

// column (b, c) -> column (-b, -c), both as storage indices b * 32 + c
__host__ __device__ constexpr int neg_col(int j) {
  return (((NV - (j >> 5)) & 31) << 5) | ((NV - (j & 31)) & 31);
}
// element (b, c) of plane `plane`: rows padded to 33 elements, so that row
// and column accesses of a warp are both free of bank conflicts and every
// element of a line sits at a constant offset from the line's start
constexpr int RSTR = 33, PSTR = 32 * RSTR;  // row and plane strides (complex elements)
__device__ __forceinline__ int widx(int plane, int b, int c) { return plane * PSTR + b * RSTR + c; }

// One warp transforms one 32 x 32 plane in place (src/collision/
// inelastic_collisions.py:212-214 restricted to the plane's two axes):
//   IFFT_c, IFFT_b, multiply by f(a, b, c), FFT_b, FFT_c.
// F_ROW = false: `fr` points at f[a][0][lane] in global memory (row stride 32);
// F_ROW = true: `fr` points at this lane's 32 values f[a][0..31][lane],
// contiguous and 16-byte aligned (shared memory).
template <bool F_ROW = false, bool PK = false>
__device__ __forceinline__ void plane_pass(float2* P, const float* fr, int lane) {
  float2 x[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) x[c] = P[lane * RSTR + c];
  fft_line<32, +1, PK>(x);
  static_for<0, 32>([&](auto ci) {
    constexpr int c = decltype(ci)::value;
    P[lane * RSTR + c] = x[pos(32, c)];
  });
  __syncwarp();
#pragma unroll
  for (int b = 0; b < 32; ++b) x[b] = P[b * RSTR + lane];
  fft_line<32, +1, PK>(x);
  float2 y[32];
  if constexpr (F_ROW) {
    static_for<0, 8>([&](auto qi) {
      constexpr int q = decltype(qi)::value;
      const float4 fv = reinterpret_cast<const float4*>(fr)[q];
      y[4 * q] = cscale(x[pos(32, 4 * q)], fv.x);
      y[4 * q + 1] = cscale(x[pos(32, 4 * q + 1)], fv.y);
      y[4 * q + 2] = cscale(x[pos(32, 4 * q + 2)], fv.z);
      y[4 * q + 3] = cscale(x[pos(32, 4 * q + 3)], fv.w);
    });
  } else {
    static_for<0, 32>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      y[b] = cscale(x[pos(32, b)], fr[b * 32]);
    });
  }
  fft_line<32, -1, PK>(y);
  static_for<0, 32>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    P[k * RSTR + lane] = y[pos(32, k)];
  });
  __syncwarp();
#pragma unroll
  for (int c = 0; c < 32; ++c) x[c] = P[lane * RSTR + c];
  fft_line<32, -1, PK>(x);
  static_for<0, 32>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    P[lane * RSTR + k] = x[pos(32, k)];
  });
}

// Thread -> column pairs of the Hermitian accumulator: each thread owns a
// column pair {j, -j} (one slot) or two self-conjugate columns (two slots).
// Warps 0..14 take rows 1..15 (every column); warp 15 takes rows 0 and 16, one
// row per half-warp, so that its shared-memory accesses are conflict-free like
// the other warps'.  ucols[t] = (column, column, first slot, 1 if two
// self-conjugate columns); colslot[j] = (slot, kind) with kind 0 for the
// representative of a pair, 1 for its negated partner, 2 for a self-conjugate
// column.  Returns false if the map does not cover every column exactly once.
bool build_column_map(std::vector<int4>& uc, std::vector<int2>& cs);
}  // namespace gc
}  // namespace pii
