// The fast-spectral operator in 2D velocity (config["collision-model"]["dim"]
// = 2, the J_0 kernel on a circle quadrature), templated on the working
// precision T and the grid size NV.
//
// A cell's grid is one NV x NV plane [b][c] (c fastest, b = first velocity
// axis).  Every 2D transform is a plane pass: NV threads own one plane, each
// transforms a row along c in registers, the plane is transposed through
// padded shared memory and each thread transforms a column along b.  Per item
// (cell, pair) (src/collision/inelastic_collisions.py:208-218):
//   k2_pair : load exp_rs(k) f^(k) (per-axis phase rows), IFFT_c, IFFT_b, * f,
//             FFT_b, FFT_c, * gain_rs(k)   -> chunk buffer
//   k2_reduce: G[cell] (+)= sum over the chunk's pairs
//   k2_finish: IFFT2 of Y1 = G + heat_bath lapl f^ and Y2 = lossk f^,
//             q = (Re Y1 - f Re Y2) / n^2                         (:218-227)
// with f^ from k2_fwd (FFT_c, FFT_b of f).  The tables are the plan's: phase
// rows 0 (b) and 1 (c) with 1/n^2 folded into row 0, gsinc / lossk built with J_0.
#pragma once
#include <algorithm>

#include "fft_reg.cuh"
#include "pii_internal.cuh"

namespace pii {

template <int NV>
struct Geo2 {
  static constexpr int N2 = NV * NV;
  static constexpr int PPB = (128 / NV) > 0 ? (128 / NV) : 1;  // planes per block
  static constexpr int THREADS = PPB * NV;
  static constexpr int LD = NV + 1;  // padded row stride (complex elements)
};

// thread t of plane g: row pass on row t, then column pass on column t
template <int NV, int DIR, typename V>
__device__ __forceinline__ void row_fft(V* row) {
  V x[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) x[c] = row[c];
  fft_line<NV, DIR>(x);
  static_for<0, NV>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    row[k] = x[pos(NV, k)];
  });
}

template <int NV, int DIR, typename V>
__device__ __forceinline__ void col_fft(V* col, int ld) {
  V x[NV];
#pragma unroll
  for (int b = 0; b < NV; ++b) x[b] = col[b * ld];
  fft_line<NV, DIR>(x);
  static_for<0, NV>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    col[k * ld] = x[pos(NV, k)];
  });
}

// f (FP64) -> fT (precision T) and f^ = FFT2(f)
template <typename T, int NV>
__global__ void __launch_bounds__(Geo2<NV>::THREADS) k2_fwd(const double* f, c2<T>* fhat, T* fT, int64_t cells) {
  using V = c2<T>;
  constexpr int N2 = Geo2<NV>::N2, LD = Geo2<NV>::LD, PPB = Geo2<NV>::PPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  const int64_t P0 = int64_t(blockIdx.x) * PPB;
  const int here = int((cells - P0) < PPB ? (cells - P0) : PPB);
  const int g = threadIdx.x / NV, t = threadIdx.x - g * NV;
  const bool active = g < here;
  for (int e = threadIdx.x; e < here * N2; e += blockDim.x) {
    const double v = f[P0 * N2 + e];
    fT[P0 * N2 + e] = T(v);
    const int gg = e / N2, rem = e - gg * N2;
    S[(gg * NV + rem / NV) * LD + rem % NV] = mk<V>(T(v), T(0));
  }
  __syncthreads();
  if (active) row_fft<NV, -1>(S + (g * NV + t) * LD);
  __syncthreads();
  if (active) col_fft<NV, -1>(S + g * NV * LD + t, LD);
  __syncthreads();
  for (int e = threadIdx.x; e < here * N2; e += blockDim.x) {
    const int gg = e / N2, rem = e - gg * N2;
    fhat[P0 * N2 + e] = S[(gg * NV + rem / NV) * LD + rem % NV];
  }
}

struct Pair2Args {
  const void* fhat;  // [cells][N2]
  const void* fT;    // [cells][N2]
  void* buf;         // [items][N2]
  int64_t c0, np, p0, items;
  int ns;
  Tables tab;
};

// one (cell, pair) item per plane: gain_rs * FFT2(IFFT2(exp_rs f^) * f)
template <typename T, int NV>
__global__ void __launch_bounds__(Geo2<NV>::THREADS) k2_pair(Pair2Args a) {
  using V = c2<T>;
  constexpr int N2 = Geo2<NV>::N2, LD = Geo2<NV>::LD, PPB = Geo2<NV>::PPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  const int64_t P0 = int64_t(blockIdx.x) * PPB;
  const int here = int((a.items - P0) < PPB ? (a.items - P0) : PPB);
  const int g = threadIdx.x / NV, t = threadIdx.x - g * NV;
  const bool active = g < here;
  // load exp_rs(k_b, k_c) f^(k_b, k_c)
  for (int e = threadIdx.x; e < here * N2; e += blockDim.x) {
    const int gg = e / N2, rem = e - gg * N2;
    const int64_t item = P0 + gg;
    const int64_t ci = item / a.np;
    const int64_t pair = a.p0 + (item - ci * a.np);
    const int b = rem / NV, c = rem - b * NV;
    const V* ep = reinterpret_cast<const V*>(a.tab.ephase) + pair * 3 * NV;
    const V fh = reinterpret_cast<const V*>(a.fhat)[(a.c0 + ci) * N2 + rem];
    S[(gg * NV + b) * LD + c] = cmul(fh, cmul(ep[b], ep[NV + c]));
  }
  __syncthreads();
  if (active) row_fft<NV, +1>(S + (g * NV + t) * LD);
  __syncthreads();
  if (active) {
    const int64_t item = P0 + g;
    const int64_t cell = a.c0 + item / a.np;
    const T* fr = reinterpret_cast<const T*>(a.fT) + cell * N2 + t;  // f[cell][b][c = t]
    V* col = S + g * NV * LD + t;
    V x[NV];
#pragma unroll
    for (int b = 0; b < NV; ++b) x[b] = col[b * LD];
    fft_line<NV, +1>(x);
    V y[NV];
    static_for<0, NV>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      y[b] = cscale(x[pos(NV, b)], fr[b * NV]);
    });
    fft_line<NV, -1>(y);
    static_for<0, NV>([&](auto ki) {
      constexpr int k = decltype(ki)::value;
      col[k * LD] = y[pos(NV, k)];
    });
  }
  __syncthreads();
  if (active) {
    // row k_b = t: FFT_c, then * gain(k_b, k_c) and store
    const int64_t item = P0 + g;
    const int64_t ci = item / a.np;
    const int64_t pair = a.p0 + (item - ci * a.np);
    const int ir = int(pair / a.ns);
    const V* gp = reinterpret_cast<const V*>(a.tab.gphase) + pair * 3 * NV;
    const T* gs = reinterpret_cast<const T*>(a.tab.gsinc) + int64_t(ir) * (a.tab.M + 1);
    V* row = S + (g * NV + t) * LD;
    V x[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) x[c] = row[c];
    fft_line<NV, -1>(x);
    const int kb = kval(t, NV);
    const V gb = gp[t];
    V* out = reinterpret_cast<V*>(a.buf) + item * N2 + int64_t(t) * NV;
    static_for<0, NV>([&](auto ci2) {
      constexpr int c = decltype(ci2)::value;
      constexpr int kc = kval(c, NV);
      const V gg = cscale(cmul(gb, gp[NV + c]), gs[kb * kb + kc * kc]);
      out[c] = cmul(x[pos(NV, c)], gg);
    });
  }
}

// G[cell] (+)= sum over the chunk's pairs of buf[item]
template <typename T>
__global__ void __launch_bounds__(256) k2_reduce(c2<T>* G, const c2<T>* buf, int64_t c0, int64_t cells, int64_t np,
                                                  int64_t N2, int first) {
  using V = c2<T>;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * N2) return;
  const int64_t ci = gid / N2, e = gid - ci * N2;
  const V* src = buf + ci * np * N2 + e;
  V s = first ? mk<V>(T(0), T(0)) : G[(c0 + ci) * N2 + e];
  for (int64_t p = 0; p < np; ++p) s = cadd(s, src[p * N2]);
  G[(c0 + ci) * N2 + e] = s;
}

// q = (Re IFFT2(G + hb lapl f^) - with_loss f Re IFFT2(lossk f^)) / n^2
template <typename T, int NV>
__global__ void __launch_bounds__(Geo2<NV>::THREADS) k2_finish(const c2<T>* G, const c2<T>* fhat, const double* f,
                                                                double* q, int64_t cells, int with_loss, double hb,
                                                                Tables tab) {
  using V = c2<T>;
  constexpr int N2 = Geo2<NV>::N2, LD = Geo2<NV>::LD, PPB = Geo2<NV>::PPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  const int64_t P0 = int64_t(blockIdx.x) * PPB;
  const int here = int((cells - P0) < PPB ? (cells - P0) : PPB);
  const int g = threadIdx.x / NV, t = threadIdx.x - g * NV;
  const bool active = g < here;
  const T* lk = reinterpret_cast<const T*>(tab.lossk);
  const T* lp = reinterpret_cast<const T*>(tab.lapl);
  T re[2][NV];
#pragma unroll
  for (int which = 0; which < 2; ++which) {
    for (int e = threadIdx.x; e < here * N2; e += blockDim.x) {
      const int gg = e / N2, rem = e - gg * N2;
      const int b = rem / NV, c = rem - b * NV;
      const int kb = kval(b, NV), kc = kval(c, NV);
      const int m = kb * kb + kc * kc;
      const V fv = fhat[P0 * N2 + e];
      V y;
      if (which == 0) {
        const V gv = G[P0 * N2 + e];
        const T l = T(hb) * lp[m];
        y = mk<V>(gv.x + l * fv.x, gv.y + l * fv.y);
      } else {
        y = cscale(fv, lk[m]);
      }
      S[(gg * NV + b) * LD + c] = y;
    }
    __syncthreads();
    if (active) row_fft<NV, +1>(S + (g * NV + t) * LD);
    __syncthreads();
    if (active) {
      V* col = S + g * NV * LD + t;
      V x[NV];
#pragma unroll
      for (int b = 0; b < NV; ++b) x[b] = col[b * LD];
      fft_line<NV, +1>(x);
      static_for<0, NV>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        re[which][b] = x[pos(NV, b)].x;
      });
    }
    __syncthreads();
  }
  if (active) {
    const int64_t base = (P0 + g) * N2 + t;  // element (b, c = t)
    const double inv = 1.0 / double(N2);
#pragma unroll
    for (int b = 0; b < NV; ++b) {
      double v = double(re[0][b]);
      if (with_loss) v -= f[base + b * NV] * double(re[1][b]);
      q[base + b * NV] = v * inv;
    }
  }
}

template <typename T, int NV>
struct Collide2D {
  static int prepare() {
    static PerDeviceOnce once;
    if (once.done()) return PII_OK;
    const int bytes = Geo2<NV>::PPB * NV * Geo2<NV>::LD * int(sizeof(c2<T>));
    PII_CUDA(cudaFuncSetAttribute(k2_fwd<T, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    PII_CUDA(cudaFuncSetAttribute(k2_pair<T, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    PII_CUDA(cudaFuncSetAttribute(k2_finish<T, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    once.set();
    return PII_OK;
  }

  // Lap_v f alone: forward transform, zero gain sum, finishing pass with heat_bath = 1, no loss
  static int laplacian(pii_plan* p, const double* f, double* out, int64_t cells, cudaStream_t s) {
    using V = c2<T>;
    constexpr int PPB = Geo2<NV>::PPB, TH = Geo2<NV>::THREADS;
    PII_TRY(prepare());
    const int smem = PPB * NV * Geo2<NV>::LD * int(sizeof(V));
    const unsigned cell_blocks = unsigned((cells + PPB - 1) / PPB);
    k2_fwd<T, NV><<<cell_blocks, TH, smem, s>>>(f, static_cast<V*>(p->fhat), static_cast<T*>(p->fT), cells);
    PII_CHECK_LAUNCH();
    PII_CUDA(cudaMemsetAsync(p->G, 0, size_t(cells) * size_t(Geo2<NV>::N2) * sizeof(V), s));
    k2_finish<T, NV><<<cell_blocks, TH, smem, s>>>(static_cast<const V*>(p->G), static_cast<const V*>(p->fhat), f,
                                                    out, cells, 0, 1.0, p->tab);
    PII_CHECK_LAUNCH();
    return PII_OK;
  }

  static int run(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb, cudaStream_t s) {
    using V = c2<T>;
    constexpr int N2 = Geo2<NV>::N2, PPB = Geo2<NV>::PPB, TH = Geo2<NV>::THREADS;
    PII_TRY(prepare());
    const int smem = PPB * NV * Geo2<NV>::LD * int(sizeof(V));
    const unsigned cell_blocks = unsigned((cells + PPB - 1) / PPB);
    {
      StageTimer st(p, ST_FWD_PLANE, s);
      k2_fwd<T, NV><<<cell_blocks, TH, smem, s>>>(f, static_cast<V*>(p->fhat), static_cast<T*>(p->fT), cells);
    }
    PII_CHECK_LAUNCH();
    // chunks of Cc cells x Pc pairs that fit the L2-sized buffer
    int64_t Cc = std::max<int64_t>(1, (p->chunk_points + N2 - 1) / N2);
    Cc = std::min<int64_t>(Cc, std::min<int64_t>(cells, p->chunk_items));
    const int64_t Pc = std::max<int64_t>(1, std::min<int64_t>(p->Q, p->chunk_items / Cc));
    for (int64_t c0 = 0; c0 < cells; c0 += Cc) {
      const int64_t cc = std::min(Cc, cells - c0);
      for (int64_t p0 = 0; p0 < p->Q; p0 += Pc) {
        const int64_t np = std::min(Pc, int64_t(p->Q) - p0);
        Pair2Args a{};
        a.fhat = p->fhat;
        a.fT = p->fT;
        a.buf = p->buf;
        a.c0 = c0;
        a.np = np;
        a.p0 = p0;
        a.items = cc * np;
        a.ns = p->ns;
        a.tab = p->tab;
        {
          StageTimer st(p, ST_PAIR_PLANE, s);
          k2_pair<T, NV><<<unsigned((a.items + PPB - 1) / PPB), TH, smem, s>>>(a);
        }
        PII_CHECK_LAUNCH();
        {
          StageTimer st(p, ST_REDUCE, s);
          k2_reduce<T><<<unsigned((cc * N2 + 255) / 256), 256, 0, s>>>(
              static_cast<V*>(p->G), static_cast<const V*>(p->buf), c0, cc, np, N2, p0 == 0 ? 1 : 0);
        }
        PII_CHECK_LAUNCH();
      }
    }
    {
      StageTimer st(p, ST_FINISH, s);
      k2_finish<T, NV><<<cell_blocks, TH, smem, s>>>(static_cast<const V*>(p->G), static_cast<const V*>(p->fhat), f,
                                                      q, cells, with_loss, hb, p->tab);
    }
    PII_CHECK_LAUNCH();
    return PII_OK;
  }
};

}  // namespace pii

#define PII_INSTANTIATE_2D(T, NV) template struct pii::Collide2D<T, NV>;
