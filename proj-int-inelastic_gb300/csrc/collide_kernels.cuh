// Kernels of the batched fast-spectral collision operator, templated on the
// working precision T (float / double) and the velocity grid size NV.
//
// A cell's velocity grid is stored [a][b][c] (c fastest), a = first velocity
// axis.  Every 3D transform is split into
//   * a column pass: one thread owns one (b, c) column and transforms along a
//     in registers (loads and stores coalesced across threads), and
//   * a plane pass: NV threads own one a-plane; each transforms a row along c
//     in registers, the plane is transposed through padded shared memory and
//     each thread transforms a column along b.
//
// Q+(f,f) for one quadrature pair (r, sigma) -- an "item" (cell, pair) -- is
// (src/collision/inelastic_collisions.py:208-218)
//   A   = IFFT3(exp_rs(k) * fhat)          column pass  (k_col<PSTART>)
//   Bk  = FFT3(A * f)                      plane pass   (k_pair_plane: IFFT_c,
//                                          IFFT_b, * f, FFT_b, FFT_c) + column
//                                          pass (k_col<PEND>: FFT_a, * gain_rs)
//   G  += sum_items gain_rs(k) * Bk        (k_reduce)
// and the final step (:218-227) is one inverse 3D FFT of
//   Y1 = G + heat_bath * lapl * fhat  and  Y2 = lossk * fhat
// with q = Re(Y1) - f Re(Y2)              (k_col<IPREP> + k_finish).
// Intermediates of a chunk of items live in one buffer sized to stay L2-resident.
#pragma once
#include <type_traits>
#include "fft_reg.cuh"
#include "pack.cuh"
#include "pii_internal.cuh"

namespace pii {

template <int NV>
struct Geo {
  static constexpr int N2 = NV * NV;
  static constexpr int N3 = NV * NV * NV;
  static constexpr int PPB = (128 / NV) > 0 ? (128 / NV) : 1;  // planes per block
  static constexpr int THREADS = PPB * NV;
  static constexpr int LD = NV + 1;  // padded row stride (complex elements)
};

struct ColArgs {
  const void* src;     // input grid(s)
  void* dst;           // output grid(s)
  const void* fhat;    // spectra of f (IPREP)
  int64_t items;       // number of grid items in the launch
  int64_t c0;          // first cell of the chunk
  int64_t p0;          // first pair of the chunk
  int64_t np;          // pairs per cell in the chunk
  int ns;              // n_sigma
  double hb;           // heat bath coefficient (IPREP)
  const int* reps;     // _PK modes: representative pair of each antipodal pass
  Tables tab;
};



// ---------------------------------------------------------------------------
// column pass along a
// ---------------------------------------------------------------------------
template <typename T, int NV, int MODE>
__global__ void __launch_bounds__(128) k_col(ColArgs args) {
  using V = c2<T>;
  constexpr int N2 = Geo<NV>::N2;
  constexpr int N3 = Geo<NV>::N3;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= args.items * N2) return;
  const int64_t item = gid / N2;
  const int j = int(gid - item * N2);
  const int jb = j / NV, jc = j - jb * NV;
  const int kb = kval(jb, NV), kc = kval(jc, NV);
  V x[NV];

  if constexpr (MODE == COL_FWD) {
    V* g = reinterpret_cast<V*>(args.dst) + item * N3 + j;
#pragma unroll
    for (int a = 0; a < NV; ++a) x[a] = g[a * N2];
    fft_line<NV, -1>(x);
    static_for<0, NV>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      g[a * N2] = x[pos(NV, a)];
    });
  } else if constexpr (MODE == COL_PSTART) {
    const int64_t ci = item / args.np;
    const int64_t pair = args.p0 + (item - ci * args.np);
    const V* fh = reinterpret_cast<const V*>(args.src) + (args.c0 + ci) * N3 + j;
    const V* ep = reinterpret_cast<const V*>(args.tab.ephase) + pair * 3 * NV;
    const V ebc = cmul(ep[NV + jb], ep[2 * NV + jc]);
#pragma unroll
    for (int a = 0; a < NV; ++a) x[a] = cmul(fh[a * N2], cmul(ep[a], ebc));
    fft_line<NV, +1>(x);
    V* out = reinterpret_cast<V*>(args.dst) + item * N3 + j;
    static_for<0, NV>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      out[a * N2] = x[pos(NV, a)];
    });
  } else if constexpr (MODE == COL_PEND) {
    const int64_t ci = item / args.np;
    const int64_t pair = args.p0 + (item - ci * args.np);
    const int ir = int(pair / args.ns);
    V* io = reinterpret_cast<V*>(args.dst) + item * N3 + j;
#pragma unroll
    for (int a = 0; a < NV; ++a) x[a] = io[a * N2];
    fft_line<NV, -1>(x);
    const int64_t cell = args.c0 + ci;  // its restitution set, when the plan has one per cell
    const V* gp = reinterpret_cast<const V*>(args.tab.gphase) + cell * args.tab.gph_stride + pair * 3 * NV;
    const T* gs =
        reinterpret_cast<const T*>(args.tab.gsinc) + cell * args.tab.gs_stride + int64_t(ir) * (args.tab.M + 1);
    const V gbc = cmul(gp[NV + jb], gp[2 * NV + jc]);
    const int mbc = kb * kb + kc * kc;
    static_for<0, NV>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      constexpr int ka = kval(a, NV);
      const V g = cscale(cmul(gp[a], gbc), gs[mbc + ka * ka]);
      io[a * N2] = cmul(x[pos(NV, a)], g);
    });
  } else if constexpr (MODE == COL_PSTART_PK) {
    // the antipodal pass's input f^ t (real phase t), transformed along a
    const int64_t ci = item / args.np;
    const int pair = args.reps[args.p0 + (item - ci * args.np)];
    const V* fh = reinterpret_cast<const V*>(args.src) + (args.c0 + ci) * N3 + j;
    const V* ep = reinterpret_cast<const V*>(args.tab.ephase) + int64_t(pair) * 3 * NV;
    T cp, cm, th;
    pack_t_consts<T, V, NV>(ep, jb, jc, cp, cm, th);
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      const V e = ep[a];
      const T t = a == NV / 2 ? th : e.x * cp + e.y * cm;
      x[a] = cscale(fh[a * N2], t);
    }
    fft_line<NV, +1>(x);
    V* out = reinterpret_cast<V*>(args.dst) + item * N3 + j;
    static_for<0, NV>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      out[a * N2] = x[pos(NV, a)];
    });
  } else if constexpr (MODE == COL_PEND_PK) {
    // forward transform along a, then the REAL coefficient 2 s(k) times the radial sinc
    const int64_t ci = item / args.np;
    const int pair = args.reps[args.p0 + (item - ci * args.np)];
    const int ir = pair / args.ns;
    V* io = reinterpret_cast<V*>(args.dst) + item * N3 + j;
#pragma unroll
    for (int a = 0; a < NV; ++a) x[a] = io[a * N2];
    fft_line<NV, -1>(x);
    const int64_t cell = args.c0 + ci;  // its restitution set, when the plan has one per cell
    const V* gp = reinterpret_cast<const V*>(args.tab.gphase) + cell * args.tab.gph_stride + int64_t(pair) * 3 * NV;
    const T* gs =
        reinterpret_cast<const T*>(args.tab.gsinc) + cell * args.tab.gs_stride + int64_t(ir) * (args.tab.M + 1);
    T dp, dm, sh;
    pack_s_consts<T, V, NV>(gp, jb, jc, dp, dm, sh);
    const int mbc = kb * kb + kc * kc;
    static_for<0, NV>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      constexpr int ka = kval(a, NV);
      const V g = gp[a];
      const T sv = a == NV / 2 ? sh : g.x * dp - g.y * dm;
      io[a * N2] = cscale(x[pos(NV, a)], T(2) * sv * gs[mbc + ka * ka]);
    });
  } else {  // COL_IPREP: item = cell in chunk; outputs Y1 -> dst[2 item], Y2 -> dst[2 item + 1]
    const int64_t cell = args.c0 + item;
    const V* gg = reinterpret_cast<const V*>(args.src) + cell * N3 + j;
    const V* fh = reinterpret_cast<const V*>(args.fhat) + cell * N3 + j;
    const T* lk = reinterpret_cast<const T*>(args.tab.lossk);
    const T* lp = reinterpret_cast<const T*>(args.tab.lapl);
    const T hb = T(args.hb);
    const int mbc = kb * kb + kc * kc;
    V y[NV];
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      const int ka = kval(a, NV);
      const int m = mbc + ka * ka;
      const V fv = fh[a * N2];
      const V gv = gg[a * N2];
      const T l = hb * lp[m];
      x[a] = mk<V>(gv.x + l * fv.x, gv.y + l * fv.y);
      y[a] = cscale(fv, lk[m]);
    }
    fft_line<NV, +1>(x);
    fft_line<NV, +1>(y);
    V* o1 = reinterpret_cast<V*>(args.dst) + (2 * item) * N3 + j;
    V* o2 = o1 + N3;
    static_for<0, NV>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      o1[a * N2] = x[pos(NV, a)];
      o2[a * N2] = y[pos(NV, a)];
    });
  }
}

// ---------------------------------------------------------------------------
// plane passes
// ---------------------------------------------------------------------------
// cooperative, coalesced copy of the block's PPB consecutive planes
template <typename V, int NV>
__device__ __forceinline__ void load_planes(V* S, const V* src, int nplanes_here) {
  constexpr int N2 = Geo<NV>::N2, LD = Geo<NV>::LD;
  for (int e = threadIdx.x; e < nplanes_here * N2; e += blockDim.x) {
    const int g = e / N2, rem = e - g * N2;
    const int b = rem / NV, c = rem - b * NV;
    S[(g * NV + b) * LD + c] = src[e];
  }
}
template <typename V, int NV>
__device__ __forceinline__ void store_planes(const V* S, V* dst, int nplanes_here) {
  constexpr int N2 = Geo<NV>::N2, LD = Geo<NV>::LD;
  for (int e = threadIdx.x; e < nplanes_here * N2; e += blockDim.x) {
    const int g = e / N2, rem = e - g * N2;
    const int b = rem / NV, c = rem - b * NV;
    dst[e] = S[(g * NV + b) * LD + c];
  }
}

// forward FFT along c then b of real input planes; also writes f in precision T
template <typename T, int NV>
__global__ void __launch_bounds__(Geo<NV>::THREADS) k_fwd_plane(const double* f, c2<T>* fhat, T* fT,
                                                                 int64_t nplanes) {
  using V = c2<T>;
  constexpr int N2 = Geo<NV>::N2, LD = Geo<NV>::LD, PPB = Geo<NV>::PPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  const int64_t P0 = int64_t(blockIdx.x) * PPB;
  const int here = int((nplanes - P0) < PPB ? (nplanes - P0) : PPB);
  const int g = threadIdx.x / NV, t = threadIdx.x - g * NV;
  const bool active = g < here;
  for (int e = threadIdx.x; e < here * N2; e += blockDim.x) {
    const double v = f[P0 * N2 + e];
    fT[P0 * N2 + e] = T(v);
    const int gg = e / N2, rem = e - gg * N2;
    const int b = rem / NV, c = rem - b * NV;
    S[(gg * NV + b) * LD + c] = mk<V>(T(v), T(0));
  }
  __syncthreads();
  V x[NV];
  V* row = S + (g * NV + t) * LD;
  if (active) {
#pragma unroll
    for (int c = 0; c < NV; ++c) x[c] = row[c];
    fft_line<NV, -1>(x);
    static_for<0, NV>([&](auto ki) {
      constexpr int k = decltype(ki)::value;
      row[k] = x[pos(NV, k)];
    });
  }
  __syncthreads();
  V* col = S + g * NV * LD + t;
  if (active) {
#pragma unroll
    for (int b = 0; b < NV; ++b) x[b] = col[b * LD];
    fft_line<NV, -1>(x);
    static_for<0, NV>([&](auto ki) {
      constexpr int k = decltype(ki)::value;
      col[k * LD] = x[pos(NV, k)];
    });
  }
  __syncthreads();
  store_planes<V, NV>(S, fhat + P0 * N2, here);
}

// pair plane pass: IFFT_c, IFFT_b, multiply by f, FFT_b, FFT_c (in place)
template <typename T, int NV>
__global__ void __launch_bounds__(Geo<NV>::THREADS) k_pair_plane(c2<T>* buf, const T* fT, int64_t c0,
                                                                  int64_t np, int64_t nplanes) {
  using V = c2<T>;
  constexpr int N2 = Geo<NV>::N2, N3 = Geo<NV>::N3, LD = Geo<NV>::LD, PPB = Geo<NV>::PPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  const int64_t P0 = int64_t(blockIdx.x) * PPB;
  const int here = int((nplanes - P0) < PPB ? (nplanes - P0) : PPB);
  const int g = threadIdx.x / NV, t = threadIdx.x - g * NV;
  const bool active = g < here;
  load_planes<V, NV>(S, buf + P0 * N2, here);
  __syncthreads();
  V x[NV];
  V* row = S + (g * NV + t) * LD;
  V* col = S + g * NV * LD + t;
  if (active) {
#pragma unroll
    for (int c = 0; c < NV; ++c) x[c] = row[c];
    fft_line<NV, +1>(x);
    static_for<0, NV>([&](auto ki) {
      constexpr int k = decltype(ki)::value;
      row[k] = x[pos(NV, k)];
    });
  }
  __syncthreads();
  if (active) {
    const int64_t P = P0 + g;
    const int64_t item = P / NV;
    const int a = int(P - item * NV);
    const int64_t cell = c0 + item / np;
    const T* fr = fT + cell * N3 + int64_t(a) * N2 + t;  // f[cell][a][b][c = t]
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
#pragma unroll
    for (int c = 0; c < NV; ++c) x[c] = row[c];
    fft_line<NV, -1>(x);
    static_for<0, NV>([&](auto ki) {
      constexpr int k = decltype(ki)::value;
      row[k] = x[pos(NV, k)];
    });
  }
  __syncthreads();
  store_planes<V, NV>(S, buf + P0 * N2, here);
}

// final plane pass: inverse transforms of Y1, Y2 along b and c, then
// q = (Re Y1 - with_loss * f * Re Y2) / n^3
template <typename T, int NV>
__global__ void __launch_bounds__(Geo<NV>::THREADS) k_finish(const c2<T>* buf, const double* f, double* q,
                                                              int64_t c0, int64_t nplanes, int with_loss) {
  using V = c2<T>;
  constexpr int N2 = Geo<NV>::N2, N3 = Geo<NV>::N3, LD = Geo<NV>::LD, PPB = Geo<NV>::PPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S = reinterpret_cast<V*>(smem_raw);
  const int64_t P0 = int64_t(blockIdx.x) * PPB;
  const int here = int((nplanes - P0) < PPB ? (nplanes - P0) : PPB);
  const int g = threadIdx.x / NV, t = threadIdx.x - g * NV;
  const bool active = g < here;
  V x[NV];
  T re[2][NV];
  V* row = S + (g * NV + t) * LD;
  V* col = S + g * NV * LD + t;
#pragma unroll
  for (int which = 0; which < 2; ++which) {
    // planes of Y_which: item i = P / NV sits at buf[(2 i + which) N3 + a N2]
    for (int e = threadIdx.x; e < here * N2; e += blockDim.x) {
      const int gg = e / N2, rem = e - gg * N2;
      const int64_t P = P0 + gg;
      const int64_t item = P / NV;
      const int a = int(P - item * NV);
      const int b = rem / NV, c = rem - b * NV;
      S[(gg * NV + b) * LD + c] = buf[(2 * item + which) * N3 + int64_t(a) * N2 + rem];
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int c = 0; c < NV; ++c) x[c] = row[c];
      fft_line<NV, +1>(x);
      static_for<0, NV>([&](auto ki) {
        constexpr int k = decltype(ki)::value;
        row[k] = x[pos(NV, k)];
      });
    }
    __syncthreads();
    if (active) {
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
    const int64_t P = P0 + g;
    const int64_t item = P / NV;
    const int a = int(P - item * NV);
    const int64_t base = (c0 + item) * N3 + int64_t(a) * N2 + t;
    const double inv = 1.0 / double(N3);
#pragma unroll
    for (int b = 0; b < NV; ++b) {
      double v = double(re[0][b]);
      if (with_loss) v -= f[base + b * NV] * double(re[1][b]);
      q[base + b * NV] = v * inv;
    }
  }
}

// G[cell] (+)= sum over the chunk's pairs of buf[item]
template <typename T>
__global__ void __launch_bounds__(256) k_reduce(c2<T>* G, const c2<T>* buf, int64_t c0, int64_t cells,
                                                 int64_t np, int64_t N3, int first) {
  using V = c2<T>;
  const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= cells * N3) return;
  const int64_t ci = gid / N3, e = gid - ci * N3;
  const V* src = buf + ci * np * N3 + e;
  // eight independent partial sums: eight loads of the chunk in flight per thread
  V s[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) s[u] = mk<V>(T(0), T(0));
  int64_t p = 0;
  for (; p + 8 <= np; p += 8) {
    V v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = src[(p + u) * N3];
#pragma unroll
    for (int u = 0; u < 8; ++u) s[u] = cadd(s[u], v[u]);
  }
  for (; p < np; ++p) s[0] = cadd(s[0], src[p * N3]);
  V t = cadd(cadd(cadd(s[0], s[1]), cadd(s[2], s[3])), cadd(cadd(s[4], s[5]), cadd(s[6], s[7])));
  if (!first) t = cadd(t, G[(c0 + ci) * N3 + e]);
  G[(c0 + ci) * N3 + e] = t;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <typename T, int NV>
static int set_smem_attrs() {
  using V = c2<T>;
  static PerDeviceOnce once;
  if (once.done()) return PII_OK;
  const int bytes = Geo<NV>::PPB * NV * Geo<NV>::LD * int(sizeof(V));
  PII_CUDA(cudaFuncSetAttribute(k_fwd_plane<T, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  PII_CUDA(cudaFuncSetAttribute(k_pair_plane<T, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  PII_CUDA(cudaFuncSetAttribute(k_finish<T, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  once.set();
  return PII_OK;
}

template <typename T, int NV>
static ColArgs col_args(pii_plan* p) {
  ColArgs a{};
  a.tab = p->tab;
  a.ns = p->ns;
  return a;
}

template <typename T, int NV>
int CollideKernels<T, NV>::prepare() {
  return set_smem_attrs<T, NV>();
}

template <typename T, int NV>
int CollideKernels<T, NV>::fwd(pii_plan* p, const double* f, int64_t c0, int64_t cells, cudaStream_t s) {
  using V = c2<T>;
  constexpr int N3 = Geo<NV>::N3, PPB = Geo<NV>::PPB, N2 = Geo<NV>::N2;
  PII_TRY((set_smem_attrs<T, NV>()));
  const int smem = PPB * NV * Geo<NV>::LD * int(sizeof(V));
  const int64_t nplanes = cells * NV;
  V* fhat = reinterpret_cast<V*>(p->fhat) + c0 * N3;
  T* fT = reinterpret_cast<T*>(p->fT) + c0 * N3;
  {
    StageTimer st(p, ST_FWD_PLANE, s);
    k_fwd_plane<T, NV><<<unsigned((nplanes + PPB - 1) / PPB), Geo<NV>::THREADS, smem, s>>>(f + c0 * N3, fhat, fT,
                                                                                           nplanes);
  }
  PII_CHECK_LAUNCH();
  ColArgs a = col_args<T, NV>(p);
  a.dst = fhat;
  a.items = cells;
  {
    StageTimer st(p, ST_COL_FWD, s);
    k_col<T, NV, COL_FWD><<<unsigned((cells * N2 + 127) / 128), 128, 0, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

template <typename T, int NV>
int CollideKernels<T, NV>::pairs(pii_plan* p, int64_t c0, int64_t cells, int64_t p0, int64_t np, bool first,
                                 cudaStream_t s, bool packed) {
  using V = c2<T>;
  constexpr int N3 = Geo<NV>::N3, PPB = Geo<NV>::PPB, N2 = Geo<NV>::N2;
  const int smem = PPB * NV * Geo<NV>::LD * int(sizeof(V));
  const int64_t items = cells * np;
  ColArgs a = col_args<T, NV>(p);
  a.src = p->fhat;
  a.dst = p->buf;
  a.items = items;
  a.c0 = c0;
  a.p0 = p0;
  a.np = np;
  a.reps = p->ap_reps;
  const unsigned colblocks = unsigned((items * N2 + 127) / 128);
  bool tc = false;
  if constexpr (std::is_same<T, float>::value && NV == 64) tc = p->dft_path == 1;
  if (tc) {
    PII_TRY(col_tc_run(p, packed ? COL_PSTART_PK : COL_PSTART, items, c0, p0, np, s));
  } else {
    StageTimer st(p, ST_COL_PSTART, s);
    if (packed)
      k_col<T, NV, COL_PSTART_PK><<<colblocks, 128, 0, s>>>(a);
    else
      k_col<T, NV, COL_PSTART><<<colblocks, 128, 0, s>>>(a);
    PII_CHECK_LAUNCH();
  }
  const int64_t nplanes = items * NV;
  {
    StageTimer st(p, ST_PAIR_PLANE, s);
    k_pair_plane<T, NV><<<unsigned((nplanes + PPB - 1) / PPB), Geo<NV>::THREADS, smem, s>>>(
        reinterpret_cast<V*>(p->buf), reinterpret_cast<const T*>(p->fT), c0, np, nplanes);
  }
  PII_CHECK_LAUNCH();
  if (tc) {
    PII_TRY(col_tc_run(p, packed ? COL_PEND_PK : COL_PEND, items, c0, p0, np, s));
  } else {
    StageTimer st(p, ST_COL_PEND, s);
    if (packed)
      k_col<T, NV, COL_PEND_PK><<<colblocks, 128, 0, s>>>(a);
    else
      k_col<T, NV, COL_PEND><<<colblocks, 128, 0, s>>>(a);
    PII_CHECK_LAUNCH();
  }
  {
    StageTimer st(p, ST_REDUCE, s);
    k_reduce<T><<<unsigned((cells * N3 + 255) / 256), 256, 0, s>>>(
        reinterpret_cast<V*>(p->G), reinterpret_cast<const V*>(p->buf), c0, cells, np, N3, first ? 1 : 0);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

template <typename T, int NV>
int CollideKernels<T, NV>::finish(pii_plan* p, const double* f, double* q, int64_t c0, int64_t cells,
                                  int with_loss, double hb, cudaStream_t s) {
  using V = c2<T>;
  constexpr int PPB = Geo<NV>::PPB, N2 = Geo<NV>::N2;
  const int smem = PPB * NV * Geo<NV>::LD * int(sizeof(V));
  ColArgs a = col_args<T, NV>(p);
  a.src = p->G;
  a.fhat = p->fhat;
  a.dst = p->buf;
  a.items = cells;
  a.c0 = c0;
  a.hb = hb;
  {
    StageTimer st(p, ST_COL_IPREP, s);
    k_col<T, NV, COL_IPREP><<<unsigned((cells * N2 + 127) / 128), 128, 0, s>>>(a);
  }
  PII_CHECK_LAUNCH();
  const int64_t nplanes = cells * NV;
  {
    StageTimer st(p, ST_FINISH, s);
    k_finish<T, NV><<<unsigned((nplanes + PPB - 1) / PPB), Geo<NV>::THREADS, smem, s>>>(
        reinterpret_cast<const V*>(p->buf), f, q, c0, nplanes, with_loss);
  }
  PII_CHECK_LAUNCH();
  return PII_OK;
}

}  // namespace pii

#define PII_INSTANTIATE(T, NV) template struct pii::CollideKernels<T, NV>;
