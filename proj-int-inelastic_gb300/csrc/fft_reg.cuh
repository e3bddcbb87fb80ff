// In-register mixed-radix FFTs for one velocity line of length N = 2^a 3^b.
//
// Each thread holds a whole line in a register array.  The transform is a
// recursive decimation-in-frequency (DIF) Cooley-Tukey with radix 4 / 2 / 3
// stages; every index and every twiddle is a compile-time constant, so after
// inlining the line stays in registers and the twiddles are immediates.
//
// Output order: after dif<N>() the coefficient X[k] sits at register
// position pos<N>(k) (a generalised digit reversal), which callers resolve at
// compile time when they store or re-order the line.
//
// Sign convention (the reference's numpy/pyfftw/cuFFT convention,
// src/collision/inelastic_collisions.py:139-186): DIR = -1 is the unnormalised
// forward transform  X[k] = sum_j x[j] exp(-2 pi i jk/N);  DIR = +1 is the
// unnormalised inverse (the 1/N factor is applied by the callers).
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

#define PII_HD __host__ __device__ __forceinline__

namespace pii {

// ---------------------------------------------------------------------------
// constexpr trigonometry (double), used only to build compile-time twiddles.
// cos / sin of 2*pi*num/den, reduced to [0, pi/4] by the octant symmetries and
// evaluated with Taylor series (error < 1e-17 on [0, pi/4]).
// ---------------------------------------------------------------------------
constexpr double kPi = 3.141592653589793238462643383279502884;

#define PII_CX __host__ __device__ constexpr

PII_CX double taylor_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 14; ++k) {
    term *= -x2 / double((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
PII_CX double taylor_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 14; ++k) {
    term *= -x2 / double((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// returns (cos, sin) of 2*pi*num/den exactly reduced with integer arithmetic
struct CS {
  double c, s;
};
PII_CX CS cs_turn(long long num, long long den) {
  // reduce num/den into [0, 1) turns
  long long m = num % den;
  if (m < 0) m += den;
  // work in units of 1/(8 den) turns: octant index = floor(8 m / den)
  long long t8 = 8 * m;
  long long oct = t8 / den;               // 0..7
  long long rem = t8 - oct * den;         // in [0, den): fraction of an octant
  // angle within octant: theta = (rem/den) * (pi/4)
  double th = double(rem) / double(den) * (kPi / 4.0);
  // for odd octants use the complement so the series argument stays <= pi/4
  double c0 = 0, s0 = 0;
  if (oct % 2 == 0) {
    c0 = taylor_cos(th);
    s0 = taylor_sin(th);
  } else {
    double th2 = double(den - rem) / double(den) * (kPi / 4.0);
    // angle = (oct+1)*pi/4 - th2
    c0 = taylor_cos(th2);
    s0 = taylor_sin(th2);
  }
  // compose with the octant base angle
  // even octant: angle = oct*pi/4 + th ; odd: angle = (oct+1)*pi/4 - th2
  long long base = (oct % 2 == 0) ? oct : oct + 1;  // multiple of pi/4, 0..8
  base %= 8;
  const double r2 = 0.70710678118654752440084436210484903928;
  double bc = 0, bs = 0;
  switch (base) {
    case 0: bc = 1; bs = 0; break;
    case 1: bc = r2; bs = r2; break;
    case 2: bc = 0; bs = 1; break;
    case 3: bc = -r2; bs = r2; break;
    case 4: bc = -1; bs = 0; break;
    case 5: bc = -r2; bs = -r2; break;
    case 6: bc = 0; bs = -1; break;
    default: bc = r2; bs = -r2; break;
  }
  double sgn = (oct % 2 == 0) ? 1.0 : -1.0;  // +th or -th2
  double s1 = sgn * s0;
  // exact for the pure-axis bases (bc or bs zero, +-1); the diagonal bases
  // never occur with a non-zero remainder in odd octants (base is even there)
  return CS{bc * c0 - bs * s1, bs * c0 + bc * s1};
}

// ---------------------------------------------------------------------------
// complex helpers on float2 / double2
// ---------------------------------------------------------------------------
template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using c2 = typename cplx<T>::type;

template <typename V> PII_HD V mk(decltype(V::x) a, decltype(V::x) b) {
  V v; v.x = a; v.y = b; return v;
}
template <typename V> PII_HD V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <typename V> PII_HD V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <typename V> PII_HD V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj-free multiply accumulate: acc += a*b
template <typename V> PII_HD V cfma(V a, V b, V acc) {
  return mk<V>(acc.x + a.x * b.x - a.y * b.y, acc.y + a.x * b.y + a.y * b.x);
}
template <typename V> PII_HD V cscale(V a, decltype(V::x) s) { return mk<V>(a.x * s, a.y * s); }

// multiply by DIR * i  (DIR = +1: i, DIR = -1: -i)
template <int DIR, typename V> PII_HD V mul_i(V a) {
  if constexpr (DIR > 0) return mk<V>(-a.y, a.x);
  else return mk<V>(a.y, -a.x);
}

// Butterfly arithmetic of the FP32 transforms on the packed FP32x2 pipe
// (add / sub / fma .f32x2: one instruction for both components of a complex
// value, rounded like the scalar instructions).  Device code only; the host
// and FP64 paths use the scalar helpers above.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned long long f2pk(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2up(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 f2add(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2pk(a)), "l"(f2pk(b)));
  return f2up(d);
}
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2pk(a)), "l"(f2pk(b)));
  return f2up(d);
}
// a * b + c, componentwise
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2pk(a)), "l"(f2pk(b)), "l"(f2pk(c)));
  return f2up(d);
}
#define PII_F32X2 1
#else
#define PII_F32X2 0
#endif
// butterfly sum / difference: packed on the device for float2 when PK (the
// pairing constraint of the packed operands costs registers, so each kernel
// chooses: faster where registers are left, slower where they are not)
template <bool PK, typename V> PII_HD V bsum(V a, V b) {
#if PII_F32X2
  if constexpr (PK && std::is_same_v<V, float2>) return f2add(a, b);
#endif
  return cadd(a, b);
}
template <bool PK, typename V> PII_HD V bdif(V a, V b) {
#if PII_F32X2
  if constexpr (PK && std::is_same_v<V, float2>) return f2sub(a, b);
#endif
  return csub(a, b);
}
// a + DIR * i * d (scalar: the packed form would need d's components swapped)
template <int DIR, typename V> PII_HD V b_add_i(V a, V d) { return cadd(a, mul_i<DIR>(d)); }

// multiply by exp(DIR * 2 pi i * num / den) with compile-time constants
template <long long NUM, long long DEN, int DIR, typename V>
PII_HD V twiddle(V a) {
  using S = decltype(V::x);
  constexpr long long m = ((NUM % DEN) + DEN) % DEN;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (4 * m == DEN) {
    return mul_i<DIR>(a);
  } else if constexpr (2 * m == DEN) {
    return mk<V>(-a.x, -a.y);
  } else if constexpr (4 * m == 3 * DEN) {
    return mul_i<-DIR>(a);
  } else {
    constexpr CS w = cs_turn(m, DEN);
    constexpr S wr = S(w.c);
    constexpr S wi = S(DIR * w.s);
    return mk<V>(a.x * wr - a.y * wi, a.x * wi + a.y * wr);
  }
}

// ---------------------------------------------------------------------------
// compile-time loops
// ---------------------------------------------------------------------------
template <int I, int END, typename F>
PII_HD void static_for(F&& f) {
  if constexpr (I < END) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, END>(f);
  }
}

PII_CX int pick_radix(int n) { return (n % 4 == 0) ? 4 : ((n % 2 == 0) ? 2 : 3); }

// position of coefficient k after dif<N>()
PII_CX int pos(int n, int k) {
  // unroll the recursion: at each level, block index q = k mod R, M = n / R
  int base = 0;
  while (n > 1) {
    int r = pick_radix(n);
    int m = n / r;
    int q = k % r;
    base += q * m;
    k /= r;
    n = m;
  }
  return base;
}

// small DFTs on y[0..R-1] (in place, natural order in and out)
template <int R, int DIR, bool PK = false, typename V>
PII_HD void small_dft(V* y) {
  using S = decltype(V::x);
  if constexpr (R == 2) {
    V a = y[0], b = y[1];
    y[0] = bsum<PK>(a, b);
    y[1] = bdif<PK>(a, b);
  } else if constexpr (R == 4) {
    V a0 = bsum<PK>(y[0], y[2]), a1 = bdif<PK>(y[0], y[2]);
    V b0 = bsum<PK>(y[1], y[3]), d = bdif<PK>(y[1], y[3]);
    y[0] = bsum<PK>(a0, b0);
    y[2] = bdif<PK>(a0, b0);
    y[1] = b_add_i<DIR>(a1, d);
    y[3] = b_add_i<-DIR>(a1, d);
  } else {  // R == 3
    constexpr S c = S(-0.5);
    constexpr S s = S(DIR * 0.86602540378443864676372317075293618);
    V t = cadd(y[1], y[2]);
    V d = csub(y[1], y[2]);
    V m0 = cadd(y[0], t);
    V m1 = mk<V>(y[0].x + c * t.x, y[0].y + c * t.y);
    // i*s*d
    V m2 = mk<V>(-s * d.y, s * d.x);
    y[0] = m0;
    y[1] = cadd(m1, m2);
    y[2] = csub(m1, m2);
  }
}

// in-place DIF on x[O + S*j], j in [0, N)
template <int N, int S, int O, int DIR, bool PK = false, typename V>
PII_HD void dif(V* x) {
  if constexpr (N > 1) {
    constexpr int R = pick_radix(N);
    constexpr int M = N / R;
    static_for<0, M>([&](auto mi) {
      constexpr int m = decltype(mi)::value;
      V y[R];
      static_for<0, R>([&](auto ji) {
        constexpr int j = decltype(ji)::value;
        y[j] = x[O + S * (m + j * M)];
      });
      small_dft<R, DIR, PK>(y);
      static_for<0, R>([&](auto qi) {
        constexpr int q = decltype(qi)::value;
        x[O + S * (m + q * M)] = twiddle<(long long)m * q, N, DIR>(y[q]);
      });
    });
    static_for<0, R>([&](auto qi) {
      constexpr int q = decltype(qi)::value;
      dif<M, S, O + S * q * M, DIR, PK>(x);
    });
  }
}

// Full line transform; on return x[pos(N,k)] holds X[k].  PK: the radix-2 / 4
// butterflies' sums and differences on the packed FP32x2 pipe (FP32 only).
template <int N, int DIR, bool PK = false, typename V>
PII_HD void fft_line(V* x) {
  dif<N, 1, 0, DIR, PK>(x);
}

// Re-order a transformed line into natural order (compile-time register renaming).
template <int N, typename V>
PII_HD void to_natural(const V* x, V* y) {
  static_for<0, N>([&](auto ki) {
    constexpr int k = decltype(ki)::value;
    y[k] = x[pos(N, k)];
  });
}

// signed spectral index of storage position i: fftshift(arange(-n/2, n/2))
PII_CX int kval(int i, int n) { return i < n / 2 ? i : i - n; }

}  // namespace pii
