// In-register DFT building blocks for the pencil FFT passes.
//
// dft<N, DIR>(v) transforms N complex values held in registers:
//   X[k] = sum_n v[n] * exp(DIR * 2*pi*i * n*k / N),   DIR = -1 forward, +1 inverse
// (unnormalised; the 1/N of the inverse transform is folded into the pointwise
// multiply of the operator). Sizes 2, 3, 4, 5 are written out; composite sizes
// are split Cooley-Tukey style N = A*B with compile-time twiddles, so every
// index and every constant resolves at compile time and the array stays in
// registers.
#pragma once
#include <cuda_runtime.h>

namespace ef {

// ---- compile-time trigonometry (double, then rounded to float) ------------------
__host__ __device__ constexpr double ce_pi() { return 3.14159265358979323846264338327950288; }

// sin/cos of pi*num/den by Taylor series after exact integer range reduction
__host__ __device__ constexpr double ce_sin_series(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int i = 1; i < 30; ++i) {
    term *= -x2 / double((2 * i) * (2 * i + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ce_cos_series(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int i = 1; i < 30; ++i) {
    term *= -x2 / double((2 * i - 1) * (2 * i));
    sum += term;
  }
  return sum;
}
// reduce num/den to (-1, 1] so the angle lies in (-pi, pi]
__host__ __device__ constexpr double ce_reduce(long num, long den) {
  long r = num % (2 * den);
  if (r < 0) r += 2 * den;
  if (r > den) r -= 2 * den;
  return double(r) / double(den);
}
__host__ __device__ constexpr double ce_cospi(long num, long den) {
  return ce_cos_series(ce_pi() * ce_reduce(num, den));
}
__host__ __device__ constexpr double ce_sinpi(long num, long den) {
  return ce_sin_series(ce_pi() * ce_reduce(num, den));
}

// ---- complex helpers -------------------------------------------------------------
// With EF_F32X2 (the default) additions, subtractions and scalings use the paired
// fp32 instructions of sm_100 and later (one instruction for the real and imaginary
// parts; IEEE round-to-nearest per component, so results equal the scalar forms:
// a - b is computed as b * (-1) + a, whose product is exact).
#ifndef EF_F32X2
#define EF_F32X2 1
#endif
#if EF_F32X2
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return __fmul2_rn(a, make_float2(s, s)); }
// a + (sx * b.y, sy * b.x): the building block of a +/- i b
__device__ __forceinline__ float2 cadd_swapped(float2 a, float2 b, float sx, float sy) {
  return __ffma2_rn(make_float2(b.y, b.x), make_float2(sx, sy), a);
}
#else
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cadd_swapped(float2 a, float2 b, float sx, float sy) {
  return make_float2(fmaf(sx, b.y, a.x), fmaf(sy, b.x, a.y));
}
#endif
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// multiply by DIR*i  (i.e. +i for DIR=+1, -i for DIR=-1)
template <int DIR>
__device__ __forceinline__ float2 mul_dir_i(float2 a) {
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// a + DIR*i*b and a - DIR*i*b
template <int DIR>
__device__ __forceinline__ float2 cadd_i(float2 a, float2 b) {
  return DIR > 0 ? cadd_swapped(a, b, -1.f, 1.f) : cadd_swapped(a, b, 1.f, -1.f);
}
template <int DIR>
__device__ __forceinline__ float2 csub_i(float2 a, float2 b) {
  return DIR > 0 ? cadd_swapped(a, b, 1.f, -1.f) : cadd_swapped(a, b, -1.f, 1.f);
}

// twiddle exp(DIR * 2 pi i * num / den) as a compile-time constant
template <int DIR, long NUM, long DEN>
__device__ __forceinline__ float2 ctw() {
  constexpr float c = float(ce_cospi(2 * NUM, DEN));
  constexpr float s = float(DIR * ce_sinpi(2 * NUM, DEN));
  return make_float2(c, s);
}

template <int N, int DIR>
struct DFT;

template <int DIR>
struct DFT<1, DIR> {
  template <typename A>
  __device__ __forceinline__ static void run(A& v) {}
};

template <int DIR>
struct DFT<2, DIR> {
  template <typename A>
  __device__ __forceinline__ static void run(A& v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <int DIR>
struct DFT<3, DIR> {
  template <typename A>
  __device__ __forceinline__ static void run(A& v) {
    constexpr float h = 0.8660254037844386f;  // sqrt(3)/2
    float2 x0 = v[0], x1 = v[1], x2 = v[2];
    float2 t1 = cadd(x1, x2);
    float2 d = cscale(csub(x1, x2), h);
    float2 m = make_float2(x0.x - 0.5f * t1.x, x0.y - 0.5f * t1.y);
    v[0] = cadd(x0, t1);
    v[1] = cadd_i<DIR>(m, d);
    v[2] = csub_i<DIR>(m, d);
  }
};

template <int DIR>
struct DFT<4, DIR> {
  template <typename A>
  __device__ __forceinline__ static void run(A& v) {
    float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    float2 c = cadd(v[1], v[3]), e = csub(v[1], v[3]);
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd_i<DIR>(b, e);
    v[3] = csub_i<DIR>(b, e);
  }
};

template <int DIR>
struct DFT<5, DIR> {
  template <typename A>
  __device__ __forceinline__ static void run(A& v) {
    // X_k = x0 + sum_{n=1..4} x_n w^{nk}, paired as (x1+x4), (x2+x3)
    constexpr float c1 = float(ce_cospi(2, 5)), c2 = float(ce_cospi(4, 5));
    constexpr float s1 = float(ce_sinpi(2, 5)), s2 = float(ce_sinpi(4, 5));
    float2 x0 = v[0];
    float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    float2 m1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    float2 m2 = make_float2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    float2 r1 = mul_dir_i<DIR>(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
    float2 r2 = mul_dir_i<DIR>(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
    v[0] = cadd(x0, cadd(a1, a2));
    v[1] = cadd(m1, r1);
    v[4] = csub(m1, r1);
    v[2] = cadd(m2, r2);
    v[3] = csub(m2, r2);
  }
};

// composite N = A*B: n = B*n1 + n2, k = k1 + A*k2
template <int N>
struct Split {
  static constexpr int A = (N % 4 == 0 && N > 4) ? 4 : (N % 2 == 0 ? 2 : (N % 3 == 0 ? 3 : 5));
  static constexpr int B = N / A;
};

template <typename T, int N>
struct RegArr {
  T d[N];
  __device__ __forceinline__ T& operator[](int i) { return d[i]; }
};

template <int N, int DIR>
struct DFT {
  template <typename Arr>
  __device__ __forceinline__ static void run(Arr& v) {
    constexpr int A = Split<N>::A, B = Split<N>::B;
    float2 y[N];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      RegArr<float2, A> t;
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) t[n1] = v[B * n1 + n2];
      DFT<A, DIR>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = t[k1];
    }
    twiddle_all<0>(y);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      RegArr<float2, B> t;
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) t[n2] = y[n2 * A + k1];
      DFT<B, DIR>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = t[k2];
    }
  }

  // y[n2*A + k1] *= W_N^{n2*k1}, unrolled with compile-time constants
  template <int I>
  __device__ __forceinline__ static void twiddle_all(float2 (&y)[N]) {
    if constexpr (I < N) {
      constexpr int A = Split<N>::A;
      constexpr int n2 = I / A, k1 = I % A;
      constexpr int p = n2 * k1;
      if constexpr (p != 0) {
        if constexpr ((4 * p) % N == 0) {          // exact quarter turns: (DIR i)^q
          constexpr int q = (4 * p / N) % 4;
          if constexpr (q == 1) y[I] = mul_dir_i<DIR>(y[I]);
          else if constexpr (q == 2) y[I] = make_float2(-y[I].x, -y[I].y);
          else if constexpr (q == 3) y[I] = mul_dir_i<-DIR>(y[I]);
        } else {
          y[I] = cmul(y[I], ctw<DIR, long(p), long(N)>());
        }
      }
      twiddle_all<I + 1>(y);
    }
  }
};

}  // namespace ef
