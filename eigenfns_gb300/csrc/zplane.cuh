// Three-pass fused Maxwell operator for grid edges whose xy-plane fits in one
// CTA's shared memory (G = 32, 48, 64, 96, 128).
//
// One application of Θ (or of the transverse-projection preconditioner, or a
// fused Chebyshev / KPM step) to a sub-batch of vectors makes three passes over
// a workspace W laid out plane-major, [v][component][z][kx][ky] complex64:
//
//   Z-in   z-pencils, inverse: reads the transverse amplitudes (a, b), builds the
//          Cartesian curl c1 t1 + c2 t2 (frame recomputed per voxel), inverse DFT
//          along z, writes W. A tile is 16 consecutive ky at one kx, so every
//          z-plane receives 128 contiguous bytes per component.
//   Plane  one (vector, component, z) plane per task, held in shared memory:
//          inverse DFT along ky then kx, pointwise w(r) (eps^-1 or eps, with the
//          inverse transform's 1/G^3 folded in), forward DFT along x then y. The
//          first step reads W and the last writes W directly (coalesced rows).
//   Z-out  z-pencils, forward, projection onto (t1, t2), curl and the epilogue
//          (plain output, Chebyshev step, KPM step with fp64 partial sums).
//
// Compulsory traffic per voxel and vector is 16 B in + 16 B out (+ the epilogue's
// extra operands); W (48 B per voxel per vector) is written once, read and
// rewritten once by the plane pass and read once more, and is sized so that a
// sub-batch's W stays in L2 between the passes.
//
// Each DFT of length G = R1*R2 runs in place as two register steps over a buffer
// (the "four-step" split): step A gives an item the R1 samples n = t2 + R2*n1,
// applies DFT_R1 and the twiddle W_G^(t2*k1) and writes the results back to the
// same slots (slot t2 + R2*k1 holds k1); step B gives an item the R2 contiguous
// slots R2*k1 .. R2*k1+R2-1, applies DFT_R2 and writes back, so slot R2*k1 + k2
// holds output index k1 + R1*k2 (a digit-reversed order). The plane pass keeps
// that order through the pointwise multiply (its table is stored permuted to
// match) and then runs the transposed steps B^T, A^T (DFT_R2; twiddle; DFT_R1),
// which take the digit-reversed order back to natural order, so no transpose
// or reorder pass is ever needed.
#pragma once
#include <vector>

#include "common.cuh"
#include "dft.cuh"
#include "fft_passes.cuh"
#include "status.h"

namespace ef {

constexpr int kZT = 16;      // z-pass tile: consecutive ky rows at one kx
constexpr int kZThreads = 128;

struct P3Args {
  const float2* X;     // Z-in input block (m,2,N) at the sub-batch start; T1 for recurrences
  float2* W;           // workspace (mb,3,G,G,G), plane-major
  float2* out;         // Z-out output (m,2,N)
  float2* T0;          // recurrence T0 (in), T2 (out, same slot)
  float2* Y;           // bandpass accumulator
  const float2* Z;     // KPM-count probe
  double* partials;    // (mb, tiles, 2)
  const float* kax;
  const uint32_t* swap;
  const float* wperm;  // plane-pass multiplier, permuted to the digit-reversed slot order
  const float2* tw;    // (G) exp(+2 pi i j / G)
  float kn_floor;
  float s;             // 2 / lambda_max
  float c0, c1;        // recurrence coefficients
};

// twiddle W_G^(DIR * j) from the shared table of exp(+2 pi i j / G)
template <int DIR>
__device__ __forceinline__ float2 twid(const float2* tw_s, int j) {
  const float2 t = tw_s[j];
  return DIR > 0 ? t : make_float2(t.x, -t.y);
}

// R contiguous complex values from/to shared memory as 16-byte words (R even,
// address 16-byte aligned)
template <int R>
__device__ __forceinline__ void lds_row(const float2* p, float2 (&u)[R]) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < R / 2; ++i) {
    const float4 w = q[i];
    u[2 * i] = make_float2(w.x, w.y);
    u[2 * i + 1] = make_float2(w.z, w.w);
  }
}
template <int R>
__device__ __forceinline__ void sts_row(float2* p, const float2 (&u)[R]) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int i = 0; i < R / 2; ++i) q[i] = make_float4(u[2 * i].x, u[2 * i].y, u[2 * i + 1].x, u[2 * i + 1].y);
}

// ---------------------------------------------------------------------------------
// Z-in: z-pencils, inverse, with the transverse -> Cartesian build.
// grid (G*G/16, mb); X points at the sub-batch's first vector.
template <int R1, int R2, int BUILD>
__global__ void __launch_bounds__(kZThreads) zin_kernel(P3Args a) {
  constexpr int G = R1 * R2, T = kZT, ZRS = G + 2;
  static_assert(R2 % 2 == 0 && G % T == 0, "z-in split");
  __shared__ float2 tw_s[G];
  extern __shared__ float4 zin_smem[];
  float2* buf = reinterpret_cast<float2*>(zin_smem);   // [3][T][ZRS]
  for (int i = threadIdx.x; i < G; i += kZThreads) tw_s[i] = a.tw[i];
  __syncthreads();
  const long long N = (long long)G * G * G, GG = (long long)G * G;
  const int kx = blockIdx.x / (G / T), ky0 = (blockIdx.x % (G / T)) * T;
  const int v = blockIdx.y;
  const float2* Xa = a.X + (long long)v * 2 * N;
  const float2* Xb = Xa + N;
  for (int it = threadIdx.x; it < T * R2; it += kZThreads) {
    const int t2 = it % R2, r = it / R2, ky = ky0 + r;
    const long long rb = ((long long)kx * G + ky) * G;
    float2 av[R1], bv[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      av[n1] = Xa[rb + t2 + R2 * n1];
      bv[n1] = Xb[rb + t2 + R2 * n1];
    }
    float2 cx[R1], cy[R1], cz[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      const Frame f = frame_at(a.kax, a.swap, G, kx, ky, t2 + R2 * n1);
      float2 c1, c2;
      if (BUILD == BUILD_THETA) {           // c1 = -i kn b, c2 = i kn a
        c1 = make_float2(f.kn * bv[n1].y, -f.kn * bv[n1].x);
        c2 = make_float2(-f.kn * av[n1].y, f.kn * av[n1].x);
      } else {                              // c1 = i b / knr, c2 = -i a / knr
        const float ik = 1.0f / fmaxf(f.kn, a.kn_floor);
        c1 = make_float2(-bv[n1].y * ik, bv[n1].x * ik);
        c2 = make_float2(av[n1].y * ik, -av[n1].x * ik);
      }
      cx[n1] = make_float2(c1.x * f.t1x + c2.x * f.t2x, c1.y * f.t1x + c2.y * f.t2x);
      cy[n1] = make_float2(c1.x * f.t1y + c2.x * f.t2y, c1.y * f.t1y + c2.y * f.t2y);
      cz[n1] = make_float2(c1.x * f.t1z + c2.x * f.t2z, c1.y * f.t1z + c2.y * f.t2z);
    }
    DFT<R1, +1>::run(cx);
    DFT<R1, +1>::run(cy);
    DFT<R1, +1>::run(cz);
    float2* b0 = buf + r * ZRS + t2;
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      float2 x = cx[k1], y = cy[k1], z = cz[k1];
      if (k1 > 0 && t2 > 0) {
        const float2 w = twid<+1>(tw_s, t2 * k1);
        x = cmul(x, w); y = cmul(y, w); z = cmul(z, w);
      }
      b0[0 * T * ZRS + R2 * k1] = x;
      b0[1 * T * ZRS + R2 * k1] = y;
      b0[2 * T * ZRS + R2 * k1] = z;
    }
  }
  __syncthreads();
  float2* Wv = a.W + (long long)v * 3 * N;
  for (int it = threadIdx.x; it < 3 * T * R1; it += kZThreads) {
    const int r = it % T, k1 = (it / T) % R1, c = it / (T * R1);
    float2 u[R2];
    lds_row<R2>(buf + (c * T + r) * ZRS + R2 * k1, u);
    DFT<R2, +1>::run(u);
    float2* dst = Wv + (long long)c * N + (long long)kx * G + ky0 + r;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) dst[(long long)(k1 + R1 * k2) * GG] = u[k2];
  }
}

// ---------------------------------------------------------------------------------
// Plane pass: PL consecutive (vector, component, z) planes per CTA, in place in W.
// grid (3*G*mb / PL). Rows of a plane are kx, columns ky.
template <int R1, int R2, int PL, int NT>
__global__ void __launch_bounds__(NT) plane_kernel(P3Args a) {
  constexpr int G = R1 * R2, RS = G + 2, PSZ = G * RS, NROW = PL * G;
  static_assert(R2 % 2 == 0, "plane split");
  __shared__ float2 tw_s[G];
  extern __shared__ float4 plane_smem[];
  float2* S = reinterpret_cast<float2*>(plane_smem);  // [PL][G][RS]
  for (int i = threadIdx.x; i < G; i += NT) tw_s[i] = a.tw[i];
  __syncthreads();
  const long long GG = (long long)G * G;
  const long long P0 = (long long)blockIdx.x * PL;
  float2* Wp = a.W + P0 * GG;

  // y inverse, step A: global -> shared
  for (int it = threadIdx.x; it < NROW * R2; it += NT) {
    const int t2 = it % R2, row = it / R2;
    float2 u[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) u[n1] = Wp[(long long)row * G + t2 + R2 * n1];
    DFT<R1, +1>::run(u);
    float2* d = S + row * RS + t2;
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) d[R2 * k1] = (k1 && t2) ? cmul(u[k1], twid<+1>(tw_s, t2 * k1)) : u[k1];
  }
  __syncthreads();
  // y inverse, step B
  for (int it = threadIdx.x; it < NROW * R1; it += NT) {
    const int row = it % NROW, k1 = it / NROW;
    float2 u[R2];
    float2* p = S + row * RS + R2 * k1;
    lds_row<R2>(p, u);
    DFT<R2, +1>::run(u);
    sts_row<R2>(p, u);
  }
  __syncthreads();
  // x inverse, step A
  for (int it = threadIdx.x; it < PL * G * R2; it += NT) {
    const int q = it % G, t2 = (it / G) % R2, pl = it / (G * R2);
    float2* col = S + pl * PSZ + q;
    float2 u[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) u[n1] = col[(t2 + R2 * n1) * RS];
    DFT<R1, +1>::run(u);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1)
      col[(t2 + R2 * k1) * RS] = (k1 && t2) ? cmul(u[k1], twid<+1>(tw_s, t2 * k1)) : u[k1];
  }
  __syncthreads();
  // x inverse step B, pointwise multiply, x forward step B^T
  for (int it = threadIdx.x; it < PL * G * R1; it += NT) {
    const int q = it % G, k1 = (it / G) % R1, pl = it / (G * R1);
    const int z = (int)((P0 + pl) % G);
    float2* col = S + pl * PSZ + (R2 * k1) * RS + q;
    float2 u[R2];
#pragma unroll
    for (int j = 0; j < R2; ++j) u[j] = col[j * RS];
    DFT<R2, +1>::run(u);
    const float4* wq = reinterpret_cast<const float4*>(a.wperm + (long long)z * GG + ((long long)k1 * G + q) * R2);
#pragma unroll
    for (int j = 0; j < R2 / 4; ++j) {
      const float4 w = __ldg(wq + j);
      u[4 * j + 0] = cscale(u[4 * j + 0], w.x);
      u[4 * j + 1] = cscale(u[4 * j + 1], w.y);
      u[4 * j + 2] = cscale(u[4 * j + 2], w.z);
      u[4 * j + 3] = cscale(u[4 * j + 3], w.w);
    }
    DFT<R2, -1>::run(u);
#pragma unroll
    for (int j = 0; j < R2; ++j) col[j * RS] = u[j];
  }
  __syncthreads();
  // x forward, step A^T: twiddle, DFT_R1, natural kx order
  for (int it = threadIdx.x; it < PL * G * R2; it += NT) {
    const int q = it % G, t2 = (it / G) % R2, pl = it / (G * R2);
    float2* col = S + pl * PSZ + q;
    float2 u[R1];
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      const float2 x = col[(R2 * k1 + t2) * RS];
      u[k1] = (k1 && t2) ? cmul(x, twid<-1>(tw_s, t2 * k1)) : x;
    }
    DFT<R1, -1>::run(u);
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) col[(t2 + R2 * n1) * RS] = u[n1];
  }
  __syncthreads();
  // y forward, step B^T
  for (int it = threadIdx.x; it < NROW * R1; it += NT) {
    const int row = it % NROW, k1 = it / NROW;
    float2 u[R2];
    float2* p = S + row * RS + R2 * k1;
    lds_row<R2>(p, u);
    DFT<R2, -1>::run(u);
    sts_row<R2>(p, u);
  }
  __syncthreads();
  // y forward, step A^T: shared -> global, natural ky order
  for (int it = threadIdx.x; it < NROW * R2; it += NT) {
    const int t2 = it % R2, row = it / R2;
    const float2* s = S + row * RS + t2;
    float2 u[R1];
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) u[k1] = (k1 && t2) ? cmul(s[R2 * k1], twid<-1>(tw_s, t2 * k1)) : s[R2 * k1];
    DFT<R1, -1>::run(u);
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) Wp[(long long)row * G + t2 + R2 * n1] = u[n1];
  }
}

// ---------------------------------------------------------------------------------
// Z-out: z-pencils, forward, projection, curl and epilogue. The split here puts the
// large factor first (R1 >= 8) and a small power of two last, so that step B holds
// the 3 components of R2 outputs per item in registers and consecutive items write
// consecutive kz. Shared-memory slots are swizzled in 16-byte words within each
// step-B block so that 8 items with consecutive k1 read 8 distinct bank groups.
template <int CPB>
__device__ __forceinline__ int zswz(int pos) {
  const int ch = pos >> 1, blk = ch / CPB;
  const int f = CPB >= 8 ? (blk & 7) : (CPB == 4 ? ((blk >> 1) & 3) : (CPB == 2 ? ((blk >> 2) & 1) : 0));
  return (((ch ^ f)) << 1) | (pos & 1);
}

// grid (G*G/16, mb); per-vector pointers (out, X, T0, Y, Z) at the sub-batch start.
template <int R1, int R2, int EPI>
__global__ void __launch_bounds__(kZThreads) zout_kernel(P3Args a) {
  constexpr int G = R1 * R2, T = kZT, ZRS = G + 2, CPB = R2 / 2;
  static_assert(R2 == 4 || R2 == 8 || R2 == 16, "z-out split: R2 a power of two 4..16");
  static_assert(R1 >= 8 && G % T == 0, "z-out split: R1 >= 8");
  __shared__ float2 tw_s[G];
  __shared__ double red[kZThreads / 32];
  extern __shared__ float4 zout_smem[];
  float2* buf = reinterpret_cast<float2*>(zout_smem);   // [3][T][ZRS]
  for (int i = threadIdx.x; i < G; i += kZThreads) tw_s[i] = a.tw[i];
  __syncthreads();
  const long long N = (long long)G * G * G, GG = (long long)G * G;
  const int kx = blockIdx.x / (G / T), ky0 = (blockIdx.x % (G / T)) * T;
  const int v = blockIdx.y;
  const float2* Wv = a.W + (long long)v * 3 * N;
  for (int it = threadIdx.x; it < 3 * T * R2; it += kZThreads) {
    const int r = it % T, t2 = (it / T) % R2, c = it / (T * R2);
    const float2* src = Wv + (long long)c * N + (long long)kx * G + ky0 + r;
    float2 u[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) u[n1] = src[(long long)(t2 + R2 * n1) * GG];
    DFT<R1, -1>::run(u);
    float2* d = buf + (c * T + r) * ZRS;
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1)
      d[zswz<CPB>(t2 + R2 * k1)] = (k1 && t2) ? cmul(u[k1], twid<-1>(tw_s, t2 * k1)) : u[k1];
  }
  __syncthreads();
  const long long vo = (long long)v * 2 * N;
  double acc0 = 0.0, acc1 = 0.0;
  for (int it = threadIdx.x; it < T * R1; it += kZThreads) {
    const int k1 = it % R1, r = it / R1, ky = ky0 + r;
    float2 dx[R2], dy[R2], dz[R2];
#pragma unroll
    for (int h = 0; h < CPB; ++h) {
      const int pos = zswz<CPB>(R2 * k1 + 2 * h);
      const float4 wx = *reinterpret_cast<const float4*>(buf + (0 * T + r) * ZRS + pos);
      const float4 wy = *reinterpret_cast<const float4*>(buf + (1 * T + r) * ZRS + pos);
      const float4 wz = *reinterpret_cast<const float4*>(buf + (2 * T + r) * ZRS + pos);
      dx[2 * h] = make_float2(wx.x, wx.y); dx[2 * h + 1] = make_float2(wx.z, wx.w);
      dy[2 * h] = make_float2(wy.x, wy.y); dy[2 * h + 1] = make_float2(wy.z, wy.w);
      dz[2 * h] = make_float2(wz.x, wz.y); dz[2 * h + 1] = make_float2(wz.z, wz.w);
    }
    DFT<R2, -1>::run(dx);
    DFT<R2, -1>::run(dy);
    DFT<R2, -1>::run(dz);
    float f0 = 0.f, f1acc = 0.f;
    const long long rowo = ((long long)kx * G + ky) * G;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      const int kz = k1 + R1 * k2;
      const long long idx = rowo + kz;
      const Frame f = frame_at(a.kax, a.swap, G, kx, ky, kz);
      const float2 p1 = make_float2(f.t1x * dx[k2].x + f.t1y * dy[k2].x + f.t1z * dz[k2].x,
                                    f.t1x * dx[k2].y + f.t1y * dy[k2].y + f.t1z * dz[k2].y);
      const float2 p2 = make_float2(f.t2x * dx[k2].x + f.t2y * dy[k2].x + f.t2z * dz[k2].x,
                                    f.t2x * dx[k2].y + f.t2y * dy[k2].y + f.t2z * dz[k2].y);
      float2 o0, o1;
      if (EPI == EPI_PRECOND) {
        const float ik = 1.0f / fmaxf(f.kn, a.kn_floor);
        o0 = make_float2(-p2.y * ik, p2.x * ik);    // i f2 / knr
        o1 = make_float2(p1.y * ik, -p1.x * ik);    // -i f1 / knr
      } else {
        o0 = make_float2(f.kn * p2.y, -f.kn * p2.x);  // -i kn f2
        o1 = make_float2(-f.kn * p1.y, f.kn * p1.x);  //  i kn f1
      }
      if (EPI == EPI_THETA || EPI == EPI_PRECOND) {
        a.out[vo + idx] = o0;
        a.out[vo + N + idx] = o1;
      } else {
        const float2 t1a = a.X[vo + idx], t1b = a.X[vo + N + idx];
        const float2 b0 = make_float2(a.s * o0.x - t1a.x, a.s * o0.y - t1a.y);
        const float2 b1 = make_float2(a.s * o1.x - t1b.x, a.s * o1.y - t1b.y);
        if (EPI == EPI_CHEB_FIRST) {
          a.out[vo + idx] = b0;
          a.out[vo + N + idx] = b1;
          a.Y[vo + idx] = make_float2(a.c0 * t1a.x + a.c1 * b0.x, a.c0 * t1a.y + a.c1 * b0.y);
          a.Y[vo + N + idx] = make_float2(a.c0 * t1b.x + a.c1 * b1.x, a.c0 * t1b.y + a.c1 * b1.y);
        } else if (EPI == EPI_KPM_FIRST || EPI == EPI_KPM_COUNT_FIRST) {
          a.out[vo + idx] = b0;
          a.out[vo + N + idx] = b1;
          f0 += t1a.x * t1a.x + t1a.y * t1a.y + t1b.x * t1b.x + t1b.y * t1b.y;
          f1acc += t1a.x * b0.x + t1a.y * b0.y + t1b.x * b1.x + t1b.y * b1.y;
        } else {
          const float2 p0 = a.T0[vo + idx], p1v = a.T0[vo + N + idx];
          const float2 n0 = make_float2(2.f * b0.x - p0.x, 2.f * b0.y - p0.y);
          const float2 n1 = make_float2(2.f * b1.x - p1v.x, 2.f * b1.y - p1v.y);
          a.T0[vo + idx] = n0;
          a.T0[vo + N + idx] = n1;
          if (EPI == EPI_CHEB) {
            const float2 y0 = a.Y[vo + idx], y1 = a.Y[vo + N + idx];
            a.Y[vo + idx] = make_float2(fmaf(a.c1, n0.x, y0.x), fmaf(a.c1, n0.y, y0.y));
            a.Y[vo + N + idx] = make_float2(fmaf(a.c1, n1.x, y1.x), fmaf(a.c1, n1.y, y1.y));
          } else if (EPI == EPI_KPM) {
            f0 += t1a.x * t1a.x + t1a.y * t1a.y + t1b.x * t1b.x + t1b.y * t1b.y;
            f1acc += n0.x * t1a.x + n0.y * t1a.y + n1.x * t1b.x + n1.y * t1b.y;
          } else {  // EPI_KPM_COUNT: <Z, T2>
            const float2 z0 = a.Z[vo + idx], z1 = a.Z[vo + N + idx];
            f0 += z0.x * n0.x + z0.y * n0.y + z1.x * n1.x + z1.y * n1.y;
          }
        }
      }
    }
    acc0 += (double)f0;
    acc1 += (double)f1acc;
  }
  if (EPI >= EPI_KPM) {
    const double s0 = block_sum(acc0, red);
    const double s1 = block_sum(acc1, red);
    if (threadIdx.x == 0) {
      double* p = a.partials + ((long long)v * gridDim.x + blockIdx.x) * 2;
      p[0] = s0;
      p[1] = s1;
    }
  }
}

// ---------------------------------------------------------------------------------
// Plan of one grid edge for the three-pass operator.
using Launch3 = void (*)(dim3, size_t, cudaStream_t, const P3Args&);

struct Plan3 {
  int G;
  int in_R1, in_R2;        // z-in split (DFT_R1 strided, DFT_R2 contiguous)
  int pl_R1, pl_R2, PL, NT;  // plane split, planes per CTA, threads
  int out_R1, out_R2;      // z-out split
  size_t smem_z, smem_plane;
  Launch3 zin[2];          // BUILD_THETA, BUILD_PRECOND
  Launch3 plane;
  Launch3 zout[8];         // EpiMode
};

template <int R1, int R2, int B>
void launch_zin(dim3 g, size_t s, cudaStream_t st, const P3Args& a) {
  set_smem_once(zin_kernel<R1, R2, B>, s);
  ef_count_launches(1);
  zin_kernel<R1, R2, B><<<g, kZThreads, s, st>>>(a);
}
template <int R1, int R2, int PL, int NT>
void launch_plane(dim3 g, size_t s, cudaStream_t st, const P3Args& a) {
  set_smem_once(plane_kernel<R1, R2, PL, NT>, s);
  ef_count_launches(1);
  plane_kernel<R1, R2, PL, NT><<<g, NT, s, st>>>(a);
}
template <int R1, int R2, int E>
void launch_zout(dim3 g, size_t s, cudaStream_t st, const P3Args& a) {
  set_smem_once(zout_kernel<R1, R2, E>, s);
  ef_count_launches(1);
  zout_kernel<R1, R2, E><<<g, kZThreads, s, st>>>(a);
}

template <int IR1, int IR2, int PR1, int PR2, int PL, int NT, int OR1, int OR2>
Plan3 make_plan3() {
  constexpr int G = IR1 * IR2;
  static_assert(PR1 * PR2 == G && OR1 * OR2 == G, "splits of one grid edge");
  static_assert((3 * G) % PL == 0, "planes per CTA divide 3G");
  static_assert(PR2 % 4 == 0, "plane multiplier rows are read as float4");
  Plan3 p;
  p.G = G;
  p.in_R1 = IR1; p.in_R2 = IR2;
  p.pl_R1 = PR1; p.pl_R2 = PR2; p.PL = PL; p.NT = NT;
  p.out_R1 = OR1; p.out_R2 = OR2;
  p.smem_z = (size_t)3 * kZT * (G + 2) * sizeof(float2);
  p.smem_plane = (size_t)PL * G * (G + 2) * sizeof(float2);
  p.zin[0] = launch_zin<IR1, IR2, BUILD_THETA>;
  p.zin[1] = launch_zin<IR1, IR2, BUILD_PRECOND>;
  p.plane = launch_plane<PR1, PR2, PL, NT>;
  p.zout[0] = launch_zout<OR1, OR2, EPI_THETA>;
  p.zout[1] = launch_zout<OR1, OR2, EPI_PRECOND>;
  p.zout[2] = launch_zout<OR1, OR2, EPI_CHEB>;
  p.zout[3] = launch_zout<OR1, OR2, EPI_CHEB_FIRST>;
  p.zout[4] = launch_zout<OR1, OR2, EPI_KPM>;
  p.zout[5] = launch_zout<OR1, OR2, EPI_KPM_FIRST>;
  p.zout[6] = launch_zout<OR1, OR2, EPI_KPM_COUNT>;
  p.zout[7] = launch_zout<OR1, OR2, EPI_KPM_FIRST>;
  return p;
}

// plans3.cu appends the grid edges of the three-pass operator
void add_plans3(std::vector<Plan3>& v);

}  // namespace ef
