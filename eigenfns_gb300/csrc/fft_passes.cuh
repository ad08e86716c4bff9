// Pencil FFT passes of the fused Maxwell operator.
//
// One application of Θ (or of the transverse-projection preconditioner) to a
// sub-batch of vectors is five passes over a 3-component workspace E
// (mb, 3, G, G, G) complex64, all in place after the first:
//
//   A  z-pencils, inverse: builds the Cartesian curl c1 t1 + c2 t2 from the
//      transverse amplitudes (frame recomputed per voxel from 1-D tables),
//      then transforms along z                                     X -> E
//   B  y-pencils, inverse                                          E -> E
//   C  x-pencils: inverse, pointwise w(r) (eps^-1 or eps, with 1/G^3 folded
//      in), forward                                                E -> E
//   D  y-pencils, forward                                          E -> E
//   E  z-pencils, forward, then the projection onto (t1, t2), the curl and a
//      fused epilogue (plain output, Chebyshev step, KPM step)     E -> out
//
// Each pencil of length G = R1*R2 is transformed in two register steps with
// one shared-memory exchange: step 1 gives each work item the R1 elements
// n = t2 + R2*n1, applies DFT_R1 and the twiddle W_G^(t2*k1); step 2 gives
// each item the R2 values of one k1 and applies DFT_R2, producing output
// frequencies f = k1 + R1*k2. Global loads and stores are arranged so that
// consecutive threads touch consecutive addresses (along z for the z-passes,
// across z-columns for the y- and x-passes).
#pragma once
#include "common.cuh"
#include "dft.cuh"

namespace ef {

constexpr int kThreads = 256;

// tile-size caps (tuning knobs; the defaults are the tuned values)
#ifndef EF_NZ_CAP
#define EF_NZ_CAP 32          // y/x passes: z-columns per tile
#endif
#ifndef EF_NRZ_ITEMS
#define EF_NRZ_ITEMS 256      // z passes: work items per tile
#endif

template <int R1_, int R2_>
struct Geo {
  static constexpr int R1 = R1_, R2 = R2_, G = R1_ * R2_;
  static constexpr int XS = R2_ + 1;                       // exchange row stride
  static constexpr int PS0 = R1_ * XS > G ? R1_ * XS : G;
  static constexpr int PS = (PS0 % 2 == 0) ? PS0 + 1 : PS0;  // odd pencil stride
  // z-pass rows per tile: largest divisor of G*G with NR*G <= 1024
  static constexpr int nr_pick() {
    int c = 1024 / G > 0 ? 1024 / G : 1;
    while (c > 1 && !((G * G) % c == 0)) --c;
    return c;
  }
  static constexpr int NR = nr_pick();
  // z-pass rows per tile: pass A (this split R1 <= R2) runs NRA*R2 items in its first
  // step, pass E (R1 >= R2) runs NRE*R1 in its second; both stay within 256 items
  // and 64 KB of exchange buffer
  static constexpr int nrz_pick(int per_row) {
    int c = EF_NRZ_ITEMS / per_row > 0 ? EF_NRZ_ITEMS / per_row : 1;
    while (c > 1 && (((G * G) % c) != 0 || 3 * c * PS * 8 > 64 * 1024)) --c;
    return c;
  }
  static constexpr int NRA = nrz_pick(R2_);
  static constexpr int NRE = nrz_pick(R1_);
  // y/x-pass z-columns per tile: largest divisor of G not above EF_NZ_CAP
  static constexpr int nz_pick() {
    int c = G < EF_NZ_CAP ? G : EF_NZ_CAP;
    while (c > 1 && (G % c != 0 || 2 * c * PS * 8 > 80 * 1024)) --c;
    return c;
  }
  static constexpr int NZ = nz_pick();
};

// epilogue modes of pass E
enum EpiMode : int {
  EPI_THETA = 0,     // out = (-i kn f2, i kn f1)
  EPI_PRECOND = 1,   // out = (i f2 / knr, -i f1 / knr)
  EPI_CHEB = 2,      // T2 = 2(s Θ T1 - T1) - T0 -> T0 slot, Y += c T2
  EPI_CHEB_FIRST = 3,// T1 = s Θ T0 - T0 -> out, Y = c0 T0 + c1 T1
  EPI_KPM = 4,       // T2 = 2(s Θ T1 - T1) - T0 -> T0 slot, partials <T1,T1>, <T2,T1>
  EPI_KPM_FIRST = 5, // T1 = s Θ Z - Z -> out, partials <Z,Z>, <Z,T1>
  EPI_KPM_COUNT = 6, // T2 as EPI_KPM, partial <Z,T2>
  EPI_KPM_COUNT_FIRST = 7, // T1 = s Θ Z - Z -> out, partials <Z,Z>, <Z,T1>
};

// pointwise multiplier kinds of pass C
enum WMode : int {
  W_INV_EPS = 0,     // inverse, * eps^-1/N, forward (Θ)
  W_EPS = 1,         // inverse, * eps/N, forward (preconditioner)
  W_INV_ONLY = 2,    // inverse only, * 1/N * scale[v]          (h_realspace)
  W_INV_ONLY_EPS = 3 // inverse only, * eps^-1/N * scale[v]    (e_realspace)
};
// build kinds of pass A
enum BuildMode : int { BUILD_THETA = 0, BUILD_PRECOND = 1, BUILD_CART = 2 };

struct PassArgs {
  const float2* X;    // operator input block (m,2,N) (pass A); T1 for recurrences
  float2* E;          // workspace (mb,3,N)
  float2* out;        // pass E output (m,2,N)
  float2* T0;         // recurrence T0 (in), T2 (out, same slot)
  float2* Y;          // bandpass accumulator
  const float2* Z;    // KPM-count probe
  double* partials;   // (mb, tiles, 2)
  const float* kax;
  const uint32_t* swap;
  const float* w;     // pass C multiplier (N)
  const float2* tw;   // (G) exp(+2 pi i j / G)
  const float* vscale;// per-vector scale of the inverse-only x pass
  float inv_n;        // 1 / G^3
  float kn_floor;
  float s;            // 2 / lambda_max
  float c0, c1;       // recurrence coefficients
  int G;
};

template <class GEO>
__device__ __forceinline__ void load_twiddles(float2* tw_s, const float2* tw) {
  for (int i = threadIdx.x; i < GEO::G; i += blockDim.x) tw_s[i] = tw[i];
}

template <int DIR>
__device__ __forceinline__ float2 tw_get(const float2* tw_s, int idx) {
  float2 t = tw_s[idx];
  return DIR > 0 ? t : make_float2(t.x, -t.y);
}

// step 1 from shared memory (natural order) into the exchange buffer
template <class GEO, int DIR>
__device__ __forceinline__ void step1_smem(const float2* nat, float2* exch, const float2* tw_s,
                                           int q, int t2) {
  float2 v[GEO::R1];
#pragma unroll
  for (int n1 = 0; n1 < GEO::R1; ++n1) v[n1] = nat[q * GEO::PS + t2 + GEO::R2 * n1];
  DFT<GEO::R1, DIR>::run(v);
#pragma unroll
  for (int k1 = 0; k1 < GEO::R1; ++k1) {
    float2 r = (k1 == 0 || t2 == 0) ? v[k1] : cmul(v[k1], tw_get<DIR>(tw_s, t2 * k1));
    exch[q * GEO::PS + k1 * GEO::XS + t2] = r;
  }
}

// step 1 from global memory (elements base + (t2 + R2*n1) * stride)
template <class GEO, int DIR>
__device__ __forceinline__ void step1_global(const float2* __restrict__ src, long long base,
                                             long long stride, float2* exch, const float2* tw_s,
                                             int q, int t2) {
  float2 v[GEO::R1];
#pragma unroll
  for (int n1 = 0; n1 < GEO::R1; ++n1) v[n1] = src[base + (long long)(t2 + GEO::R2 * n1) * stride];
  DFT<GEO::R1, DIR>::run(v);
#pragma unroll
  for (int k1 = 0; k1 < GEO::R1; ++k1) {
    float2 r = (k1 == 0 || t2 == 0) ? v[k1] : cmul(v[k1], tw_get<DIR>(tw_s, t2 * k1));
    exch[q * GEO::PS + k1 * GEO::XS + t2] = r;
  }
}

// step 2: read one k1 row of the exchange buffer, DFT_R2; u[k2] is frequency k1 + R1*k2
template <class GEO, int DIR>
__device__ __forceinline__ void step2_load(const float2* exch, int q, int k1, float2 (&u)[GEO::R2]) {
#pragma unroll
  for (int t2 = 0; t2 < GEO::R2; ++t2) u[t2] = exch[q * GEO::PS + k1 * GEO::XS + t2];
  DFT<GEO::R2, DIR>::run(u);
}

// ---------------------------------------------------------------------------------
// Pass A: z-pencils, inverse, with the transverse -> Cartesian build. GEO is the
// split with the small factor first (R1 <= R2): a first-step item owns voxels
// z = t2 + R2*n1 of one row, loads (a, b), computes the frame once per voxel and
// transforms all 3 Cartesian components in registers.
// grid (G*G/NRA, mb); X points at the sub-batch's first vector.
template <class GEO, int BUILD>
__global__ void __launch_bounds__(kThreads) pass_a_kernel(PassArgs a) {
  constexpr int G = GEO::G, NR = GEO::NRA, NP = 3 * NR, R1 = GEO::R1, R2 = GEO::R2;
  extern __shared__ float2 smem[];
  float2* exch = smem;
  float2* tw_s = exch + NP * GEO::PS;
  load_twiddles<GEO>(tw_s, a.tw);
  __syncthreads();
  const long long N = (long long)G * G * G;
  const int v = blockIdx.y;
  const int row0 = blockIdx.x * NR;
  const float2* Xa = a.X + (long long)v * 2 * N;
  const float2* Xb = Xa + N;
  for (int it = threadIdx.x; it < NR * R2; it += blockDim.x) {
    const int r = it / R2, t2 = it % R2;
    const int row = row0 + r, x = row / G, y = row % G;
    float2 cx[R1], cy[R1], cz[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      const int z = t2 + R2 * n1;
      const long long idx = (long long)row * G + z;
      const Frame f = frame_at(a.kax, a.swap, G, x, y, z);
      const float2 av = Xa[idx], bv = Xb[idx];
      float2 c1, c2;
      if (BUILD == BUILD_THETA) {           // c1 = -i kn b, c2 = i kn a
        c1 = make_float2(f.kn * bv.y, -f.kn * bv.x);
        c2 = make_float2(-f.kn * av.y, f.kn * av.x);
      } else if (BUILD == BUILD_PRECOND) {  // c1 = i b / knr, c2 = -i a / knr
        const float ik = 1.0f / fmaxf(f.kn, a.kn_floor);
        c1 = make_float2(-bv.y * ik, bv.x * ik);
        c2 = make_float2(av.y * ik, -av.x * ik);
      } else {                               // Cartesian H: a t1 + b t2
        c1 = av;
        c2 = bv;
      }
      cx[n1] = make_float2(c1.x * f.t1x + c2.x * f.t2x, c1.y * f.t1x + c2.y * f.t2x);
      cy[n1] = make_float2(c1.x * f.t1y + c2.x * f.t2y, c1.y * f.t1y + c2.y * f.t2y);
      cz[n1] = make_float2(c1.x * f.t1z + c2.x * f.t2z, c1.y * f.t1z + c2.y * f.t2z);
    }
    DFT<R1, +1>::run(cx);
    DFT<R1, +1>::run(cy);
    DFT<R1, +1>::run(cz);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      float2 tw = make_float2(1.f, 0.f);
      if (k1 != 0 && t2 != 0) tw = tw_get<+1>(tw_s, t2 * k1);
      const int o = k1 * GEO::XS + t2;
      exch[(0 * NR + r) * GEO::PS + o] = (k1 && t2) ? cmul(cx[k1], tw) : cx[k1];
      exch[(1 * NR + r) * GEO::PS + o] = (k1 && t2) ? cmul(cy[k1], tw) : cy[k1];
      exch[(2 * NR + r) * GEO::PS + o] = (k1 && t2) ? cmul(cz[k1], tw) : cz[k1];
    }
  }
  __syncthreads();
  float2* E = a.E + (long long)v * 3 * N;
  for (int it = threadIdx.x; it < NP * R1; it += blockDim.x) {
    const int q = it / R1, k1 = it % R1;
    float2 u[R2];
    step2_load<GEO, +1>(exch, q, k1, u);
    const int j = q / NR, r = q % NR;
    float2* dst = E + (long long)j * N + (long long)(row0 + r) * G;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) dst[k1 + R1 * k2] = u[k2];
  }
}

// ---------------------------------------------------------------------------------
// Pass B / D: y-pencils in place. grid (G/NZ, G, 3*mb).
template <class GEO, int DIR>
__global__ void __launch_bounds__(kThreads) pass_y_kernel(PassArgs a) {
  constexpr int G = GEO::G, NZ = GEO::NZ;
  extern __shared__ float2 smem[];
  float2* exch = smem;
  float2* tw_s = exch + NZ * GEO::PS;
  load_twiddles<GEO>(tw_s, a.tw);
  __syncthreads();
  const long long N = (long long)G * G * G;
  const int z0 = blockIdx.x * NZ, x = blockIdx.y;
  float2* E = a.E + (long long)blockIdx.z * N;
  const long long base = (long long)x * G * G + z0;
  for (int it = threadIdx.x; it < NZ * GEO::R2; it += blockDim.x) {
    int q = it % NZ, t2 = it / NZ;
    step1_global<GEO, DIR>(E, base + q, G, exch, tw_s, q, t2);
  }
  __syncthreads();
  for (int it = threadIdx.x; it < NZ * GEO::R1; it += blockDim.x) {
    int q = it % NZ, k1 = it / NZ;
    float2 u[GEO::R2];
    step2_load<GEO, DIR>(exch, q, k1, u);
#pragma unroll
    for (int k2 = 0; k2 < GEO::R2; ++k2) E[base + q + (long long)(k1 + GEO::R1 * k2) * G] = u[k2];
  }
}

// ---------------------------------------------------------------------------------
// Pass C: x-pencils in place: inverse, multiply by w, forward. grid (G/NZ, G, 3*mb).
template <class GEO, int WM>
__global__ void __launch_bounds__(kThreads) pass_c_kernel(PassArgs a) {
  constexpr int G = GEO::G, NZ = GEO::NZ;
  constexpr bool INV_ONLY = (WM == W_INV_ONLY || WM == W_INV_ONLY_EPS);
  extern __shared__ float2 smem[];
  float2* nat = smem;
  float2* exch = smem + NZ * GEO::PS;
  float2* tw_s = exch + NZ * GEO::PS;
  load_twiddles<GEO>(tw_s, a.tw);
  __syncthreads();
  const long long N = (long long)G * G * G;
  const long long GG = (long long)G * G;
  const int z0 = blockIdx.x * NZ, y = blockIdx.y;
  float2* E = a.E + (long long)blockIdx.z * N;
  const long long base = (long long)y * G + z0;
  for (int it = threadIdx.x; it < NZ * GEO::R2; it += blockDim.x) {
    int q = it % NZ, t2 = it / NZ;
    step1_global<GEO, +1>(E, base + q, GG, exch, tw_s, q, t2);
  }
  __syncthreads();
  float vs = 1.0f;
  if (INV_ONLY && a.vscale) vs = a.vscale[blockIdx.z / 3];
  for (int it = threadIdx.x; it < NZ * GEO::R1; it += blockDim.x) {
    int q = it % NZ, k1 = it / NZ;
    float2 u[GEO::R2];
    step2_load<GEO, +1>(exch, q, k1, u);
#pragma unroll
    for (int k2 = 0; k2 < GEO::R2; ++k2) {
      int xx = k1 + GEO::R1 * k2;
      if (INV_ONLY) {
        float wv = (WM == W_INV_ONLY) ? a.inv_n : a.w[xx * GG + base + q];
        E[base + q + (long long)xx * GG] = cscale(u[k2], wv * vs);
      } else {
        nat[q * GEO::PS + xx] = cscale(u[k2], a.w[xx * GG + base + q]);
      }
    }
  }
  if (INV_ONLY) return;
  __syncthreads();
  for (int it = threadIdx.x; it < NZ * GEO::R2; it += blockDim.x) {
    int q = it % NZ, t2 = it / NZ;
    step1_smem<GEO, -1>(nat, exch, tw_s, q, t2);
  }
  __syncthreads();
  for (int it = threadIdx.x; it < NZ * GEO::R1; it += blockDim.x) {
    int q = it % NZ, k1 = it / NZ;
    float2 u[GEO::R2];
    step2_load<GEO, -1>(exch, q, k1, u);
#pragma unroll
    for (int k2 = 0; k2 < GEO::R2; ++k2) E[base + q + (long long)(k1 + GEO::R1 * k2) * GG] = u[k2];
  }
}

// ---------------------------------------------------------------------------------
// Pass E: z-pencils, forward, projection and epilogue. grid (G*G/NR, mb).
// Per-vector vectors (out, X, T0, Y, Z) point at the sub-batch's first vector.
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  }
  return s;
}

// Pass E: z-pencils, forward, then projection, curl and the epilogue. GEO is the
// split with the large factor first (R1 >= R2): a second-step item owns outputs
// z = k1 + R1*k2 of one row for all 3 components, so the frame is computed once
// per voxel and the projection happens in registers.
// grid (G*G/NRE, mb); per-vector pointers (out, X, T0, Y, Z) at the sub-batch start.
template <class GEO, int EPI>
__global__ void __launch_bounds__(kThreads) pass_e_kernel(PassArgs a) {
  constexpr int G = GEO::G, NR = GEO::NRE, NP = 3 * NR, R1 = GEO::R1, R2 = GEO::R2;
  extern __shared__ float2 smem[];
  float2* exch = smem;
  float2* tw_s = exch + NP * GEO::PS;
  __shared__ double red[kThreads / 32];
  load_twiddles<GEO>(tw_s, a.tw);
  __syncthreads();
  const long long N = (long long)G * G * G;
  const int v = blockIdx.y;
  const int row0 = blockIdx.x * NR;
  const float2* E = a.E + (long long)v * 3 * N;
  for (int it = threadIdx.x; it < NP * R2; it += blockDim.x) {
    const int q = it / R2, t2 = it % R2;
    const int j = q / NR, r = q % NR;
    step1_global<GEO, -1>(E, (long long)j * N + (long long)(row0 + r) * G, 1, exch, tw_s, q, t2);
  }
  __syncthreads();
  const long long vo = (long long)v * 2 * N;
  double acc0 = 0.0, acc1 = 0.0;
  for (int it = threadIdx.x; it < NR * R1; it += blockDim.x) {
    const int r = it / R1, k1 = it % R1;
    const int row = row0 + r, x = row / G, y = row % G;
    float2 dx[R2], dy[R2], dz[R2];
    step2_load<GEO, -1>(exch, 0 * NR + r, k1, dx);
    step2_load<GEO, -1>(exch, 1 * NR + r, k1, dy);
    step2_load<GEO, -1>(exch, 2 * NR + r, k1, dz);
    float f0 = 0.f, f1acc = 0.f;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      const int z = k1 + R1 * k2;
      const long long idx = (long long)row * G + z;
      const Frame f = frame_at(a.kax, a.swap, G, x, y, z);
      const float2 f1 = make_float2(f.t1x * dx[k2].x + f.t1y * dy[k2].x + f.t1z * dz[k2].x,
                                    f.t1x * dx[k2].y + f.t1y * dy[k2].y + f.t1z * dz[k2].y);
      const float2 f2 = make_float2(f.t2x * dx[k2].x + f.t2y * dy[k2].x + f.t2z * dz[k2].x,
                                    f.t2x * dx[k2].y + f.t2y * dy[k2].y + f.t2z * dz[k2].y);
      float2 o0, o1;
      if (EPI == EPI_PRECOND) {
        const float ik = 1.0f / fmaxf(f.kn, a.kn_floor);
        o0 = make_float2(-f2.y * ik, f2.x * ik);   // i f2 / knr
        o1 = make_float2(f1.y * ik, -f1.x * ik);   // -i f1 / knr
      } else {
        o0 = make_float2(f.kn * f2.y, -f.kn * f2.x); // -i kn f2
        o1 = make_float2(-f.kn * f1.y, f.kn * f1.x); //  i kn f1
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
          const float2 p0 = a.T0[vo + idx], p1 = a.T0[vo + N + idx];
          const float2 n0 = make_float2(2.f * b0.x - p0.x, 2.f * b0.y - p0.y);
          const float2 n1 = make_float2(2.f * b1.x - p1.x, 2.f * b1.y - p1.y);
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

}  // namespace ef
