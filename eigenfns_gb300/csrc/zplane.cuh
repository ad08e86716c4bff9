// Three-pass fused Maxwell operator (grid edges 32, 48, 64, 96, 128, 192, 256).
//
// One application of Θ (or of the transverse-projection preconditioner, or a
// fused Chebyshev / KPM step) to a sub-batch of vectors makes three passes over
// a workspace W laid out plane-major, [v][component][z][kx][ky] complex64:
//
//   Z-in   z-pencils, inverse: reads the transverse amplitudes (a, b), builds the
//          Cartesian curl c1 t1 + c2 t2 (frame recomputed per voxel), inverse DFT
//          along z, writes W. A tile is 16 consecutive ky at one kx, so every
//          z-plane receives 128 contiguous bytes per component.
//   Plane  one (vector, component, z, x-class) sub-plane per task, held in shared
//          memory: inverse DFT along ky then kx, pointwise w(r) (eps^-1 or eps, with
//          the inverse transform's 1/G^3 folded in), forward DFT along x then y. The
//          first step reads W and the last writes W directly (coalesced rows).
//
// Large grid edges split the x transform between the passes so that a sub-plane
// fits in shared memory (and several fit per SM at 128): with G = Q * GX, the z-in
// pass also applies the first radix-Q step of the inverse x DFT across the Q rows
// kx' + GX*j of its tile (DFT_Q over j, then the twiddle W_G^(s kx')), leaving Q
// sub-planes of GX x G per z whose rows are the real-space x = Q n' + s after the
// plane pass's GX-point transform; the z-out pass applies the matching last step of
// the forward x DFT (twiddle W_G^(-s kx'), DFT_Q over s) before its z transform.
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
constexpr int kZThreads = 256;
// resident z-pass CTAs per SM the register budget is sized for: three up to G = 128
// (50 KB of shared memory each), two above (75-100 KB)
constexpr int z_min_blocks(int G) { return G <= 128 ? 3 : 2; }

// Work items are distributed over the threads in compile-time rounds, so that a
// thread's loads of all its items can be issued together.
#define EF_ITEMS(ITEMS, NT, ...)                                                           \
  _Pragma("unroll") for (int round_ = 0; round_ < ((ITEMS) + (NT) - 1) / (NT); ++round_) { \
    const int it = (int)threadIdx.x + round_ * (NT);                                       \
    if ((ITEMS) % (NT) == 0 || it < (ITEMS)) { __VA_ARGS__ }                               \
  }

// A z-pass tile is kZT rows: row r = j*TY + t has kx = kx0 + j*(G/Q), ky = ky0 + t
// (TY = kZT/Q consecutive ky at each of the Q x-classes' kx).
// Per-tile frame inputs staged in shared memory by the z passes: K_z for every z,
// K_x and K_y of the tile's rows, and the reference-axis switch bit of each (row, z).
template <int G, int Q>
struct ZFrame {
  static constexpr int TY = kZT / Q, GX = G / Q;
  float kz[G];
  float ky[TY];
  float kx[Q];
  uint8_t sw[kZT * G];
  __device__ __forceinline__ void load(const float* __restrict__ kax, const uint32_t* __restrict__ swap,
                                       int kx0, int ky0) {
    for (int i = threadIdx.x; i < G; i += blockDim.x) kz[i] = kax[2 * G + i];
    for (int i = threadIdx.x; i < TY; i += blockDim.x) ky[i] = kax[G + ky0 + i];
    for (int i = threadIdx.x; i < Q; i += blockDim.x) kx[i] = kax[kx0 + i * GX];
    for (int i = threadIdx.x; i < kZT * G; i += blockDim.x) {
      const int r = i / G, z = i % G;
      const unsigned b = ((unsigned)(kx0 + (r / TY) * GX) * G + ky0 + r % TY) * G + z;
      sw[i] = (uint8_t)((__ldg(swap + (b >> 5)) >> (b & 31)) & 1u);
    }
  }
  __device__ __forceinline__ Frame at(int r, int z) const {
    return make_frame(kx[r / TY], ky[r % TY], kz[z], sw[r * G + z] != 0);
  }
};

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
// Z-in: z-pencils, inverse, with the transverse -> Cartesian build, then (Q > 1) the
// first radix-Q step of the inverse x transform. grid (G*G/16, mb); X points at the
// sub-batch's first vector. W sub-plane (v, c, z, s) is GX x G at ((v*3+c)*G+z)*Q+s.
template <int R1, int R2, int Q, int BUILD>
__global__ void __launch_bounds__(kZThreads, z_min_blocks(R1 * R2)) zin_kernel(P3Args a) {
  constexpr int G = R1 * R2, T = kZT, ZRS = G + 2, NT = kZThreads, TY = T / Q, GX = G / Q;
  static_assert(R2 % 2 == 0 && G % T == 0 && T % Q == 0 && G % Q == 0, "z-in split");
  __shared__ float2 tw_s[G];
  __shared__ ZFrame<G, Q> fr;
  extern __shared__ float4 zin_smem[];
  float2* buf = reinterpret_cast<float2*>(zin_smem);   // [3][T][ZRS]
  constexpr unsigned N = (unsigned)G * G * G, GG = (unsigned)G * G;
  const int kx0 = blockIdx.x / (G / TY), ky0 = (blockIdx.x % (G / TY)) * TY;
  for (int i = threadIdx.x; i < G; i += NT) tw_s[i] = a.tw[i];
  fr.load(a.kax, a.swap, kx0, ky0);
  __syncthreads();
  const float2* Xa = a.X + (size_t)blockIdx.y * 2 * N;
  const float2* Xb = Xa + N;
  EF_ITEMS(T * R2, NT, {
    const int t2 = it % R2, r = it / R2;
    const unsigned rb = ((unsigned)(kx0 + (r / TY) * GX) * G + ky0 + r % TY) * G + t2;
    float2 av[R1], bv[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      av[n1] = Xa[rb + R2 * n1];
      bv[n1] = Xb[rb + R2 * n1];
    }
    float2 cx[R1], cy[R1], cz[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      const Frame f = fr.at(r, t2 + R2 * n1);
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
  })
  __syncthreads();
  float2* Wv = a.W + (size_t)blockIdx.y * 3 * N;
  EF_ITEMS(3 * T * R1, NT, {
    const int r = it % T, k1 = (it / T) % R1, c = it / (T * R1);
    float2 u[R2];
    float2* p = buf + (c * T + r) * ZRS + R2 * k1;
    lds_row<R2>(p, u);
    DFT<R2, +1>::run(u);
    if constexpr (Q == 1) {
      float2* dst = Wv + (size_t)c * N + (unsigned)kx0 * G + ky0 + r;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) dst[(unsigned)(k1 + R1 * k2) * GG] = u[k2];
    } else {
      sts_row<R2>(p, u);                    // slot R2*k1 + k2 now holds z = k1 + R1*k2
    }
  })
  if constexpr (Q > 1) {
    __syncthreads();
    // first radix-Q step of the inverse x DFT over the tile's Q x-classes
    EF_ITEMS(3 * TY * G, NT, {
      const int t = it % TY, pos = (it / TY) % G, c = it / (TY * G);
      const int z = pos / R2 + R1 * (pos % R2);
      float2 u[Q];
#pragma unroll
      for (int j = 0; j < Q; ++j) u[j] = buf[(c * T + j * TY + t) * ZRS + pos];
      DFT<Q, +1>::run(u);
      float2* dst = Wv + ((size_t)(c * G + z) * Q) * (GX * G) + (unsigned)kx0 * G + ky0 + t;
#pragma unroll
      for (int sidx = 0; sidx < Q; ++sidx)
        dst[(size_t)sidx * (GX * G)] = (sidx && kx0) ? cmul(u[sidx], twid<+1>(tw_s, sidx * kx0)) : u[sidx];
    })
  }
}

// ---------------------------------------------------------------------------------
// Plane pass: PL consecutive sub-planes (GX rows = x, GY = G columns = y) per CTA, in
// place in W. grid (3*G*Q*mb / PL).
template <int XR1, int XR2, int YR1, int YR2, int PL, int NT>
__global__ void __launch_bounds__(NT) plane_kernel(P3Args a) {
  constexpr int GX = XR1 * XR2, GY = YR1 * YR2, Q = GY / GX, RS = GY + 2, PSZ = GX * RS;
  constexpr int NROW = PL * GX;
  static_assert(XR2 % 4 == 0 && YR2 % 2 == 0 && GY % GX == 0, "plane split");
  __shared__ float2 tw_s[GY];                        // W_GY^j; W_GX^j = tw_s[Q*j]
  extern __shared__ float4 plane_smem[];
  float2* S = reinterpret_cast<float2*>(plane_smem);  // [PL][GX][RS]
  for (int i = threadIdx.x; i < GY; i += NT) tw_s[i] = a.tw[i];
  __syncthreads();
  constexpr unsigned SP = (unsigned)GX * GY;         // sub-plane size
  const size_t P0 = (size_t)blockIdx.x * PL;
  float2* Wp = a.W + P0 * SP;

  // y inverse, step A: global -> shared
  EF_ITEMS(NROW * YR2, NT, {
    const int t2 = it % YR2, row = it / YR2;
    float2 u[YR1];
#pragma unroll
    for (int n1 = 0; n1 < YR1; ++n1) u[n1] = Wp[(unsigned)row * GY + t2 + YR2 * n1];
    DFT<YR1, +1>::run(u);
    float2* d = S + row * RS + t2;
#pragma unroll
    for (int k1 = 0; k1 < YR1; ++k1) d[YR2 * k1] = (k1 && t2) ? cmul(u[k1], twid<+1>(tw_s, t2 * k1)) : u[k1];
  })
  __syncthreads();
  // y inverse, step B
  EF_ITEMS(NROW * YR1, NT, {
    const int row = it % NROW, k1 = it / NROW;
    float2 u[YR2];
    float2* p = S + row * RS + YR2 * k1;
    lds_row<YR2>(p, u);
    DFT<YR2, +1>::run(u);
    sts_row<YR2>(p, u);
  })
  __syncthreads();
  // the pointwise factors of the x step B items, fetched now so that their latency
  // overlaps the x step A; sub-plane (z, s) table at ((z*Q + s) * GX * GY)
  constexpr int XB_ROUNDS = (PL * GY * XR1 + NT - 1) / NT;
  float4 wpre[XB_ROUNDS][XR2 / 4];
  EF_ITEMS(PL * GY * XR1, NT, {
    const int q = it % GY, k1 = (it / GY) % XR1, pl = it / (GY * XR1);
    const size_t P = P0 + pl;
    const unsigned zs = (unsigned)(P % ((size_t)GY * Q));       // z*Q + s
    const float4* wq = reinterpret_cast<const float4*>(a.wperm + zs * SP + ((unsigned)k1 * GY + q) * XR2);
#pragma unroll
    for (int j = 0; j < XR2 / 4; ++j) wpre[round_][j] = __ldg(wq + j);
  })
  // x inverse, step A (columns of length GX; twiddles W_GX = tw_s[Q*.])
  EF_ITEMS(PL * GY * XR2, NT, {
    const int q = it % GY, t2 = (it / GY) % XR2, pl = it / (GY * XR2);
    float2* col = S + pl * PSZ + q;
    float2 u[XR1];
#pragma unroll
    for (int n1 = 0; n1 < XR1; ++n1) u[n1] = col[(t2 + XR2 * n1) * RS];
    DFT<XR1, +1>::run(u);
#pragma unroll
    for (int k1 = 0; k1 < XR1; ++k1)
      col[(t2 + XR2 * k1) * RS] = (k1 && t2) ? cmul(u[k1], twid<+1>(tw_s, Q * t2 * k1)) : u[k1];
  })
  __syncthreads();
  // x inverse step B, pointwise multiply, x forward step B^T
  EF_ITEMS(PL * GY * XR1, NT, {
    const int q = it % GY, k1 = (it / GY) % XR1, pl = it / (GY * XR1);
    float2* col = S + pl * PSZ + (XR2 * k1) * RS + q;
    const float4* w4 = wpre[round_];
    float2 u[XR2];
#pragma unroll
    for (int j = 0; j < XR2; ++j) u[j] = col[j * RS];
    DFT<XR2, +1>::run(u);
#pragma unroll
    for (int j = 0; j < XR2 / 4; ++j) {
      u[4 * j + 0] = cscale(u[4 * j + 0], w4[j].x);
      u[4 * j + 1] = cscale(u[4 * j + 1], w4[j].y);
      u[4 * j + 2] = cscale(u[4 * j + 2], w4[j].z);
      u[4 * j + 3] = cscale(u[4 * j + 3], w4[j].w);
    }
    DFT<XR2, -1>::run(u);
#pragma unroll
    for (int j = 0; j < XR2; ++j) col[j * RS] = u[j];
  })
  __syncthreads();
  // x forward, step A^T: twiddle, DFT_XR1, natural x order
  EF_ITEMS(PL * GY * XR2, NT, {
    const int q = it % GY, t2 = (it / GY) % XR2, pl = it / (GY * XR2);
    float2* col = S + pl * PSZ + q;
    float2 u[XR1];
#pragma unroll
    for (int k1 = 0; k1 < XR1; ++k1) {
      const float2 x = col[(XR2 * k1 + t2) * RS];
      u[k1] = (k1 && t2) ? cmul(x, twid<-1>(tw_s, Q * t2 * k1)) : x;
    }
    DFT<XR1, -1>::run(u);
#pragma unroll
    for (int n1 = 0; n1 < XR1; ++n1) col[(t2 + XR2 * n1) * RS] = u[n1];
  })
  __syncthreads();
  // y forward, step B^T
  EF_ITEMS(NROW * YR1, NT, {
    const int row = it % NROW, k1 = it / NROW;
    float2 u[YR2];
    float2* p = S + row * RS + YR2 * k1;
    lds_row<YR2>(p, u);
    DFT<YR2, -1>::run(u);
    sts_row<YR2>(p, u);
  })
  __syncthreads();
  // y forward, step A^T: shared -> global, natural ky order
  EF_ITEMS(NROW * YR2, NT, {
    const int t2 = it % YR2, row = it / YR2;
    const float2* sp = S + row * RS + t2;
    float2 u[YR1];
#pragma unroll
    for (int k1 = 0; k1 < YR1; ++k1) u[k1] = (k1 && t2) ? cmul(sp[YR2 * k1], twid<-1>(tw_s, t2 * k1)) : sp[YR2 * k1];
    DFT<YR1, -1>::run(u);
#pragma unroll
    for (int n1 = 0; n1 < YR1; ++n1) Wp[(unsigned)row * GY + t2 + YR2 * n1] = u[n1];
  })
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
template <int R1, int R2, int Q, int EPI>
__global__ void __launch_bounds__(kZThreads, z_min_blocks(R1 * R2)) zout_kernel(P3Args a) {
  constexpr int G = R1 * R2, T = kZT, ZRS = G + 2, CPB = R2 / 2, NT = kZThreads;
  constexpr int TY = T / Q, GX = G / Q;
  static_assert(R2 == 4 || R2 == 8 || R2 == 16, "z-out split: R2 a power of two 4..16");
  static_assert(R1 >= 8 && G % T == 0 && T % Q == 0, "z-out split: R1 >= 8");
  __shared__ float2 tw_s[G];
  __shared__ double red[NT / 32];
  __shared__ ZFrame<G, Q> fr;
  extern __shared__ float4 zout_smem[];
  float2* buf = reinterpret_cast<float2*>(zout_smem);   // [3][T][ZRS]
  constexpr unsigned N = (unsigned)G * G * G, GG = (unsigned)G * G;
  const int kx0 = blockIdx.x / (G / TY), ky0 = (blockIdx.x % (G / TY)) * TY;
  for (int i = threadIdx.x; i < G; i += NT) tw_s[i] = a.tw[i];
  fr.load(a.kax, a.swap, kx0, ky0);
  const float2* Wv = a.W + (size_t)blockIdx.y * 3 * N;
  if constexpr (Q > 1) {
    __syncthreads();
    // last radix-Q step of the forward x DFT: twiddle W_G^(-s kx0), DFT_Q over s; the
    // natural-z values land in the swizzled slots the z step A reads and rewrites
    EF_ITEMS(3 * TY * G, NT, {
      const int t = it % TY, z = (it / TY) % G, c = it / (TY * G);
      const float2* src = Wv + ((size_t)(c * G + z) * Q) * (GX * G) + (unsigned)kx0 * G + ky0 + t;
      float2 u[Q];
#pragma unroll
      for (int sidx = 0; sidx < Q; ++sidx) {
        const float2 v = src[(size_t)sidx * (GX * G)];
        u[sidx] = (sidx && kx0) ? cmul(v, twid<-1>(tw_s, sidx * kx0)) : v;
      }
      DFT<Q, -1>::run(u);
#pragma unroll
      for (int j = 0; j < Q; ++j) buf[(c * T + j * TY + t) * ZRS + zswz<CPB>(z)] = u[j];
    })
  }
  __syncthreads();
  EF_ITEMS(3 * T * R2, NT, {
    const int r = it % T, t2 = (it / T) % R2, c = it / (T * R2);
    float2* d = buf + (c * T + r) * ZRS;
    float2 u[R1];
    if constexpr (Q == 1) {
      const float2* src = Wv + (size_t)c * N + (unsigned)kx0 * G + ky0 + r + (unsigned)t2 * GG;
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) u[n1] = src[(unsigned)(R2 * n1) * GG];
    } else {
      // this item reads and rewrites the same R1 slots, so no other item's data moves
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) u[n1] = d[zswz<CPB>(t2 + R2 * n1)];
    }
    DFT<R1, -1>::run(u);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1)
      d[zswz<CPB>(t2 + R2 * k1)] = (k1 && t2) ? cmul(u[k1], twid<-1>(tw_s, t2 * k1)) : u[k1];
  })
  __syncthreads();
  const size_t vo = (size_t)blockIdx.y * 2 * N;
  double acc0 = 0.0, acc1 = 0.0;
  EF_ITEMS(T * R1, NT, {
    const int k1 = it % R1, r = it / R1, ky = ky0 + r % TY, kx = kx0 + (r / TY) * GX;
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
    const unsigned rowo = ((unsigned)kx * G + ky) * G;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      const int kz = k1 + R1 * k2;
      const size_t idx = rowo + kz;
      const Frame f = fr.at(r, kz);
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
  })
  if (EPI >= EPI_KPM) {
    const double s0 = block_sum(acc0, red);
    const double s1 = block_sum(acc1, red);
    if (threadIdx.x == 0) {
      double* p = a.partials + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 2;
      p[0] = s0;
      p[1] = s1;
    }
  }
}

// ---------------------------------------------------------------------------------
// Plan of one grid edge for the three-pass operator.
using Launch3 = void (*)(dim3, size_t, cudaStream_t, const P3Args&);

struct Plan3 {
  int G, Q;                // grid edge, x-classes (sub-planes per z)
  int in_R1, in_R2;        // z-in split (DFT_R1 strided, DFT_R2 contiguous)
  int x_R1, x_R2;          // sub-plane x split (length G/Q)
  int y_R1, y_R2;          // sub-plane y split (length G)
  int PL, NT;              // sub-planes per CTA, threads
  int out_R1, out_R2;      // z-out split
  size_t smem_z, smem_plane;
  Launch3 zin[2];          // BUILD_THETA, BUILD_PRECOND
  Launch3 plane;
  Launch3 zout[8];         // EpiMode
};

template <int R1, int R2, int Q, int B>
void launch_zin(dim3 g, size_t s, cudaStream_t st, const P3Args& a) {
  set_smem_once(zin_kernel<R1, R2, Q, B>, s);
  ef_count_launches(1);
  zin_kernel<R1, R2, Q, B><<<g, kZThreads, s, st>>>(a);
}
template <int XR1, int XR2, int YR1, int YR2, int PL, int NT>
void launch_plane(dim3 g, size_t s, cudaStream_t st, const P3Args& a) {
  set_smem_once(plane_kernel<XR1, XR2, YR1, YR2, PL, NT>, s);
  ef_count_launches(1);
  plane_kernel<XR1, XR2, YR1, YR2, PL, NT><<<g, NT, s, st>>>(a);
}
template <int R1, int R2, int Q, int E>
void launch_zout(dim3 g, size_t s, cudaStream_t st, const P3Args& a) {
  set_smem_once(zout_kernel<R1, R2, Q, E>, s);
  ef_count_launches(1);
  zout_kernel<R1, R2, Q, E><<<g, kZThreads, s, st>>>(a);
}

template <int Q, int IR1, int IR2, int XR1, int XR2, int YR1, int YR2, int PL, int NT, int OR1, int OR2>
Plan3 make_plan3() {
  constexpr int G = IR1 * IR2;
  static_assert(YR1 * YR2 == G && OR1 * OR2 == G && XR1 * XR2 * Q == G, "splits of one grid edge");
  static_assert((3 * G * Q) % PL == 0, "sub-planes per CTA divide 3GQ");
  static_assert(XR2 % 4 == 0, "plane multiplier rows are read as float4");
  Plan3 p;
  p.G = G; p.Q = Q;
  p.in_R1 = IR1; p.in_R2 = IR2;
  p.x_R1 = XR1; p.x_R2 = XR2; p.y_R1 = YR1; p.y_R2 = YR2;
  p.PL = PL; p.NT = NT;
  p.out_R1 = OR1; p.out_R2 = OR2;
  p.smem_z = (size_t)3 * kZT * (G + 2) * sizeof(float2);
  p.smem_plane = (size_t)PL * (G / Q) * (G + 2) * sizeof(float2);
  p.zin[0] = launch_zin<IR1, IR2, Q, BUILD_THETA>;
  p.zin[1] = launch_zin<IR1, IR2, Q, BUILD_PRECOND>;
  p.plane = launch_plane<XR1, XR2, YR1, YR2, PL, NT>;
  p.zout[0] = launch_zout<OR1, OR2, Q, EPI_THETA>;
  p.zout[1] = launch_zout<OR1, OR2, Q, EPI_PRECOND>;
  p.zout[2] = launch_zout<OR1, OR2, Q, EPI_CHEB>;
  p.zout[3] = launch_zout<OR1, OR2, Q, EPI_CHEB_FIRST>;
  p.zout[4] = launch_zout<OR1, OR2, Q, EPI_KPM>;
  p.zout[5] = launch_zout<OR1, OR2, Q, EPI_KPM_FIRST>;
  p.zout[6] = launch_zout<OR1, OR2, Q, EPI_KPM_COUNT>;
  p.zout[7] = launch_zout<OR1, OR2, Q, EPI_KPM_FIRST>;   // first count step: same epilogue
  return p;
}

// plans3.cu appends the grid edges of the three-pass operator
void add_plans3(std::vector<Plan3>& v);

}  // namespace ef
