// Block linear algebra on complex64 vector blocks.
//
// Reference: eigenfns/solver.py -- gram (:35-43, true-fp32 X^H Y), combine and
// the tensordot rotations (:49-57, :106, :125, :256, :261-262, :274), row norms and
// Rayleigh quotients (:228-238), residual R = HX - lam X (:229), random start
// blocks (:196-205); eigenfns/chebyshev.py:248 and scripts/exp/exp_kpm_dos.py:139-140
// (Rademacher probes).
//
// Gram: each CTA owns a 32x32 output tile and one K-chunk (split-K). Products and
// short runs of sums are fp32 on the CUDA cores; every 256 k-values the fp32 run
// is flushed into an fp64 accumulator, and the chunks are reduced in fp64 in a
// fixed order, so results are deterministic and the long sums keep fp64 accuracy.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "dft.cuh"
#include "status.h"

using namespace ef;

namespace {

constexpr int GT = 32;      // gram output tile edge
constexpr int GBK = 32;     // k-values per shared-memory stage
constexpr int GFLUSH = 8;   // stages per fp64 flush (256 k-values)
constexpr int GTHREADS = 64;

__global__ void __launch_bounds__(GTHREADS) gram_kernel(const float2* __restrict__ A,
                                                        const float2* __restrict__ B, int ma, int mb,
                                                        long long K, long long kchunk,
                                                        double2* __restrict__ partial) {
  __shared__ float2 As[GBK][GT + 1];
  __shared__ float2 Bs[GBK][GT + 1];
  const int tid = threadIdx.x;
  const int ti = tid & 7, tj = tid >> 3;
  const int i0 = blockIdx.x * GT, j0 = blockIdx.y * GT;
  const long long kbeg = (long long)blockIdx.z * kchunk;
  long long kend = kbeg + kchunk;
  if (kend > K) kend = K;
  float accr[4][4], acci[4][4];
  double dr[4][4], di[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) { accr[r][c] = acci[r][c] = 0.f; dr[r][c] = di[r][c] = 0.0; }
  int stage = 0;
  for (long long k0 = kbeg; k0 < kend; k0 += GBK) {
    // cooperative load of a 32 x 32 tile of A and of B (row, k), transposed into smem
#pragma unroll
    for (int l = 0; l < (GT * GBK) / GTHREADS; ++l) {
      int e = tid + l * GTHREADS;
      int row = e / GBK, kk = e % GBK;
      long long k = k0 + kk;
      float2 va = make_float2(0.f, 0.f), vb = make_float2(0.f, 0.f);
      if (k < kend) {
        if (i0 + row < ma) va = A[(long long)(i0 + row) * K + k];
        if (j0 + row < mb) vb = B[(long long)(j0 + row) * K + k];
      }
      As[kk][row] = va;
      Bs[kk][row] = vb;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < GBK; ++kk) {
      float2 a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ti + 8 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tj + 8 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          // conj(a) * b
          accr[r][c] = fmaf(a[r].x, b[c].x, fmaf(a[r].y, b[c].y, accr[r][c]));
          acci[r][c] = fmaf(a[r].x, b[c].y, fmaf(-a[r].y, b[c].x, acci[r][c]));
        }
    }
    __syncthreads();
    if (++stage == GFLUSH) {
      stage = 0;
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          dr[r][c] += (double)accr[r][c];
          di[r][c] += (double)acci[r][c];
          accr[r][c] = acci[r][c] = 0.f;
        }
    }
  }
  // partials are entry-major, (ma*mb, nsplit), so the reduction reads contiguous runs
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int i = i0 + ti + 8 * r, j = j0 + tj + 8 * c;
      if (i < ma && j < mb)
        partial[((long long)i * mb + j) * gridDim.z + blockIdx.z] =
            make_double2(dr[r][c] + (double)accr[r][c], di[r][c] + (double)acci[r][c]);
    }
}

// Pipelined variant for 16-byte aligned rows of even length: 128 threads own a 32x32
// tile (2 x 4 outputs each), tiles of A and B rows stream through two shared-memory
// stages with cp.async while the previous stage is multiplied. fp32 inside the CTA's
// K-chunk, fp64 across chunks.
constexpr int PG_THREADS = 128;
constexpr int PG_BK = 32;                 // complex k-values per stage
constexpr int PG_LD = PG_BK + 2;          // row stride in float2 (272 B, 16-byte aligned)

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__global__ void __launch_bounds__(PG_THREADS) gram_pipe_kernel(const float2* __restrict__ A,
                                                               const float2* __restrict__ B, int ma,
                                                               int mb, long long K, long long kchunk,
                                                               double2* __restrict__ partial) {
  __shared__ __align__(16) float2 As[2][GT][PG_LD];
  __shared__ __align__(16) float2 Bs[2][GT][PG_LD];
  const int tid = threadIdx.x;
  const int ti = tid & 15, tj = tid >> 4;   // rows ti, ti+16; cols tj + 8c
  const int i0 = blockIdx.x * GT, j0 = blockIdx.y * GT;
  const long long kbeg = (long long)blockIdx.z * kchunk;
  long long kend = kbeg + kchunk;
  if (kend > K) kend = K;
  const int nst = (int)((kend - kbeg + PG_BK - 1) / PG_BK);
  // each stage: 32 rows x 16 chunks of 16 B for A and for B = 1024 copies, 8 per thread
  auto issue = [&](int stage, int buf) {
    const long long k0 = kbeg + (long long)stage * PG_BK;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      int e = tid + l * PG_THREADS;      // 0..511
      int row = e >> 4, ch = e & 15;     // chunk of 2 complex values
      long long k = k0 + 2 * ch;
      long long left = kend - k;
      int bytes = left >= 2 ? 16 : (left == 1 ? 8 : 0);
      int ra = i0 + row, rb = j0 + row;
      const float2* ga = A + (long long)(ra < ma ? ra : 0) * K + (bytes ? k : 0);
      const float2* gb = B + (long long)(rb < mb ? rb : 0) * K + (bytes ? k : 0);
      cp_async16(&As[buf][row][2 * ch], ga, ra < ma ? bytes : 0);
      cp_async16(&Bs[buf][row][2 * ch], gb, rb < mb ? bytes : 0);
    }
    cp_async_commit();
  };
  // two fp32 levels: a stage's 32 products, then the chunk's sum of stage sums
  float accr[2][4], acci[2][4], totr[2][4], toti[2][4];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) accr[r][c] = acci[r][c] = totr[r][c] = toti[r][c] = 0.f;
  if (nst > 0) issue(0, 0);
  for (int st = 0; st < nst; ++st) {
    const int buf = st & 1;
    if (st + 1 < nst) {
      issue(st + 1, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < PG_BK; ++kk) {
      float2 a0 = As[buf][ti][kk], a1 = As[buf][ti + 16][kk];
      float2 b[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[buf][tj + 8 * c][kk];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        accr[0][c] = fmaf(a0.x, b[c].x, fmaf(a0.y, b[c].y, accr[0][c]));
        acci[0][c] = fmaf(a0.x, b[c].y, fmaf(-a0.y, b[c].x, acci[0][c]));
        accr[1][c] = fmaf(a1.x, b[c].x, fmaf(a1.y, b[c].y, accr[1][c]));
        acci[1][c] = fmaf(a1.x, b[c].y, fmaf(-a1.y, b[c].x, acci[1][c]));
      }
    }
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        totr[r][c] += accr[r][c];
        toti[r][c] += acci[r][c];
        accr[r][c] = acci[r][c] = 0.f;
      }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int i = i0 + ti + 16 * r, j = j0 + tj + 8 * c;
      if (i < ma && j < mb)
        partial[((long long)i * mb + j) * gridDim.z + blockIdx.z] =
            make_double2((double)totr[r][c], (double)toti[r][c]);
    }
}

// one warp per Gram entry: lanes stride the entry's contiguous split partials, then a
// fixed shuffle tree (deterministic run to run)
__global__ void gram_reduce_kernel(const double2* __restrict__ partial, int nsplit, int n,
                                   double2* __restrict__ G) {
  const int e = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= n) return;
  const double2* p = partial + (long long)e * nsplit;
  double sr = 0.0, si = 0.0;
  for (int s = lane; s < nsplit; s += 32) {
    double2 v = p[s];
    sr += v.x;
    si += v.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (lane == 0) G[e] = make_double2(sr, si);
}

int gram_splits(int ma, int mb, long long K) {
  long long tiles = (long long)((ma + GT - 1) / GT) * ((mb + GT - 1) / GT);
  long long target = 4096 / (tiles > 0 ? tiles : 1);
  long long maxs = (K + 255) / 256;     // at least 256 k-values per chunk (small K: more CTAs)
  long long s = target < maxs ? target : maxs;
  if (s < 1) s = 1;
  return (int)s;
}

// ---- rotation ---------------------------------------------------------------------
constexpr int RT = 32;      // outputs per thread
constexpr int RTHREADS = 256;

__global__ void __launch_bounds__(RTHREADS) rotate_kernel(const float2* __restrict__ C,
                                                          const float2* S, float2* out, int m_in,
                                                          int m_out, long long K, int mode) {
  extern __shared__ float4 Cs4[];  // (m_in, RT) slice of C for this output tile, 2 complex per float4
  float2* Cs = reinterpret_cast<float2*>(Cs4);
  const int i0 = blockIdx.y * RT;
  const int nt = (m_out - i0) < RT ? (m_out - i0) : RT;
  for (int e = threadIdx.x; e < m_in * RT; e += blockDim.x) {
    int j = e / RT, ii = e % RT;
    Cs[e] = (ii < nt) ? C[(long long)j * m_out + i0 + ii] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  constexpr int JU = 4;   // rows of S loaded together
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
       k += (long long)gridDim.x * blockDim.x) {
    float2 acc[RT];
#pragma unroll
    for (int ii = 0; ii < RT; ++ii) acc[ii] = make_float2(0.f, 0.f);
    int j = 0;
    for (; j + JU <= m_in; j += JU) {
      float2 sv[JU];
#pragma unroll
      for (int u = 0; u < JU; ++u) sv[u] = S[(long long)(j + u) * K + k];
#pragma unroll
      for (int u = 0; u < JU; ++u) {
        const float4* cj = Cs4 + (j + u) * (RT / 2);
#pragma unroll
        for (int h = 0; h < RT / 2; ++h) {
          float4 c = cj[h];
          float2 s2 = sv[u];
          acc[2 * h].x = fmaf(c.x, s2.x, fmaf(-c.y, s2.y, acc[2 * h].x));
          acc[2 * h].y = fmaf(c.x, s2.y, fmaf(c.y, s2.x, acc[2 * h].y));
          acc[2 * h + 1].x = fmaf(c.z, s2.x, fmaf(-c.w, s2.y, acc[2 * h + 1].x));
          acc[2 * h + 1].y = fmaf(c.z, s2.y, fmaf(c.w, s2.x, acc[2 * h + 1].y));
        }
      }
    }
    for (; j < m_in; ++j) {
      float2 s2 = S[(long long)j * K + k];
      const float4* cj = Cs4 + j * (RT / 2);
#pragma unroll
      for (int h = 0; h < RT / 2; ++h) {
        float4 c = cj[h];
        acc[2 * h].x = fmaf(c.x, s2.x, fmaf(-c.y, s2.y, acc[2 * h].x));
        acc[2 * h].y = fmaf(c.x, s2.y, fmaf(c.y, s2.x, acc[2 * h].y));
        acc[2 * h + 1].x = fmaf(c.z, s2.x, fmaf(-c.w, s2.y, acc[2 * h + 1].x));
        acc[2 * h + 1].y = fmaf(c.z, s2.y, fmaf(c.w, s2.x, acc[2 * h + 1].y));
      }
    }
#pragma unroll
    for (int ii = 0; ii < RT; ++ii) {
      if (ii < nt) {
        float2* o = out + (long long)(i0 + ii) * K + k;
        if (mode == 0) *o = acc[ii];
        else if (mode > 0) { float2 v = *o; *o = make_float2(v.x + acc[ii].x, v.y + acc[ii].y); }
        else { float2 v = *o; *o = make_float2(v.x - acc[ii].x, v.y - acc[ii].y); }
      }
    }
  }
}

// Tiled variant for 16-byte aligned rows of even length and m_out <= 64 per CTA row:
// a CTA owns 128 k-columns for up to 8*TI outputs; S rows (16 at a time) and the
// matching C rows stream through two cp.async shared-memory stages; each thread keeps
// a 4 (k) x TI (outputs) complex register tile, so every shared load feeds 8-16 FMAs.
constexpr int RK_T = 256, RK_KT = 128, RK_JB = 16;

template <int TI>
__global__ void __launch_bounds__(RK_T) rotate_tiled_kernel(const float2* __restrict__ C,
                                                            const float2* S, float2* out, int m_in,
                                                            int m_out, long long K, int mode) {
  constexpr int MO = 8 * TI;                            // outputs per CTA
  __shared__ __align__(16) float2 Ss[2][RK_JB][RK_KT];  // 32 KB
  __shared__ __align__(16) float2 Cs[2][RK_JB][MO];
  const int tid = threadIdx.x, kg = tid & 31, ig = tid >> 5;
  const long long k0 = (long long)blockIdx.x * RK_KT;
  const int i0 = blockIdx.y * MO;
  const int nst = (m_in + RK_JB - 1) / RK_JB;
  auto issue = [&](int st, int buf) {
    const int j0 = st * RK_JB;
    // S: 16 rows x 128 complex = 1024 chunks of 16 B, 4 per thread
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const int e = tid + l * RK_T;
      const int r = e >> 6, ch = e & 63;               // row, chunk of 2 complex
      const long long k = k0 + 2 * ch;
      const long long left = K - k;
      int bytes = left >= 2 ? 16 : (left == 1 ? 8 : 0);
      if (j0 + r >= m_in) bytes = 0;
      const float2* g = S + (long long)(j0 + r < m_in ? j0 + r : 0) * K + (bytes ? k : 0);
      unsigned sa = (unsigned)__cvta_generic_to_shared(&Ss[buf][r][2 * ch]);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(g), "r"(bytes));
    }
    // C: 16 rows x MO complex; chunks of 2 complex
    for (int e = tid; e < RK_JB * MO / 2; e += RK_T) {
      const int r = e / (MO / 2), ch = e % (MO / 2);
      const int i = i0 + 2 * ch;
      int bytes = 0;
      if (j0 + r < m_in && i < m_out) bytes = (i + 1 < m_out) ? 16 : 8;
      const float2* g = C + (long long)(j0 + r < m_in ? j0 + r : 0) * m_out + (bytes ? i : 0);
      unsigned sa = (unsigned)__cvta_generic_to_shared(&Cs[buf][r][2 * ch]);
      // C rows are 8-byte aligned only: copy as two 8-byte pieces
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(g), "r"(bytes >= 8 ? 8 : 0));
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa + 8), "l"(g + (bytes == 16 ? 1 : 0)),
                   "r"(bytes == 16 ? 8 : 0));
    }
    asm volatile("cp.async.commit_group;\n" ::);
  };
  float2 acc[4][TI];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < TI; ++t) acc[q][t] = make_float2(0.f, 0.f);
  issue(0, 0);
  for (int st = 0; st < nst; ++st) {
    const int buf = st & 1;
    if (st + 1 < nst) {
      issue(st + 1, buf ^ 1);
      asm volatile("cp.async.wait_group 1;\n" ::);
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::);
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < RK_JB; ++jj) {
      const float4 s01 = *reinterpret_cast<const float4*>(&Ss[buf][jj][4 * kg]);
      const float4 s23 = *reinterpret_cast<const float4*>(&Ss[buf][jj][4 * kg + 2]);
      const float2 sv[4] = {make_float2(s01.x, s01.y), make_float2(s01.z, s01.w),
                            make_float2(s23.x, s23.y), make_float2(s23.z, s23.w)};
#pragma unroll
      for (int t2 = 0; t2 < TI; t2 += 2) {
        const float4 cc = *reinterpret_cast<const float4*>(&Cs[buf][jj][ig * TI + t2]);
        const float2 c0 = make_float2(cc.x, cc.y), c1 = make_float2(cc.z, cc.w);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          acc[q][t2].x = fmaf(c0.x, sv[q].x, fmaf(-c0.y, sv[q].y, acc[q][t2].x));
          acc[q][t2].y = fmaf(c0.x, sv[q].y, fmaf(c0.y, sv[q].x, acc[q][t2].y));
          acc[q][t2 + 1].x = fmaf(c1.x, sv[q].x, fmaf(-c1.y, sv[q].y, acc[q][t2 + 1].x));
          acc[q][t2 + 1].y = fmaf(c1.x, sv[q].y, fmaf(c1.y, sv[q].x, acc[q][t2 + 1].y));
        }
      }
    }
    __syncthreads();
  }
  // every S column of this CTA's k-range has been read: outputs may alias S when gridDim.y == 1
#pragma unroll
  for (int t = 0; t < TI; ++t) {
    const int i = i0 + ig * TI + t;
    if (i >= m_out) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long k = k0 + 4 * kg + q;
      if (k >= K) continue;
      float2* o = out + (long long)i * K + k;
      if (mode == 0) *o = acc[q][t];
      else if (mode > 0) { float2 v = *o; *o = make_float2(v.x + acc[q][t].x, v.y + acc[q][t].y); }
      else { float2 v = *o; *o = make_float2(v.x - acc[q][t].x, v.y - acc[q][t].y); }
    }
  }
}

// ---- per-row statistics ----------------------------------------------------------
// For each row i: <A_i, B_i> (complex), |A_i|^2, |B_i|^2. Products in fp32, runs of
// 32 float4 loads flushed into fp64, chunks reduced in fp64 in a fixed order. SAME: B is
// A (row norms of one block): each value is loaded once and used as both operands, the
// same arithmetic on half the traffic.
constexpr int DTHREADS = 256;

template <bool SAME>
__global__ void __launch_bounds__(DTHREADS) rowstats_kernel(const float4* __restrict__ A,
                                                            const float4* __restrict__ B,
                                                            long long K2, long long kchunk,
                                                            double4* partial) {
  __shared__ double red[4][DTHREADS / 32];
  const int row = blockIdx.y;
  const long long kb = (long long)blockIdx.x * kchunk;
  long long ke = kb + kchunk;
  if (ke > K2) ke = K2;
  const float4* a = A + (long long)row * K2;
  const float4* b = B + (long long)row * K2;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  constexpr int U = 4;
  for (long long k0 = kb; k0 < ke; k0 += (long long)U * 8 * blockDim.x) {
    // 8 rounds of U independent loads, summed in fp32, then flushed to fp64
    float f[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
    for (int r = 0; r < 8; ++r) {
      float4 x[U], y[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        long long k = k0 + ((long long)r * U + u) * blockDim.x + threadIdx.x;
        bool ok = k < ke;
        x[u] = ok ? a[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (!SAME) y[u] = ok ? b[k] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        float4 p = x[u], q = SAME ? x[u] : y[u];
        f[0] = fmaf(p.x, q.x, fmaf(p.y, q.y, fmaf(p.z, q.z, fmaf(p.w, q.w, f[0]))));
        f[1] = fmaf(p.x, q.y, fmaf(-p.y, q.x, fmaf(p.z, q.w, fmaf(-p.w, q.z, f[1]))));
        f[2] = fmaf(p.x, p.x, fmaf(p.y, p.y, fmaf(p.z, p.z, fmaf(p.w, p.w, f[2]))));
        f[3] = fmaf(q.x, q.x, fmaf(q.y, q.y, fmaf(q.z, q.z, fmaf(q.w, q.w, f[3]))));
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) s[q] += (double)f[q];
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) red[q][threadIdx.x >> 5] = s[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < DTHREADS / 32; ++w)
#pragma unroll
      for (int q = 0; q < 4; ++q) t[q] += red[q][w];
    partial[(long long)row * gridDim.x + blockIdx.x] = make_double4(t[0], t[1], t[2], t[3]);
  }
}

// R = HX - lam[row] X and |R|^2 per row (fp32 runs flushed to fp64)
__global__ void __launch_bounds__(DTHREADS) residual_norm_kernel(const float4* __restrict__ HX,
                                                                 const float4* __restrict__ X,
                                                                 const double* __restrict__ lam,
                                                                 float4* R, long long K2,
                                                                 long long kchunk, double* partial) {
  __shared__ double red[DTHREADS / 32];
  const int row = blockIdx.y;
  const long long kb = (long long)blockIdx.x * kchunk;
  long long ke = kb + kchunk;
  if (ke > K2) ke = K2;
  const float l = (float)lam[row];
  const float4* h = HX + (long long)row * K2;
  const float4* x = X + (long long)row * K2;
  float4* r = R + (long long)row * K2;
  double s = 0.0;
  constexpr int U = 4;
  for (long long k0 = kb; k0 < ke; k0 += (long long)U * 8 * blockDim.x) {
    float f = 0.f;
#pragma unroll 2
    for (int q = 0; q < 8; ++q) {
      float4 hv[U], xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        long long k = k0 + ((long long)q * U + u) * blockDim.x + threadIdx.x;
        bool ok = k < ke;
        hv[u] = ok ? h[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        xv[u] = ok ? x[k] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        long long k = k0 + ((long long)q * U + u) * blockDim.x + threadIdx.x;
        float4 v = make_float4(hv[u].x - l * xv[u].x, hv[u].y - l * xv[u].y, hv[u].z - l * xv[u].z,
                               hv[u].w - l * xv[u].w);
        if (k < ke) r[k] = v;
        f = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, f))));
      }
    }
    s += (double)f;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < DTHREADS / 32; ++w) t += red[w];
    partial[(long long)row * gridDim.x + blockIdx.x] = t;
  }
}

__global__ void sum_rows_kernel(const double* partial, int nchunk, int m, double* out) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  double t = 0.0;
  for (int c = 0; c < nchunk; ++c) t += partial[(long long)row * nchunk + c];
  out[row] = t;
}

__global__ void rowstats_reduce_kernel(const double4* partial, int nchunk, int m, double4* out) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = 0; c < nchunk; ++c) {
    double4 p = partial[(long long)row * nchunk + c];
    t[0] += p.x; t[1] += p.y; t[2] += p.z; t[3] += p.w;
  }
  out[row] = make_double4(t[0], t[1], t[2], t[3]);
}

// rows of odd complex length fall back to the scalar kernel below
__global__ void __launch_bounds__(DTHREADS) rowstats_scalar_kernel(const float2* __restrict__ A,
                                                                   const float2* __restrict__ B,
                                                                   long long K, long long kchunk,
                                                                   double4* partial) {
  __shared__ double red[4][DTHREADS / 32];
  const int row = blockIdx.y;
  const long long kb = (long long)blockIdx.x * kchunk;
  long long ke = kb + kchunk;
  if (ke > K) ke = K;
  const float2* a = A + (long long)row * K;
  const float2* b = B + (long long)row * K;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long k = kb + threadIdx.x; k < ke; k += blockDim.x) {
    float2 x = a[k], y = b[k];
    s[0] += (double)x.x * y.x + (double)x.y * y.y;
    s[1] += (double)x.x * y.y - (double)x.y * y.x;
    s[2] += (double)x.x * x.x + (double)x.y * x.y;
    s[3] += (double)y.x * y.x + (double)y.y * y.y;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) red[q][threadIdx.x >> 5] = s[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < DTHREADS / 32; ++w)
#pragma unroll
      for (int q = 0; q < 4; ++q) t[q] += red[q][w];
    partial[(long long)row * gridDim.x + blockIdx.x] = make_double4(t[0], t[1], t[2], t[3]);
  }
}

int rowdot_chunks(long long K) {
  long long c = (K + 65535) / 65536;
  if (c < 1) c = 1;
  if (c > 1024) c = 1024;
  return (int)c;
}

// ---- elementwise --------------------------------------------------------------------
__global__ void residual_kernel(const float2* HX, const float2* X, const double* lam, float2* R,
                                long long K, long long total) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    float l = (float)lam[i / K];
    float2 h = HX[i], x = X[i];
    R[i] = make_float2(h.x - l * x.x, h.y - l * x.y);
  }
}

__global__ void scale_rows_kernel(float2* X, const double* scale, long long K, long long total) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    float s = (float)scale[i / K];
    float2 x = X[i];
    X[i] = make_float2(x.x * s, x.y * s);
  }
}

__global__ void axpby_kernel(const float2* X, float2* Y, long long n, float a, float b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float2 x = X[i], y = Y[i];
    Y[i] = make_float2(a * x.x + b * y.x, a * x.y + b * y.y);
  }
}

// splitmix64 finaliser; the same words as the oracle's counter generator
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void rand_kernel(const float* kax, int G, float2* X, long long total, uint64_t key,
                            int kind) {
  const long long N = (long long)G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    uint64_t w = mix64(key + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull);
    long long vox = i % N;
    int z = vox % G, y = (vox / G) % G, x = vox / ((long long)G * G);
    bool live = !(kax[x] == 0.f && kax[G + y] == 0.f && kax[2 * G + z] == 0.f);
    float2 v;
    if (kind == EF_RAND_NORMAL) {
      float u1 = ((float)(w >> 40) + 0.5f) * 5.9604644775390625e-08f;
      float u2 = ((float)((w >> 16) & 0xFFFFFFull) + 0.5f) * 5.9604644775390625e-08f;
      float r = sqrtf(-2.0f * logf(u1));
      float ang = 6.2831855f * u2;
      float sn, cs;
      sincosf(ang, &sn, &cs);
      v = make_float2(r * cs, r * sn);
    } else {
      float re = ((w >> 63) & 1ull) ? -1.f : 1.f;
      if (kind == EF_RAND_RADEMACHER) {
        v = make_float2(re, 0.f);
      } else {
        float im = ((w >> 62) & 1ull) ? -1.f : 1.f;
        const float h = 0.70710678f;
        v = make_float2(re * h, im * h);
      }
    }
    X[i] = live ? v : make_float2(0.f, 0.f);
  }
}

__global__ void mask_kernel(const float* kax, int G, float2* X, long long total) {
  const long long N = (long long)G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long vox = i % N;
    int z = vox % G, y = (vox / G) % G, x = vox / ((long long)G * G);
    if (kax[x] == 0.f && kax[G + y] == 0.f && kax[2 * G + z] == 0.f) X[i] = make_float2(0.f, 0.f);
  }
}

int grid_for(long long total) {
  long long b = (total + 255) / 256;
  const long long cap = 16LL * ef::sm_count();     // two waves of 8 resident 256-thread CTAs
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

// ---- Gram with a fixed scratch area owned by the library --------------------------
// ef_gram_noalloc serves callers that have no way to hand the library device
// scratch memory: a host program in another language whose only device memory is
// the vectors it already owns, or a service running under a fixed device-memory
// budget that forbids allocations after start-up. Its split-K partial sums live in
// this file-scope array instead of a caller-provided work buffer. Every GPU that
// loads the library holds the array until the process exits.
constexpr size_t kNoallocScratchBytes = (size_t)8 << 20;   // 8 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};   // device address of the array, per device

// The array's name in host code is only a stand-in: ask the runtime for its device
// address, once per device, with that device current.
int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ef_fail(EF_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return ef_fail(EF_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return ef_fail(EF_ERR_CUDA, "cudaGetSymbolAddress of the gram scratch failed");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return EF_OK;
}
}  // namespace

// ef_gram runs on the tensor cores (ef_gram_tc) from 16 x 32 up (measured at K = 4.2M:
// 32x32 0.53 vs 0.79 ms, 64x32 0.73 vs 1.49, 96x96 3.5 vs 6.5) and on the CUDA cores
// below, where the tensor-core kernel's fixed cost per K-stage dominates;
// EF_GRAM_KERNEL=tc|simt overrides
inline bool gram_use_tc(int ma, int mb) { return (long long)ma * mb >= 16 * 32; }

namespace ef {
bool gram_tune_get(int ma, int mb, int* kernel, int* units);
int* tc_error_dev();
int tc_rotate_max_rows(int m_out, int mode);
int tc_rotate_launch(const float* C, int ldc, const float* S, float* out, int m_in, int m_out,
                     long long K, int mode, cudaStream_t st);
}  // namespace ef

extern "C" {

size_t ef_gram_workspace_bytes(int ma, int mb, long long K) {
  if (ma <= 0 || mb <= 0 || K <= 0) return 0;
  const size_t simt = (size_t)gram_splits(ma, mb, K) * ma * mb * sizeof(double2) + 256;
  const size_t tc = ef_gram_tc_workspace_bytes(ma, mb, K);
  return simt > tc ? simt : tc;
}

int ef_gram(const float* A, const float* B, int ma, int mb, long long K, double* G, void* work,
            size_t work_bytes, void* stream) {
  if (!A || !B || !G || ma <= 0 || mb <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad gram arguments");
  if (!work || work_bytes < ef_gram_workspace_bytes(ma, mb, K))
    return ef_fail(EF_ERR_WORKSPACE, "gram work buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  const bool pipe = (K % 2 == 0) && ((((uintptr_t)A) | ((uintptr_t)B)) % 16 == 0);
  int tuned = 0;
  ef::gram_tune_get(ma, mb, &tuned, nullptr);
  const char* kern = getenv("EF_GRAM_KERNEL");
  const bool tc = kern ? strcmp(kern, "tc") == 0 : (tuned ? tuned == 1 : gram_use_tc(ma, mb));
  if (tc && pipe) return ef_gram_tc(A, B, ma, mb, K, G, ef::tc_error_dev(), work, work_bytes, stream);
  int ns = gram_splits(ma, mb, K);
  long long kchunk = (K + ns - 1) / ns;
  kchunk = (kchunk + GBK - 1) / GBK * GBK;
  ns = (int)((K + kchunk - 1) / kchunk);
  dim3 grid((ma + GT - 1) / GT, (mb + GT - 1) / GT, ns);
  ef_count_launches(1);
  if (pipe)
    gram_pipe_kernel<<<grid, PG_THREADS, 0, st>>>((const float2*)A, (const float2*)B, ma, mb, K,
                                                  kchunk, (double2*)work);
  else
    gram_kernel<<<grid, GTHREADS, 0, st>>>((const float2*)A, (const float2*)B, ma, mb, K, kchunk,
                                          (double2*)work);
  int n = ma * mb;
  ef_count_launches(1);
  gram_reduce_kernel<<<(n + 7) / 8, 256, 0, st>>>((const double2*)work, ns, n, (double2*)G);
  return ef_check_launch();
}

int ef_gram_noalloc(const float* A, const float* B, int ma, int mb, long long K, double* G,
                    void* stream) {
  if (!A || !B || !G || ma <= 0 || mb <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad gram arguments");
  const size_t per_split = (size_t)ma * mb * sizeof(double2);
  if (per_split > kNoallocScratchBytes)
    return ef_fail(EF_ERR_TOO_LARGE, "gram_noalloc: ma*mb*16 bytes exceeds the fixed 8 MiB scratch");
  void* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != EF_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int ns = gram_splits(ma, mb, K);
  const int cap = (int)(kNoallocScratchBytes / per_split);
  if (ns > cap) ns = cap;
  long long kchunk = (K + ns - 1) / ns;
  kchunk = (kchunk + GBK - 1) / GBK * GBK;
  ns = (int)((K + kchunk - 1) / kchunk);
  dim3 grid((ma + GT - 1) / GT, (mb + GT - 1) / GT, ns);
  const bool pipe = (K % 2 == 0) && ((((uintptr_t)A) | ((uintptr_t)B)) % 16 == 0);
  ef_count_launches(2);
  if (pipe)
    gram_pipe_kernel<<<grid, PG_THREADS, 0, st>>>((const float2*)A, (const float2*)B, ma, mb, K,
                                                  kchunk, (double2*)scratch);
  else
    gram_kernel<<<grid, GTHREADS, 0, st>>>((const float2*)A, (const float2*)B, ma, mb, K, kchunk,
                                          (double2*)scratch);
  int n = ma * mb;
  gram_reduce_kernel<<<(n + 7) / 8, 256, 0, st>>>((const double2*)scratch, ns, n, (double2*)G);
  return ef_check_launch();
}

int ef_rotate(const float* C, const float* S, float* out, int m_in, int m_out, long long K, int mode,
              void* stream) {
  if (!C || !S || !out || m_in <= 0 || m_out <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad rotate arguments");
  const bool tiled = (K % 2 == 0) && ((((uintptr_t)S) | ((uintptr_t)out)) % 16 == 0);
  const int TIc = m_out <= 16 ? 2 : (m_out <= 32 ? 4 : 8);
  int ty = tiled ? (m_out + 8 * TIc - 1) / (8 * TIc) : (m_out + RT - 1) / RT;
  const char* s0 = (const char*)S;
  const char* s1 = s0 + (size_t)m_in * K * sizeof(float2);
  const char* o0 = (const char*)out;
  const char* o1 = o0 + (size_t)m_out * K * sizeof(float2);
  bool overlap = (o0 < s1) && (s0 < o1);
  if (overlap && !(o0 == s0 && m_out <= 32 && ty == 1))
    return ef_fail(EF_ERR_INVALID, "rotate: out may alias S only exactly and with m_out <= 32");
  cudaStream_t st = (cudaStream_t)stream;
  const char* kern = getenv("EF_ROTATE_KERNEL");
  const bool simt = kern && strcmp(kern, "simt") == 0;
  if (!simt && tiled) {
    // tensor cores: output groups of <= 64 columns; a pass holds a bounded number of
    // input rows (the accumulate modes also stage the current output)
    if (overlap) {
      if (m_in <= ef::tc_rotate_max_rows(m_out, mode))
        return ef::tc_rotate_launch(C, m_out, S, out, m_in, m_out, K, mode, st);
    } else {
      int rc = EF_OK;
      for (int i0 = 0; i0 < m_out && rc == EF_OK; i0 += 64) {
        const int mo = m_out - i0 < 64 ? m_out - i0 : 64;
        const int cap0 = ef::tc_rotate_max_rows(mo, mode);
        const int chunk = m_in <= cap0 ? cap0 : ef::tc_rotate_max_rows(mo, 1);
        for (int j0 = 0; j0 < m_in && rc == EF_OK; j0 += chunk) {
          const int mi = m_in - j0 < chunk ? m_in - j0 : chunk;
          const int md = j0 == 0 ? mode : (mode == 0 ? 1 : mode);
          rc = ef::tc_rotate_launch(C + 2 * ((long long)j0 * m_out + i0), m_out, S + 2 * (long long)j0 * K,
                                    out + 2 * (long long)i0 * K, mi, mo, K, md, st);
        }
      }
      return rc;
    }
  }
  if ((size_t)m_in * RT * sizeof(float2) > 200 * 1024) return ef_fail(EF_ERR_TOO_LARGE, "m_in too large for rotate");
  if (tiled) {
    dim3 g((unsigned)((K + RK_KT - 1) / RK_KT), ty);
    ef_count_launches(1);
    if (TIc == 2)
      rotate_tiled_kernel<2><<<g, RK_T, 0, st>>>((const float2*)C, (const float2*)S, (float2*)out, m_in, m_out, K, mode);
    else if (TIc == 4)
      rotate_tiled_kernel<4><<<g, RK_T, 0, st>>>((const float2*)C, (const float2*)S, (float2*)out, m_in, m_out, K, mode);
    else
      rotate_tiled_kernel<8><<<g, RK_T, 0, st>>>((const float2*)C, (const float2*)S, (float2*)out, m_in, m_out, K, mode);
    return ef_check_launch();
  }
  size_t smem = (size_t)m_in * RT * sizeof(float2);
  set_smem_once(rotate_kernel, smem);
  long long bx = (K + RTHREADS - 1) / RTHREADS;
  long long cap = (8LL * ef::sm_count() + ty - 1) / ty;
  if (bx > cap) bx = cap;
  ef_count_launches(1);
  rotate_kernel<<<dim3((unsigned)bx, ty), RTHREADS, smem, st>>>((const float2*)C, (const float2*)S,
                                                                (float2*)out, m_in, m_out, K, mode);
  return ef_check_launch();
}

static size_t rowstats_partial_bytes(int m, long long K) {
  return (size_t)m * rowdot_chunks(K) * sizeof(double4) + 256;
}

size_t ef_rowdot_workspace_bytes(int m, long long K) {
  if (m <= 0 || K <= 0) return 0;
  return rowstats_partial_bytes(m, K) + (size_t)m * sizeof(double4) + 512;
}

int ef_rowstats(const float* A, const float* B, int m, long long K, double* out, void* work,
                size_t work_bytes, void* stream) {
  if (!A || !B || !out || m <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad rowstats arguments");
  if (!work || work_bytes < rowstats_partial_bytes(m, K)) return ef_fail(EF_ERR_WORKSPACE, "rowstats work buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  int nc = rowdot_chunks(K);
  bool vec = (K % 2 == 0) && (((uintptr_t)A | (uintptr_t)B) % 16 == 0);
  if (vec) {
    long long K2 = K / 2;
    long long kchunk = (K2 + nc - 1) / nc;
    ef_count_launches(1);
    if (A == B)
      rowstats_kernel<true><<<dim3(nc, m), DTHREADS, 0, st>>>((const float4*)A, (const float4*)B, K2,
                                                             kchunk, (double4*)work);
    else
      rowstats_kernel<false><<<dim3(nc, m), DTHREADS, 0, st>>>((const float4*)A, (const float4*)B, K2,
                                                              kchunk, (double4*)work);
  } else {
    long long kchunk = (K + nc - 1) / nc;
    ef_count_launches(1);
    rowstats_scalar_kernel<<<dim3(nc, m), DTHREADS, 0, st>>>((const float2*)A, (const float2*)B, K,
                                                            kchunk, (double4*)work);
  }
  ef_count_launches(1);
  rowstats_reduce_kernel<<<(m + 127) / 128, 128, 0, st>>>((const double4*)work, nc, m, (double4*)out);
  return ef_check_launch();
}

__global__ void rowdot_pick_kernel(const double4* s, int m, double2* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = make_double2(s[i].x, s[i].y);
}

int ef_rowdot(const float* A, const float* B, int m, long long K, double* out, void* work,
              size_t work_bytes, void* stream) {
  if (!A || !B || !out || m <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad rowdot arguments");
  if (!work || work_bytes < ef_rowdot_workspace_bytes(m, K)) return ef_fail(EF_ERR_WORKSPACE, "rowdot work buffer too small");
  size_t pb = (rowstats_partial_bytes(m, K) + 255) / 256 * 256;
  double4* stats = reinterpret_cast<double4*>(reinterpret_cast<char*>(work) + pb);
  int r = ef_rowstats(A, B, m, K, (double*)stats, work, pb, stream);
  if (r != EF_OK) return r;
  ef_count_launches(1);
  rowdot_pick_kernel<<<(m + 127) / 128, 128, 0, (cudaStream_t)stream>>>(stats, m, (double2*)out);
  return ef_check_launch();
}

int ef_residual(const float* HX, const float* X, const double* lam, float* R, int m, long long K,
                void* stream) {
  if (!HX || !X || !lam || !R || m <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad residual arguments");
  long long total = (long long)m * K;
  ef_count_launches(1);
  residual_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>((const float2*)HX, (const float2*)X,
                                                                      lam, (float2*)R, K, total);
  return ef_check_launch();
}

int ef_residual_norms(const float* HX, const float* X, const double* lam, float* R, int m,
                      long long K, double* r2, void* work, size_t work_bytes, void* stream) {
  if (!HX || !X || !lam || !R || !r2 || m <= 0 || K <= 0)
    return ef_fail(EF_ERR_INVALID, "bad residual_norms arguments");
  if ((K % 2) != 0 || ((((uintptr_t)HX) | ((uintptr_t)X) | ((uintptr_t)R)) % 16) != 0)
    return ef_fail(EF_ERR_INVALID, "residual_norms needs even K and 16-byte aligned rows");
  int nc = rowdot_chunks(K);
  if (!work || work_bytes < (size_t)m * nc * sizeof(double) + 256)
    return ef_fail(EF_ERR_WORKSPACE, "residual_norms work buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  long long K2 = K / 2;
  long long kchunk = (K2 + nc - 1) / nc;
  ef_count_launches(2);
  residual_norm_kernel<<<dim3(nc, m), DTHREADS, 0, st>>>((const float4*)HX, (const float4*)X, lam,
                                                        (float4*)R, K2, kchunk, (double*)work);
  sum_rows_kernel<<<(m + 127) / 128, 128, 0, st>>>((const double*)work, nc, m, r2);
  return ef_check_launch();
}

int ef_scale_rows(float* X, const double* scale, int m, long long K, void* stream) {
  if (!X || !scale || m <= 0 || K <= 0) return ef_fail(EF_ERR_INVALID, "bad scale arguments");
  long long total = (long long)m * K;
  ef_count_launches(1);
  scale_rows_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>((float2*)X, scale, K, total);
  return ef_check_launch();
}

int ef_axpby(const float* X, float* Y, long long n_complex, double a, double b, void* stream) {
  if (!X || !Y || n_complex <= 0) return ef_fail(EF_ERR_INVALID, "bad axpby arguments");
  ef_count_launches(1);
  axpby_kernel<<<grid_for(n_complex), 256, 0, (cudaStream_t)stream>>>((const float2*)X, (float2*)Y,
                                                                       n_complex, (float)a, (float)b);
  return ef_check_launch();
}

int ef_rand_block(const ef_op* op, float* X, int m, uint64_t seed, uint64_t stream_id, int kind,
                  void* stream) {
  const ef::Op* o = op;
  if (!o || !X || m <= 0 || kind < 0 || kind > 2) return ef_fail(EF_ERR_INVALID, "bad rand arguments");
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + stream_id * 0xC2B2AE3D27D4EB4Full + 1ull;
  // key = mix(seed * phi + stream * c2 + 1), computed on the host like the oracle
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  uint64_t key = z ^ (z >> 31);
  long long total = (long long)m * 2 * o->N;
  ef_count_launches(1);
  rand_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(o->kax, o->G, (float2*)X, total, key, kind);
  return ef_check_launch();
}

int ef_apply_mask(const ef_op* op, float* X, int m, void* stream) {
  const ef::Op* o = op;
  if (!o || !X || m <= 0) return ef_fail(EF_ERR_INVALID, "bad mask arguments");
  long long total = (long long)m * 2 * o->N;
  ef_count_launches(1);
  mask_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(o->kax, o->G, (float2*)X, total);
  return ef_check_launch();
}

}  // extern "C"
