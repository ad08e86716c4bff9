// Gram matrices on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// G[i][j] = sum_k conj(A[i,k]) B[j,k] over complex64 rows, computed as real
// products over the interleaved (re, im) storage:
//   Re G = A_r . B_r^T            A_r[i] = (ar0, ai0, ar1, ai1, ...)
//   Im G = A'_r . B_r^T           A'_r[i] = (-ai0, ar0, -ai1, ar1, ...)
// Rows [0, 64) of the M = 128 MMA operand hold up to 64 rows of A, rows [64, 128)
// the matching rows of A'; a CTA covers 64 rows of A and NB <= 64 rows of B
// (larger shapes tile over grid.x / grid.y). Three TF32 products per pair give
// fp32-class products (x = hi + lo, hi = round-to-tf32(x)):
//   D += A_hi B_hi + A_hi B_lo + A_lo B_hi        (.kind::tf32, fp32 accumulate)
// Tensor-core fp32 accumulation is not round-to-nearest over long chains, so a
// CTA's K-chunk is cut into segments of SEG stages that accumulate alternately
// into two TMEM regions; every finished segment is read back (tcgen05.ld) and
// added into fp64 registers, one TMEM lane (= one row) per thread, while the
// next segment's MMAs run in the other region. Chunks are reduced in fp64.
//
// Pipeline per 16-complex stage: all 128 threads convert the stage they prefetched
// into registers (hi/lo split, A' swap) and store it with 16-byte stores into the
// no-swizzle K-major core-matrix layout, prefetch the next stage, fence the
// async proxy, and thread 0 issues the stage's 12 MMAs and commits them to the
// stage buffer's mbarrier. Every mbarrier wait is bounded; on timeout the kernel
// sets an error flag, skips the rest, frees its TMEM and returns.
//
// Reference: gram, eigenfns/solver.py:35-43 (true-fp32 X^H Y; the reference
// forbids plain TF32, which floors the Gram at ~1e-3).
#include <cstdint>

#include "common.cuh"
#include "status.h"
#include "tc_common.cuh"

namespace {

using namespace ef::tc;

constexpr int TC_THREADS = 128;
constexpr int TC_KB = 32;            // real k-values (tf32) per stage = 16 complex
constexpr int TC_M = 128;
constexpr int TC_SEG = 8;            // stages per TMEM accumulation segment

// byte offset of (row r, k-quad q) in an operand tile: core matrices of 8 rows x 16 B,
// K-adjacent core matrices 128 B apart, 8-row groups (TC_KB/4)*128 = 1024 B apart
__device__ __forceinline__ int quad_off(int r, int q) {
  return (((r >> 3) * (TC_KB / 4) + q) << 7) + ((r & 7) << 4);
}

__device__ __forceinline__ uint64_t gram_desc(uint32_t addr) {
  return smem_desc(addr, 128, (TC_KB / 4) * 128);
}

__host__ __device__ constexpr int tmem_cols(int nb) {
  return 2 * nb <= 32 ? 32 : (2 * nb <= 64 ? 64 : (2 * nb <= 128 ? 128 : 256));
}

template <int NB>
__global__ void __launch_bounds__(TC_THREADS) tc_gram_kernel(const float* __restrict__ A,
                                                             const float* __restrict__ B, int ma,
                                                             int mb, long long K, long long kchunk,
                                                             double* __restrict__ partial,
                                                             int* __restrict__ err) {
  constexpr int TILE_A = TC_M * TC_KB * 4;      // 16 KB
  constexpr int TILE_B = NB * TC_KB * 4;
  constexpr int STAGE = 2 * TILE_A + 2 * TILE_B;
  constexpr int ITEMS_MAX = (64 + NB) * 8;       // float4 per stage
  constexpr int PER_T = (ITEMS_MAX + TC_THREADS - 1) / TC_THREADS;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t stage_bar[2];
  __shared__ __align__(8) uint64_t seg_bar[2];
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * NB;
  const int mrows = (ma - i0) < 64 ? (ma - i0) : 64;
  const int nrows = (mb - j0) < NB ? (mb - j0) : NB;
  const long long kbeg = (long long)blockIdx.z * kchunk;
  long long kend = kbeg + kchunk;
  if (kend > K) kend = K;
  const int nst = (int)((kend - kbeg + (TC_KB / 2) - 1) / (TC_KB / 2));
  const int items = (mrows + nrows) * 8;

  if (tid == 0) {
    abort_s = 0;
    mbar_init(&stage_bar[0], 1);
    mbar_init(&stage_bar[1], 1);
    mbar_init(&seg_bar[0], 1);
    mbar_init(&seg_bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int e = tid; e < 2 * STAGE / 16; e += TC_THREADS)
    reinterpret_cast<float4*>(smem)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_base_s)), "r"(tmem_cols(NB)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_s;
  const uint32_t idesc = idesc_tf32(TC_M, NB);

  // stage loads: item e -> (row, quad q): rows [0, mrows) of A then [0, nrows) of B
  float4 pre[PER_T];
  auto prefetch = [&](int st) {
    const long long kc0 = kbeg + (long long)st * (TC_KB / 2);
#pragma unroll
    for (int u = 0; u < PER_T; ++u) {
      const int e = tid + u * TC_THREADS;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (e < items) {
        const int r = e >> 3, q = e & 7;
        const long long kc = kc0 + 2 * q;
        const float* src = (r < mrows) ? A + ((long long)(i0 + r) * K + kc) * 2
                                       : B + ((long long)(j0 + r - mrows) * K + kc) * 2;
        if (kc + 1 < kend) v = __ldg(reinterpret_cast<const float4*>(src));
        else if (kc < kend) v = make_float4(__ldg(src), __ldg(src + 1), 0.f, 0.f);
      }
      pre[u] = v;
    }
  };
  double acc[NB];
#pragma unroll
  for (int c = 0; c < NB; ++c) acc[c] = 0.0;
  uint32_t sph[2] = {0u, 0u}, gph[2] = {0u, 0u};
  int drained = 0;   // segments already added into acc
  const int nseg = (nst + TC_SEG - 1) / TC_SEG;

  auto drain = [&](int seg) -> bool {
    const int reg = seg & 1;
    if (!mbar_wait(&seg_bar[reg], gph[reg])) return false;
    gph[reg] ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(reg * NB);
#pragma unroll
    for (int c0 = 0; c0 < NB; c0 += 8) {
      uint32_t v[8];
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                     "=r"(v[6]), "=r"(v[7])
                   : "r"(taddr + c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[c0 + t] += (double)__uint_as_float(v[t]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    return true;
  };

  if (nst > 0) prefetch(0);
  for (int st = 0; st < nst; ++st) {
    const int buf = st & 1;
    unsigned char* sb = smem + buf * STAGE;
    if (st >= 2) {
      if (tid == 0 && !mbar_wait(&stage_bar[buf], sph[buf])) abort_s = 1;
      sph[buf] ^= 1u;
      __syncthreads();
      if (abort_s) break;
    }
    // convert the prefetched stage: A rows -> (A, A') hi/lo, B rows -> B hi/lo
#pragma unroll
    for (int u = 0; u < PER_T; ++u) {
      const int e = tid + u * TC_THREADS;
      if (e < items) {
        const int r = e >> 3, q = e & 7;
        const float4 v = pre[u];
        const float4 h = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
        const float4 l = make_float4(tf32_rn(v.x - h.x), tf32_rn(v.y - h.y), tf32_rn(v.z - h.z),
                                     tf32_rn(v.w - h.w));
        if (r < mrows) {
          *reinterpret_cast<float4*>(sb + quad_off(r, q)) = h;
          *reinterpret_cast<float4*>(sb + TILE_A + quad_off(r, q)) = l;
          // A' = (-ai, ar) per complex: swap within the pairs and negate the new real part
          *reinterpret_cast<float4*>(sb + quad_off(64 + r, q)) = make_float4(-h.y, h.x, -h.w, h.z);
          *reinterpret_cast<float4*>(sb + TILE_A + quad_off(64 + r, q)) = make_float4(-l.y, l.x, -l.w, l.z);
        } else {
          const int rb = r - mrows;
          *reinterpret_cast<float4*>(sb + 2 * TILE_A + quad_off(rb, q)) = h;
          *reinterpret_cast<float4*>(sb + 2 * TILE_A + TILE_B + quad_off(rb, q)) = l;
        }
      }
    }
    if (st + 1 < nst) prefetch(st + 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    const int seg = st / TC_SEG;
    const bool seg_first = (st % TC_SEG) == 0;
    const bool seg_last = ((st % TC_SEG) == TC_SEG - 1) || (st == nst - 1);
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + (uint32_t)((seg & 1) * NB);
      const uint32_t aHi = smem_u32(sb), aLo = smem_u32(sb + TILE_A);
      const uint32_t bHi = smem_u32(sb + 2 * TILE_A), bLo = smem_u32(sb + 2 * TILE_A + TILE_B);
#pragma unroll
      for (int s = 0; s < TC_KB / 8; ++s) {   // 8 tf32 = 2 core matrices per MMA
        const uint32_t off = s * 256;
        mma_tf32(d, gram_desc(aHi + off), gram_desc(bHi + off), idesc, (seg_first && s == 0) ? 0u : 1u);
        mma_tf32(d, gram_desc(aHi + off), gram_desc(bLo + off), idesc, 1u);
        mma_tf32(d, gram_desc(aLo + off), gram_desc(bHi + off), idesc, 1u);
      }
      mma_commit(&stage_bar[buf]);
      if (seg_last) mma_commit(&seg_bar[seg & 1]);
    }
    // one stage into a segment, drain the previous one (its region is reused two segments on)
    if ((st % TC_SEG) == 1 && seg >= 1 && drained == seg - 1) {
      if (!drain(seg - 1)) atomicExch(&abort_s, 1);
      ++drained;
    }
  }
  __syncthreads();
  if (!abort_s) {
    while (drained < nseg) {
      if (!drain(drained)) { abort_s = 1; break; }
      ++drained;
    }
  }
  __syncthreads();
  if (!abort_s && nst > 0) {
    const int row = warp * 32 + lane;
    double* out = partial + (long long)blockIdx.z * ma * mb * 2;
    const bool re = row < mrows, im = row >= 64 && row - 64 < mrows;
    const int i = i0 + (re ? row : row - 64);
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      if (c < nrows) {
        if (re) out[((long long)i * mb + j0 + c) * 2] = acc[c];
        if (im) out[((long long)i * mb + j0 + c) * 2 + 1] = acc[c];
      }
    }
  } else if (abort_s && tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols(NB))
                 : "memory");
  }
}

__global__ void tc_gram_reduce_kernel(const double* partial, int nsplit, int n, double* G) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double sr = 0.0, si = 0.0;
  for (int s = 0; s < nsplit; ++s) {
    sr += partial[((long long)s * n + e) * 2];
    si += partial[((long long)s * n + e) * 2 + 1];
  }
  G[2 * e] = sr;
  G[2 * e + 1] = si;
}

int tc_nb(int mb) { return mb <= 16 ? 16 : (mb <= 32 ? 32 : 64); }

int tc_splits(int ma, int mb, long long K) {
  const int nb = tc_nb(mb);
  long long tiles = (long long)((ma + 63) / 64) * ((mb + nb - 1) / nb);
  long long target = (152 * 3) / (tiles > 0 ? tiles : 1);
  if (target < 1) target = 1;
  long long maxs = (K + 1023) / 1024;                   // >= 1024 complex per chunk
  long long s = target < maxs ? target : maxs;
  return (int)(s < 1 ? 1 : s);
}

template <int NB>
void launch_tc(dim3 grid, cudaStream_t st, const float* A, const float* B, int ma, int mb, long long K,
               long long kchunk, double* part, int* err) {
  const size_t smem = (size_t)2 * (2 * TC_M * TC_KB * 4 + 2 * NB * TC_KB * 4) + 1024;
  ef::set_smem_once(tc_gram_kernel<NB>, smem);
  tc_gram_kernel<NB><<<grid, TC_THREADS, smem, st>>>(A, B, ma, mb, K, kchunk, part, err);
}

}  // namespace

extern "C" size_t ef_gram_tc_workspace_bytes(int ma, int mb, long long K) {
  if (ma <= 0 || mb <= 0 || K <= 0) return 0;
  return (size_t)tc_splits(ma, mb, K) * ma * mb * 2 * sizeof(double) + 512;
}

extern "C" int ef_gram_tc(const float* A, const float* B, int ma, int mb, long long K, double* G,
                          int* err_dev, void* work, size_t work_bytes, void* stream) {
  if (!A || !B || !G || !err_dev || ma <= 0 || mb <= 0 || K <= 0)
    return ef_fail(EF_ERR_INVALID, "bad gram_tc arguments");
  if (((uintptr_t)A | (uintptr_t)B) % 16 != 0 || (K % 2) != 0)
    return ef_fail(EF_ERR_INVALID, "gram_tc needs 16-byte aligned rows of even length");
  if (!work || work_bytes < ef_gram_tc_workspace_bytes(ma, mb, K))
    return ef_fail(EF_ERR_WORKSPACE, "gram_tc work buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = tc_nb(mb);
  int ns = tc_splits(ma, mb, K);
  long long kchunk = (K + ns - 1) / ns;
  kchunk = (kchunk + 15) / 16 * 16;
  ns = (int)((K + kchunk - 1) / kchunk);
  dim3 grid((ma + 63) / 64, (mb + nb - 1) / nb, ns);
  ef_count_launches(2);
  if (nb == 16) launch_tc<16>(grid, st, A, B, ma, mb, K, kchunk, (double*)work, err_dev);
  else if (nb == 32) launch_tc<32>(grid, st, A, B, ma, mb, K, kchunk, (double*)work, err_dev);
  else launch_tc<64>(grid, st, A, B, ma, mb, K, kchunk, (double*)work, err_dev);
  int n = ma * mb;
  tc_gram_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>((const double*)work, ns, n, G);
  return ef_check_launch();
}
