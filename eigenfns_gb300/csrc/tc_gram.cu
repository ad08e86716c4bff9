// Gram matrices on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// G[i][j] = sum_k conj(A[i,k]) B[j,k] over complex64 rows, computed as real
// products over the interleaved (re, im) storage:
//   Re G = A_r . B_r^T            A_r[i] = (ar0, ai0, ar1, ai1, ...)
//   Im G = A'_r . B_r^T           A'_r[i] = (-ai0, ar0, -ai1, ar1, ...)
// The two operands are stacked as the M = 128 rows of one MMA: rows [0, ma) hold
// A, rows [64, 64 + ma) hold A'; ma <= 64 per CTA (larger ma tiles over grid.x).
// B supplies N = mb rows (<= 256). Accuracy of fp32 products with three TF32
// products per pair (x = hi + lo, hi = round-to-tf32(x)):
//   D += A_hi B_hi + A_hi B_lo + A_lo B_hi          (.kind::tf32, fp32 accumulate)
// Converter threads load each K-stage from global memory, split it and store
// the six operand tiles in the no-swizzle K-major core-matrix layout (8 rows x
// 16 bytes per core matrix); one thread issues the MMAs and commits them to an
// mbarrier that guards the stage's buffer. Every mbarrier wait is bounded: on
// timeout the kernel records an error flag, drains, frees its TMEM and returns.
//
// Reference: gram, eigenfns/solver.py:35-43 (true-fp32 X^H Y; the reference
// forbids plain TF32, which floors the Gram at ~1e-3).
#include <cstdint>

#include "common.cuh"
#include "status.h"

namespace {

constexpr int TC_THREADS = 128;      // 4 warps: converters; warp 0 lane 0 issues MMAs
constexpr int TC_KB = 32;            // real k-values (tf32) per stage = 16 complex
constexpr int TC_M = 128;
constexpr int TC_STAGES = 2;
constexpr unsigned long long TC_SPIN_LIMIT = 1ull << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// element (r, k) of an operand tile with R rows and TC_KB k-values, no swizzle:
// core matrices of 8 rows x 4 k (16 B rows), K-adjacent core matrices 128 B apart,
// 8-row groups (TC_KB/4)*128 = 1024 B apart.
__device__ __forceinline__ int tile_off(int r, int k) {
  return (((r >> 3) * (TC_KB / 4) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  const uint64_t lbo = 128, sbo = (TC_KB / 4) * 128;
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;               // descriptor version for tcgen05
  return d;                             // base offset 0, swizzle none
}

// kind::tf32 instruction descriptor: D f32, A/B tf32, both K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                      // D format: f32
         | (2u << 7)                    // A format: tf32
         | (2u << 10)                   // B format: tf32
         | ((uint32_t)(N >> 3) << 17)
         | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// bounded wait on an mbarrier phase; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  uint32_t a = smem_u32(bar);
  for (unsigned long long it = 0; it < TC_SPIN_LIMIT; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(TC_THREADS) tc_gram_kernel(const float* __restrict__ A,
                                                             const float* __restrict__ B, int ma,
                                                             int mb, long long K, long long kchunk,
                                                             int ncols, double* __restrict__ partial,
                                                             int* __restrict__ err) {
  // operand tiles per stage: MA_hi, MA_lo (128 rows), B_hi, B_lo (nb rows, padded to 16)
  extern __shared__ __align__(1024) unsigned char smem[];
  const int nb = ncols;                       // N of the MMA: mb rounded up to 16
  const int tileA = TC_M * TC_KB * 4;         // bytes
  const int tileB = nb * TC_KB * 4;
  const int stage_bytes = 2 * tileA + 2 * tileB;
  __shared__ __align__(8) uint64_t bars[TC_STAGES];
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = blockIdx.x * 64;             // this CTA's rows of A
  const int mrows = (ma - i0) < 64 ? (ma - i0) : 64;
  const long long kbeg = (long long)blockIdx.z * kchunk;       // complex index
  long long kend = kbeg + kchunk;
  if (kend > K) kend = K;
  const int nst = (int)((kend - kbeg + (TC_KB / 2) - 1) / (TC_KB / 2));

  if (tid == 0) {
    abort_s = 0;
    for (int s = 0; s < TC_STAGES; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // zero every stage once: padding rows stay zero for the whole kernel
  for (int e = tid; e < TC_STAGES * stage_bytes / 16; e += TC_THREADS)
    reinterpret_cast<float4*>(smem)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_base_s)), "r"(nb <= 32 ? 32 : (nb <= 64 ? 64 : (nb <= 128 ? 128 : 256)))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_s;
  const uint32_t idesc = idesc_tf32(TC_M, nb);
  uint32_t phase[TC_STAGES] = {0u, 0u};

  for (int st = 0; st < nst; ++st) {
    const int buf = st % TC_STAGES;
    unsigned char* sb = smem + buf * stage_bytes;
    float* Ahi = reinterpret_cast<float*>(sb);
    float* Alo = reinterpret_cast<float*>(sb + tileA);
    float* Bhi = reinterpret_cast<float*>(sb + 2 * tileA);
    float* Blo = reinterpret_cast<float*>(sb + 2 * tileA + tileB);
    if (st >= TC_STAGES) {
      // the MMAs that read this buffer two stages ago must have completed
      bool ok = true;
      if (tid == 0) {
        ok = mbar_wait(&bars[buf], phase[buf]);
        if (!ok) abort_s = 1;
      }
      phase[buf] ^= 1u;
      __syncthreads();
      if (abort_s) break;
    }
    const long long kc0 = kbeg + (long long)st * (TC_KB / 2);   // first complex index of the stage
    // A rows: 16 complex = 32 floats per row per stage, 8 float4 per row
    for (int e = tid; e < 64 * 8; e += TC_THREADS) {
      int r = e >> 3, q = e & 7;              // q-th float4: complex pair (2q, 2q+1)
      long long kc = kc0 + 2 * q;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < mrows && kc < kend) {
        const float* src = A + ((long long)(i0 + r) * K + kc) * 2;
        if (kc + 1 < kend) v = *reinterpret_cast<const float4*>(src);
        else v = make_float4(src[0], src[1], 0.f, 0.f);
      }
      float vv[4] = {v.x, v.y, v.z, v.w};
      float sw[4] = {-v.y, v.x, -v.w, v.z};    // A' = conj-swap: Im G = A' . B
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        int k = 4 * q + t;
        float h = tf32_rn(vv[t]);
        Ahi[tile_off(r, k) >> 2] = h;
        Alo[tile_off(r, k) >> 2] = tf32_rn(vv[t] - h);
        float h2 = tf32_rn(sw[t]);
        Ahi[tile_off(64 + r, k) >> 2] = h2;
        Alo[tile_off(64 + r, k) >> 2] = tf32_rn(sw[t] - h2);
      }
    }
    for (int e = tid; e < nb * 8; e += TC_THREADS) {
      int r = e >> 3, q = e & 7;
      long long kc = kc0 + 2 * q;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      int j = blockIdx.y * 256 + r;
      if (r < nb && j < mb && kc < kend) {
        const float* src = B + ((long long)j * K + kc) * 2;
        if (kc + 1 < kend) v = *reinterpret_cast<const float4*>(src);
        else v = make_float4(src[0], src[1], 0.f, 0.f);
      }
      float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        int k = 4 * q + t;
        float h = tf32_rn(vv[t]);
        Bhi[tile_off(r, k) >> 2] = h;
        Blo[tile_off(r, k) >> 2] = tf32_rn(vv[t] - h);
      }
    }
    // make the generic-proxy stores visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t aHi = smem_u32(Ahi), aLo = smem_u32(Alo), bHi = smem_u32(Bhi), bLo = smem_u32(Blo);
#pragma unroll
      for (int s = 0; s < TC_KB / 8; ++s) {  // 8 tf32 (32 B = 2 core matrices) per MMA
        const uint32_t off = s * 256;
        const uint32_t acc0 = (st > 0 || s > 0) ? 1u : 0u;
        mma_tf32(tmem, smem_desc(aHi + off), smem_desc(bHi + off), idesc, acc0);
        mma_tf32(tmem, smem_desc(aHi + off), smem_desc(bLo + off), idesc, 1u);
        mma_tf32(tmem, smem_desc(aLo + off), smem_desc(bHi + off), idesc, 1u);
      }
      mma_commit(&bars[buf]);
    }
  }
  // drain: wait for the last commit of every stage still in flight
  __syncthreads();
  if (tid == 0 && !abort_s) {
    int last = nst - 1;
    for (int s = 0; s < TC_STAGES && s <= last; ++s) {
      int st = last - s;
      int buf = st % TC_STAGES;
      if (!mbar_wait(&bars[buf], phase[buf])) { abort_s = 1; break; }
      phase[buf] ^= 1u;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!abort_s && nst > 0) {
    // warp w reads TMEM lanes 32w..32w+31 = rows of [A; pad; A'; pad]
    const int row = warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    double* out = partial + (long long)blockIdx.z * ma * mb * 2;
    for (int c0 = 0; c0 < nb; c0 += 8) {
      uint32_t v[8];
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                     "=r"(v[6]), "=r"(v[7])
                   : "r"(taddr + c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        int j = blockIdx.y * 256 + c0 + t;
        if (j >= mb || c0 + t >= nb) continue;
        float val = __uint_as_float(v[t]);
        if (row < mrows) out[((long long)(i0 + row) * mb + j) * 2] = (double)val;
        else if (row >= 64 && row - 64 < mrows) out[((long long)(i0 + row - 64) * mb + j) * 2 + 1] = (double)val;
      }
    }
  } else if (abort_s && tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(nb <= 32 ? 32 : (nb <= 64 ? 64 : (nb <= 128 ? 128 : 256)))
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

int tc_splits(int ma, int mb, long long K) {
  long long tiles = (long long)((ma + 63) / 64) * ((mb + 255) / 256);
  long long target = 1216 / (tiles > 0 ? tiles : 1);   // 152 SMs x 8
  long long maxs = (K + 1023) / 1024;                   // >= 1024 complex per chunk
  long long s = target < maxs ? target : maxs;
  return (int)(s < 1 ? 1 : s);
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
  if (mb > 256) return ef_fail(EF_ERR_TOO_LARGE, "gram_tc: mb above 256");
  if (((uintptr_t)A | (uintptr_t)B) % 16 != 0 || (K % 2) != 0)
    return ef_fail(EF_ERR_INVALID, "gram_tc needs 16-byte aligned rows of even length");
  if (!work || work_bytes < ef_gram_tc_workspace_bytes(ma, mb, K))
    return ef_fail(EF_ERR_WORKSPACE, "gram_tc work buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  int ns = tc_splits(ma, mb, K);
  long long kchunk = (K + ns - 1) / ns;
  kchunk = (kchunk + 15) / 16 * 16;
  ns = (int)((K + kchunk - 1) / kchunk);
  int nb = ((mb < 256 ? mb : 256) + 15) / 16 * 16;
  if (nb < 16) nb = 16;
  size_t smem = (size_t)TC_STAGES * (2 * TC_M * TC_KB * 4 + 2 * nb * TC_KB * 4) + 1024;
  cudaFuncSetAttribute(tc_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid((ma + 63) / 64, (mb + 255) / 256, ns);
  ef_count_launches(2);
  tc_gram_kernel<<<grid, TC_THREADS, smem, st>>>(A, B, ma, mb, K, kchunk, nb, (double*)work, err_dev);
  int n = ma * mb;
  tc_gram_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>((const double*)work, ns, n, G);
  return ef_check_launch();
}
