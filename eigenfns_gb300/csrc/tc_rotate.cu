// Block rotations out_i (+/-)= sum_j C[j][i] S_j on the tcgen05 tensor cores.
//
// Real view: a complex64 row of K values is 2K interleaved floats s_j[p]. With
// D1[p][i] = sum_j s_j[p] Re C[j][i] and D2[p][i] = sum_j s_j[p] Im C[j][i]:
//   Re out_i[k] = D1[2k][i] - D2[2k+1][i]      Im out_i[k] = D1[2k+1][i] + D2[2k][i]
// so one real GEMM D (2K x 2m_out) = S^T (2K x m_in) . [Re C | Im C] (m_in x 2m_out)
// followed by a neighbour exchange (adjacent TMEM lanes = adjacent threads of a warp)
// gives the complex result. Three TF32 products per pair (x = hi + lo) give
// fp32-class accuracy: D += A_hi B_hi + A_hi B_lo + A_lo B_hi.
// The accumulate modes out (+/-)= ... fold the current output into the same GEMM:
// its m_out rows are appended to S with identity coefficients and C is negated for
// subtraction, so every mode ends in a plain store.
//
// Tiles are 128 real positions (M = 128 TMEM lanes); N = 2 * m_out padded to 8.
// A persistent CTA (448 threads) walks its tiles with four warp roles:
//   warp 13     loads: one bulk copy (TMA engine) per 512-byte row of a 16-row x
//               128-position stage into an 8-deep raw ring (mbarrier byte counts);
//   warps 0-7   convert: read the raw stage (one position per thread), split hi/lo,
//               store 16-byte quads into a 3-deep ring of K-major operand stages;
//   warp 12     one thread issues the MMAs of each stage into one of two TMEM
//               accumulators and commits them to the stage's "empty" barrier;
//   warps 8-11  drain a finished accumulator (tcgen05.ld, one lane per thread),
//               combine D1/D2 with a lane exchange and store.
// The coefficient operand [Re C | Im C] (hi and lo) is built once per CTA and stays
// resident in shared memory. Every mbarrier wait is bounded: on timeout the kernel
// sets the library's device error flag and stops issuing work, waits (bounded) for
// its own copies and MMAs and frees its TMEM.
//
// Reference: tensordot(C.T, S) in combine / rotations, eigenfns/solver.py:49-57,106,125.
#include <cstdint>

#include "common.cuh"
#include "status.h"
#include "tc_common.cuh"

namespace {

using namespace ef::tc;

constexpr int TR_THREADS = 448;
constexpr int TR_CONV = 256;              // converter threads (warps 0-7)
constexpr int TR_EPI0 = 256;              // first epilogue thread (warps 8-11)
constexpr int TR_MMA_WARP = 12;
constexpr int TR_LOAD_WARP = 13;
constexpr int TR_M = 128;                 // real positions per tile
constexpr int TR_JC = 16;                 // rows of S per stage
constexpr int TR_NBUF = 3;                // operand stages in the ring
constexpr int TR_OP_HALF = TR_M * TR_JC * 4;       // 8 KB: hi or lo of one stage
constexpr int TR_OP_BYTES = 2 * TR_OP_HALF;        // 16 KB per stage
constexpr int TR_RAW = 8;                 // raw stages in flight (power of two)
constexpr int TR_RAW_BYTES = TR_JC * TR_M * 4;     // 8 KB per raw stage (row-major)
constexpr int TR_SMEM_MAX = 227 * 1024 - 1024;   // dynamic part; static barriers take the rest

__device__ int g_tc_error = 0;

struct TrArgs {
  const float2* C;      // (m_in, ldc) complex, columns [0, m_out) used
  const float* S;       // m_in rows of n2 floats
  float* out;           // m_out rows of n2 floats (also the identity rows when mode != 0)
  long long n2;         // 2K
  long long ntiles;
  int ldc, m_in, m_tot, m_out, mp, nch;
  float sign;           // -1 for subtraction
};

// 14 warps: at most 4 per SM sub-partition, so 128 registers a thread fit
__global__ void __maxnreg__(128) tc_rotate_kernel(const TrArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t op_full[TR_NBUF], op_empty[TR_NBUF];
  __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done_bar;
  __shared__ __align__(8) uint64_t raw_full[TR_RAW], raw_empty[TR_RAW];
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int N = 2 * a.mp;
  const int kj = a.nch * TR_JC;            // padded rows of the coefficient operand
  const uint32_t b_half = (uint32_t)N * kj * 4;
  unsigned char* raw = smem + TR_NBUF * TR_OP_BYTES;
  unsigned char* bops = raw + TR_RAW * TR_RAW_BYTES;
  const uint32_t tcols = tmem_cols_for(2 * N);

  if (tid == 0) {
    abort_s = 0;
    for (int b = 0; b < TR_NBUF; ++b) {
      mbar_init(&op_full[b], TR_CONV);
      mbar_init(&op_empty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 128);
    }
    mbar_init(&done_bar, 1);
    for (int b = 0; b < TR_RAW; ++b) {
      mbar_init(&raw_full[b], 1);
      mbar_init(&raw_empty[b], TR_CONV);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // coefficient operand, K-major core matrices: row n (D column), column j (row of S)
  // rows [0, mp) = Re C[:, n], rows [mp, 2mp) = Im C[:, n - mp]; rows j >= m_in of
  // the inputs are the current output (identity coefficients); zero padding elsewhere
  for (int e = tid; e < (int)(2 * b_half / 16); e += TR_THREADS)
    reinterpret_cast<float4*>(bops)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  const int kq = kj / 4;
  auto put = [&](int n, int j, float x) {
    const float hi = tf32_rn(x), lo = tf32_rn(x - hi);
    const uint32_t off = (uint32_t)(((n >> 3) * kq + (j >> 2)) * 128 + (n & 7) * 16 + (j & 3) * 4);
    *reinterpret_cast<float*>(bops + off) = hi;
    *reinterpret_cast<float*>(bops + b_half + off) = lo;
  };
  for (int e = tid; e < a.m_in * a.m_out; e += TR_THREADS) {
    const int j = e / a.m_out, i = e - j * a.m_out;
    const float2 c = a.C[(long long)j * a.ldc + i];
    put(i, j, a.sign * c.x);
    put(a.mp + i, j, a.sign * c.y);
  }
  for (int i = tid; i < a.m_tot - a.m_in; i += TR_THREADS) put(i, a.m_in + i, 1.f);
  fence_async_smem();
  if (warp == TR_MMA_WARP) tmem_alloc(&tmem_base_s, tcols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = tmem_base_s;
  const long long my_tiles =
      (a.ntiles > blockIdx.x) ? (a.ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
  const long long nstages = my_tiles * a.nch;

  if (warp < 8) {
    // ---------------- converters ----------------
    // each thread owns position p and rows 8h..8h+7 of a stage (conflict-free reads)
    const int p = tid & (TR_M - 1), h = tid >> 7;
    long long cur_tile = blockIdx.x;
    int cur_c = 0;
    for (long long s = 0; s < nstages; ++s) {
      const int slot = (int)(s & (TR_RAW - 1));
      const uint32_t ur = (uint32_t)(s / TR_RAW);
      if (abort_s) break;
      if (!mbar_wait(&raw_full[slot], ur & 1)) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      const float* rs = reinterpret_cast<const float*>(raw + slot * TR_RAW_BYTES) + p;
      const bool pin = cur_tile * TR_M + p < a.n2;
      const int j0 = cur_c * TR_JC + h * 8;
      float v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = (pin && j0 + r < a.m_tot) ? rs[(h * 8 + r) * TR_M] : 0.f;
      mbar_arrive(&raw_empty[slot]);
      if (++cur_c == a.nch) {
        cur_c = 0;
        cur_tile += gridDim.x;
      }
      const int o = (int)(s % TR_NBUF);
      const uint32_t u = (uint32_t)(s / TR_NBUF);
      if (!mbar_wait(&op_empty[o], (u + 1) & 1)) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      unsigned char* base = smem + o * TR_OP_BYTES;
#pragma unroll
      for (int qq = 0; qq < 2; ++qq) {
        const int q = h * 2 + qq;
        const float4 x = make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
        const float4 hi = make_float4(tf32_rn(x.x), tf32_rn(x.y), tf32_rn(x.z), tf32_rn(x.w));
        const float4 lo = make_float4(tf32_rn(x.x - hi.x), tf32_rn(x.y - hi.y), tf32_rn(x.z - hi.z),
                                      tf32_rn(x.w - hi.w));
        const int off = (((p >> 3) * (TR_JC / 4) + q) << 7) + ((p & 7) << 4);
        *reinterpret_cast<float4*>(base + off) = hi;
        *reinterpret_cast<float4*>(base + TR_OP_HALF + off) = lo;
      }
      fence_async_smem();
      mbar_arrive(&op_full[o]);
    }
  } else if (warp < 12) {
    // ---------------- epilogue ----------------
    const int p = tid - TR_EPI0;                       // = 32 * (warp % 4) + lane
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const bool even = (p & 1) == 0;
    for (long long k = 0; k < my_tiles; ++k) {
      if (abort_s) break;
      const int ab = (int)(k & 1);
      if (!mbar_wait(&acc_full[ab], (uint32_t)((k >> 1) & 1))) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      fence_after_sync();
      const long long tile = blockIdx.x + k * (long long)gridDim.x;
      const long long pos = tile * TR_M + p;
      const bool pin = pos < a.n2;
      const uint32_t ta = lane_base + (uint32_t)(ab * N);
      for (int i0 = 0; i0 < a.mp; i0 += 8) {
        float d1[8], d2[8];
        tmem_ld8x2(ta + i0, ta + a.mp + i0, d1, d2);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const float w = __shfl_xor_sync(0xffffffffu, d2[t], 1);
          const float val = even ? d1[t] - w : d1[t] + w;
          if (pin && i0 + t < a.m_out) a.out[(long long)(i0 + t) * a.n2 + pos] = val;
        }
      }
      fence_before_sync();
      mbar_arrive(&acc_empty[ab]);
    }
  } else if (warp == TR_MMA_WARP && lane == 0) {
    // ---------------- MMA issue ----------------
    const uint32_t idesc = idesc_tf32(TR_M, N);
    const uint32_t b_hi = smem_u32(bops);
    const uint32_t b_sbo = (uint32_t)kq * 128;
    const uint64_t a_desc0 = smem_desc(smem_u32(smem), 128, (TR_JC / 4) * 128);
    const uint64_t b_desc0 = smem_desc(b_hi, 128, b_sbo);
    bool issued = false;
    for (long long k = 0; k < my_tiles && !abort_s; ++k) {
      const int ab = (int)(k & 1);
      if (!mbar_wait(&acc_empty[ab], (uint32_t)(((k >> 1) + 1) & 1))) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      fence_after_sync();
      const uint32_t d = tmem + (uint32_t)(ab * N);
      for (int c = 0; c < a.nch; ++c) {
        const long long s = k * a.nch + c;
        const int o = (int)(s % TR_NBUF);
        if (!mbar_wait(&op_full[o], (uint32_t)((s / TR_NBUF) & 1))) {
          abort_s = 1;
          atomicExch(&g_tc_error, 1);
          break;
        }
        fence_after_sync();
        // descriptors differ from the base ones only in the start-address field
        const uint64_t ah0 = a_desc0 + (uint64_t)((o * TR_OP_BYTES) >> 4);
        const uint64_t bh0 = b_desc0 + (uint64_t)((c * (TR_JC / 4) * 128) >> 4);
#pragma unroll
        for (int g = 0; g < TR_JC / 8; ++g) {
          if (c * TR_JC + g * 8 >= a.m_tot) break;      // all-zero rows: nothing to add
          const uint64_t ah = ah0 + (uint64_t)(g * 256 >> 4), al = ah + (uint64_t)(TR_OP_HALF >> 4);
          const uint64_t bh = bh0 + (uint64_t)(g * 256 >> 4), bl = bh + (uint64_t)(b_half >> 4);
          mma_tf32(d, ah, bh, idesc, (c | g) ? 1u : 0u);
          mma_tf32(d, ah, bl, idesc, 1u);
          mma_tf32(d, al, bh, idesc, 1u);
        }
        mma_commit(&op_empty[o]);
        issued = true;
      }
      if (abort_s) break;
      mma_commit(&acc_full[ab]);
    }
    if (abort_s && issued) {
      // let this thread's MMAs finish before the TMEM they write is freed
      mma_commit(&done_bar);
      mbar_wait(&done_bar, 0);
    }
  }
  if (warp == TR_LOAD_WARP) {
    // ---------------- loader ----------------
    // one bulk copy (TMA engine) per row of a stage: 16 rows x up to 512 B, completing
    // on the slot's raw_full barrier; rows beyond the inputs are not copied (the
    // converters read zeros for them)
    long long tile = blockIdx.x;
    int c = 0;
    long long issued = 0;
    for (long long s = 0; s < nstages; ++s) {
      const int slot = (int)(s & (TR_RAW - 1));
      const uint32_t ur = (uint32_t)(s / TR_RAW);
      if (abort_s) break;
      bool ok = true;
      if (lane == 0) ok = mbar_wait(&raw_empty[slot], (ur + 1) & 1);
      if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) {
        if (lane == 0) {
          abort_s = 1;
          atomicExch(&g_tc_error, 1);
        }
        break;
      }
      const long long pos0 = tile * TR_M;
      const long long left = a.n2 - pos0;
      const uint32_t row_bytes = (uint32_t)(left >= TR_M ? TR_M * 4 : left * 4);
      int nrows = a.m_tot - c * TR_JC;
      nrows = nrows < 0 ? 0 : (nrows > TR_JC ? TR_JC : nrows);
      if (lane == 0) mbar_arrive_expect_tx(&raw_full[slot], row_bytes * (uint32_t)nrows);
      __syncwarp();
      if (lane < nrows) {
        const int j = c * TR_JC + lane;
        const float* src = (j < a.m_in) ? a.S + (long long)j * a.n2 + pos0
                                        : a.out + (long long)(j - a.m_in) * a.n2 + pos0;
        bulk_copy_g2s(raw + slot * TR_RAW_BYTES + lane * (TR_M * 4), src, row_bytes, &raw_full[slot]);
      }
      issued = s + 1;
      if (++c == a.nch) {
        c = 0;
        tile += gridDim.x;
      }
    }
    // no copy may still be landing when the CTA exits: wait for the last issued phases
    if (lane == 0)
      for (long long s = issued - TR_RAW > 0 ? issued - TR_RAW : 0; s < issued; ++s)
        mbar_wait(&raw_full[(int)(s & (TR_RAW - 1))], (uint32_t)((s / TR_RAW) & 1));
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == TR_MMA_WARP) tmem_dealloc(tmem, tcols);
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cached[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 1;
  }
  return cached[dev];
}

size_t tr_smem(int m_tot, int mp) {
  const int nch = (m_tot + TR_JC - 1) / TR_JC;
  return (size_t)TR_NBUF * TR_OP_BYTES + (size_t)TR_RAW * TR_RAW_BYTES +
         (size_t)2 * (2 * mp) * (nch * TR_JC) * 4;
}

}  // namespace

namespace ef {

// largest number of input rows (S rows plus, in the accumulate modes, the m_out
// output rows) one tensor-core pass holds for m_out outputs; 0 when m_out > 64
int tc_rotate_max_rows(int m_out) {
  if (m_out <= 0 || m_out > 64) return 0;
  const int mp = (m_out + 7) / 8 * 8;
  int rows = 0;
  while (tr_smem(rows + TR_JC, mp) <= (size_t)TR_SMEM_MAX) rows += TR_JC;
  return rows;
}

// one pass: m_out <= 64, m_in + (mode ? m_out : 0) <= tc_rotate_max_rows(m_out);
// S and out 16-byte aligned, K even
int tc_rotate_launch(const float* C, int ldc, const float* S, float* out, int m_in, int m_out,
                     long long K, int mode, cudaStream_t st) {
  TrArgs a;
  a.C = (const float2*)C;
  a.S = S;
  a.out = out;
  a.n2 = 2 * K;
  a.ntiles = (a.n2 + TR_M - 1) / TR_M;
  a.ldc = ldc;
  a.m_in = m_in;
  a.m_out = m_out;
  a.m_tot = m_in + (mode != 0 ? m_out : 0);
  a.mp = (m_out + 7) / 8 * 8;
  a.nch = (a.m_tot + TR_JC - 1) / TR_JC;
  a.sign = mode < 0 ? -1.f : 1.f;
  const size_t smem = tr_smem(a.m_tot, a.mp);
  ef::set_smem_once(tc_rotate_kernel, smem);
  long long grid = sm_count();
  if (grid > a.ntiles) grid = a.ntiles;
  ef_count_launches(1);
  tc_rotate_kernel<<<(unsigned)grid, TR_THREADS, smem, st>>>(a);
  return ef_check_launch();
}

// reads and clears the tensor-core kernels' device error flag (synchronises the device)
int tc_error_flag(int* flag) {
  int v = 0, zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
  if (e != cudaSuccess) return ef_fail(EF_ERR_CUDA, cudaGetErrorString(e));
  *flag = v;
  return EF_OK;
}

}  // namespace ef

extern "C" int ef_tc_error(int* flag) {
  if (!flag) return ef_fail(EF_ERR_INVALID, "null flag");
  return ef::tc_error_flag(flag);
}
