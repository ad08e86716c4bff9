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
// its m_out rows are appended to S (from the next 32-row boundary) with identity
// coefficients and C is negated for subtraction, so every mode ends in a plain store.
//
// Tiles are 128 real positions (M = 128 TMEM lanes); N = 2 * m_out padded to 8.
// A persistent CTA (448 threads) walks its tiles with four warp roles:
//   warp 13     loads: one 2-D TMA box (32 rows x 128 positions, 16 KB, zero fill
//               outside the matrix) per stage into a raw shared-memory ring;
//   warps 0-7   convert: each thread owns one position (= one TMEM lane) and 16 rows
//               of the stage, splits hi/lo and writes them with tcgen05.st into a
//               ring of TMEM operand stages (the MMA's A operand lives in TMEM);
//   warp 12     one thread issues the MMAs of each stage (A from TMEM, the resident
//               coefficient operand B from shared memory) into one of two TMEM
//               accumulators and commits them to the stage's "empty" barrier;
//   warps 8-11  drain a finished accumulator (tcgen05.ld, one lane per thread),
//               combine D1/D2 with a lane exchange and store.
// Every mbarrier wait is bounded: on timeout the kernel sets the library's device
// error flag and stops issuing work, waits (bounded) for its own copies and MMAs and
// frees its TMEM.
//
// Reference: tensordot(C.T, S) in combine / rotations, eigenfns/solver.py:49-57,106,125.
#include <cuda.h>

#include <cstdint>

#include "common.cuh"
#include "status.h"
#include "tc_common.cuh"
#include "tmap.h"

namespace {

using namespace ef::tc;

constexpr int TR_THREADS = 448;
constexpr int TR_CONV = 256;              // converter threads (warps 0-7)
constexpr int TR_EPI0 = 256;              // first epilogue thread (warps 8-11)
constexpr int TR_MMA_WARP = 12;
constexpr int TR_LOAD_WARP = 13;
constexpr int TR_M = 128;                 // real positions per tile
constexpr int TR_JC = 32;                 // rows of S per stage
constexpr int TR_RPT = TR_JC / 2;         // rows per converter thread (two warps per lane quarter)
constexpr int TR_NBUF_MAX = 8;            // TMEM operand stages (hi + lo: 2*TR_JC columns each)
constexpr int TR_RAW = 6;                 // raw shared-memory stages
constexpr int TR_RAW_BYTES = TR_JC * TR_M * 4;     // 16 KB per raw stage (row-major box)
constexpr int TR_SMEM_MAX = 227 * 1024 - 1024;   // dynamic part; static barriers take the rest
constexpr int TR_SMEM_MIN = 120 * 1024;          // keeps one CTA (and its TMEM) per SM

__device__ int g_tc_error = 0;

struct TrArgs {
  const float2* C;      // (m_in, ldc) complex, columns [0, m_out) used
  float* out;           // m_out rows of n2 floats
  long long n2;         // 2K
  long long ntiles;
  int ldc, m_in, m_out, mp, ncs, nch, nbuf;
  float sign;           // -1 for subtraction
};

// 14 warps: at most 4 per SM sub-partition, so 128 registers a thread fit
__global__ void __maxnreg__(128) tc_rotate_kernel(const TrArgs a, const __grid_constant__ CUtensorMap map_s,
                                                  const __grid_constant__ CUtensorMap map_o) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t op_full[TR_NBUF_MAX], op_empty[TR_NBUF_MAX];
  __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done_bar;
  __shared__ __align__(8) uint64_t raw_full[TR_RAW], raw_empty[TR_RAW];
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int N = 2 * a.mp;
  const int kj = a.nch * TR_JC;            // rows of the coefficient operand
  const uint32_t b_half = (uint32_t)N * kj * 4;
  // TMA box destinations: align the raw ring to 1024 bytes
  unsigned char* raw = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
  unsigned char* bops = raw + TR_RAW * TR_RAW_BYTES;
  const uint32_t col_a = (uint32_t)(2 * N);                // first TMEM operand column
  const uint32_t tcols = tmem_cols_for(2 * N + a.nbuf * 2 * TR_JC);

  if (tid == 0) {
    abort_s = 0;
    for (int b = 0; b < a.nbuf; ++b) {
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
  // coefficient operand, K-major core matrices: row n (D column), column j (input row)
  // rows [0, mp) = Re C[:, n], rows [mp, 2mp) = Im C[:, n - mp]. Inputs j < 16*ncs are
  // S rows (coefficient 0 past m_in), inputs 16*ncs + i are output rows i (identity).
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
  if (a.nch > a.ncs)
    for (int i = tid; i < a.m_out; i += TR_THREADS) put(i, a.ncs * TR_JC + i, 1.f);
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
    // warp w writes TMEM lane quarter w % 4; thread = position p = lane of its quarter;
    // warps 0-3 take rows [0, TR_RPT) of a stage, warps 4-7 rows [TR_RPT, TR_JC)
    const int q4 = warp & 3, hv = warp >> 2;
    const int p = q4 * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(q4 * 32) << 16);
    int o = 0;
    uint32_t uo = 0;                                   // operand ring slot and its use count
    for (long long s = 0; s < nstages; ++s) {
      const int slot = (int)(s % TR_RAW);
      if (abort_s) break;
      if (!mbar_wait(&raw_full[slot], (uint32_t)((s / TR_RAW) & 1))) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      const float* rs = reinterpret_cast<const float*>(raw + slot * TR_RAW_BYTES) + p;
      float hi[TR_RPT], lo[TR_RPT];
#pragma unroll
      for (int r = 0; r < TR_RPT; ++r) {
        const float x = rs[(hv * TR_RPT + r) * TR_M];
        split_tf32(x, hi[r], lo[r]);
      }
      // the split values must exist before the raw slot goes back to the loader: an arrive
      // issued while the shared loads are still in flight lets the next TMA box land
      // under them (the compiler may otherwise sink the arithmetic below the arrive)
#pragma unroll
      for (int r = 0; r < TR_RPT; ++r) asm volatile("" ::"f"(hi[r]), "f"(lo[r]) : "memory");
      mbar_arrive(&raw_empty[slot]);
      if (!mbar_wait(&op_empty[o], (uo + 1) & 1)) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      fence_after_sync();
      const uint32_t col = col_a + (uint32_t)(o * 2 * TR_JC + hv * TR_RPT);
#pragma unroll
      for (int r8 = 0; r8 < TR_RPT; r8 += 8) {
        tmem_st8(lane_base + col + r8, *reinterpret_cast<const float(*)[8]>(hi + r8));
        tmem_st8(lane_base + col + TR_JC + r8, *reinterpret_cast<const float(*)[8]>(lo + r8));
      }
      tmem_wait_st();
      fence_before_sync();
      mbar_arrive(&op_full[o]);
      if (++o == a.nbuf) {
        o = 0;
        ++uo;
      }
    }
  } else if (warp < 12) {
    // ---------------- epilogue ----------------
    const int p = tid - TR_EPI0;                       // = 32 * (warp % 4) + lane
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const bool even = (p & 1) == 0;
    for (long long k = 0; k < my_tiles; ++k) {
      if (abort_s) break;
      const int ab = (int)(k & 1);
      if (!mbar_wait(&acc_full[ab], (uint32_t)((k >> 1) & 1), 128)) {
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
    const uint64_t b_desc0 = smem_desc(smem_u32(bops), 128, (uint32_t)kq * 128);
    bool issued = false;
    int o = 0;
    uint32_t uo = 0;                                   // operand ring slot and its use count
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
        if (!mbar_wait(&op_full[o], uo & 1)) {
          abort_s = 1;
          atomicExch(&g_tc_error, 1);
          break;
        }
        fence_after_sync();
        const uint32_t a_hi = tmem + col_a + (uint32_t)(o * 2 * TR_JC), a_lo = a_hi + TR_JC;
        // descriptors differ from the base one only in the start-address field
        const uint64_t bh0 = b_desc0 + (uint64_t)((c * (TR_JC / 4) * 128) >> 4);
#pragma unroll
        for (int g = 0; g < TR_JC / 8; ++g) {
          const uint64_t bh = bh0 + (uint64_t)(g * 256 >> 4), bl = bh + (uint64_t)(b_half >> 4);
          mma_tf32_ts(d, a_hi + 8 * g, bh, idesc, (c | g) ? 1u : 0u);
          mma_tf32_ts(d, a_hi + 8 * g, bl, idesc, 1u);
          mma_tf32_ts(d, a_lo + 8 * g, bh, idesc, 1u);
        }
        mma_commit(&op_empty[o]);
        issued = true;
        if (++o == a.nbuf) {
          o = 0;
          ++uo;
        }
      }
      if (abort_s) break;
      mma_commit(&acc_full[ab]);
    }
    if (abort_s && issued) {
      // let this thread's MMAs finish before the TMEM they write is freed
      mma_commit(&done_bar);
      mbar_wait(&done_bar, 0);
    }
  } else if (warp == TR_LOAD_WARP && lane == 0) {
    // ---------------- loader ----------------
    // one 2-D TMA box per stage: rows [16c, 16c + 16) of S (chunks c < ncs) or of the
    // output (chunks c >= ncs), positions [128 t, 128 t + 128); outside the matrix the
    // box reads zeros. The transaction count is the full box.
    long long tile = blockIdx.x;
    int c = 0;
    long long issued = 0;
    for (long long s = 0; s < nstages; ++s) {
      const int slot = (int)(s % TR_RAW);
      if (abort_s) break;
      if (!mbar_wait(&raw_empty[slot], (uint32_t)(((s / TR_RAW) + 1) & 1), 64)) {
        abort_s = 1;
        atomicExch(&g_tc_error, 1);
        break;
      }
      mbar_arrive_expect_tx(&raw_full[slot], TR_RAW_BYTES);
      const int x = (int)(tile * TR_M);
      if (c < a.ncs) tma_load_2d(raw + slot * TR_RAW_BYTES, &map_s, x, c * TR_JC, &raw_full[slot]);
      else tma_load_2d(raw + slot * TR_RAW_BYTES, &map_o, x, (c - a.ncs) * TR_JC, &raw_full[slot]);
      issued = s + 1;
      if (++c == a.nch) {
        c = 0;
        tile += gridDim.x;
      }
    }
    // no copy may still be landing when the CTA exits: wait for the last issued phases
    for (long long s = issued - TR_RAW > 0 ? issued - TR_RAW : 0; s < issued; ++s)
      mbar_wait(&raw_full[(int)(s % TR_RAW)], (uint32_t)((s / TR_RAW) & 1));
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == TR_MMA_WARP) tmem_dealloc(tmem, tcols);
}

size_t tr_smem(int nch, int mp) {
  const size_t s = (size_t)TR_RAW * TR_RAW_BYTES + (size_t)2 * (2 * mp) * (nch * TR_JC) * 4 + 1024;
  return s < (size_t)TR_SMEM_MIN ? (size_t)TR_SMEM_MIN : s;
}

int chunks_for(int m_in, int m_out, int mode) {
  return (m_in + TR_JC - 1) / TR_JC + (mode != 0 ? (m_out + TR_JC - 1) / TR_JC : 0);
}

}  // namespace

namespace ef {

// largest number of S rows one tensor-core pass holds for m_out outputs in `mode`
// (the accumulate modes also stage the m_out output rows); 0 when m_out > 64
int tc_rotate_max_rows(int m_out, int mode) {
  if (m_out <= 0 || m_out > 64) return 0;
  const int mp = (m_out + 7) / 8 * 8;
  int rows = 0;
  while (tr_smem(chunks_for(rows + TR_JC, m_out, mode), mp) <= (size_t)TR_SMEM_MAX) rows += TR_JC;
  return rows;
}

// one pass: m_out <= 64, m_in <= tc_rotate_max_rows(m_out, mode); S and out 16-byte
// aligned, K even
int tc_rotate_launch(const float* C, int ldc, const float* S, float* out, int m_in, int m_out,
                     long long K, int mode, cudaStream_t st) {
  TrArgs a;
  a.C = (const float2*)C;
  a.out = out;
  a.n2 = 2 * K;
  a.ntiles = (a.n2 + TR_M - 1) / TR_M;
  a.ldc = ldc;
  a.m_in = m_in;
  a.m_out = m_out;
  a.mp = (m_out + 7) / 8 * 8;
  a.ncs = (m_in + TR_JC - 1) / TR_JC;
  a.nch = chunks_for(m_in, m_out, mode);
  a.sign = mode < 0 ? -1.f : 1.f;
  a.nbuf = (512 - 2 * 2 * a.mp) / (2 * TR_JC);          // TMEM left after the accumulators
  if (a.nbuf > TR_NBUF_MAX) a.nbuf = TR_NBUF_MAX;
  CUtensorMap ms, mo;
  if (!make_tmap_2d(&ms, S, m_in, a.n2, TR_M, TR_JC, false) ||
      !make_tmap_2d(&mo, out, m_out, a.n2, TR_M, TR_JC, false))
    return ef_fail(EF_ERR_CUDA, "rotate: tensor map encoding failed");
  const size_t smem = tr_smem(a.nch, a.mp);
  ef::set_smem_once(tc_rotate_kernel, smem);
  long long grid = ef::sm_count();
  if (grid > a.ntiles) grid = a.ntiles;
  ef_count_launches(1);
  tc_rotate_kernel<<<(unsigned)grid, TR_THREADS, smem, st>>>(a, ms, mo);
  return ef_check_launch();
}

// device address of the tensor-core kernels' error flag (current device)
int* tc_error_dev() {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_tc_error) != cudaSuccess) return nullptr;
  return (int*)p;
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

// queues a copy of the flag into host memory on a stream (the flag is not cleared)
int tc_error_flag_async(int* host_flag, cudaStream_t st) {
  cudaError_t e = cudaMemcpyFromSymbolAsync(host_flag, g_tc_error, sizeof(int), 0,
                                            cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return ef_fail(EF_ERR_CUDA, cudaGetErrorString(e));
  return EF_OK;
}

}  // namespace ef

extern "C" int ef_tc_error_async(int* host_flag, void* stream) {
  if (!host_flag) return ef_fail(EF_ERR_INVALID, "null flag");
  return ef::tc_error_flag_async(host_flag, (cudaStream_t)stream);
}

extern "C" int ef_tc_error(int* flag) {
  if (!flag) return ef_fail(EF_ERR_INVALID, "null flag");
  return ef::tc_error_flag(flag);
}
