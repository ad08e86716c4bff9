// Gram matrices on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// G[i][j] = sum_k conj(A[i,k]) B[j,k] over complex64 rows, computed as real
// products over the interleaved (re, im) storage:
//   Re G = A_r . B_r^T            A_r[i] = (ar0, ai0, ar1, ai1, ...)
//   Im G = A'_r . B_r^T           A'_r[i] = (-ai0, ar0, -ai1, ar1, ...)
// The M = 128 operand holds up to MT (32 or 64) rows of A in rows [0, MT) and the
// matching rows of A' in [MT, 2MT); the N operand holds NB rows of B as
// [B_hi; B_lo]. Per 8-real k-step two MMAs give fp32-class products (x = hi + lo):
//   D[:, 0:2NB]  += A_hi [B_hi; B_lo]^T      (hh | hl)
//   D[:, NB:2NB] += A_lo B_hi^T              (hl + lh)
// A tiles of up to 32 rows pack two K-ranges into the 128 lanes (PK = 2): lanes [0, 64)
// take the stage's reals [0, 32) and lanes [64, 128) its reals [32, 64) at the same
// k-step; B is laid out as [B1_lo; B1_hi; B2_hi; B2_lo] (1, 2: the two K-ranges), so
//   D[:, 0:4NB]  += A_hi [B1_lo; B1_hi; B2_hi; B2_lo]^T
//   D[:, NB:3NB] += A_lo [B1_hi; B2_hi]^T
// leaves each lane half's three products in its own 2NB columns (the other half's
// columns hold cross terms that are never read): half the MMAs per stage.
// Tensor-core fp32 accumulation is not round-to-nearest over long chains, so the
// accumulation is cut into segments of 32 k-steps, alternating between two TMEM
// accumulators where TMEM holds two; each finished segment is read back (tcgen05.ld)
// and added into fp32 registers while the next segment's MMAs run; a work unit's sum
// goes out in fp64 and units (K-chunks, and the two K-ranges) are reduced in fp64.
//
// A persistent CTA (576 threads) walks work units (A-tile, B-tile, K-chunk):
//   warp 17      loads: per 32-complex stage two 2-D TMA boxes (128-byte swizzle, zero
//                fill outside) of the unit's A rows and two of its B rows into a raw
//                shared-memory ring (the shared memory the operand ring leaves);
//   warps 0-11   three groups of four converter warps, taking the stages round robin
//                (a group's wait-convert-store chain per stage is longer than a stage's
//                share of HBM time, so three chains run staggered; two groups, 448
//                threads and warps shifted down by 4, where the TMEM operand ring holds
//                only two stages):
//                A rows hi/lo split and tcgen05.st into a ring of TMEM operand stages
//                (the MMA's A operand lives in TMEM, one A or A' row per lane), B rows
//                hi/lo split into a ring of K-major shared-memory stages;
//   warp 16      one thread issues each stage's MMAs and commits them;
//   warps 12-15  drain finished segments (one TMEM lane per thread, all columns)
//                and write the unit's partial sums.
// Every mbarrier wait is bounded; on timeout the kernel sets the error flag, stops,
// waits (bounded) for its own copies and MMAs and frees its TMEM.
//
// Reference: gram, eigenfns/solver.py:35-43 (true-fp32 X^H Y; the reference
// forbids plain TF32, which floors the Gram at ~1e-3).
#include <cuda.h>

#include <cstdint>

#include "common.cuh"
#include "status.h"
#include "tc_common.cuh"
#include "tmap.h"

namespace ef {
bool gram_tune_get(int ma, int mb, int* kernel, int* units);
}

namespace {

using namespace ef::tc;

constexpr int GC_GROUP = 128;         // converter threads per stage (one group of 4 warps)
constexpr int GC_KB = 64;             // reals per stage (32 complex) = 8 k-steps of 8
constexpr int GC_BOX = 32;            // reals per TMA box row (128 bytes, the swizzle width)
constexpr int GC_RAW_MAX = 12;        // raw box stages at most (the rest of shared memory)
constexpr int GC_SEG = 4;             // stages per TMEM accumulation segment (32 k-steps)
constexpr int GC_SMEM_MIN = 120 * 1024;   // keeps one CTA (and its TMEM) per SM
constexpr int GC_MIN_UNIT = 512;          // complex values per work unit at least (16 stages)
// TMEM split between accumulators and the operand ring (compile-time tuning knobs): at
// most EF_GC_NACC_MAX accumulators (1 gives their columns to the operand ring) and at
// most EF_GC_NBUF_MAX operand stages
#ifndef EF_GC_NACC_MAX
#define EF_GC_NACC_MAX 2
#endif
#ifndef EF_GC_NBUF_MAX
#define EF_GC_NBUF_MAX 4
#endif

// byte offset of (row r, k-quad q) in a K-major operand tile of QPR quads per row: core
// matrices of 8 rows x 16 B, K-adjacent core matrices 128 B apart, 8-row groups QPR*128 B
// apart
template <int QPR>
__device__ __forceinline__ int quad_off(int r, int q) {
  return (((r >> 3) * QPR + q) << 7) + ((r & 7) << 4);
}

template <int QPR>
__device__ __forceinline__ uint64_t gram_desc(uint32_t addr) {
  return smem_desc(addr, 128, QPR * 128);
}

struct GcArgs {
  double* partial;      // entry-major (ma*mb, nk) double2
  int* err;
  long long K;          // complex values per row
  long long kchunk;     // complex values per unit (multiple of 16)
  int ma, mb, mt, nit, njt, nk;
};

// TMEM budget of one configuration. PK = 1: a stage's 64 reals run through 8 k-steps,
// one accumulator is [hh | hl] (2NB columns). PK = 2 (A tiles of 32 rows): the two
// 32-real halves of a stage go to the lane halves [0, 64) and [64, 128) side by side,
// 4 k-steps per stage, and the accumulator is [1lo | 1hi | 2hi | 2lo] (4NB columns).
template <int NB, int PK>
struct GcCfg {
  static constexpr int KS = GC_KB / 8 / PK;                    // k-steps per stage
  static constexpr int QPR = GC_KB / 4 / PK;                   // B quads per operand row
  static constexpr int ACOLS = 2 * GC_KB / PK;                 // TMEM columns of one A stage (hi, lo)
  static constexpr int DCOLS = 2 * NB * PK;                    // columns of one accumulator
  static constexpr int NACC = (2 * DCOLS + 2 * ACOLS <= 512 && EF_GC_NACC_MAX >= 2) ? 2 : 1;
  static constexpr int MTMAX = 64 / PK;                        // A rows per box
  static constexpr int B_BYTES = 2 * NB * GC_KB * 4;           // [B_hi; B_lo] per stage
  // raw stage: A boxes for reals [0,32) and [32,64), then the two B boxes
  static constexpr int RAW_BYTES = (2 * MTMAX + 2 * NB) * 128;
  // operand stages: what TMEM holds after the accumulators (at most 4, and at least 4 raw
  // stages beside them in 226 KB of shared memory); the raw ring takes the rest of the
  // shared memory, which sets the bytes in flight from HBM
  static constexpr int SMEM_BUDGET = 226 * 1024 - 1024;
  static constexpr int NBUF_TMEM = (512 - NACC * DCOLS) / ACOLS < EF_GC_NBUF_MAX
                                       ? (512 - NACC * DCOLS) / ACOLS
                                       : EF_GC_NBUF_MAX;
  static constexpr int NBUF_SMEM = (SMEM_BUDGET - 4 * RAW_BYTES) / B_BYTES;
  static constexpr int NBUF = NBUF_TMEM < NBUF_SMEM ? NBUF_TMEM : NBUF_SMEM;
  static constexpr int NRAW = (SMEM_BUDGET - NBUF * B_BYTES) / RAW_BYTES < GC_RAW_MAX
                                  ? (SMEM_BUDGET - NBUF * B_BYTES) / RAW_BYTES
                                  : GC_RAW_MAX;
  static_assert(NBUF >= 2 && NRAW >= 4, "operand and raw rings");
  static constexpr int SEG = GC_SEG * PK;                      // stages per segment (32 k-steps)
  // converter groups, taking the stages round robin. A group's wait for an operand
  // buffer is by phase parity, which is only unambiguous while the buffer's previous
  // user, NBUF stages back, is a stage the waiting group has already seen retire; with
  // NG groups a group's previous stage is NG back, so NG <= NBUF.
  static constexpr int NG = NBUF >= 3 ? 3 : 2;
  static constexpr int DRAIN_WARP = 4 * NG;                    // first of the 4 drain warps
  static constexpr int MMA_WARP = DRAIN_WARP + 4;
  static constexpr int LOAD_WARP = MMA_WARP + 1;
  static constexpr int THREADS = 32 * (LOAD_WARP + 1);         // 576 (NG = 3) or 448
  // raw slots are owned by groups: stage s goes to slot (s % NG) + NG * ((s / NG) % RPG),
  // so a slot's consecutive stages belong to one group, which has consumed the slot's
  // previous phase before it waits on the next (no parity aliasing between groups)
  static constexpr int RPG = NRAW / NG;                        // raw slots per group
  static constexpr int NRAW_USED = RPG * NG;
  static_assert(RPG >= 1, "a raw slot per converter group");
};

// raw slot of stage s and how many earlier stages used that slot
template <int NG, int RPG>
__device__ __forceinline__ int raw_slot(uint32_t s) {
  return (int)(s % NG) + NG * (int)((s / NG) % RPG);
}
template <int NG, int RPG>
__device__ __forceinline__ uint32_t raw_use(uint32_t s) {
  return (s / NG) / RPG;
}

// up to 18 warps, up to 5 on one SM sub-partition, whose 16,384 registers hold 5 warps x
// 32 x 96 registers (15,360)
template <int NB, int PK>
__global__ void __maxnreg__(96) tc_gram_kernel(const GcArgs a, const __grid_constant__ CUtensorMap map_a,
                                                const __grid_constant__ CUtensorMap map_b) {
  using Cfg = GcCfg<NB, PK>;
  constexpr int GC_NBUF = Cfg::NBUF;
  constexpr int NACC = Cfg::NACC;
  constexpr int B_BYTES = Cfg::B_BYTES;
  constexpr int RAW_BYTES = Cfg::RAW_BYTES;
  constexpr int GC_RAW = Cfg::NRAW;
  constexpr int MTMAX = Cfg::MTMAX;
  constexpr int IPB = NB * (GC_KB / 4) / 128;                  // B items per B-converter thread
  constexpr uint32_t COL_A = NACC * Cfg::DCOLS;                // first TMEM operand column
  constexpr uint32_t TCOLS = tmem_cols_for(COL_A + GC_NBUF * Cfg::ACOLS);
  static_assert(COL_A + GC_NBUF * Cfg::ACOLS <= 512, "TMEM budget");
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t op_full[GC_NBUF], op_empty[GC_NBUF];
  __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done_bar;
  __shared__ __align__(8) uint64_t raw_full[GC_RAW], raw_empty[GC_RAW];
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // raw boxes use the 128-byte swizzle, which wants 1024-byte aligned stages
  unsigned char* raw = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
  unsigned char* bst = raw + GC_RAW * RAW_BYTES;
  const long long units = (long long)a.nit * a.njt * a.nk;
  const long long my_units = units > blockIdx.x ? (units - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

  if (tid == 0) {
    abort_s = 0;
    for (int b = 0; b < GC_NBUF; ++b) {
      mbar_init(&op_full[b], GC_GROUP);
      mbar_init(&op_empty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 128);
    }
    mbar_init(&done_bar, 1);
    for (int b = 0; b < GC_RAW; ++b) {
      mbar_init(&raw_full[b], 1);
      mbar_init(&raw_empty[b], GC_GROUP);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  constexpr int GC_MMA_WARP = Cfg::MMA_WARP, GC_LOAD_WARP = Cfg::LOAD_WARP, GC_NGROUPS = Cfg::NG;
  if (warp == GC_MMA_WARP) tmem_alloc(&tmem_base_s, TCOLS);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = tmem_base_s;
  constexpr uint32_t nbuf = GC_NBUF;

  // k-th unit of this CTA -> (A-tile, B-tile, K-chunk), first complex index, stages
  auto unit_of = [&](long long k, int& it, int& jt, int& kc, long long& kbeg, int& nst) {
    const long long u = blockIdx.x + k * (long long)gridDim.x;
    kc = (int)(u % a.nk);
    const long long t = u / a.nk;
    jt = (int)(t % a.njt);
    it = (int)(t / a.njt);
    kbeg = (long long)kc * a.kchunk;
    long long kend = kbeg + a.kchunk;
    if (kend > a.K) kend = a.K;
    nst = kend > kbeg ? (int)((kend - kbeg + GC_KB / 2 - 1) / (GC_KB / 2)) : 0;
  };

  if (warp < Cfg::DRAIN_WARP) {
    // ---------------- converters ----------------
    // Three groups of four warps take the stages round robin (group g the stages s with
    // s % 3 == g), so one stage's waits and TMEM stores overlap the next stages' work. In a group,
    // thread t (TMEM lane t) converts:
    //   A rows: lane l < mt is A row l, mt <= l < 2mt is A' row l - mt; PK = 1: l = t, both
    //   halves of the stage; PK = 2: l = t & 63, the half t >> 6 (reals [32 h, 32 h + 32));
    //   B items e = t + 128 u -> row e % NB, quad e / NB (consecutive threads, consecutive
    //   rows: conflict-free swizzled reads and operand stores).
    // Quads past the unit's end read zero (boxes past the matrix are zero-filled).
    const int grp = warp >> 2;
    const int t = tid & 127;
    const int rg = PK == 2 ? (t >> 6) : 0;
    const int l = PK == 2 ? (t & 63) : t;
    const bool aprime = l >= a.mt;
    const int ar = aprime ? l - a.mt : l;
    const bool aact = l < 2 * a.mt;
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    uint32_t s = 0;                                     // stage counter (32-bit ring arithmetic)
    for (long long k = 0; k < my_units && !abort_s; ++k) {
      int it, jt, kc, nst;
      long long kbeg;
      unit_of(k, it, jt, kc, kbeg, nst);
      long long kend = kbeg + a.kchunk;
      if (kend > a.K) kend = a.K;
      for (int st = 0; st < nst; ++st, ++s) {
        if ((int)(s % GC_NGROUPS) != grp) continue;
        const int slot = raw_slot<Cfg::NG, Cfg::RPG>(s);
        const int o = (int)(s % nbuf);
        if (!mbar_wait(&raw_full[slot], raw_use<Cfg::NG, Cfg::RPG>(s) & 1u) ||
            !mbar_wait(&op_empty[o], (uint32_t)(((s / nbuf) + 1) & 1))) {
          abort_s = 1;
          atomicExch(a.err, 1);
          break;
        }
        fence_after_sync();
        const long long kc0 = kbeg + (long long)st * (GC_KB / 2);
        const int rem = kend - kc0 < GC_KB ? (int)(kend - kc0) : GC_KB;   // complex left in the unit
        const unsigned char* rs = raw + slot * RAW_BYTES;
        // B rows -> shared-memory operand stage
        unsigned char* base = bst + o * B_BYTES;
#pragma unroll 4
        for (int u = 0; u < IPB; ++u) {
          const int e = t + u * 128;
          const int rb = e % NB, q = e / NB, hf = q >> 3;   // quad q of 16: box hf, its quad q & 7
          const float4 x = (2 * q < rem)
                               ? *reinterpret_cast<const float4*>(rs + (2 * MTMAX + hf * NB + rb) * 128 +
                                                                  (((q & 7) ^ (rb & 7)) << 4))
                               : make_float4(0.f, 0.f, 0.f, 0.f);
          float4 hh, ll;
          split_tf32(x.x, hh.x, ll.x);
          split_tf32(x.y, hh.y, ll.y);
          split_tf32(x.z, hh.z, ll.z);
          split_tf32(x.w, hh.w, ll.w);
          if (PK == 1) {
            *reinterpret_cast<float4*>(base + quad_off<Cfg::QPR>(rb, q)) = hh;
            *reinterpret_cast<float4*>(base + quad_off<Cfg::QPR>(NB + rb, q)) = ll;
          } else {   // rows [1lo | 1hi | 2hi | 2lo]
            *reinterpret_cast<float4*>(base + quad_off<Cfg::QPR>((hf ? 2 * NB : NB) + rb, q & 7)) = hh;
            *reinterpret_cast<float4*>(base + quad_off<Cfg::QPR>((hf ? 3 * NB : 0) + rb, q & 7)) = ll;
          }
        }
        // A rows -> TMEM operand stage
        const uint32_t col = COL_A + (uint32_t)(o * Cfg::ACOLS);
        // in quarters of 16 reals (4 quads), so that a converter thread holds 32 values
#pragma unroll 1
        for (int h4 = 0; h4 < 4 / PK; ++h4) {
          const int h2 = h4 >> 1, qh = h4 & 1;
          const int hf = PK == 2 ? rg : h2;
          float h[16], lo[16];
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) {
            const int q = 4 * qh + qq;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
            if (aact && 2 * (8 * hf + q) < rem)
              x = *reinterpret_cast<const float4*>(rs + hf * MTMAX * 128 + ar * 128 + ((q ^ (ar & 7)) << 4));
            if (aprime) x = make_float4(-x.y, x.x, -x.w, x.z);   // (-ai, ar) per complex
            h[4 * qq] = x.x;
            h[4 * qq + 1] = x.y;
            h[4 * qq + 2] = x.z;
            h[4 * qq + 3] = x.w;
          }
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            split_tf32(h[e], h[e], lo[e]);
          }
          tmem_st16(lane_base + col + h2 * GC_BOX + 16 * qh, h);
          tmem_st16(lane_base + col + GC_KB / PK + h2 * GC_BOX + 16 * qh, lo);
        }
        tmem_wait_st();
        fence_async_smem();
        fence_before_sync();
        // the raw slot goes back to the loader only now: an arrive issued while shared
        // loads from it are still in flight (their registers not yet consumed) let the
        // next TMA box land under them
        mbar_arrive(&raw_empty[slot]);
        mbar_arrive(&op_full[o]);
      }
    }
  } else if (warp < GC_MMA_WARP) {
    // ---------------- drain ----------------
    const int lq = warp & 3;
    const int L = lq * 32 + lane;                       // TMEM lane = M row
    const int rg = PK == 2 ? (lq >> 1) : 0;             // lane half (warp-uniform)
    const int l = PK == 2 ? (L & 63) : L;
    const uint32_t lane_base = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(rg * 2 * NB);
    float acc[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) acc[c] = 0.f;
    uint32_t q = 0;                                     // segment counter
    for (long long k = 0; k < my_units && !abort_s; ++k) {
      int it, jt, kc, nst;
      long long kbeg;
      unit_of(k, it, jt, kc, kbeg, nst);
      const int nseg = (nst + Cfg::SEG - 1) / Cfg::SEG;
      for (int sg = 0; sg < nseg; ++sg, ++q) {
        const int ab = (int)(q % NACC);
        if (!mbar_wait(&acc_full[ab], (uint32_t)((q / NACC) & 1), NACC == 2 ? 128u : 32u)) {
          abort_s = 1;
          atomicExch(a.err, 1);
          break;
        }
        fence_after_sync();
        const uint32_t ta = lane_base + (uint32_t)(ab * Cfg::DCOLS);
#pragma unroll
        for (int c0 = 0; c0 < NB; c0 += 8) {
          float d1[8], d2[8];
          tmem_ld8x2(ta + c0, ta + NB + c0, d1, d2);
#pragma unroll
          for (int t = 0; t < 8; ++t) acc[c0 + t] += d1[t] + d2[t];
        }
        fence_before_sync();
        mbar_arrive(&acc_empty[ab]);
      }
      if (abort_s) break;
      // unit partial: lanes [0, mt) Re of A rows, [mt, 2mt) Im (of each lane half)
      const bool re = l < a.mt, im = l >= a.mt && l < 2 * a.mt;
      const int i = it * a.mt + (re ? l : l - a.mt);
      if ((re || im) && i < a.ma) {
#pragma unroll
        for (int c = 0; c < NB; ++c) {
          const int j = jt * NB + c;
          if (j < a.mb)
            a.partial[(((long long)i * a.mb + j) * (a.nk * PK) + kc * PK + rg) * 2 + (re ? 0 : 1)] =
                (double)acc[c];
        }
      }
#pragma unroll
      for (int c = 0; c < NB; ++c) acc[c] = 0.f;
    }
  } else if (warp == GC_MMA_WARP && lane == 0) {
    // ---------------- MMA issue ----------------
    const uint32_t id1 = idesc_tf32(128, 2 * NB * PK), id2 = idesc_tf32(128, NB * PK);
    const uint64_t bdesc0 = gram_desc<Cfg::QPR>(smem_u32(bst));
    // B_hi rows, the second MMA's operand: [0, NB) for PK = 1, [NB, 3NB) for PK = 2
    constexpr uint64_t b2off = PK == 2 ? (uint64_t)(((NB / 8) * Cfg::QPR * 128) >> 4) : 0;
    uint32_t s = 0, q = 0;
    bool issued = false;
    for (long long k = 0; k < my_units && !abort_s; ++k) {
      int it, jt, kc, nst;
      long long kbeg;
      unit_of(k, it, jt, kc, kbeg, nst);
      for (int st = 0; st < nst; ++st, ++s) {
        const bool seg_first = (st % Cfg::SEG) == 0;
        const bool seg_last = (st % Cfg::SEG) == Cfg::SEG - 1 || st == nst - 1;
        const int ab = (int)(q % NACC);
        if (seg_first && !mbar_wait(&acc_empty[ab], (uint32_t)(((q / NACC) + 1) & 1))) {
          abort_s = 1;
          atomicExch(a.err, 1);
          break;
        }
        const int o = (int)(s % nbuf);
        if (!mbar_wait(&op_full[o], (uint32_t)((s / nbuf) & 1))) {
          abort_s = 1;
          atomicExch(a.err, 1);
          break;
        }
        fence_after_sync();
        const uint32_t d = tmem + (uint32_t)(ab * Cfg::DCOLS);
        const uint32_t a_hi = tmem + COL_A + (uint32_t)(o * Cfg::ACOLS), a_lo = a_hi + GC_KB / PK;
        // descriptors differ from the base one only in the start-address field
        const uint64_t bB = bdesc0 + (uint64_t)((o * B_BYTES) >> 4);
#pragma unroll
        for (int g = 0; g < Cfg::KS; ++g) {
          const uint64_t off = (uint64_t)(g * 256 >> 4);
          mma_tf32_ts(d, a_hi + 8 * g, bB + off, id1, (seg_first && g == 0) ? 0u : 1u);
          mma_tf32_ts(d + NB, a_lo + 8 * g, bB + b2off + off, id2, 1u);
        }
        mma_commit(&op_empty[o]);
        issued = true;
        if (seg_last) {
          mma_commit(&acc_full[ab]);
          ++q;
        }
      }
    }
    if (abort_s && issued) {
      mma_commit(&done_bar);
      mbar_wait(&done_bar, 0);
    }
  } else if (warp == GC_LOAD_WARP && lane == 0) {
    // ---------------- loader ----------------
    // per stage two 2-D boxes of the unit's A rows and two of its B rows (16 complex =
    // 128 B per row and box), counted on raw_full in bytes
    uint32_t s = 0, issued = 0;
    for (long long k = 0; k < my_units && !abort_s; ++k) {
      int it, jt, kc, nst;
      long long kbeg;
      unit_of(k, it, jt, kc, kbeg, nst);
      const int i0 = it * a.mt, j0 = jt * NB;
      for (int st = 0; st < nst; ++st, ++s) {
        const int slot = raw_slot<Cfg::NG, Cfg::RPG>(s);
        if (!mbar_wait(&raw_empty[slot], (raw_use<Cfg::NG, Cfg::RPG>(s) + 1u) & 1u, 64u)) {
          abort_s = 1;
          atomicExch(a.err, 1);
          break;
        }
        const long long kc0 = kbeg + (long long)st * (GC_KB / 2);
        unsigned char* dst = raw + slot * RAW_BYTES;
        mbar_arrive_expect_tx(&raw_full[slot], (uint32_t)((2 * a.mt + 2 * NB) * 128));
        for (int hf = 0; hf < 2; ++hf) {
          const int x = (int)(2 * kc0) + hf * GC_BOX;
          tma_load_2d(dst + hf * MTMAX * 128, &map_a, x, i0, &raw_full[slot]);
          tma_load_2d(dst + (2 * MTMAX + hf * NB) * 128, &map_b, x, j0, &raw_full[slot]);
        }
        issued = s + 1;
      }
    }
    // no copy may still be landing when the CTA exits: wait for the last issued phases
    for (uint32_t t = issued > (uint32_t)Cfg::NRAW_USED ? issued - Cfg::NRAW_USED : 0; t < issued; ++t)
      mbar_wait(&raw_full[raw_slot<Cfg::NG, Cfg::RPG>(t)], raw_use<Cfg::NG, Cfg::RPG>(t) & 1u);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == GC_MMA_WARP) tmem_dealloc(tmem, TCOLS);
}

// one warp per Gram entry over its contiguous unit partials, fixed shuffle tree; with
// ld_t > 0 the computed (n / ld_t, ld_t) matrix is B^H A and entry e goes out conjugated
// to its transposed place in G = A^H B
__global__ void tc_gram_reduce_kernel(const double2* __restrict__ partial, int nsplit, int n,
                                      int ld_t, double2* __restrict__ G) {
  const int e = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= n) return;
  const double2* p = partial + (long long)e * nsplit;
  double sr = 0.0, si = 0.0;
  for (int s = lane; s < nsplit; s += 32) {
    sr += p[s].x;
    si += p[s].y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if (lane == 0) {
    if (ld_t > 0) G[(long long)(e % ld_t) * (n / ld_t) + e / ld_t] = make_double2(sr, -si);
    else G[e] = make_double2(sr, si);
  }
}

int tc_nb(int mb) { return mb <= 16 ? 16 : (mb <= 32 ? 32 : 64); }

template <int NB, int PK>
size_t gc_smem() {
  using Cfg = GcCfg<NB, PK>;
  const size_t s = (size_t)Cfg::NBUF * Cfg::B_BYTES + (size_t)Cfg::NRAW * Cfg::RAW_BYTES + 1024;
  return s < (size_t)GC_SMEM_MIN ? (size_t)GC_SMEM_MIN : s;
}

struct GcPlan {
  int mt, nb, pk, nit, njt, nk;
  long long kchunk;
};

// A tiles of up to 32 rows fill the 128 TMEM lanes with both halves of a stage (pk = 2)
// unless EF_GRAM_TC_PACK=0
bool gc_pack_enabled() {
  const char* e = getenv("EF_GRAM_TC_PACK");
  return !(e && e[0] == '0');
}

// G = A^H B with more than 32 rows of A and at most 32 of B runs as (B^H A)^H, the
// 32-row side in the packed A tiles (64x32 0.82 ms this way against 0.92 unpacked, 96x32
// 1.59 against 1.81, at K = 4.2M)
bool gc_swap(int ma, int mb) { return ma > 32 && mb <= 32 && gc_pack_enabled(); }

// units per SM: the autotuner's choice for the caller's (ma, mb), else 2
int gc_units(int ma, int mb) {
  int units = 0;
  ef::gram_tune_get(ma, mb, nullptr, &units);
  return units > 0 ? units : 2;
}

GcPlan gc_plan(int ma, int mb, long long K, int units) {
  GcPlan p;
  p.mt = ma <= 32 ? 32 : 64;
  p.pk = (p.mt == 32 && gc_pack_enabled()) ? 2 : 1;
  p.nb = tc_nb(mb);
  p.nit = (ma + p.mt - 1) / p.mt;
  p.njt = (mb + p.nb - 1) / p.nb;
  const long long tiles = (long long)p.nit * p.njt;
  const long long sms = ef::sm_count();
  long long nk = (units * sms + tiles - 1) / tiles;           // about `units` units per SM
  // >= GC_MIN_UNIT complex per unit: at small K (grids of 32^3-64^3) the units, not the
  // SMs, would otherwise run out (2048 per unit left 32 of 152 SMs busy at 32^3)
  const long long maxk = (K + GC_MIN_UNIT - 1) / GC_MIN_UNIT;
  if (nk > maxk) nk = maxk;
  if (nk < 1) nk = 1;
  long long kchunk = (K + nk - 1) / nk;
  kchunk = (kchunk + GC_KB / 2 - 1) / (GC_KB / 2) * (GC_KB / 2);
  p.kchunk = kchunk;
  p.nk = (int)((K + kchunk - 1) / kchunk);
  return p;
}

template <int NB, int PK>
int launch_gc(const GcPlan& p, cudaStream_t st, const float* A, const float* B, int ma, int mb,
               long long K, double* part, int* err) {
  GcArgs a;
  a.partial = part;
  a.err = err;
  a.K = K;
  a.kchunk = p.kchunk;
  a.ma = ma;
  a.mb = mb;
  a.mt = p.mt;
  a.nit = p.nit;
  a.njt = p.njt;
  a.nk = p.nk;

  CUtensorMap ma_map, mb_map;
  if (!ef::make_tmap_2d(&ma_map, A, ma, 2 * K, GC_BOX, p.mt, true) ||
      !ef::make_tmap_2d(&mb_map, B, mb, 2 * K, GC_BOX, NB, true))
    return ef_fail(EF_ERR_CUDA, "gram_tc: tensor map encoding failed");
  const size_t smem = gc_smem<NB, PK>();
  ef::set_smem_once(tc_gram_kernel<NB, PK>, smem);
  long long units = (long long)p.nit * p.njt * p.nk;
  long long grid = ef::sm_count();
  if (grid > units) grid = units;
  tc_gram_kernel<NB, PK><<<(unsigned)grid, GcCfg<NB, PK>::THREADS, smem, st>>>(a, ma_map, mb_map);
  return EF_OK;
}

}  // namespace

extern "C" size_t ef_gram_tc_workspace_bytes(int ma, int mb, long long K) {
  if (ma <= 0 || mb <= 0 || K <= 0) return 0;
  const int u = gc_units(ma, mb);
  const GcPlan p = gc_swap(ma, mb) ? gc_plan(mb, ma, K, u) : gc_plan(ma, mb, K, u);
  return (size_t)p.nk * p.pk * ma * mb * 2 * sizeof(double) + 512;
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
  const int units = gc_units(ma, mb);
  const bool swap = gc_swap(ma, mb);
  if (swap) {
    const float* t = A;
    A = B;
    B = t;
    const int tm = ma;
    ma = mb;
    mb = tm;
  }
  const GcPlan p = gc_plan(ma, mb, K, units);
  ef_count_launches(2);
  int rc;
  double* part = (double*)work;
  if (p.pk == 2) {
    if (p.nb == 16) rc = launch_gc<16, 2>(p, st, A, B, ma, mb, K, part, err_dev);
    else if (p.nb == 32) rc = launch_gc<32, 2>(p, st, A, B, ma, mb, K, part, err_dev);
    else rc = launch_gc<64, 2>(p, st, A, B, ma, mb, K, part, err_dev);
  } else {
    if (p.nb == 16) rc = launch_gc<16, 1>(p, st, A, B, ma, mb, K, part, err_dev);
    else if (p.nb == 32) rc = launch_gc<32, 1>(p, st, A, B, ma, mb, K, part, err_dev);
    else rc = launch_gc<64, 1>(p, st, A, B, ma, mb, K, part, err_dev);
  }
  if (rc != EF_OK) return rc;
  const int n = ma * mb;
  tc_gram_reduce_kernel<<<(n + 7) / 8, 256, 0, st>>>((const double2*)work, p.nk * p.pk, n,
                                                     swap ? mb : 0, (double2*)G);
  return ef_check_launch();
}
