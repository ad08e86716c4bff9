// Arithmetic-rate probe: a long chain of independent fp32 fused multiply-adds per
// thread (scalar FFMA or the paired FFMA2 of sm_100 and later), for measuring the
// FP32 roof the Θ pipeline's FFT work is compared against. Each thread carries eight
// independent accumulators so that the FMA pipes, not the dependency latency, bound
// the rate; the results are stored so that nothing is optimised away.
#include "common.cuh"
#include "status.h"

namespace {

constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) fma_probe_kernel(float* out, int iters, float b, float c) {
  float a0 = threadIdx.x * 1e-6f, a1 = a0 + 1e-3f, a2 = a0 + 2e-3f, a3 = a0 + 3e-3f;
  float a4 = a0 + 4e-3f, a5 = a0 + 5e-3f, a6 = a0 + 6e-3f, a7 = a0 + 7e-3f;
  for (int i = 0; i < iters; ++i) {
    a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
    a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void __launch_bounds__(kProbeThreads) fma2_probe_kernel(float* out, int iters, float b, float c) {
  const float2 bb = make_float2(b, b), cc = make_float2(c, c);
  float2 a0 = make_float2(threadIdx.x * 1e-6f, 1e-3f), a1 = make_float2(2e-3f, 3e-3f);
  float2 a2 = make_float2(4e-3f, 5e-3f), a3 = make_float2(6e-3f, 7e-3f);
  for (int i = 0; i < iters; ++i) {
    a0 = __ffma2_rn(a0, bb, cc); a1 = __ffma2_rn(a1, bb, cc);
    a2 = __ffma2_rn(a2, bb, cc); a3 = __ffma2_rn(a3, bb, cc);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0.x + a0.y + a1.x + a1.y + a2.x + a2.y + a3.x + a3.y;
}

}  // namespace

extern "C" {

long long ef_fma_probe_flops(int blocks, int iters) {
  return 2LL * 8 * (long long)iters * blocks * kProbeThreads;
}

int ef_fma_probe(float* out, int blocks, int iters, int paired, void* stream) {
  if (!out || blocks <= 0 || iters <= 0) return ef_fail(EF_ERR_INVALID, "fma_probe: bad arguments");
  ef_count_launches(1);
  if (paired)
    fma2_probe_kernel<<<blocks, kProbeThreads, 0, (cudaStream_t)stream>>>(out, iters, 0.999f, 1e-7f);
  else
    fma_probe_kernel<<<blocks, kProbeThreads, 0, (cudaStream_t)stream>>>(out, iters, 0.999f, 1e-7f);
  return ef_check_launch();
}

}  // extern "C"
