// Shared definitions of the eigenfns_gb300 CUDA library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>


#include "../../include/eigenfns_gb300.h"

namespace ef {

// Operator handle: one scalar-eps problem (grid, box, Bloch k) resident on the device.
struct Op {
  int G;            // grid edge
  int R1, R2;       // pencil FFT split G = R1 * R2
  long long N;      // G^3 voxels
  double L;         // box edge
  double k[3];      // Bloch k in units of 2 pi / L
  float kn_floor;   // half the smallest nonzero |k+G|
  double eps_mean_inv;
  int device;
  // device tables (owned)
  float* kax;       // (3, G) per-axis k+G components, fp64-rounded
  uint32_t* swap;   // (ceil(N/32)) reference-axis switch bit per voxel
  float* inv_eps;   // (N) 1/eps / N  (the inverse FFT's 1/N folded in)
  float* eps_n;     // (N) eps / N
  float* eps_raw;   // (N) eps as given (for field outputs)
  float2* tw;       // (G) exp(+2 pi i j / G)
  // three-pass operator (zplane.cuh) only: eps^-1/N and eps/N per plane z in the
  // digit-reversed slot order of the plane pass, [z][k1][q][j]
  float* wperm_inv;
  float* wperm_eps;
  // pipeline selection (ef_op_configure): 0 automatic, 3 three-pass, 5 five-pass;
  // sub-batch workspace cap in bytes (0 = default)
  int passes;
  size_t subbatch_bytes;
};

// Frame at one voxel, computed from the per-axis tables exactly as the reference
// builds it: t1 = K x ref / |K x ref|, t2 = K x t1 / |K x t1|, ref = z unless the
// switch bit selects x, both zero where K = 0.
struct Frame {
  float kn, t1x, t1y, t1z, t2x, t2y, t2z;
};

__device__ __forceinline__ Frame make_frame(float Kx, float Ky, float Kz, bool sw) {
  Frame f;
  f.kn = sqrtf(Kx * Kx + Ky * Ky + Kz * Kz);
  float ax, ay, az;
  if (!sw) { ax = Ky; ay = -Kx; az = 0.f; }       // K x z
  else     { ax = 0.f; ay = Kz; az = -Ky; }       // K x x
  float n1sq = ax * ax + ay * ay + az * az;
  if (n1sq == 0.f) {
    f.t1x = f.t1y = f.t1z = f.t2x = f.t2y = f.t2z = 0.f;
    return f;
  }
  // normalise with one reciprocal square root each (a few ulp, like the fp64
  // frame rounded to fp32)
  const float r1 = rsqrtf(n1sq);
  ax *= r1; ay *= r1; az *= r1;
  float bx = Ky * az - Kz * ay;
  float by = Kz * ax - Kx * az;
  float bz = Kx * ay - Ky * ax;
  float n2sq = bx * bx + by * by + bz * bz;
  const float r2 = n2sq > 0.f ? rsqrtf(n2sq) : 1.f;
  f.t1x = ax; f.t1y = ay; f.t1z = az;
  f.t2x = bx * r2; f.t2y = by * r2; f.t2z = bz * r2;
  return f;
}

__device__ __forceinline__ Frame frame_at(const float* __restrict__ kax,
                                          const uint32_t* __restrict__ swap, int G,
                                          int x, int y, int z) {
  long long idx = ((long long)x * G + y) * G + z;
  bool sw = (swap[idx >> 5] >> (idx & 31)) & 1u;
  return make_frame(kax[x], kax[G + y], kax[2 * G + z], sw);
}

// Raise a kernel's dynamic shared-memory limit once per (kernel, device), and
// again only for a larger size: the attribute call costs far more than a launch,
// and the pipeline launches its kernels hundreds of times per solve.
void set_smem_limit(const void* kernel, size_t smem);

// number of SMs of the current device (queried once per device)
int sm_count();

template <class K>
inline void set_smem_once(K kernel, size_t smem) {
  if (smem > 48 * 1024) set_smem_limit(reinterpret_cast<const void*>(kernel), smem);
}

}  // namespace ef

// the opaque handle of the C ABI is the operator record itself
struct ef_op : public ef::Op {};
