// Sub-voxel-averaging rasterizer of periodic rod networks (benchmark inputs).
//
// The reference rasterizes binary, centre-sampled voxels (eigenfns/structure.py:51-151);
// the benchmark structures call for eps averaged over s^3 regular sub-samples per
// voxel. A rod is a flat-capped cylinder (the reference's membership test: axial
// 0 <= t <= |q-p| and radial distance <= r, structure.py:135-138) and wraps across
// the periodic box. A sub-sample inside any rod counts once; eps of a voxel is
// eps_bg + (eps_rod - eps_bg) * (inside sub-samples) / s^3. Geometry is fp64 so the
// result matches a numpy evaluation of the same test.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "status.h"

namespace {

__global__ void mark_kernel(const double* rods, int n_rods, int G, int s, double L,
                            unsigned int* bits) {
  const int r = blockIdx.x;
  if (r >= n_rods) return;
  const double* R = rods + 7 * (long long)r;
  const double px = R[0], py = R[1], pz = R[2];
  const double vx = R[3] - px, vy = R[4] - py, vz = R[5] - pz;
  const double rad = R[6];
  // explicit rounding (no FMA contraction) so the arithmetic is numpy's, bit for bit
  const double len = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz)));
  if (!(len > 0.0)) return;
  const double ux = vx / len, uy = vy / len, uz = vz / len;
  const int GS = G * s;
  const double h = L / GS;  // sub-sample spacing; sample a sits at (a + 0.5) h
  int lo[3], hi[3];
  const double pmin[3] = {fmin(px, R[3]), fmin(py, R[4]), fmin(pz, R[5])};
  const double pmax[3] = {fmax(px, R[3]), fmax(py, R[4]), fmax(pz, R[5])};
  for (int d = 0; d < 3; ++d) {
    lo[d] = (int)floor((pmin[d] - rad) / h - 0.5) - 1;
    hi[d] = (int)ceil((pmax[d] + rad) / h - 0.5) + 1;
  }
  const long long nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
  const long long total = nx * ny * nz;
  const double r2 = __dmul_rn(rad, rad);
  for (long long e = threadIdx.x; e < total; e += blockDim.x) {
    int a = lo[0] + (int)(e / (ny * nz));
    int b = lo[1] + (int)((e / nz) % ny);
    int c = lo[2] + (int)(e % nz);
    double X = __dsub_rn(__dmul_rn(a + 0.5, h), px);
    double Y = __dsub_rn(__dmul_rn(b + 0.5, h), py);
    double Z = __dsub_rn(__dmul_rn(c + 0.5, h), pz);
    double t = __dadd_rn(__dadd_rn(__dmul_rn(X, ux), __dmul_rn(Y, uy)), __dmul_rn(Z, uz));
    if (t < 0.0 || t > len) continue;
    double rx = __dsub_rn(X, __dmul_rn(t, ux));
    double ry = __dsub_rn(Y, __dmul_rn(t, uy));
    double rz = __dsub_rn(Z, __dmul_rn(t, uz));
    if (__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)) > r2) continue;
    int wa = ((a % GS) + GS) % GS, wb = ((b % GS) + GS) % GS, wc = ((c % GS) + GS) % GS;
    long long idx = ((long long)wa * GS + wb) * GS + wc;
    atomicOr(bits + (idx >> 5), 1u << (idx & 31));
  }
}

__global__ void average_kernel(const unsigned int* bits, int G, int s, double eps_rod,
                               double eps_bg, float* eps) {
  const long long N = (long long)G * G * G;
  const int GS = G * s;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    int z = i % G, y = (i / G) % G, x = i / ((long long)G * G);
    int cnt = 0;
    for (int a = 0; a < s; ++a)
      for (int b = 0; b < s; ++b)
        for (int c = 0; c < s; ++c) {
          long long idx = ((long long)(x * s + a) * GS + (y * s + b)) * GS + (z * s + c);
          cnt += (bits[idx >> 5] >> (idx & 31)) & 1u;
        }
    double f = (double)cnt / (double)(s * s * s);
    eps[i] = (float)__dadd_rn(eps_bg, __dmul_rn(eps_rod - eps_bg, f));
  }
}

}  // namespace

extern "C" int ef_rasterize_rods(int grid, double box_size, const double* rods_host, int n_rods,
                                 int sub, double eps_rod, double eps_bg, float* eps_host) {
  if (grid <= 0 || sub <= 0 || n_rods < 0 || !(box_size > 0.0) || !eps_host || (n_rods && !rods_host))
    return ef_fail(EF_ERR_INVALID, "bad rasterizer arguments");
  const long long GS = (long long)grid * sub;
  const long long nbits = GS * GS * GS;
  const long long N = (long long)grid * grid * grid;
  unsigned int* bits = nullptr;
  double* rods = nullptr;
  float* eps = nullptr;
  cudaError_t e = cudaMalloc(&bits, (size_t)((nbits + 31) / 32) * 4);
  if (e == cudaSuccess) e = cudaMemset(bits, 0, (size_t)((nbits + 31) / 32) * 4);
  if (e == cudaSuccess && n_rods) e = cudaMalloc(&rods, (size_t)n_rods * 7 * sizeof(double));
  if (e == cudaSuccess && n_rods)
    e = cudaMemcpy(rods, rods_host, (size_t)n_rods * 7 * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&eps, (size_t)N * sizeof(float));
  if (e == cudaSuccess) {
    ef_count_launches(n_rods ? 2 : 1);
    if (n_rods) mark_kernel<<<n_rods, 256>>>(rods, n_rods, grid, sub, box_size, bits);
    average_kernel<<<2048, 256>>>(bits, grid, sub, eps_rod, eps_bg, eps);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(eps_host, eps, (size_t)N * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(bits);
  cudaFree(rods);
  cudaFree(eps);
  if (e != cudaSuccess) return ef_fail(EF_ERR_CUDA, cudaGetErrorString(e));
  return EF_OK;
}
