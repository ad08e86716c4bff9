// Maxwell operator handle and the fused FFT pipeline entry points.
//
// Reference: eigenfns/operator.py (make_basis :44-79, _theta_block :82-95,
// _precondition_block :98-101, _precondition_fancy_block :104-127,
// MaxwellOperator :130-184), the Chebyshev recurrence of
// eigenfns/interior.py:336-354 and the KPM recurrences of
// eigenfns/chebyshev.py:254-263 and scripts/exp/exp_kpm_dos.py:141-152.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "fft_passes.cuh"
#include "plan.cuh"
#include "status.h"
#include "zplane.cuh"

using namespace ef;

namespace {

const std::vector<Plan>& plans() {
  static const std::vector<Plan> v = [] {
    std::vector<Plan> p;
    add_plans_small(p);
    add_plans_mid(p);
    add_plans_large(p);
    return p;
  }();
  return v;
}

const Plan* find_plan(int G) {
  for (const Plan& p : plans()) if (p.G == G) return &p;
  return nullptr;
}

const std::vector<Plan3>& plans3() {
  static const std::vector<Plan3> v = [] {
    std::vector<Plan3> p;
    add_plans3(p);
    return p;
  }();
  return v;
}

const Plan3* plan3_of_grid(int G) {
  for (const Plan3& p : plans3()) if (p.G == G) return &p;
  return nullptr;
}

// The three-pass operator serves the grid edges it has a plan for, unless the handle
// was configured for the five-pass pencil pipeline (ef_op_configure) or, for handles
// left on automatic, EF_THETA_PASSES=5 is set (comparisons).
const Plan3* find_plan3(const ef_op* op) {
  if (op->passes == 5) return nullptr;
  if (op->passes == 0) {
    static const bool five = [] {
      const char* e = std::getenv("EF_THETA_PASSES");
      return e && std::atoi(e) == 5;
    }();
    if (five) return nullptr;
  }
  return plan3_of_grid(op->G);
}

// Plane-pass multiplier in the slot order the plane pass sees between its inverse
// and forward transforms: in sub-plane (z, s), slot (row XR2*k1 + j, column q) holds
// real-space x = Q*(k1 + XR1*j) + s and y = q/YR2 + YR1*(q%YR2); stored
// [z][s][k1][q][j] so that one item's XR2 factors are contiguous.
void permute_plane_table(const std::vector<float>& w, const Plan3& p, std::vector<float>& out) {
  const int G = p.G, Q = p.Q, XR1 = p.x_R1, XR2 = p.x_R2, YR1 = p.y_R1, YR2 = p.y_R2;
  out.resize(w.size());
  size_t o = 0;
  for (int z = 0; z < G; ++z)
    for (int s = 0; s < Q; ++s)
      for (int k1 = 0; k1 < XR1; ++k1)
        for (int q = 0; q < G; ++q) {
          const int yr = q / YR2 + YR1 * (q % YR2);
          for (int j = 0; j < XR2; ++j) {
            const int xr = Q * (k1 + XR1 * j) + s;
            out[o++] = w[((size_t)xr * G + yr) * G + z];
          }
        }
}

// ---- host-side fp64 frame tables (operator.py:46-59) -----------------------------
void axis_wavevectors(int G, double L, const double k[3], std::vector<double>& K) {
  // 2*pi*fftfreq(G, d=L/G) + 2*pi*k/L, evaluated in numpy's operation order
  K.assign(3 * (size_t)G, 0.0);
  const double d = L / G;
  const double val = 1.0 / (G * d);
  const int Np = (G - 1) / 2 + 1;
  const double twopi = 2.0 * M_PI;
  for (int ax = 0; ax < 3; ++ax) {
    const double k0 = twopi * k[ax] / L;
    for (int i = 0; i < G; ++i) {
      long n = (i < Np) ? i : (long)i - G;
      K[(size_t)ax * G + i] = twopi * ((double)n * val) + k0;
    }
  }
}

__global__ void basis_kernel(const float* kax, const uint32_t* swap, int G, float* kn, float* t,
                             float* mask) {
  const long long N = (long long)G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    int z = i % G, y = (i / G) % G, x = i / ((long long)G * G);
    Frame f = frame_at(kax, swap, G, x, y, z);
    if (kn) kn[i] = f.kn;
    if (mask) mask[i] = f.kn > 0.f ? 1.f : 0.f;
    if (t) {
      t[0 * N + i] = f.t1x; t[1 * N + i] = f.t1y; t[2 * N + i] = f.t1z;
      t[3 * N + i] = f.t2x; t[4 * N + i] = f.t2y; t[5 * N + i] = f.t2z;
    }
  }
}

__global__ void precond_simple_kernel(const float* kax, int G, const float2* X, float2* Y,
                                      long long total, float scale) {
  const long long N = (long long)G * G * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long vox = i % N;
    int z = vox % G, y = (vox / G) % G, x = vox / ((long long)G * G);
    float Kx = kax[x], Ky = kax[G + y], Kz = kax[2 * G + z];
    float kn = sqrtf(Kx * Kx + Ky * Ky + Kz * Kz);
    float d = kn * kn + scale;
    float2 v = X[i];
    Y[i] = make_float2(v.x / d, v.y / d);
  }
}

// finalize per-vector sums of the pass-E partials (deterministic order)
enum FinMode { FIN_KPM_FIRST = 0, FIN_KPM_STEP = 1, FIN_COUNT_FIRST = 2, FIN_COUNT_STEP = 3 };

__global__ void finalize_kernel(const double* partials, int tiles, int mode, double* out, int ld,
                                int k, double c0, double c1) {
  __shared__ double r0[256], r1[256];
  const int v = blockIdx.x;
  double s0 = 0.0, s1 = 0.0;
  for (int t = threadIdx.x; t < tiles; t += blockDim.x) {
    s0 += partials[((long long)v * tiles + t) * 2];
    s1 += partials[((long long)v * tiles + t) * 2 + 1];
  }
  r0[threadIdx.x] = s0;
  r1[threadIdx.x] = s1;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      r0[threadIdx.x] += r0[threadIdx.x + o];
      r1[threadIdx.x] += r1[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double d0 = r0[0], d1 = r1[0];
    double* row = out + (long long)v * ld;
    if (mode == FIN_KPM_FIRST) { row[0] = d0; row[1] = d1; }
    else if (mode == FIN_KPM_STEP) { row[2 * k] = 2.0 * d0 - row[0]; row[2 * k + 1] = 2.0 * d1 - row[1]; }
    else if (mode == FIN_COUNT_FIRST) { row[0] = c0 * d0 + c1 * d1; }
    else { row[0] += c0 * d0; }
  }
}

// Sub-batch workspace cap: the three-pass workspace of one sub-batch should stay in
// L2 (126 MB) next to the streamed input and output, so it defaults to 64 MB (one
// vector at 128^3); EF_SUBBATCH_BYTES overrides it for both pipelines.
size_t subbatch_cap_bytes(const ef_op* op, bool three_pass) {
  if (op->subbatch_bytes > 0) return op->subbatch_bytes;
  const char* e = std::getenv("EF_SUBBATCH_BYTES");
  if (e) {
    long long v = std::atoll(e);
    if (v > 0) return (size_t)v;
  }
  return (size_t)(three_pass ? 64 : 96) << 20;
}

struct Sizes {
  long long N;
  const Plan3* p3;     // three-pass plan, or null for the five-pass pipeline
  int tiles;           // last-pass tiles per vector (one partial each)
  int tiles_a;         // pass-A tiles per vector
  size_t per_vec;      // E bytes per vector
  size_t per_vec_part; // partial bytes per vector
};

Sizes sizes_of(const ef_op* op, const Plan* p) {
  Sizes s;
  s.N = op->N;
  s.p3 = find_plan3(op);
  s.tiles = s.p3 ? (op->G * op->G) / kZT : (op->G * op->G) / p->NRE;
  s.tiles_a = (op->G * op->G) / p->NRA;
  s.per_vec = (size_t)3 * s.N * sizeof(float2);
  s.per_vec_part = ((size_t)s.tiles * 2 * sizeof(double) + 255) / 256 * 256;
  return s;
}

int mb_cap(const ef_op* op, const Sizes& s) {
  size_t cap = subbatch_cap_bytes(op, s.p3 != nullptr) / s.per_vec;
  return cap < 1 ? 1 : (int)(cap > 4096 ? 4096 : cap);
}

struct Pipe {
  int build;   // BuildMode
  int wmode;   // WMode (0/1)
  int epi;     // EpiMode
  int fin;     // -1 none, else FinMode
};

// Run the operator pipeline (three-pass where the grid edge has a plan, else the
// five-pass pencil pipeline) on m vectors in sub-batches.
int run_pipe(const ef_op* op, const Pipe& pp, const float2* X, float2* out, float2* T0, float2* Y,
             const float2* Z, int m, float s, float c0, float c1, double* fin_out, int fin_ld,
             int fin_k, double fc0, double fc1, void* work, size_t work_bytes, cudaStream_t st) {
  if (!op || m <= 0 || !X) return ef_fail(EF_ERR_INVALID, "null operator/input or m <= 0");
  const Plan* p = find_plan(op->G);
  if (!p) return ef_fail(EF_ERR_UNSUPPORTED, "no FFT plan for this grid");
  Sizes sz = sizes_of(op, p);
  if (!work) return ef_fail(EF_ERR_WORKSPACE, "work buffer is null");
  int mb = mb_cap(op, sz);
  if (mb > m) mb = m;
  size_t need1 = sz.per_vec + sz.per_vec_part + 256;
  if (work_bytes < need1) return ef_fail(EF_ERR_WORKSPACE, "work buffer smaller than one vector's workspace");
  int fit = (int)((work_bytes - 256) / (sz.per_vec + sz.per_vec_part));
  if (fit < mb) mb = fit;
  float2* E = reinterpret_cast<float2*>(work);
  size_t e_bytes = (size_t)mb * sz.per_vec;
  double* partials = reinterpret_cast<double*>(reinterpret_cast<char*>(work) + (e_bytes + 255) / 256 * 256);
  const int G = op->G, NZ = p->NZ, PS = p->PS;
  const size_t smem_a = (size_t)(3 * p->NRA * p->PSA + G) * sizeof(float2);
  const size_t smem_e = (size_t)(3 * p->NRE * p->PSE + G) * sizeof(float2);
  const size_t smem_y = (size_t)(NZ * PS + G) * sizeof(float2);
  const size_t smem_c = (size_t)(2 * NZ * PS + G) * sizeof(float2);
  const long long N2 = 2 * op->N;
  for (int v0 = 0; v0 < m; v0 += mb) {
    const int nb = (m - v0) < mb ? (m - v0) : mb;
    const long long off = (long long)v0 * N2;
    if (sz.p3) {
      const Plan3* q = sz.p3;
      P3Args a;
      std::memset(&a, 0, sizeof(a));
      a.X = X + off;
      a.W = E;
      a.out = out ? out + off : nullptr;
      a.T0 = T0 ? T0 + off : nullptr;
      a.Y = Y ? Y + off : nullptr;
      a.Z = Z ? Z + off : nullptr;
      a.partials = partials;
      a.kax = op->kax;
      a.swap = op->swap;
      a.wperm = pp.wmode == W_EPS ? op->wperm_eps : op->wperm_inv;
      a.tw = op->tw;
      a.kn_floor = op->kn_floor;
      a.s = s;
      a.c0 = c0;
      a.c1 = c1;
      q->zin[pp.build == BUILD_PRECOND ? 1 : 0](dim3(sz.tiles, nb), q->smem_z, st, a);
      q->plane(dim3(3 * G * q->Q * nb / q->PL), q->smem_plane, st, a);
      q->zout[pp.epi](dim3(sz.tiles, nb), q->smem_z, st, a);
    } else {
      PassArgs a;
      std::memset(&a, 0, sizeof(a));
      a.X = X + off;
      a.E = E;
      a.out = out ? out + off : nullptr;
      a.T0 = T0 ? T0 + off : nullptr;
      a.Y = Y ? Y + off : nullptr;
      a.Z = Z ? Z + off : nullptr;
      a.partials = partials;
      a.kax = op->kax;
      a.swap = op->swap;
      a.w = pp.wmode == W_EPS ? op->eps_n : op->inv_eps;
      a.tw = op->tw;
      a.inv_n = 1.0f / (float)op->N;
      a.kn_floor = op->kn_floor;
      a.s = s;
      a.c0 = c0;
      a.c1 = c1;
      a.G = G;
      p->a[pp.build](dim3(sz.tiles_a, nb), smem_a, st, a);
      p->y[0](dim3(G / NZ, G, 3 * nb), smem_y, st, a);
      p->c[pp.wmode](dim3(G / NZ, G, 3 * nb), smem_c, st, a);
      p->y[1](dim3(G / NZ, G, 3 * nb), smem_y, st, a);
      p->e[pp.epi](dim3(sz.tiles, nb), smem_e, st, a);
    }
    if (pp.fin >= 0) {
      double* o = (pp.fin == FIN_COUNT_FIRST || pp.fin == FIN_COUNT_STEP) ? fin_out + v0 : fin_out + (long long)v0 * fin_ld;
      ef_count_launches(1);
      finalize_kernel<<<nb, 256, 0, st>>>(partials, sz.tiles, pp.fin, o, pp.fin >= FIN_COUNT_FIRST ? 1 : fin_ld, fin_k, fc0, fc1);
    }
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return ef_fail(EF_ERR_CUDA, cudaGetErrorString(err));
  return EF_OK;
}

}  // namespace

// ---- field outputs: energy density and participation sums ------------------------
// u(r) = eps(r) * sum_c |E_c(r)|^2 per mode (run_modes.py:119-124) and the sums
// (sum u, sum u^2) in fp64 behind the participation ratio PR = (sum u)^2 / sum u^2
// (localization.py:23-29). One CTA row per mode; block partials reduced in fp64.
constexpr int kEnergyBlocks = 152;

__global__ void __launch_bounds__(256) energy_kernel(const float2* __restrict__ E, const float* __restrict__ eps,
                                                     long long N, float* __restrict__ u,
                                                     double* __restrict__ partial) {
  const int v = blockIdx.y;
  const float2* e0 = E + (long long)v * 3 * N;
  double s1 = 0.0, s2 = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 a = e0[i], b = e0[N + i], c = e0[2 * N + i];
    const float val = eps[i] * (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y);
    if (u) u[(long long)v * N + i] = val;
    s1 += (double)val;
    s2 += (double)val * (double)val;
  }
  __shared__ double r1[8], r2[8];
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    r1[w] = s1;
    r2[w] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0.0, t2 = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      t1 += r1[k];
      t2 += r2[k];
    }
    partial[((long long)v * gridDim.x + blockIdx.x) * 2] = t1;
    partial[((long long)v * gridDim.x + blockIdx.x) * 2 + 1] = t2;
  }
}

__global__ void energy_reduce_kernel(const double* __restrict__ partial, double* __restrict__ sums) {
  const int v = blockIdx.x, lane = threadIdx.x;
  double t1 = 0.0, t2 = 0.0;
  for (int b = lane; b < kEnergyBlocks; b += 32) {
    t1 += partial[((long long)v * kEnergyBlocks + b) * 2];
    t2 += partial[((long long)v * kEnergyBlocks + b) * 2 + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    t1 += __shfl_down_sync(0xffffffffu, t1, o);
    t2 += __shfl_down_sync(0xffffffffu, t2, o);
  }
  if (lane == 0) {
    sums[2 * v] = t1;
    sums[2 * v + 1] = t2;
  }
}

extern "C" {

int ef_supported_grid(int grid) { return find_plan(grid) != nullptr; }

int ef_op_create(int grid, double box_size, double kx, double ky, double kz, const float* eps_host,
                 ef_op** out) {
  if (!out) return ef_fail(EF_ERR_INVALID, "out is null");
  *out = nullptr;
  if (!eps_host || grid <= 0 || !(box_size > 0.0)) return ef_fail(EF_ERR_INVALID, "bad grid, box size or eps");
  const Plan* p = find_plan(grid);
  if (!p) return ef_fail(EF_ERR_UNSUPPORTED, "grid edge has no FFT plan");
  if (!std::isfinite(kx) || !std::isfinite(ky) || !std::isfinite(kz))
    return ef_fail(EF_ERR_INVALID, "non-finite k");
  const int G = grid;
  const long long N = (long long)G * G * G;
  for (long long i = 0; i < N; ++i)
    if (!std::isfinite(eps_host[i]) || !(eps_host[i] > 0.0f))
      return ef_fail(EF_ERR_NONFINITE, "eps must be finite and positive");
  ef_op* op = new ef_op();
  std::memset(static_cast<ef::Op*>(op), 0, sizeof(ef::Op));
  op->G = G; op->R1 = p->R1; op->R2 = p->R2; op->N = N; op->L = box_size;
  op->k[0] = kx; op->k[1] = ky; op->k[2] = kz;
  cudaGetDevice(&op->device);
  std::vector<double> K;
  axis_wavevectors(G, box_size, op->k, K);
  std::vector<float> kaxf(3 * (size_t)G);
  for (size_t i = 0; i < kaxf.size(); ++i) kaxf[i] = (float)K[i];
  std::vector<uint32_t> swap((size_t)((N + 31) / 32), 0u);
  double knmin = INFINITY;
  for (int x = 0; x < G; ++x)
    for (int y = 0; y < G; ++y)
      for (int z = 0; z < G; ++z) {
        double a0 = K[x], a1 = K[G + y], a2 = K[2 * G + z];
        double kn = std::sqrt((a0 * a0 + a1 * a1) + a2 * a2);
        bool sw = std::fabs(a2) > 0.9 * std::fmax(kn, 1e-300);
        long long i = ((long long)x * G + y) * G + z;
        if (sw) swap[i >> 5] |= (1u << (i & 31));
        float knf = (float)kn;
        if (knf > 0.0f && knf < knmin) knmin = knf;
      }
  op->kn_floor = (float)(0.5 * knmin);
  std::vector<float> inv((size_t)N), epsn((size_t)N);
  double acc = 0.0;
  const float invN = (float)(1.0 / (double)N);
  for (long long i = 0; i < N; ++i) {
    float ie = 1.0f / eps_host[i];
    acc += ie;
    inv[i] = ie * invN;
    epsn[i] = eps_host[i] * invN;
  }
  op->eps_mean_inv = acc / (double)N;
  const Plan3* p3 = plan3_of_grid(G);
  std::vector<float> pinv, peps;
  if (p3) {
    permute_plane_table(inv, *p3, pinv);
    permute_plane_table(epsn, *p3, peps);
  }
  std::vector<float2> tw(G);
  for (int j = 0; j < G; ++j) {
    double ang = 2.0 * M_PI * (double)j / (double)G;
    tw[j] = make_float2((float)std::cos(ang), (float)std::sin(ang));
  }
  cudaError_t e = cudaSuccess;
  e = cudaMalloc(&op->kax, kaxf.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&op->swap, swap.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&op->inv_eps, (size_t)N * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&op->eps_n, (size_t)N * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&op->eps_raw, (size_t)N * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&op->tw, (size_t)G * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(op->kax, kaxf.data(), kaxf.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(op->swap, swap.data(), swap.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(op->inv_eps, inv.data(), (size_t)N * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(op->eps_n, epsn.data(), (size_t)N * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(op->eps_raw, eps_host, (size_t)N * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(op->tw, tw.data(), (size_t)G * sizeof(float2), cudaMemcpyHostToDevice);
  if (p3) {
    if (e == cudaSuccess) e = cudaMalloc(&op->wperm_inv, (size_t)N * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&op->wperm_eps, (size_t)N * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(op->wperm_inv, pinv.data(), (size_t)N * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(op->wperm_eps, peps.data(), (size_t)N * sizeof(float), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    ef_op_destroy(op);
    return ef_fail(EF_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = op;
  return EF_OK;
}

int ef_op_destroy(ef_op* op) {
  if (!op) return EF_OK;
  cudaFree(op->kax);
  cudaFree(op->swap);
  cudaFree(op->inv_eps);
  cudaFree(op->eps_n);
  cudaFree(op->eps_raw);
  cudaFree(op->tw);
  cudaFree(op->wperm_inv);
  cudaFree(op->wperm_eps);
  delete op;
  return EF_OK;
}

int ef_op_configure(ef_op* op, int passes, size_t subbatch_bytes) {
  if (!op) return ef_fail(EF_ERR_INVALID, "null operator");
  if (passes != 0 && passes != 3 && passes != 5) return ef_fail(EF_ERR_INVALID, "passes must be 0, 3 or 5");
  if (passes == 3 && !plan3_of_grid(op->G))
    return ef_fail(EF_ERR_UNSUPPORTED, "no three-pass plan for this grid edge");
  op->passes = passes;
  op->subbatch_bytes = subbatch_bytes;
  return EF_OK;
}

int ef_op_pipeline(const ef_op* op) {
  if (!op) return 0;
  return find_plan3(op) ? 3 : 5;
}

int ef_op_info(const ef_op* op, int* grid, double* kn_floor, double* eps_mean_inv) {
  if (!op) return ef_fail(EF_ERR_INVALID, "null operator");
  if (grid) *grid = op->G;
  if (kn_floor) *kn_floor = op->kn_floor;
  if (eps_mean_inv) *eps_mean_inv = op->eps_mean_inv;
  return EF_OK;
}

int ef_op_basis(const ef_op* op, float* kn_dev, float* t_dev, void* stream) {
  if (!op) return ef_fail(EF_ERR_INVALID, "null operator");
  ef_count_launches(1);
  basis_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(op->kax, op->swap, op->G, kn_dev, t_dev, nullptr);
  return ef_check_launch();
}

int ef_op_mask(const ef_op* op, float* mask_dev, void* stream) {
  if (!op || !mask_dev) return ef_fail(EF_ERR_INVALID, "null argument");
  ef_count_launches(1);
  basis_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(op->kax, op->swap, op->G, nullptr, nullptr, mask_dev);
  return ef_check_launch();
}

size_t ef_op_workspace_bytes(const ef_op* op, int m) {
  if (!op || m <= 0) return 0;
  const Plan* p = find_plan(op->G);
  if (!p) return 0;
  Sizes sz = sizes_of(op, p);
  int mb = mb_cap(op, sz);
  if (mb > m) mb = m;
  return (size_t)mb * (sz.per_vec + sz.per_vec_part) + 512;
}

int ef_theta(const ef_op* op, const float* X, float* Y, int m, void* work, size_t work_bytes,
             void* stream) {
  if (!Y) return ef_fail(EF_ERR_INVALID, "null output");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_THETA, -1};
  return run_pipe(op, pp, (const float2*)X, (float2*)Y, nullptr, nullptr, nullptr, m, 0.f, 0.f,
                  0.f, nullptr, 0, 0, 0.0, 0.0, work, work_bytes, (cudaStream_t)stream);
}

int ef_precondition(const ef_op* op, const float* X, float* Y, int m, void* work,
                    size_t work_bytes, void* stream) {
  if (!Y) return ef_fail(EF_ERR_INVALID, "null output");
  Pipe pp{BUILD_PRECOND, W_EPS, EPI_PRECOND, -1};
  return run_pipe(op, pp, (const float2*)X, (float2*)Y, nullptr, nullptr, nullptr, m, 0.f, 0.f,
                  0.f, nullptr, 0, 0, 0.0, 0.0, work, work_bytes, (cudaStream_t)stream);
}

int ef_precondition_simple(const ef_op* op, const float* X, float* Y, int m, float scale,
                           void* stream) {
  if (!op || !X || !Y || m <= 0) return ef_fail(EF_ERR_INVALID, "null argument or m <= 0");
  long long total = (long long)m * 2 * op->N;
  ef_count_launches(1);
  precond_simple_kernel<<<2048, 256, 0, (cudaStream_t)stream>>>(op->kax, op->G, (const float2*)X,
                                                                 (float2*)Y, total, scale);
  return ef_check_launch();
}

static int realspace(const ef_op* op, const float* X, float* out, const float* vscale, int m,
                     int build, int wmode, cudaStream_t st) {
  if (!op || !X || !out || m <= 0) return ef_fail(EF_ERR_INVALID, "null argument or m <= 0");
  const Plan* p = find_plan(op->G);
  if (!p) return ef_fail(EF_ERR_UNSUPPORTED, "no FFT plan for this grid");
  const int G = op->G, NZ = p->NZ, PS = p->PS;
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.X = (const float2*)X;
  a.E = (float2*)out;
  a.kax = op->kax;
  a.swap = op->swap;
  a.w = op->inv_eps;
  a.tw = op->tw;
  a.vscale = vscale;
  a.inv_n = 1.0f / (float)op->N;
  a.kn_floor = op->kn_floor;
  a.G = G;
  const int tiles = G * G / p->NRA;
  p->a[build](dim3(tiles, m), (size_t)(3 * p->NRA * p->PSA + G) * sizeof(float2), st, a);
  p->y[0](dim3(G / NZ, G, 3 * m), (size_t)(NZ * PS + G) * sizeof(float2), st, a);
  p->c[wmode](dim3(G / NZ, G, 3 * m), (size_t)(2 * NZ * PS + G) * sizeof(float2), st, a);
  return ef_check_launch();
}

int ef_h_realspace(const ef_op* op, const float* X, float* H, int m, void* stream) {
  return realspace(op, X, H, nullptr, m, BUILD_CART, W_INV_ONLY, (cudaStream_t)stream);
}

int ef_e_realspace(const ef_op* op, const float* X, const float* vec_scale_dev, float* Eout, int m,
                   void* stream) {
  if (!vec_scale_dev) return ef_fail(EF_ERR_INVALID, "null vec_scale");
  return realspace(op, X, Eout, vec_scale_dev, m, BUILD_THETA, W_INV_ONLY_EPS, (cudaStream_t)stream);
}

int ef_energy_workspace_bytes(const ef_op* op, int m) {
  if (!op || m <= 0) return 0;
  return (int)((size_t)m * kEnergyBlocks * 2 * sizeof(double) + 256);
}

int ef_energy_density(const ef_op* op, const float* E, float* u, double* sums, int m, void* work,
                      size_t work_bytes, void* stream) {
  if (!op || !E || !sums || m <= 0) return ef_fail(EF_ERR_INVALID, "bad energy_density arguments");
  if (!work || work_bytes < (size_t)ef_energy_workspace_bytes(op, m))
    return ef_fail(EF_ERR_WORKSPACE, "energy_density work buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  ef_count_launches(2);
  energy_kernel<<<dim3(kEnergyBlocks, m), 256, 0, st>>>((const float2*)E, op->eps_raw, op->N, u,
                                                         (double*)work);
  energy_reduce_kernel<<<m, 32, 0, st>>>((const double*)work, sums);
  return ef_check_launch();
}

int ef_cheb_first(const ef_op* op, const float* T0, float* T1, float* Y, int m, double s, float c0,
                  float c1, void* work, size_t work_bytes, void* stream) {
  if (!T1 || !Y) return ef_fail(EF_ERR_INVALID, "null output");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_CHEB_FIRST, -1};
  return run_pipe(op, pp, (const float2*)T0, (float2*)T1, nullptr, (float2*)Y, nullptr, m, (float)s,
                  c0, c1, nullptr, 0, 0, 0.0, 0.0, work, work_bytes, (cudaStream_t)stream);
}

int ef_cheb_step(const ef_op* op, const float* T1, float* T0, float* Y, int m, double s, float ck,
                 void* work, size_t work_bytes, void* stream) {
  if (!T0 || !Y) return ef_fail(EF_ERR_INVALID, "null output");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_CHEB, -1};
  return run_pipe(op, pp, (const float2*)T1, nullptr, (float2*)T0, (float2*)Y, nullptr, m, (float)s,
                  0.f, ck, nullptr, 0, 0, 0.0, 0.0, work, work_bytes, (cudaStream_t)stream);
}

int ef_kpm_first(const ef_op* op, const float* Z, float* T1, int m, double s, double* mom, int ld_mom,
                 void* work, size_t work_bytes, void* stream) {
  if (!T1 || !mom || ld_mom < 2) return ef_fail(EF_ERR_INVALID, "bad output arguments");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_KPM_FIRST, FIN_KPM_FIRST};
  return run_pipe(op, pp, (const float2*)Z, (float2*)T1, nullptr, nullptr, nullptr, m, (float)s, 0.f,
                  0.f, mom, ld_mom, 0, 0.0, 0.0, work, work_bytes, (cudaStream_t)stream);
}

int ef_kpm_step(const ef_op* op, const float* T1, float* T0, int m, double s, int k, double* mom,
                int ld_mom, void* work, size_t work_bytes, void* stream) {
  if (!T0 || !mom || k < 1 || ld_mom < 2 * k + 2) return ef_fail(EF_ERR_INVALID, "bad output arguments");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_KPM, FIN_KPM_STEP};
  return run_pipe(op, pp, (const float2*)T1, nullptr, (float2*)T0, nullptr, nullptr, m, (float)s, 0.f,
                  0.f, mom, ld_mom, k, 0.0, 0.0, work, work_bytes, (cudaStream_t)stream);
}

int ef_kpm_count_first(const ef_op* op, const float* Z, float* T1, int m, double s, double c0,
                       double c1, double* est, void* work, size_t work_bytes, void* stream) {
  if (!T1 || !est) return ef_fail(EF_ERR_INVALID, "bad output arguments");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_KPM_FIRST, FIN_COUNT_FIRST};
  return run_pipe(op, pp, (const float2*)Z, (float2*)T1, nullptr, nullptr, nullptr, m, (float)s, 0.f,
                  0.f, est, 1, 0, c0, c1, work, work_bytes, (cudaStream_t)stream);
}

int ef_kpm_count_step(const ef_op* op, const float* T1, float* T0, const float* Z, int m, double s,
                      double ck, double* est, void* work, size_t work_bytes, void* stream) {
  if (!T0 || !Z || !est) return ef_fail(EF_ERR_INVALID, "bad arguments");
  Pipe pp{BUILD_THETA, W_INV_EPS, EPI_KPM_COUNT, FIN_COUNT_STEP};
  return run_pipe(op, pp, (const float2*)T1, nullptr, (float2*)T0, nullptr, (const float2*)Z, m,
                  (float)s, 0.f, 0.f, est, 1, 0, ck, 0.0, work, work_bytes, (cudaStream_t)stream);
}

}  // extern "C"
