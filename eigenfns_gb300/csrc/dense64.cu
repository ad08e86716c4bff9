// Small dense fp64 problems on the device, batched one CTA per problem:
//   ef_cholqr_f64  Cholesky-QR coefficients of a Gram matrix (G = R^H R, C = R^-1)
//   ef_eigh_f64    eigendecomposition of a Hermitian matrix by cyclic Jacobi
// Matrices are complex128, row-major, n <= 96 (the Rayleigh-Ritz size 3m for block
// m = 32). GB300's fp64 rate is low (about 1/64 of its fp32 rate), so these pay where
// many small problems run side by side (one CTA each) or where they remove a
// device-to-host round trip; a single large eigenproblem is faster on the host.
#include <cmath>

#include "common.cuh"
#include "status.h"

namespace {

constexpr int kDenseThreads = 256;
constexpr int kDenseMaxN = 96;

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconjmul(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Cholesky G = R^H R (R upper) in shared memory, then C = R^-1 (upper). A pivot at or
// below tol * max diag(G) marks a dead direction, as SVQB's drop does: its row of R and
// its entries of C are zero, so ef_rotate(C, X) leaves a zero row there (the other rows
// are orthonormalised within the live span). status[b] = number of dead directions.
__global__ void __launch_bounds__(kDenseThreads) cholqr_kernel(const double2* __restrict__ Gall, int n,
                                                               long long sG, float2* __restrict__ Call,
                                                               long long sC, int* status, double tol) {
  extern __shared__ double2 dsm[];
  double2* A = dsm;                                        // n x n
  double* diag = reinterpret_cast<double*>(A + n * n);     // R[j][j], 0 for a dead direction
  __shared__ int ndead;
  __shared__ double dmax;
  const double2* G = Gall + blockIdx.x * sG;
  float2* C = Call + blockIdx.x * sC;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) A[i] = G[i];
  if (threadIdx.x == 0) {
    ndead = 0;
    double m = 0.0;
    for (int i = 0; i < n; ++i) m = fmax(m, G[i * n + i].x);
    dmax = m;
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const double piv = A[j * n + j].x;    // every thread reads the same value
    const bool live = piv > tol * dmax;
    const double r = live ? sqrt(piv) : 0.0;
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
      const double2 v = A[j * n + i];
      A[j * n + i] = live ? make_double2(v.x / r, v.y / r) : make_double2(0.0, 0.0);
    }
    if (threadIdx.x == 0) {
      diag[j] = r;
      A[j * n + j] = make_double2(r, 0.0);
      if (!live) ++ndead;
    }
    __syncthreads();
    if (live) {
      // trailing update of the upper triangle: A[p][q] -= conj(R[j][p]) R[j][q], p <= q
      const int m = n - j - 1;
      for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
        const int p = j + 1 + t / m, q = j + 1 + t % m;
        if (q < p) continue;
        const double2 u = zconjmul(A[j * n + p], A[j * n + q]);
        A[p * n + q].x -= u.x;
        A[p * n + q].y -= u.y;
      }
    }
    __syncthreads();
  }
  // C = R^-1 column by column (thread i owns column i) on the live directions:
  // C[i][i] = 1/R[i][i], C[k][i] = -(sum_{l=k+1..i} R[k][l] C[l][i]) / R[k][k]; dead
  // directions have zero rows and columns. Column i is kept in the (free) lower triangle
  // of A, transposed: C[k][i] at A[i][k].
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    A[i * n + i] = make_double2(diag[i] > 0.0 ? 1.0 / diag[i] : 0.0, 0.0);
    for (int k = i - 1; k >= 0; --k) {
      double2 s = make_double2(0.0, 0.0);
      if (diag[k] > 0.0) {
        for (int l = k + 1; l <= i; ++l) {
          const double2 pr = zmul(A[k * n + l], A[i * n + l]);   // R[k][l] C[l][i]
          s.x += pr.x;
          s.y += pr.y;
        }
        s = make_double2(-s.x / diag[k], -s.y / diag[k]);
      }
      A[i * n + k] = s;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int k = t / n, i = t % n;
    const double2 v = k <= i ? A[i * n + k] : make_double2(0.0, 0.0);
    C[t] = make_float2((float)v.x, (float)v.y);
  }
  if (threadIdx.x == 0) status[blockIdx.x] = ndead;
}

// Round-robin pairing of n (even) indices, round r: slot k pairs idx(k) with idx(n-1-k)
__device__ __forceinline__ int rr_index(int k, int r, int n) {
  if (k == 0) return 0;
  return 1 + ((k - 1 + r) % (n - 1));
}

__device__ double block_sum_d(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;   // every thread returns the total
}

// Cyclic Jacobi on a Hermitian matrix held in shared memory; V accumulates in global
// memory (work). Each round applies n/2 disjoint rotations at once: rows, then columns.
// The rotation J = [[c, s], [-s e, c e]] with e = exp(-i arg A[p][q]) and (c, s) the real
// symmetric Jacobi rotation of [[A_pp, |A_pq|], [|A_pq|, A_qq]] zeroes A[p][q].
__global__ void __launch_bounds__(kDenseThreads) jacobi_kernel(const double2* __restrict__ Aall, int n,
                                                               long long sA, double* __restrict__ wall,
                                                               double2* __restrict__ Vall,
                                                               double2* __restrict__ work, int* status,
                                                               int max_sweeps) {
  extern __shared__ double2 dsm[];
  const int ne = n + (n & 1);              // padded to even with a zero row and column
  double2* A = dsm;                        // ne x ne
  double2* rot = A + ne * ne;              // per pair: (c, s), e
  int* pairs = reinterpret_cast<int*>(rot + ne);
  __shared__ double red[kDenseThreads / 32];
  const double2* Ain = Aall + blockIdx.x * sA;
  double2* V = work + (long long)blockIdx.x * ne * ne;
  for (int t = threadIdx.x; t < ne * ne; t += blockDim.x) {
    const int i = t / ne, j = t % ne;
    A[t] = (i < n && j < n) ? Ain[i * n + j] : make_double2(0.0, 0.0);
    V[t] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // off-diagonal sum of squares (summed directly, no cancellation) against the total
    double off = 0.0, tot = 0.0;
    for (int t = threadIdx.x; t < ne * ne; t += blockDim.x) {
      const double2 v = A[t];
      const double m2 = v.x * v.x + v.y * v.y;
      tot += m2;
      if (t / ne != t % ne) off += m2;
    }
    off = block_sum_d(off, red);
    tot = block_sum_d(tot, red);
    if (!(off > 1e-26 * tot)) break;       // uniform across the block; ~1e-13 relative
    for (int r = 0; r < ne - 1; ++r) {
      for (int k = threadIdx.x; k < ne / 2; k += blockDim.x) {
        int p = rr_index(k, r, ne), q = rr_index(ne - 1 - k, r, ne);
        if (p > q) { const int t = p; p = q; q = t; }
        pairs[2 * k] = p;
        pairs[2 * k + 1] = q;
        const double2 c = A[p * ne + q];
        const double ac = sqrt(c.x * c.x + c.y * c.y);
        double cs = 1.0, sn = 0.0, ex = 1.0, ey = 0.0;
        if (ac > 0.0) {
          const double tau = (A[q * ne + q].x - A[p * ne + p].x) / (2.0 * ac);
          const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          cs = 1.0 / sqrt(1.0 + t * t);
          sn = t * cs;
          ex = c.x / ac;
          ey = -c.y / ac;                  // e = exp(-i phi)
        }
        rot[2 * k] = make_double2(cs, sn);
        rot[2 * k + 1] = make_double2(ex, ey);
      }
      __syncthreads();
      // rows: A <- J^H A on rows p, q
      for (int t = threadIdx.x; t < (ne / 2) * ne; t += blockDim.x) {
        const int k = t / ne, j = t % ne;
        const int p = pairs[2 * k], q = pairs[2 * k + 1];
        const double cs = rot[2 * k].x, sn = rot[2 * k].y;
        const double2 e = rot[2 * k + 1];
        const double2 ap = A[p * ne + j];
        const double2 aq = zmul(make_double2(e.x, -e.y), A[q * ne + j]);   // conj(e) A_q
        A[p * ne + j] = make_double2(cs * ap.x - sn * aq.x, cs * ap.y - sn * aq.y);
        A[q * ne + j] = make_double2(sn * ap.x + cs * aq.x, sn * ap.y + cs * aq.y);
      }
      __syncthreads();
      // columns: A <- A J and V <- V J on columns p, q
      for (int t = threadIdx.x; t < (ne / 2) * ne; t += blockDim.x) {
        const int k = t / ne, i = t % ne;
        const int p = pairs[2 * k], q = pairs[2 * k + 1];
        const double cs = rot[2 * k].x, sn = rot[2 * k].y;
        const double2 e = rot[2 * k + 1];
        const double2 ap = A[i * ne + p], aq = zmul(A[i * ne + q], e);
        A[i * ne + p] = make_double2(cs * ap.x - sn * aq.x, cs * ap.y - sn * aq.y);
        A[i * ne + q] = make_double2(sn * ap.x + cs * aq.x, sn * ap.y + cs * aq.y);
        const double2 vp = V[i * ne + p], vq = zmul(V[i * ne + q], e);
        V[i * ne + p] = make_double2(cs * vp.x - sn * vq.x, cs * vp.y - sn * vq.y);
        V[i * ne + q] = make_double2(sn * vp.x + cs * vq.x, sn * vp.y + cs * vq.y);
      }
      __syncthreads();
    }
  }
  // eigenvalues ascending (rank sort, ties by index) and the matching columns of V
  double* w = wall + (long long)blockIdx.x * n;
  double2* Vout = Vall + (long long)blockIdx.x * n * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double wi = A[i * ne + i].x;
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double wj = A[j * ne + j].x;
      rank += (wj < wi) || (wj == wi && j < i);
    }
    w[rank] = wi;
    for (int r = 0; r < n; ++r) Vout[r * n + rank] = V[r * ne + i];
  }
  if (threadIdx.x == 0) status[blockIdx.x] = (sweep >= max_sweeps) ? 1 : 0;
}

}  // namespace

extern "C" {

int ef_cholqr_f64(const double* G, int n, int batch, float* C, int* status, double tol,
                  void* stream) {
  if (!G || !C || !status || n <= 0 || n > kDenseMaxN || batch <= 0 || !(tol >= 0.0))
    return ef_fail(EF_ERR_INVALID, "cholqr_f64: bad arguments (1 <= n <= 96)");
  const size_t smem = (size_t)n * n * sizeof(double2) + (size_t)n * sizeof(double);
  ef::set_smem_once(cholqr_kernel, smem);
  ef_count_launches(1);
  cholqr_kernel<<<batch, kDenseThreads, smem, (cudaStream_t)stream>>>(
      (const double2*)G, n, (long long)n * n, (float2*)C, (long long)n * n, status, tol);
  return ef_check_launch();
}

size_t ef_eigh_f64_workspace_bytes(int n, int batch) {
  if (n <= 0 || batch <= 0) return 0;
  const size_t ne = (size_t)n + (n & 1);
  return (size_t)batch * ne * ne * sizeof(double2);
}

int ef_eigh_f64(const double* A, int n, int batch, double* w, double* V, void* work,
                size_t work_bytes, int* status, void* stream) {
  if (!A || !w || !V || !status || n <= 0 || n > kDenseMaxN || batch <= 0)
    return ef_fail(EF_ERR_INVALID, "eigh_f64: bad arguments (1 <= n <= 96)");
  if (!work || work_bytes < ef_eigh_f64_workspace_bytes(n, batch))
    return ef_fail(EF_ERR_WORKSPACE, "eigh_f64: work buffer too small");
  const int ne = n + (n & 1);
  const size_t smem = (size_t)ne * ne * sizeof(double2) + (size_t)ne * sizeof(double2) +
                      (size_t)ne * sizeof(int);
  ef::set_smem_once(jacobi_kernel, smem);
  ef_count_launches(1);
  jacobi_kernel<<<batch, kDenseThreads, smem, (cudaStream_t)stream>>>(
      (const double2*)A, n, (long long)n * n, w, (double2*)V, (double2*)work, status, 40);
  return ef_check_launch();
}

}  // extern "C"
