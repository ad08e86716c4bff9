// Grouped block operations: one host call applies an operation to the blocks of a set
// of instances (solves of one shape: the same grid edge and block sizes, any k-point or
// structure). The blocks of all instances live in stacked device arrays; instance i's
// operand starts at base + i * stride (strides count complex64 values for vector blocks
// and coefficient matrices, complex128 entries for Gram outputs, doubles for the row
// statistics, eigenvalues and scales), and `inst` lists the n
// instances the call covers (host memory). Each instance's work is exactly the
// single-instance call on its own operands, queued in list order on one stream with
// the workspace reused, so a grouped solve computes bit for bit what its instances
// compute alone; the grouping removes the per-instance host calls.
//
// Reference: the per-instance operations are eigenfns/operator.py:82-95,104-127 (Θ and
// the preconditioner) and eigenfns/solver.py:35-57,228-238 (Gram, rotations, row
// statistics, residuals); the reference has no grouped form.
#include <cstddef>

#include "eigenfns_gb300.h"
#include "status.h"

namespace {

inline const float* at(const float* base, int i, long long stride) {
  return base + 2 * (long long)i * stride;
}
inline float* at(float* base, int i, long long stride) { return base + 2 * (long long)i * stride; }
inline double* atd(double* base, int i, long long stride) { return base + (long long)i * stride; }
inline const double* atd(const double* base, int i, long long stride) {
  return base + (long long)i * stride;
}

bool bad_list(const int* inst, int n) { return n < 0 || (n > 0 && !inst); }
int invalid() { return ef_fail(EF_ERR_INVALID, "group: null instance list or operator table"); }

}  // namespace

extern "C" {

int ef_group_theta(const ef_op* const* ops, const int* inst, int n, const float* X, long long x_stride,
                   float* Y, long long y_stride, int m, void* work, size_t work_bytes, void* stream) {
  if (bad_list(inst, n) || !ops) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_theta(ops[i], at(X, i, x_stride), at(Y, i, y_stride), m, work, work_bytes, stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

int ef_group_precondition(const ef_op* const* ops, const int* inst, int n, const float* X,
                          long long x_stride, float* Y, long long y_stride, int m, void* work,
                          size_t work_bytes, void* stream) {
  if (bad_list(inst, n) || !ops) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_precondition(ops[i], at(X, i, x_stride), at(Y, i, y_stride), m, work, work_bytes,
                                   stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

int ef_group_gram(const int* inst, int n, const float* A, long long a_stride, const float* B,
                  long long b_stride, int ma, int mb, long long K, double* G, long long g_stride,
                  void* work, size_t work_bytes, void* stream) {
  if (bad_list(inst, n)) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_gram(at(A, i, a_stride), at(B, i, b_stride), ma, mb, K, atd(G, i, 2 * g_stride),
                           work, work_bytes, stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

int ef_group_rotate(const int* inst, int n, const float* C, long long c_stride, const float* S,
                    long long s_stride, float* out, long long o_stride, int m_in, int m_out, long long K,
                    int mode, void* stream) {
  if (bad_list(inst, n)) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_rotate(at(C, i, c_stride), at(S, i, s_stride), at(out, i, o_stride), m_in, m_out, K,
                             mode, stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

int ef_group_rowstats(const int* inst, int n, const float* A, long long a_stride, const float* B,
                      long long b_stride, int m, long long K, double* out, long long out_stride,
                      void* work, size_t work_bytes, void* stream) {
  if (bad_list(inst, n)) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_rowstats(at(A, i, a_stride), at(B, i, b_stride), m, K, atd(out, i, out_stride), work,
                               work_bytes, stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

int ef_group_residual_norms(const int* inst, int n, const float* HX, long long h_stride, const float* X,
                            long long x_stride, const double* lam, long long lam_stride, float* R,
                            long long r_stride, int m, long long K, double* r2, long long r2_stride,
                            void* work, size_t work_bytes, void* stream) {
  if (bad_list(inst, n)) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_residual_norms(at(HX, i, h_stride), at(X, i, x_stride), atd(lam, i, lam_stride),
                                     at(R, i, r_stride), m, K, atd(r2, i, r2_stride), work, work_bytes,
                                     stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

int ef_group_scale_rows(const int* inst, int n, float* X, long long x_stride, const double* scale,
                        long long s_stride, int m, long long K, void* stream) {
  if (bad_list(inst, n)) return invalid();
  for (int j = 0; j < n; ++j) {
    const int i = inst[j];
    const int rc = ef_scale_rows(at(X, i, x_stride), atd(scale, i, s_stride), m, K, stream);
    if (rc != EF_OK) return rc;
  }
  return EF_OK;
}

}  // extern "C"
