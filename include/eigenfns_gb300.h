/* eigenfns_gb300 -- C ABI of the GB300 Maxwell eigensolver hot path.
 *
 * A thin, stream-ordered C interface over hand-written sm_103a CUDA kernels. It
 * replaces the device work of the reference (fhernandez93/eigenfns, JAX/XLA);
 * every entry names the reference code it stands in for. The Python package
 * `eigenfns_gb300` binds it with ctypes (eigenfns_gb300/_lib.py).
 *
 * Conventions
 *   - Complex64 arrays are interleaved (re, im) float pairs; complex128 arrays
 *     interleaved double pairs. A block of m vectors is (m, 2, G, G, G) complex64
 *     in C order (the reference's (m, 2, G, G, G) transverse amplitudes), so a
 *     vector has K = 2*G^3 complex entries.
 *   - All array arguments except `eps_host` are DEVICE pointers owned by the
 *     caller; the library never frees caller memory. `stream` is a cudaStream_t
 *     (NULL = legacy default stream). No entry point synchronises the device.
 *   - Scratch memory ("work") is passed in by the caller; the *_workspace_bytes
 *     queries give the size. The operator handle owns its eps and frame tables.
 *   - Every entry returns an int status: EF_OK or one of the codes below. The
 *     Python layer maps EF_ERR_INVALID / EF_ERR_UNSUPPORTED / EF_ERR_WORKSPACE to
 *     ValueError and the rest to RuntimeError. No entry point exits or traps.
 */
#ifndef EIGENFNS_GB300_H
#define EIGENFNS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EF_OK 0
#define EF_ERR_INVALID 1      /* null pointer, non-positive size, non-cube grid */
#define EF_ERR_UNSUPPORTED 2  /* grid edge not covered by the FFT plans */
#define EF_ERR_CUDA 3         /* a CUDA runtime call or kernel launch failed */
#define EF_ERR_WORKSPACE 4    /* work buffer smaller than required */
#define EF_ERR_NONFINITE 5    /* non-finite value in an input table */
#define EF_ERR_TOO_LARGE 6    /* size beyond a stated fixed maximum */

/* random block kinds for ef_rand_block */
#define EF_RAND_NORMAL 0          /* complex normal, re and im N(0,1) */
#define EF_RAND_RADEMACHER 1      /* real +-1 (the reference's KPM probes) */
#define EF_RAND_RADEMACHER_C 2    /* (+-1 +- i)/sqrt(2) */

typedef struct ef_op ef_op;

const char* ef_version(void);
const char* ef_status_string(int status);
/* detail text of the last failure on the calling thread */
const char* ef_last_error(void);
/* number of kernels this library has launched in the process (all threads) */
unsigned long long ef_launch_count(void);

/* 1 if the grid edge has an FFT plan (G = R1*R2, R1, R2 in {1..6, 8, 12, 16}) */
int ef_supported_grid(int grid);

/* ---- operator (eigenfns/operator.py) ------------------------------------------ */

/* MaxwellOperator.__init__ (operator.py:136-151) with make_basis (:44-79):
 * copies eps (G^3 float32, host) to the device, builds the per-axis k+G tables,
 * the reference-axis switch bits (fp64, operator.py:55-59), eps^-1 and kn_floor. */
int ef_op_create(int grid, double box_size, double kx, double ky, double kz,
                 const float* eps_host, ef_op** out);
int ef_op_destroy(ef_op* op);
/* Pipeline of the operator applications (no counterpart in the reference: the
 * autotuner's control, eigenfns_gb300/tune.py). passes = 0 automatic (three-pass
 * z / xy-plane / z pipeline where the grid edge has a plan: 32, 48, 64, 96, 128;
 * else the five-pass pencil pipeline), 3 (EF_ERR_UNSUPPORTED without a plan) or 5.
 * subbatch_bytes caps one sub-batch's workspace (0 = default: 64 MB three-pass,
 * 96 MB five-pass). Applies to ef_op_workspace_bytes and to every later call. */
int ef_op_configure(ef_op* op, int passes, size_t subbatch_bytes);
/* the pipeline the handle's operator calls use now: 3 or 5 */
int ef_op_pipeline(const ef_op* op);
/* grid_size, kn_floor (operator.py:149-151), eps_mean_inv (:148) */
int ef_op_info(const ef_op* op, int* grid, double* kn_floor, double* eps_mean_inv);
/* TransverseBasis.kn (G^3 float32) and .t (2,3,G^3 float32) (operator.py:36-37) */
int ef_op_basis(const ef_op* op, float* kn_dev, float* t_dev, void* stream);
/* the mask (kn > 0) as float32 G^3 (solver.py:162) */
int ef_op_mask(const ef_op* op, float* mask_dev, void* stream);

/* work bytes for one ef_theta / ef_precondition / recurrence call on m vectors */
size_t ef_op_workspace_bytes(const ef_op* op, int m);

/* Θ Hs for a block (m,2,G,G,G): _theta_block / MaxwellOperator.theta (operator.py:82-95,153-155) */
int ef_theta(const ef_op* op, const float* X, float* Y, int m,
             void* work, size_t work_bytes, void* stream);
/* transverse-projection preconditioner: _precondition_fancy_block /
 * MaxwellOperator.precondition (operator.py:104-127,157-161) */
int ef_precondition(const ef_op* op, const float* X, float* Y, int m,
                    void* work, size_t work_bytes, void* stream);
/* diagonal kinetic preconditioner R/(kn^2+scale): _precondition_block (operator.py:98-101,163-166) */
int ef_precondition_simple(const ef_op* op, const float* X, float* Y, int m, float scale,
                           void* stream);
/* real-space Cartesian H (m,3,G,G,G): MaxwellOperator.h_realspace (operator.py:174-176) */
int ef_h_realspace(const ef_op* op, const float* X, float* H, int m, void* stream);
/* real-space E = eps^-1 curl H * vec_scale[v] (m,3,G,G,G), vec_scale = 1/sqrt(lambda):
 * MaxwellOperator.e_realspace (operator.py:178-184) */
int ef_e_realspace(const ef_op* op, const float* X, const float* vec_scale_dev, float* Eout,
                   int m, void* stream);

/* energy density u = eps * sum_c |E_c|^2 of real-space E fields (m,3,G,G,G) complex64
 * (run_modes.py:119-124) into u (m,G,G,G) float32 (may be NULL), and per mode the fp64
 * sums (sum u, sum u^2) into sums (m,2) device doubles, from which the participation
 * ratio PR = (sum u)^2 / sum u^2 follows (localization.py:23-29) */
int ef_energy_workspace_bytes(const ef_op* op, int m);
int ef_energy_density(const ef_op* op, const float* E, float* u, double* sums, int m, void* work,
                      size_t work_bytes, void* stream);

/* ---- fused Chebyshev / KPM recurrences ------------------------------------------ */
/* Bandpass filter Y = sum_k c_k T_k(B) X with B = s*Θ - 1, s = 2/lambda_max
 * (_apply_cheb_poly, interior.py:336-354).
 * first step: T1 = B T0, Y = c0 T0 + c1 T1 (interior.py:344-346) */
int ef_cheb_first(const ef_op* op, const float* T0, float* T1, float* Y, int m, double s,
                  float c0, float c1, void* work, size_t work_bytes, void* stream);
/* later steps: T0 <- 2 B T1 - T0 (in place), Y += ck * T0 (interior.py:347-350) */
int ef_cheb_step(const ef_op* op, const float* T1, float* T0, float* Y, int m, double s,
                 float ck, void* work, size_t work_bytes, void* stream);

/* KPM moments with the doubling identities (scripts/exp/exp_kpm_dos.py:141-152).
 * mom is a device (m, ld_mom) float64 array.
 * first: T1 = B Z, mom[:,0] = <Z,Z>, mom[:,1] = <Z,T1> */
int ef_kpm_first(const ef_op* op, const float* Z, float* T1, int m, double s,
                 double* mom, int ld_mom, void* work, size_t work_bytes, void* stream);
/* step k >= 1: T0 <- 2 B T1 - T0 (= T_{k+1}), mom[:,2k] = 2<T1,T1> - mom[:,0],
 * mom[:,2k+1] = 2<T0_new,T1> - mom[:,1] */
int ef_kpm_step(const ef_op* op, const float* T1, float* T0, int m, double s, int k,
                double* mom, int ld_mom, void* work, size_t work_bytes, void* stream);
/* kpm_count_below recurrence (eigenfns/chebyshev.py:254-263): est is a device
 * float64 (m) accumulator of sum_k coef_k Re<Z, T_k>.
 * first: T1 = B Z, est = c0 <Z,Z> + c1 <Z,T1>; step: T0 <- 2 B T1 - T0, est += ck <Z,T0> */
int ef_kpm_count_first(const ef_op* op, const float* Z, float* T1, int m, double s,
                       double c0, double c1, double* est, void* work, size_t work_bytes,
                       void* stream);
int ef_kpm_count_step(const ef_op* op, const float* T1, float* T0, const float* Z, int m,
                      double s, double ck, double* est, void* work, size_t work_bytes,
                      void* stream);

/* ---- block linear algebra (eigenfns/solver.py) ------------------------------------ */
/* work bytes of ef_gram for these sizes */
size_t ef_gram_workspace_bytes(int ma, int mb, long long K);
/* G[i][j] = sum_k conj(A[i,k]) B[j,k], complex128 (ma, mb) row-major:
 * gram (solver.py:35-43) with fp32 products and a fp64 split-K reduction */
int ef_gram(const float* A, const float* B, int ma, int mb, long long K, double* G,
            void* work, size_t work_bytes, void* stream);
/* ef_gram without a work buffer, for callers that cannot provide device scratch
 * (no counterpart in the reference). The split-K partials use an 8 MiB array owned by
 * the library, held on every GPU that loads it; ma*mb*16 must not exceed 8 MiB
 * (EF_ERR_TOO_LARGE otherwise). The first call on a device looks up the array's device
 * address; make that first call before any stream capture. All calls share the array:
 * calls that can overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. Allocates nothing. */
int ef_gram_noalloc(const float* A, const float* B, int ma, int mb, long long K, double* G,
                    void* stream);
/* Gram schedule override for one (ma, mb) shape (no counterpart in the reference: set
 * by the autotuner, eigenfns_gb300/tune.py). kernel 0 = built-in choice, 1 = tensor
 * cores, 2 = CUDA cores; units_per_sm (0 = default 2) sets how many K-chunks per SM the
 * tensor-core Gram splits into. Consulted by ef_gram, ef_gram_tc and their workspace
 * queries; EF_ERR_TOO_LARGE once 256 shapes are registered. */
int ef_tune_gram(int ma, int mb, int kernel, int units_per_sm);
/* drops every ef_tune_gram override */
int ef_tune_reset(void);
/* reads and clears the sticky device flag the tensor-core Gram and rotation set when one
 * of their bounded waits ran out (never expected; results of that call are not valid).
 * Synchronises the device. */
int ef_tc_error(int* flag);
/* queues a copy of the same flag into *host_flag (pinned host memory) on `stream`,
 * without clearing it: after the stream reaches the copy, a nonzero value means a
 * tensor-core kernel queued before it on that stream (or finished before it on another)
 * timed out. The batch driver reads it per solve without synchronising the device. */
int ef_tc_error_async(int* host_flag, void* stream);
/* work bytes of ef_gram_tc for these sizes */
size_t ef_gram_tc_workspace_bytes(int ma, int mb, long long K);
/* the Gram of ef_gram (solver.py:35-43) on the tcgen05 tensor cores: 3xTF32 split
 * products (fp32-class accuracy), fp32 accumulation in TMEM per K-chunk, fp64 reduction
 * across chunks. mb <= 256, K even, 16-byte aligned rows. err_dev (a device int, not
 * NULL) is set to 1 if a bounded wait timed out (never expected; the result of that call
 * is then not valid). */
int ef_gram_tc(const float* A, const float* B, int ma, int mb, long long K, double* G, int* err_dev,
               void* work, size_t work_bytes, void* stream);
/* out_i (+/-)= sum_j C[j][i] S_j, C complex64 (m_in, m_out) row-major:
 * combine / tensordot(C.T, S) (solver.py:49-57,106,125); mode 0 set, 1 add, -1 subtract.
 * `out` may be `S` itself when m_out <= 32 (each column k is read in full before it is
 * written); otherwise it must not overlap S (EF_ERR_INVALID). Runs on the tcgen05
 * tensor cores (3xTF32 split products, fp32-class accuracy); setting the environment
 * variable EF_ROTATE_KERNEL=simt selects the fp32 CUDA-core kernel instead. */
int ef_rotate(const float* C, const float* S, float* out, int m_in, int m_out, long long K,
              int mode, void* stream);
/* ---- arithmetic-rate probe (no counterpart in the reference: measures the FP32 roof
 * the operator's FFT work is compared against) ----
 * `blocks` CTAs of 256 threads, each thread 8 independent fp32 FMA chains of `iters`
 * steps (paired = 1: four FFMA2 pairs); out holds blocks*256 floats. */
long long ef_fma_probe_flops(int blocks, int iters);
int ef_fma_probe(float* out, int blocks, int iters, int paired, void* stream);
/* ---- small dense fp64 problems on the device (solver.py:46-66, 113-126, 281-301) ----
 * Batched, one CTA per problem; matrices complex128 (n, n) row-major, 1 <= n <= 96,
 * consecutive in memory for the batch. */
/* Cholesky-QR coefficients of Gram matrices G = X^H X (gram, solver.py:35-43): C = R^-1
 * (complex64, upper triangular) with G = R^H R, so ef_rotate(C, X) orthonormalises X
 * like one pass of the reference's SVQB ortho_block (solver.py:113-126) does, within
 * the span. A pivot at or below tol * max diag(G) is a dead direction, as SVQB's drop:
 * its row and column of C are zero, so the rotated row is zero; status[b] = the number
 * of dead directions. */
int ef_cholqr_f64(const double* G, int n, int batch, float* C, int* status, double tol,
                  void* stream);
/* work bytes of ef_eigh_f64 */
size_t ef_eigh_f64_workspace_bytes(int n, int batch);
/* Hermitian eigendecomposition (numpy.linalg.eigh as used at solver.py:46-66, 281-301)
 * by cyclic Jacobi in fp64: w (batch, n) ascending, V (batch, n, n) complex128 with the
 * eigenvectors as columns; status[b] = 1 if 40 sweeps did not converge. */
int ef_eigh_f64(const double* A, int n, int batch, double* w, double* V, void* work,
                size_t work_bytes, int* status, void* stream);
/* work bytes of ef_rowdot and ef_rowstats for these sizes */
size_t ef_rowdot_workspace_bytes(int m, long long K);
/* per-row statistics in one pass, out (m, 4) float64: Re<A_i,B_i>, Im<A_i,B_i>, |A_i|^2,
 * |B_i|^2 -- Rayleigh quotients, row norms and the residual norm
 * |HX - lam X|^2 = |HX|^2 - 2 lam Re<X,HX> + lam^2 |X|^2 (solver.py:228-238) */
int ef_rowstats(const float* A, const float* B, int m, long long K, double* out, void* work,
                size_t work_bytes, void* stream);
/* per-row complex <A_i, B_i> as complex128 (m) -- row norms and Rayleigh quotients
 * (solver.py:228-235, interior.py:75-82) */
int ef_rowdot(const float* A, const float* B, int m, long long K, double* out,
              void* work, size_t work_bytes, void* stream);
/* R = HX - lam[i] X_i with lam a device float64 (m) array (solver.py:229) */
int ef_residual(const float* HX, const float* X, const double* lam, float* R, int m,
                long long K, void* stream);
/* R = HX - lam[i] X_i and r2[i] = |R_i|^2 (float64, device) in one pass; K even and
 * 16-byte aligned rows; work >= ef_rowdot_workspace_bytes(m, K) (solver.py:229-231) */
int ef_residual_norms(const float* HX, const float* X, const double* lam, float* R, int m,
                      long long K, double* r2, void* work, size_t work_bytes, void* stream);
/* X_i *= scale[i] (device float64 (m)) */
int ef_scale_rows(float* X, const double* scale, int m, long long K, void* stream);
/* Y = a X + b Y with real scalars (recurrence helpers, lanczos) */
int ef_axpby(const float* X, float* Y, long long n_complex, double a, double b, void* stream);
/* masked random block (solver.py:196-205, chebyshev.py:248, exp_kpm_dos.py:139-140);
 * kind EF_RAND_*, element i of the block uses counter i of stream `stream_id` */
int ef_rand_block(const ef_op* op, float* X, int m, uint64_t seed, uint64_t stream_id,
                  int kind, void* stream);
/* X *= mask(kn > 0) */
int ef_apply_mask(const ef_op* op, float* X, int m, void* stream);

/* ---- grouped block operations (no counterpart in the reference) ------------------ */
/* The same operation on the blocks of several instances of one shape (one grid edge and
 * block size; any k-point or structure) in one call: instance i's operand starts at
 * base + i * stride, where strides count complex64 values for vector blocks and
 * coefficient matrices, complex128 entries for Gram outputs and doubles for row
 * statistics, eigenvalues, squared norms and scales; inst[0..n) (host memory) lists the
 * instances covered. Each instance's work is the single-instance call on its operands
 * (so results equal the instance computed alone), queued in list order on `stream` with
 * one workspace sized for one instance. Replaces, per instance, the calls of
 * eigenfns/operator.py:82-95 / 104-127 and eigenfns/solver.py:35-57, 228-238. */
int ef_group_theta(const ef_op* const* ops, const int* inst, int n, const float* X,
                   long long x_stride, float* Y, long long y_stride, int m, void* work,
                   size_t work_bytes, void* stream);
int ef_group_precondition(const ef_op* const* ops, const int* inst, int n, const float* X,
                          long long x_stride, float* Y, long long y_stride, int m, void* work,
                          size_t work_bytes, void* stream);
int ef_group_gram(const int* inst, int n, const float* A, long long a_stride, const float* B,
                  long long b_stride, int ma, int mb, long long K, double* G, long long g_stride,
                  void* work, size_t work_bytes, void* stream);
int ef_group_rotate(const int* inst, int n, const float* C, long long c_stride, const float* S,
                    long long s_stride, float* out, long long o_stride, int m_in, int m_out,
                    long long K, int mode, void* stream);
int ef_group_rowstats(const int* inst, int n, const float* A, long long a_stride, const float* B,
                      long long b_stride, int m, long long K, double* out, long long out_stride,
                      void* work, size_t work_bytes, void* stream);
int ef_group_residual_norms(const int* inst, int n, const float* HX, long long h_stride,
                            const float* X, long long x_stride, const double* lam,
                            long long lam_stride, float* R, long long r_stride, int m, long long K,
                            double* r2, long long r2_stride, void* work, size_t work_bytes,
                            void* stream);
int ef_group_scale_rows(const int* inst, int n, float* X, long long x_stride, const double* scale,
                        long long s_stride, int m, long long K, void* stream);

/* ---- benchmark inputs (no counterpart in the reference) -------------------------- */
/* eps of a periodic rod network averaged over sub^3 sub-samples per voxel into
 * eps_host (G^3 float32, host). rods_host is (n_rods, 7) float64: endpoints p, q
 * (q the minimum image of the far node) and radius. Flat-capped cylinders as in
 * the reference's membership test (eigenfns/structure.py:135-138); the reference
 * itself rasterizes binary centre samples. Allocates its own device scratch. */
int ef_rasterize_rods(int grid, double box_size, const double* rods_host, int n_rods, int sub,
                      double eps_rod, double eps_bg, float* eps_host);

#ifdef __cplusplus
}
#endif

#endif /* EIGENFNS_GB300_H */
