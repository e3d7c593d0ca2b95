/*
 * tncontract_gb300 -- C ABI of the GB300 (sm_103a) engine for tncontract's
 * tensor-network hot path.
 *
 * The reference library (andrewdarmawan/tncontract) is pure Python on NumPy:
 * it has no FFI layer of its own.  Every entry point below replaces one NumPy
 * / LAPACK call (or one loop body) that the reference's Python code makes on
 * the hot path; each declaration cites that call site (path within the
 * reference project, file:line).  A binding layer (ctypes in this project,
 * see tncontract_gb300/_lib.py) calls these with device pointers it owns.
 *
 * Conventions
 *  - All pointers are device pointers unless stated otherwise; matrices are
 *    row-major (C order, like NumPy's default) with explicit leading
 *    dimensions; tensors are dense C-order arrays.
 *  - `dtype` is one of TNC_F32 / TNC_F64 / TNC_C64 / TNC_C128; complex values
 *    are (re, im) pairs like numpy.complex64 / complex128.
 *  - Scalars (alpha, beta) are passed as host `double[2]` = (re, im).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).
 *  - Functions return a TNC_* status; they never allocate device memory.
 *    Factorisations take a caller-provided workspace whose size is given by
 *    the matching *_workspace_size function.
 *  - Device-side failures (non-convergence, non-finite input, a bounded
 *    wait on a barrier, flag or step counter that gave up) are written to a
 *    device `info` word that the caller reads after synchronising; nothing
 *    traps or spins without bound.
 */
#ifndef TNCONTRACT_GB300_H
#define TNCONTRACT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { TNC_F32 = 0, TNC_F64 = 1, TNC_C64 = 2, TNC_C128 = 3 };

enum {
  TNC_OK = 0,
  TNC_ERR_ARG = 1,           /* bad shape / dtype / pointer argument       */
  TNC_ERR_NOT_CONVERGED = 2, /* Jacobi sweep cap reached                   */
  TNC_ERR_NONFINITE = 3,     /* NaN / Inf met in the input                 */
  TNC_ERR_CUDA = 4,          /* a CUDA launch or API call failed           */
  TNC_ERR_WORKSPACE = 5,     /* workspace smaller than *_workspace_size    */
  TNC_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up         */
  TNC_ERR_TOO_LARGE = 7      /* problem exceeds tnc_svd_noalloc's scratch  */
};

/* matrix operation applied to a row-major operand */
enum { TNC_OP_N = 0, TNC_OP_T = 1, TNC_OP_C = 2 /* conj-transpose */, TNC_OP_R = 3 /* conj */ };

int tnc_abi_version(void);
const char *tnc_status_string(int status);

/* Polls every bounded device-side wait makes before it gives up and records
 * TNC_ERR_TIMEOUT (grid barriers, step counters and flags of the persistent
 * factorisation kernels; twice as many for the tensor-core GEMM's mbarrier
 * waits).  Applies to the current device; polls <= 0 restores the default
 * (2^24, a few seconds).  No counterpart in the reference (which has no
 * device code); it lets a test make a wait run out. */
int tnc_set_spin_limit(long long polls);
/* One CTA waits on something nothing completes -- kind 0: a grid barrier
 * expecting two CTAs, 1: a step counter nobody publishes, 2: a flag nobody
 * sets -- until the wait limit runs out; info[0] (device int) receives the
 * error word, TNC_ERR_TIMEOUT when the bounded wait gave up as designed.
 * work: 256 bytes of device memory.  A self-test of the failure path the
 * factorisations share; the reference's counterpart of that path is
 * tensor_svd's retry and re-raise (tncontract/tensor.py:914-929). */
int tnc_wait_selftest(int kind, void *work, size_t work_bytes, int *info,
                      void *stream);
/* Kernels launched by this library since it was loaded (host counter). */
unsigned long long tnc_kernel_launches(void);

/* ------------------------------------------------------------ data movement */

/* dst = transpose(src, perm) (optionally conjugated): dst.shape[i] =
 * shape[perm[i]].  rank <= 8.  Replaces the axis moves of the reference:
 * np.rollaxis in Tensor.move_index / move_indices / consolidate_indices
 * (tncontract/tensor.py:340-394, 396-482) and the operand transposes inside
 * np.tensordot (tensor.py:735); conj=1 replaces Tensor.conjugate
 * (tensor.py:484-485). */
int tnc_permute(int dtype, const void *src, void *dst, int rank,
                const int64_t *shape, const int *perm, int conj, void *stream);

/* y[i] = alpha * (conj ? conj(x[i]) : x[i]); x may equal y.  Replaces
 * Tensor.__mul__/__rmul__ (tensor.py:95-123) and the in-place rescalings of
 * the MPS routines (onedim_core.py:301-314, 357-358, 479-484). */
int tnc_scale(int dtype, int64_t n, const double *alpha, const void *x,
              void *y, int conj, void *stream);

/* y = alpha*x + beta*y.  Replaces Tensor.__add__ (tensor.py:125-140). */
int tnc_axpby(int dtype, int64_t n, const double *alpha, const void *x,
              const double *beta, void *y, void *stream);

/* dtype conversion (real -> complex sets im = 0; complex -> real drops im). */
int tnc_cast(int src_dtype, int dst_dtype, int64_t n, const void *src,
             void *dst, void *stream);

/* out[0] = sqrt(sum |x_i|^2), accumulated in double, into a device double.
 * Replaces np.linalg.norm (tensor.py:587-590, onedim_core.py:279, 655-658). */
int tnc_nrm2(int dtype, int64_t n, const void *x, double *out, void *stream);

/* out[0..1] = sum op(x_i) y_i as (re, im) in double (device).  Used for the
 * scalar closing of inner_product_mps (onedim_core.py:1666-1683). */
int tnc_dot(int dtype, int64_t n, const void *x, const void *y, int conj_x,
            double *out, void *stream);

/* Trace over axes (axis1, axis2) of a dense tensor; dst holds the remaining
 * axes in order.  Replaces np.trace in Tensor.contract_internal
 * (tensor.py:318-334). */
int tnc_trace(int dtype, int rank, const int64_t *shape, int axis1, int axis2,
              const void *src, void *dst, void *stream);

/* A[i, :] *= f(d[i]) for a rows x cols row-major A (lda), d real (float for
 * F32/C64, double for F64/C128), f = identity (mode 0), sqrt (mode 1),
 * 1/x (mode 2) or 1/x^2 (mode 3; zero stays zero).
 * Replaces the dense diag(S) contractions that absorb singular values
 * (tensor.py:940-959, 1166-1182; onedim_core.py:347-351). */
int tnc_scale_rows(int dtype, int64_t rows, int64_t cols, const void *d,
                   int mode, void *A, int64_t lda, void *stream);
/* A[:, j] *= f(d[j]); same conventions. */
int tnc_scale_cols(int dtype, int64_t rows, int64_t cols, const void *d,
                   int mode, void *A, int64_t lda, void *stream);

/* dst[i, j] = src[i, j] for a rows x cols block with leading dimensions
 * lds / ldd.  The slicing copies of truncation, U.data[:, :, :k]
 * (onedim_core.py:340-343, tensor.py:1158-1163), and zero padding
 * (Tensor.pad_index, tensor.py:543-563). */
int tnc_copy2d(int dtype, int64_t rows, int64_t cols, const void *src,
               int64_t lds, void *dst, int64_t ldd, void *stream);

/* out = diag(d) as a dense n x n matrix (d real, see tnc_scale_rows).  The
 * S tensor of tensor_svd, np.diag(s) (tensor.py:940). */
int tnc_diag_matrix(int dtype, int64_t n, const void *d, void *out, void *stream);

/* ------------------------------------------------------------ contraction */

/* Batched GEMM on row-major operands:
 *   C_b = alpha * op(A_b) * op(B_b) + beta * C_b,  b < batch,
 * op(A_b) is m x k, op(B_b) is k x n, X_b = X + b*strideX.  This is the
 * product np.tensordot performs after matricising both operands
 * (tensor.py:735); the label -> axis resolution stays on the host. */
int tnc_gemm(int dtype, int opA, int opB, int64_t m, int64_t n, int64_t k,
             const double *alpha, const void *A, int64_t lda, int64_t strideA,
             const void *B, int64_t ldb, int64_t strideB, const double *beta,
             void *C, int64_t ldc, int64_t strideC, int64_t batch,
             void *stream);

/* Up to TNC_GEMM_GROUP_MAX independent products of different shapes in one
 * launch (CUDA-core tiles, round-to-nearest FMA): problem i computes
 * C_i = alpha_i op(A_i) op(B_i) + beta_i C_i on row-major operands as
 * tnc_gemm does (k >= 1; problems with m or n = 0 are skipped).  `problems`
 * is a HOST array.  The independent pairwise contractions of one network
 * (con's cost-ordered plan) run as one grouped launch per wave; in the
 * reference they are successive np.tensordot calls in tncontract/tncon.py:
 * 131-155. */
#define TNC_GEMM_GROUP_MAX 16
typedef struct {
  int opA, opB;
  int64_t m, n, k;
  const void *A;
  int64_t lda;
  const void *B;
  int64_t ldb;
  void *C;
  int64_t ldc;
  double alpha[2], beta[2];
} tnc_gemm_problem;
int tnc_gemm_grouped(int dtype, int count, const tnc_gemm_problem *problems,
                     void *stream);

/* tnc_gemm on the tcgen05 tensor cores for F32 / C64: TF32 split products
 * (hi*hi + hi*lo + lo*hi, FP32 accumulation in tensor memory) give
 * FP32-class accuracy; operands are split into planar K-major TF32 planes in
 * the workspace and streamed by TMA.  Same operands and ops as tnc_gemm;
 * batch <= 65535.  The product np.tensordot performs (tensor.py:735) for
 * single-precision tensors, and the absorption products of the sweep. */
int tnc_gemm_tc_workspace_size(int dtype, int64_t m, int64_t n, int64_t k,
                               int64_t batch, size_t *bytes);
int tnc_gemm_tc(int dtype, int opA, int opB, int64_t m, int64_t n, int64_t k,
                const double *alpha, const void *A, int64_t lda,
                int64_t strideA, const void *B, int64_t ldb, int64_t strideB,
                const double *beta, void *C, int64_t ldc, int64_t strideC,
                int64_t batch, void *work, size_t work_bytes, void *stream);
/* Reads and clears the tensor-core GEMM's device error flag (1 = a bounded
 * wait gave up; synchronous). */
int tnc_gemm_tc_error(void);

/* One MPO-MPS site product with the reference's fused bond layout
 * (contract_mps_mpo, onedim_core.py:1702-1704: contract over phys/physin
 * then consolidate_indices, fused bond = a*D + b):
 *   out[l*Dl + wl][po][r*Dr + wr]      (layout 0: (left, physout, right),
 *                                        the reference's label order)
 *   out[po][l*Dl + wl][r*Dr + wr]      (layout 1: (phys, left, right))
 *   = sum_p A[p][l][r] * W[po][p][wl][wr].
 * A is (d_in, chl, chr), W is (d_out, d_in, Dl, Dr). */
int tnc_mps_mpo_site(int dtype, int64_t d_in, int64_t d_out, int64_t chl,
                     int64_t chr, int64_t Dl, int64_t Dr, const void *A,
                     const void *W, void *out, int layout, void *stream);

/* ------------------------------------------------------------ factorisations */

/* Reduced QR of a row-major m x n matrix A (lda): Q is m x k (ldq = k),
 * R is k x n (ldr = n), k = min(m, n).  Householder reflectors in LAPACK's
 * convention (geqrf + ungqr), factored by one cooperative persistent launch
 * as a column-owner dataflow, Q formed explicitly.  info (device int):
 * TNC_OK or TNC_ERR_TIMEOUT.
 * Replaces np.linalg.qr(mode="reduced") in tensor_qr (tensor.py:1044). */
int tnc_qr_workspace_size(int dtype, int64_t m, int64_t n, size_t *bytes);
int tnc_qr(int dtype, int64_t m, int64_t n, const void *A, int64_t lda,
           void *Q, void *R, void *work, size_t work_bytes, int *info,
           void *stream);

/* R factor only of a dense row-major m x n matrix A (adjoint = 0; R is
 * k x n) or of its conjugate transpose A^H (adjoint = 1; R is k x m),
 * k = min(m, n); Q is not formed.  The sweep SVD preconditions its Jacobi
 * stage with the R of M^H: the rotated rows of R are S U^H of M, so U comes
 * out orthonormal whatever the spectrum, and the Jacobi converges in fewer
 * sweeps on graded matrices.  No counterpart in the reference (whose
 * tensor_svd calls LAPACK gesdd on M directly, tensor.py:915). */
int tnc_qr_r_workspace_size(int dtype, int64_t m, int64_t n, int adjoint,
                            size_t *bytes);
int tnc_qr_r(int dtype, int64_t m, int64_t n, const void *A, int adjoint,
             void *R, void *work, size_t work_bytes, int *info, void *stream);

/* Thin SVD of a row-major m x n matrix A (lda): U is m x k, S has k real
 * values sorted descending (float for F32/C64, double for F64/C128), VH is
 * k x n, k = min(m, n).  QR-preconditioned one-sided (Hestenes) Jacobi:
 * the k x k triangular factor of A^H (wide A) or A (tall A) is
 * orthogonalised with a round-robin ordering by one persistent cooperative
 * launch, rotations accumulated; U and VH follow with one GEMM against Q,
 * both orthonormal however graded the spectrum.  max_sweeps <= 0 selects
 * 40; tol <= 0 selects sqrt(k) * eps (4x that for FP32 storage).  info
 * (device, 4 ints):
 * [0] status (TNC_OK / TNC_ERR_NOT_CONVERGED / TNC_ERR_NONFINITE /
 * TNC_ERR_TIMEOUT), [1] sweeps used, [2] rotations in the last sweep.
 * Replaces np.linalg.svd(full_matrices=False) in tensor_svd (tensor.py:915)
 * and its scipy gesvd retry (tensor.py:916-929). */
int tnc_svd_workspace_size(int dtype, int64_t m, int64_t n, size_t *bytes);
int tnc_svd(int dtype, int64_t m, int64_t n, const void *A, int64_t lda,
            void *U, void *S, void *VH, int max_sweeps, double tol,
            void *work, size_t work_bytes, int *info, void *stream);

/* tnc_svd for callers that cannot provide a workspace.  No counterpart in the
 * reference: it exists for hosts where this library may not allocate and
 * the caller has no spare buffer to lend it (a plugin inside another
 * framework that owns the whole device-memory budget, a service that
 * reserves all memory at start-up).  The work area is a fixed 16 MiB
 * array inside the library image (held by every GPU that loads the library
 * until exit); a problem is accepted when tnc_svd_workspace_size(dtype, m, n)
 * is at most 16 MiB (e.g. complex128 up to 450 x 450 or 433 x 512, complex64
 * and float64 up to 647 x 647 or 531 x 1024), otherwise TNC_ERR_TOO_LARGE is
 * returned before anything is launched or written.  Same arguments and
 * results as tnc_svd otherwise.  All calls on a device share that area:
 * calls that overlap on the GPU race, so order them on one stream.  The
 * area's device address is looked up (with the device current) on the first
 * call on a device, and again after that device's context was destroyed and
 * re-created (cudaDeviceReset); make those calls before any stream
 * capture. */
int tnc_svd_noalloc(int dtype, int64_t m, int64_t n, const void *A,
                    int64_t lda, void *U, void *S, void *VH, int max_sweeps,
                    double tol, int *info, void *stream);

/* Jacobi stage of the truncating sweep SVD (left_canonise's SVD branch,
 * onedim_core.py:317-343): the rows of W = A (m <= n) or A^H (m > n),
 * min(m,n) x max(m,n), are made mutually orthogonal by one-sided Jacobi
 * rotations that are not accumulated (block ordering: half-blocks of rows
 * in registers and shared memory, one cooperative launch).  Writes W (caller
 * buffer), S = row norms sorted descending (real type of dtype) and order
 * (int64: order[i] = row of W holding the i-th singular triplet).  For a wide
 * A, rows order[:k] of W are S_k V_k^H and U_k = A (S_k V_k^H)^H S_k^-2; for
 * a tall A they are S_k U_k^H and S_k V_k^H = U_k^H A.  block_rows (2, 4, 8,
 * or 16 for rows up to 512 of types up to 8 bytes; anything else selects 8)
 * is the half-block height of the row-by-row rotation kernel, chosen per
 * shape by the caller's autotuner (0: 8); TNC_ROWS_GRAM selects, for F32 /
 * C64 rows, the Gram-form block update: each half-block pair's rotations
 * run on its 16 x 16 Gram matrix and are applied to the rows as one 16 x 16
 * product (same rotations, GEMM-shaped work; 8-row half-blocks, the
 * row-by-row kernel where fewer rows need smaller ones).
 * max(m,n) <= 1024 (512 for F64/C128).  info as for tnc_svd. */
enum { TNC_ROWS_GRAM = 32 };
int tnc_svd_rows_workspace_size(int dtype, int64_t m, int64_t n, size_t *bytes);
int tnc_svd_rows(int dtype, int64_t m, int64_t n, const void *A, void *W,
                 void *S, int64_t *order, int max_sweeps, double tol,
                 int block_rows, void *work, size_t work_bytes, int *info,
                 void *stream);

/* tnc_svd_rows where only the first nkeep rows of W must come out orthogonal
 * to every row: pairs of rows that both lie beyond nkeep (in whole
 * half-blocks) take no rotation, so those rows are orthogonal to the kept
 * ones but not among themselves, and their norms are their singular values
 * only to the accuracy of W's start.  For a start whose rows are already
 * nearly orthogonal and sorted by norm (the FP64 finish of a truncating
 * bond: the rows beyond the retained rank are discarded), this saves the
 * discarded-discarded rotations.  nkeep >= min(m, n) is tnc_svd_rows. */
int tnc_svd_rows_keep(int dtype, int64_t m, int64_t n, const void *A, void *W,
                      void *S, int64_t *order, int max_sweeps, double tol,
                      int block_rows, int64_t nkeep, void *work,
                      size_t work_bytes, int *info, void *stream);

/* tnc_svd_rows as the first stage of a finished core: the sweeps also stop
 * (status TNC_OK, info[3] = 1) after the first sweep in which no rotation
 * met a relative off-diagonal |<w_i, w_j>| / (|w_i| |w_j|) above stop_tol,
 * instead of running on to a sweep without any rotation above tol -- the
 * finishing stage (tnc_svd_rows_df / tnc_svd_rows_keep) takes the rows from
 * there and confirms their orthogonality itself.  stop_tol = 0 is
 * tnc_svd_rows. */
int tnc_svd_rows_stage(int dtype, int64_t m, int64_t n, const void *A, void *W,
                       void *S, int64_t *order, int max_sweeps, double tol,
                       double stop_tol, int block_rows, void *work,
                       size_t work_bytes, int *info, void *stream);

/* The rows of src (m x L) in decreasing-norm order: dst[i] = src[order[i]],
 * stable (equal norms keep their order; a NaN norm ranks last), rank[j] =
 * the dst row of src row j.  norms2: m doubles of the caller's device memory
 * (the squared norms).  src and dst must not overlap; m <= 65536 (the
 * ranking compares every pair of rows).  The sweep sorts each
 * bond matrix's rows before the R-only QR of M^H (a static column pivoting
 * of that QR: the Jacobi on R then needs fewer sweeps) -- part of the
 * truncating SVD of left_canonise, onedim_core.py:317-343. */
int tnc_sort_rows(int dtype, int64_t m, int64_t L, const void *src, void *dst,
                  int64_t *order, int64_t *rank, double *norms2, void *stream);
/* dst[i] = src[idx[i]] for i < n (rows of length L; device idx, every
 * value a row of src: the kernel does not check it) -- e.g. the inverse of
 * tnc_sort_rows with idx = rank.  src and dst must not overlap. */
int tnc_permute_rows(int dtype, int64_t n, int64_t L, const void *src,
                     const int64_t *idx, void *dst, void *stream);

/* The extended-precision finish of single-precision rows, in double-float
 * arithmetic on the FP32 pipe (a real number as an unevaluated pair of
 * floats, about 48 significant bits; error-free TwoSum / TwoProd and Dot2
 * inner products): GB300 issues FP32 fused multiply-adds about 70 times as
 * fast as FP64 ones.  A: m x n rows (m <= n) of dtype TNC_F32 or TNC_C64,
 * scaled by a power of two to unit Frobenius norm inside; W (m x n) receives
 * the orthogonalised rows as FP64 / complex128 elements, S (FP64) and order
 * as tnc_svd_rows for the FP64 type, and the rows are orthogonal to tol
 * relative (<= 0: 1e-7).  The finish ends without a checking sweep (info[3]
 * = 1) after a rotating sweep whose rotations were all small angles below
 * 1e-5 relative: their residual is second order (about 1e-8).  Rows beyond nkeep as in tnc_svd_rows_keep.  Rows
 * up to 800 complex / 1600 real elements.  Workspace:
 * tnc_svd_rows_workspace_size of the FP64 type.  Replaces, in the sweep,
 * the FP64 finish (tnc_cast to the FP64 type + tnc_svd_rows_keep). */
int tnc_svd_rows_df(int dtype, int64_t m, int64_t n, const void *A, void *W,
                    void *S, int64_t *order, int max_sweeps, double tol,
                    int block_rows, int64_t nkeep, void *work,
                    size_t work_bytes, int *info, void *stream);

/* dst <- rows order[0:k] of src (row length L), k read from device memory
 * (capped by kmax): mode 0 copies rows (dst k x L); mode 1 writes
 * dst[c][i] = conj(src[order[i]][c]) / S[i] (dst L x k, leading dim k).
 * The slicing U.data[:, :, :k] / V.data[:k] of onedim_core.py:340-343 on the
 * Jacobi output. */
int tnc_gather_rows(int dtype, const void *src, int64_t L, const int64_t *order,
                    const int64_t *k, int64_t kmax, const void *S, int mode,
                    void *dst, void *stream);

/* ------------------------------------------------------------ the sweep */

/* One MPO.MPS apply + svd_compress sweep run natively on one stream:
 * contract_mps_mpo followed by MatrixProductState.svd_compress with the
 * norm restored (onedim_core.py:1691-1708, 463-484; the QR branch of
 * left_canonise :267-294, the truncating SVD branch :317-343), the retained
 * rank per bond by the reference's rule (s/s_max > threshold, at most chi,
 * :332-339) capped at the storage type's rounding-noise floor.  Sites are
 * (phys, left, right) device arrays; MPO sites (physout, physin, left,
 * right).  HOST arrays: sites[n_sites] and mpo[n_sites] (device pointers),
 * mps_bonds[n_sites+1], mpo_bonds[n_sites+1] (both ends 1); out_bonds
 * [n_sites+1] and out_offsets[n_sites] (byte offset in `work` of each
 * compressed site, (phys, out_bonds[i], out_bonds[i+1])) are written.
 * Every bond matrix's rows are sorted by norm before the R-only QR
 * (tnc_sort_rows; U's rows are put back after the factorisation).
 * core: TNC_CORE_STORAGE (0) factors every bond core in the storage
 * precision; TNC_CORE_FP64 (1, F32 / C64 storage only) finishes the Jacobi of
 * each core (rows up to 512 for C64, 1024 for F32) in FP64 after the
 * storage-precision Jacobi, and takes the singular values, the truncation
 * decision and U from the finished rows (the storage-precision stage then
 * runs to 3e-6, at most 14 sweeps, and stops after its first sweep without a
 * rotation above 1e-3 (tnc_svd_rows_stage), a stall handing over to the
 * finish as well); TNC_CORE_DF (2) is the same with the finish in
 * double-float arithmetic (tnc_svd_rows_df) instead of FP64.  core_tol: the
 * finishing stage's tolerance (<= 0: 1e-7, pairs of rows orthogonal to 1e-7
 * relative, the rounding level of U's single-precision storage; the
 * singular values' error from it is second order).  The singular values
 * inherit the storage-precision stage's rounding (FP32-class relative to
 * s_max).  The core changes the workspace size.
 * out_discarded (HOST, may be NULL): n_sites-1 doubles, [i] = the fraction of
 * the squared singular values discarded at the bond between sites i and i+1.
 * *log_norm: in, the natural log of the input state's norm factor; out, that
 * of the output.  *folded = 1 when that factor (except its s_max part) was
 * representable and folded into the first site.  block_rows as for
 * tnc_svd_rows (0 = 8).  profile (HOST, may be NULL): 12 doubles, for op o
 * (0 the QR of the left sweep, 1 the R-only QR of M^H, 2 the Jacobi, 3 its
 * FP64 finish) profile[3o] += milliseconds (CUDA events on `stream`),
 * [3o+1] += calls, [3o+2] += the op's fixed algorithmic flops (for op 3 the
 * flops the FP64 Jacobi executed: 14 n^2 L per rotating sweep and 4 n^2 L for
 * the last, checking one, n rows of length L, complex; a third of that
 * real; for TNC_CORE_DF the FP32 operations of the double-float Jacobi:
 * 44 n^2 L per rotating sweep and 24 n^2 L for the checking one, complex;
 * 15 and 6 real).  Returns TNC_ERR_ARG for a zero state. */
enum { TNC_CORE_STORAGE = 0, TNC_CORE_FP64 = 1, TNC_CORE_DF = 2 };
int tnc_sweep_workspace_size(int dtype, int n_sites, int64_t d,
                             const int64_t *mps_bonds, const int64_t *mpo_bonds,
                             int core, size_t *bytes);
int tnc_sweep_apply_compress(int dtype, int n_sites, int64_t d,
                             const void *const *sites, const int64_t *mps_bonds,
                             const void *const *mpo, const int64_t *mpo_bonds,
                             int64_t chi, double threshold, int block_rows,
                             int core, double core_tol, void *work,
                             size_t work_bytes, int64_t *out_bonds,
                             int64_t *out_offsets, double *out_discarded,
                             double *log_norm, int *folded, double *profile,
                             void *stream);

/* ------------------------------------------------------------ learned rank
 * Kernels of the rank predictor (a small MLP trained on singular spectra the
 * plain method produces) and of the randomized-SVD sketch it sizes.  No
 * counterpart in the reference; they size a randomized SVD that stands in
 * for left_canonise's full SVD (onedim_core.py:317) when the predicted rank
 * is small, with the full SVD as fallback.  FP32, row-major, batch-major. */
/* out[b][o] = act(sum_i W[o][i] in[b][i] + bias[o]); act 0 identity, 1 relu, 2 sigmoid */
int tnc_dense_forward(const float *W, const float *bias, const float *in,
                      float *out, int batch, int nin, int nout, int act,
                      void *stream);
/* dW = g^T in, db = colsum(g); gin = (g W) masked by act_in > 0 when
 * relu_mask (gin may be NULL) */
int tnc_dense_backward(const float *W, const float *in, const float *act_in,
                       const float *g, float *dW, float *db, float *gin,
                       int batch, int nin, int nout, int relu_mask,
                       void *stream);
/* g = d(mean squared error)/dz for y = sigmoid(z) */
int tnc_mse_sigmoid_grad(const float *y, const float *target, float *g,
                         int batch, void *stream);
/* one Adam step with bias correction (step >= 1) */
int tnc_adam_step(float *params, const float *grads, float *m, float *v,
                  int64_t n, double lr, double beta1, double beta2,
                  double eps, int step, void *stream);
/* i.i.d. standard normal entries (complex: re and im each N(0,1)),
 * counter-based: entry i depends only on (seed, i) */
int tnc_fill_gaussian(int dtype, int64_t n, uint64_t seed, void *out,
                      void *stream);

/* Truncation decision on descending singular values S (n, real type of
 * dtype): k = #{ s_i > t } capped at chi (chi <= 0: no cap), t = threshold
 * (relative = 0) or threshold * S[0] (relative = 1).  Writes k (device
 * int64) and the discarded weight sum_{i >= k} s_i^2 (device double).  The
 * rule of truncated_svd (tensor.py:1137-1152) and of left_canonise
 * (onedim_core.py:332-339; s/s_max > threshold is s > threshold*s_max). */
int tnc_truncation_rank(int dtype, int64_t n, const void *S, int64_t chi,
                        double threshold, int relative, int64_t *k,
                        double *discarded, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TNCONTRACT_GB300_H */
