// Native driver of one MPO.MPS apply + svd_compress sweep: contract_mps_mpo
// followed by MatrixProductState.svd_compress (tncontract/onedim/
// onedim_core.py:1691-1708, 463-484; the QR branch of left_canonise :267-294,
// the truncating SVD branch :317-343 on the reversed state) with
// normalise=False and the norm restored, on device sites kept in the layout
// (phys, left, right).
//
// The same algorithm as the Python engine (tncontract_gb300/engine.py:
// apply_compress), run as one C call so that a host thread driving one
// instance never returns to the interpreter during a sweep: every per-site
// decision (R's norm, the retained rank from the spectrum) is a synchronous
// read on the caller's stream made here, with the calling thread outside
// Python.  Instances on concurrent streams then share the GPU without
// contending for the interpreter lock.
//
// Per site of the QR left sweep:   Q, R = qr(P_i as (d l) x r);  P_i = Q;
//                                  P_{i+1} <- (R / |R|) P_{i+1}.
// Per site of the SVD right sweep: M = P_i as (d r) x l, its rows sorted by
//                                  norm (M' = Pi M: a static column pivoting
//                                  of the QR below, fewer Jacobi sweeps);
//                                  R = qr_r(M'^H);  Jacobi on the rows of R
//                                  (rotated rows = S U'^H of M');  k from the
//                                  reference's rule (s / s_max > threshold, at
//                                  most chi) capped at the rounding-noise floor
//                                  4 eps |M|_F;  U' = normalised rows;
//                                  S V^H = U'^H M';  P_i = U = Pi^T U';
//                                  P_{i-1} <- P_{i-1} (S V^H)^T / s_max.
// With a finishing core (core = 1 FP64, core = 2 double-float; single-
// precision storage only) the Jacobi of every truncating bond runs twice: the
// storage-precision Jacobi above brings the rows of R to orthogonality at the
// FP32 rounding level, then the rows are sorted by norm and a one-sided
// Jacobi in FP64 (widened rows) or in double-float arithmetic on the FP32
// pipe finishes them (tolerances kCoreFp32Tol / kCoreTol: usually one
// rotating and one checking sweep); rows beyond the FP32 rank plus a margin
// are rotated against the kept rows only (they are discarded);
// the singular values, the truncation decision (s / s_max > threshold, at most
// chi) and U come from the finished rows.  The products around the core stay
// in the storage precision.
// All buffers are carved from one caller workspace sized for the un-truncated
// bond dimensions (tnc_sweep_workspace_size); nothing is allocated.
#include "tnc_common.cuh"

#include <cmath>
#include <vector>

namespace tnc {
namespace {

constexpr size_t kAlign = 256;

struct Carve {
  char* base;
  size_t off;
  void* take(size_t bytes) {
    off = (off + kAlign - 1) & ~(kAlign - 1);
    void* p = base ? base + off : nullptr;
    off += bytes;
    return p;
  }
};

struct Dims {
  std::vector<int64_t> bp;  // applied bonds b_i * D_i
  int64_t max_site = 0, max_r = 0, max_u = 0, max_sv = 0, max_kmin = 0, max_m = 0;
  size_t fact = 0;          // largest factorisation / GEMM workspace
  bool core64 = false;      // FP64-accurate Jacobi finish of the bond cores
  bool core_df = false;     // ... computed in double-float (else in FP64)
};

// Tolerances of the two Jacobi stages of an FP64 core (|<w_i, w_j>| <= tol
// |w_i| |w_j| for every pair of rows).  The FP32 stage runs to 3e-6, near its
// rounding floor (sqrt(L) eps_32 ~ 2.7e-6 at L = 512), and at most
// kCoreFp32Sweeps sweeps: a stage that stalls above the tolerance is not an
// error, the FP64 stage takes over from where it stopped.  The FP64 stage
// runs to 1e-7: U is stored back in single precision, whose rounding (6e-8
// per entry) already limits its orthogonality to that level, and the
// singular values' error from the tolerance is second order (1e-14).  From
// that start one rotating FP64 sweep and one checking sweep usually suffice
// (measured at 512 x 512: 2 FP64 sweeps, against 3 with an FP32 stage at its
// default 1.1e-5 and an FP64 stage at 1e-8).
constexpr double kCoreFp32Tol = 3e-6;
constexpr int kCoreFp32Sweeps = 14;
constexpr double kCoreTol = 1e-7;
// The FP32 stage of a finished core also stops after the first sweep whose
// rotations were all below kCoreStopTol relative: the finish converges the
// rows from there and confirms their orthogonality itself, so the FP32
// stage's own checking sweep (and its last sweeps at the rounding floor)
// are not needed.
constexpr double kCoreStopTol = 1e-3;
// Rows beyond the FP32 stage's retained rank that the FP64 stage still
// finishes against each other: the FP64 decision may retain a few more (or
// rank them differently); if it retains any row beyond, the whole finish
// runs again.
constexpr int64_t kCoreKeepMargin = 16;

// the FP64 type that finishes the Jacobi of a single-precision core
inline int core_dtype(int dt) { return dt == TNC_C64 ? TNC_C128 : TNC_F64; }
// rows of the register-resident FP64 Jacobi (complex128 rows hold 512 entries)
inline int64_t core_rows_limit(int dt) { return dt == TNC_C64 ? 512 : 1024; }

bool fp32_class(int dt) { return dt == TNC_F32 || dt == TNC_C64; }

size_t tc_ws(int dt, int64_t m, int64_t n, int64_t k, int64_t batch) {
  if (!fp32_class(dt)) return 0;
  size_t b = 0;
  if (tnc_gemm_tc_workspace_size(dt, m, n, k, batch, &b) != TNC_OK) return 0;
  return b;
}

// The sweep's absorption products of single-precision sites run on the
// tensor-core GEMM, whose error-free digit split keeps the products unbiased
// (a TF32 split accumulated with truncation in tensor memory had shrunk the
// state's norm by 1.6e-3 over the 190 products of a chi = 256 sweep); small
// products stay on the CUDA-core GEMM.
bool use_tc(int dt, int64_t m, int64_t n, int64_t k, int64_t batch) {
  return fp32_class(dt) && (m < n ? m : n) >= 64 && k >= 32 && (double)m * n * k * batch >= (double)(1 << 21) &&
         batch <= 65535;
}

int64_t rows_limit(int dt) { return fp32_class(dt) ? 1024 : 512; }

// upper bounds of every buffer over the whole sweep
int plan(int dt, int n_sites, int64_t d, const int64_t* b, const int64_t* D, int core, Dims& P) {
  if (core != 0 && core != 1 && core != 2) return TNC_ERR_ARG;
  if (core != 0 && !fp32_class(dt)) return TNC_ERR_ARG;  // the finish is of single-precision cores
  P.core64 = core != 0;
  P.core_df = core == 2;
  P.bp.resize(n_sites + 1);
  for (int i = 0; i <= n_sites; ++i) {
    if (b[i] <= 0 || D[i] <= 0) return TNC_ERR_ARG;
    P.bp[i] = b[i] * D[i];
  }
  size_t f = 0, x = 0;
  for (int i = 0; i < n_sites; ++i) {
    const int64_t l = P.bp[i], r = P.bp[i + 1];
    const int64_t site = d * l * r;
    P.max_site = site > P.max_site ? site : P.max_site;
    // QR left sweep: (d l) x r, R k x r, absorption k x r2 x r batched over d
    const int64_t rows = d * l, kq = rows < r ? rows : r;
    if (tnc_qr_workspace_size(dt, rows, r, &x) != TNC_OK) return TNC_ERR_ARG;
    f = x > f ? x : f;
    P.max_r = kq * r > P.max_r ? kq * r : P.max_r;
    if (i + 1 < n_sites) {
      const int64_t r2 = P.bp[i + 2];
      x = tc_ws(dt, kq, r2, r, d);
      f = x > f ? x : f;
    }
    // SVD right sweep: M (d r) x l, R of M^H kmin x m, U m x kmin, S V^H kmin x l
    const int64_t m = d * r, n = l, kmin = m < n ? m : n;
    P.max_m = m > P.max_m ? m : P.max_m;
    if (tnc_qr_r_workspace_size(dt, m, n, 1, &x) != TNC_OK) return TNC_ERR_ARG;
    f = x > f ? x : f;
    // the rows path runs whenever the truncated row count is within the
    // register limit, which it can be even when this bound is not
    const int64_t mr = m < rows_limit(dt) ? m : rows_limit(dt), kr = mr < n ? mr : n;
    if (tnc_svd_rows_workspace_size(dt, kr, mr, &x) != TNC_OK) return TNC_ERR_ARG;
    f = x > f ? x : f;
    if (P.core64) {
      if (tnc_svd_rows_workspace_size(core_dtype(dt), kr, mr, &x) != TNC_OK) return TNC_ERR_ARG;
      f = x > f ? x : f;
    }
    if (m > rows_limit(dt)) {
      if (tnc_svd_workspace_size(dt, kmin, m, &x) != TNC_OK) return TNC_ERR_ARG;
      f = x > f ? x : f;
    }
    x = tc_ws(dt, kmin, n, m, 1);
    f = x > f ? x : f;
    if (i > 0) {
      const int64_t lp = P.bp[i - 1];
      x = tc_ws(dt, d * lp, kmin, n, 1);
      f = x > f ? x : f;
    }
    P.max_r = kmin * m > P.max_r ? kmin * m : P.max_r;
    P.max_u = m * kmin > P.max_u ? m * kmin : P.max_u;
    P.max_sv = kmin * n > P.max_sv ? kmin * n : P.max_sv;
    P.max_kmin = kmin > P.max_kmin ? kmin : P.max_kmin;
  }
  P.fact = f;
  return TNC_OK;
}

struct Buffers {
  std::vector<void*> slot;
  void *scratch, *rbuf, *wbuf, *ubuf, *svbuf, *S, *fact;
  void *w64a = nullptr, *w64b = nullptr;  // FP64 core: widened rows, finished rows
  double* S64 = nullptr;
  int64_t* order64 = nullptr;
  int64_t* order;
  void* mpiv;                      // the bond matrix with its rows sorted by norm
  int64_t *porder, *prank;         // that sort and its inverse
  double* pnorm2;
  int64_t* kdev;
  double* dnorm;
  int* info;
};

size_t carve(Carve& c, int n_sites, int64_t d, const Dims& P, size_t es, size_t rs, Buffers& B) {
  B.slot.resize(n_sites);
  for (int i = 0; i < n_sites; ++i) B.slot[i] = c.take((size_t)d * P.bp[i] * P.bp[i + 1] * es);
  B.scratch = c.take((size_t)P.max_site * es);
  B.rbuf = c.take((size_t)P.max_r * es);
  B.wbuf = c.take((size_t)P.max_r * es);
  B.ubuf = c.take((size_t)(P.max_u > P.max_r ? P.max_u : P.max_r) * es);
  B.svbuf = c.take((size_t)P.max_sv * es);
  B.S = c.take((size_t)P.max_kmin * rs);
  B.order = (int64_t*)c.take((size_t)P.max_kmin * sizeof(int64_t));
  B.mpiv = c.take((size_t)P.max_site * es);
  B.porder = (int64_t*)c.take((size_t)P.max_m * sizeof(int64_t));
  B.prank = (int64_t*)c.take((size_t)P.max_m * sizeof(int64_t));
  B.pnorm2 = (double*)c.take((size_t)P.max_m * sizeof(double));
  B.kdev = (int64_t*)c.take(sizeof(int64_t));
  B.dnorm = (double*)c.take(sizeof(double));
  B.info = (int*)c.take(4 * sizeof(int));
  if (P.core64) {
    const size_t es64 = 2 * es;  // complex64 -> complex128, float -> double
    B.w64a = c.take((size_t)P.max_r * es64);
    B.w64b = c.take((size_t)P.max_r * es64);
    B.S64 = (double*)c.take((size_t)P.max_kmin * sizeof(double));
    B.order64 = (int64_t*)c.take((size_t)P.max_kmin * sizeof(int64_t));
  }
  B.fact = c.take(P.fact);
  return c.off;
}

int gemm_any(int dt, int opA, int opB, int64_t m, int64_t n, int64_t k, double alpha, const void* A, int64_t lda,
             int64_t sA, const void* Bm, int64_t ldb, int64_t sB, void* C, int64_t ldc, int64_t sC, int64_t batch,
             void* fact, size_t factb, cudaStream_t st) {
  const double a[2] = {alpha, 0.0}, z[2] = {0.0, 0.0};
  if (use_tc(dt, m, n, k, batch)) {
    size_t need = 0;
    if (tnc_gemm_tc_workspace_size(dt, m, n, k, batch, &need) == TNC_OK && need <= factb)
      return tnc_gemm_tc(dt, opA, opB, m, n, k, a, A, lda, sA, Bm, ldb, sB, z, C, ldc, sC, batch, fact, factb, st);
  }
  return tnc_gemm(dt, opA, opB, m, n, k, a, A, lda, sA, Bm, ldb, sB, z, C, ldc, sC, batch, st);
}

int scale(int dt, int64_t n, double s, void* x, cudaStream_t st) {
  const double a[2] = {s, 0.0};
  return tnc_scale(dt, n, a, x, x, 0, st);
}

// |x| to the host (a synchronising read on the stream)
int host_norm(int dt, int64_t n, const void* x, double* dnorm, double* out, cudaStream_t st) {
  if (int rc = tnc_nrm2(dt, n, x, dnorm, st)) return rc;
  if (cudaMemcpyAsync(out, dnorm, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return TNC_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? TNC_OK : TNC_ERR_CUDA;
}

int device_status(const int* info, cudaStream_t st) {
  int h = 0;
  if (cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return TNC_ERR_CUDA;
  return h;
}

// Optional per-op timing of a sweep on the caller's stream: for op o,
// prof[3o] += milliseconds, prof[3o+1] += calls, prof[3o+2] += the op's fixed
// algorithmic flops (QR 2mn^2 - 2n^3/3, SVD 6mn^2 + 20n^3, complex x4).
// Ops: 0 the QR of the left sweep, 1 the R-only QR of M^H, 2 the Jacobi,
// 3 the FP64 finish of the Jacobi (FP64 core only).
struct Prof {
  double* out = nullptr;
  cudaEvent_t ev[8] = {};
  bool ok = false;
  explicit Prof(double* o) : out(o) {
    if (!out) return;
    ok = true;
    for (auto& e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
  }
  ~Prof() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
  void begin(int op, cudaStream_t st) {
    if (ok) cudaEventRecord(ev[2 * op], st);
  }
  void end(int op, cudaStream_t st) {
    if (ok) cudaEventRecord(ev[2 * op + 1], st);
  }
  // after a synchronisation that covers the end event
  void add(int op, double flops) {
    if (!ok) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev[2 * op], ev[2 * op + 1]) != cudaSuccess) return;
    out[3 * op] += ms;
    out[3 * op + 1] += 1.0;
    out[3 * op + 2] += flops;
  }
};

double qr_flops(int64_t m, int64_t n, bool cplx) {
  const double mm = (double)(m > n ? m : n), nn = (double)(m < n ? m : n);
  return (2.0 * mm * nn * nn - 2.0 / 3.0 * nn * nn * nn) * (cplx ? 4.0 : 1.0);
}
double svd_flops(int64_t m, int64_t n, bool cplx) {
  const double mm = (double)(m > n ? m : n), nn = (double)(m < n ? m : n);
  return (6.0 * mm * nn * nn + 20.0 * nn * nn * nn) * (cplx ? 4.0 : 1.0);
}

template <typename R>
int64_t rank_rule(const std::vector<R>& s, int64_t chi, double threshold, double eps) {
  // the reference's rule: s / s_max > threshold, then at most chi
  // (onedim_core.py:332-339), capped at the rounding-noise floor 4 eps |M|_F
  const int64_t n = (int64_t)s.size();
  if (n == 0 || !(s[0] > 0)) return 0;
  const double smax = (double)s[0];
  double f2 = 0.0;
  for (int64_t j = 0; j < n; ++j) f2 += (double)s[j] * (double)s[j];
  const double floor = 4.0 * eps * std::sqrt(f2);
  int64_t k = 0, kn = 0;
  for (int64_t j = 0; j < n; ++j) {
    if ((double)s[j] > threshold * smax) ++k;
    if ((double)s[j] > floor) ++kn;
  }
  if (chi > 0 && k > chi) k = chi;
  if (kn < 1) kn = 1;
  return k < kn ? k : kn;
}

template <typename T>
int sweep_impl(int dt, int n_sites, int64_t d, const void* const* sites, const int64_t* b, const void* const* mpo,
               const int64_t* D, int64_t chi, double threshold, int block_rows, int core, double core_tol, void* work,
               size_t wb, int64_t* out_bonds, int64_t* out_offsets, double* out_discarded, double* log_norm,
               int* folded, double* profile, cudaStream_t st) {
  typedef typename traits<T>::real R;
  const bool cplx = traits<T>::is_complex;
  Prof prof(profile);
  Dims P;
  if (int rc = plan(dt, n_sites, d, b, D, core, P)) return rc;
  Carve c{(char*)work, 0};
  Buffers B;
  const size_t need = carve(c, n_sites, d, P, sizeof(T), sizeof(R), B);
  if (wb < need) return TNC_ERR_WORKSPACE;
  const size_t factb = P.fact;
  const double eps = traits<T>::eps;
  std::vector<int64_t> sl(n_sites), sr(n_sites);  // current bonds of every site
  // 1. apply: site i -> (d, b_i D_i, b_{i+1} D_{i+1}), fused bond a * D + w
  for (int i = 0; i < n_sites; ++i) {
    if (int rc = tnc_mps_mpo_site(dt, d, d, b[i], b[i + 1], D[i], D[i + 1], sites[i], mpo[i], B.slot[i], 1, st))
      return rc;
    sl[i] = P.bp[i];
    sr[i] = P.bp[i + 1];
  }
  // 2. QR left sweep
  double lnorm = *log_norm;
  for (int i = 0; i + 1 < n_sites; ++i) {
    const int64_t l = sl[i], r = sr[i], rows = d * l, k = rows < r ? rows : r;
    size_t qb = 0;
    if (tnc_qr_workspace_size(dt, rows, r, &qb) != TNC_OK || qb > factb) return TNC_ERR_WORKSPACE;
    // Q overwrites the site: the QR reads its input into the workspace first
    prof.begin(0, st);
    if (int rc = tnc_qr(dt, rows, r, B.slot[i], r, B.slot[i], B.rbuf, B.fact, factb, B.info, st)) return rc;
    prof.end(0, st);
    double rn = 0.0;
    if (int rc = host_norm(dt, k * r, B.rbuf, B.dnorm, &rn, st)) return rc;
    if (int stq = device_status(B.info, st)) return stq;
    prof.add(0, qr_flops(rows, r, cplx));
    if (rn > 0) lnorm += std::log(rn);
    const int64_t r2 = sr[i + 1];  // sl[i + 1] == r
    if (int rc = gemm_any(dt, TNC_OP_N, TNC_OP_N, k, r2, r, rn > 0 ? 1.0 / rn : 1.0, B.rbuf, r, 0, B.slot[i + 1], r2,
                          r * r2, B.scratch, r2, k * r2, d, B.fact, factb, st))
      return rc;
    if (cudaMemcpyAsync(B.slot[i + 1], B.scratch, (size_t)d * k * r2 * sizeof(T), cudaMemcpyDeviceToDevice, st) !=
        cudaSuccess)
      return TNC_ERR_CUDA;
    sr[i] = k;
    sl[i + 1] = k;
  }
  {
    const int i = n_sites - 1;
    double last = 0.0;
    if (int rc = host_norm(dt, d * sl[i] * sr[i], B.slot[i], B.dnorm, &last, st)) return rc;
    if (!(last > 0.0)) return TNC_ERR_ARG;  // zero state
    if (int rc = scale(dt, d * sl[i] * sr[i], 1.0 / last, B.slot[i], st)) return rc;
    lnorm += std::log(last);
  }
  // 3. truncating SVD right sweep
  double norm_acc = 1.0;
  std::vector<R> s_host((size_t)P.max_kmin);
  std::vector<double> sd;  // the spectrum the truncation decision reads
  std::vector<int64_t> ord;  // the FP64 stage's row order
  for (int i = n_sites - 1; i >= 1; --i) {
    const int64_t l = sl[i], r = sr[i], m = d * r, n = l, kmin = m < n ? m : n;
    {  // M = P_i as (d, r, l)
      const int64_t shp[3] = {d, l, r};
      const int perm[3] = {0, 2, 1};
      if (int rc = tnc_permute(dt, B.slot[i], B.scratch, 3, shp, perm, 0, st)) return rc;
    }
    const void* M = B.scratch;
    const bool rows_path = m <= rows_limit(dt);
    // rows path: M's rows in decreasing-norm order (they are graded by the
    // previous bond's spectrum), a static column pivoting of the QR of M^H
    // that cuts the Jacobi's sweeps; U's rows are put back in order below
    if (rows_path) {
      if (int rc = tnc_sort_rows(dt, m, n, B.scratch, B.mpiv, B.porder, B.prank, B.pnorm2, st)) return rc;
      M = B.mpiv;
    }
    size_t xb = 0;
    if (tnc_qr_r_workspace_size(dt, m, n, 1, &xb) != TNC_OK || xb > factb) return TNC_ERR_WORKSPACE;
    prof.begin(1, st);
    if (int rc = tnc_qr_r(dt, m, n, M, 1, B.rbuf, B.fact, factb, B.info, st)) return rc;
    prof.end(1, st);
    if (int stq = device_status(B.info, st)) return stq;
    prof.add(1, qr_flops(n, m, cplx));
    prof.begin(2, st);
    const bool core_path = P.core64 && rows_path && m <= core_rows_limit(dt);
    if (rows_path) {
      if (tnc_svd_rows_workspace_size(dt, kmin, m, &xb) != TNC_OK || xb > factb) return TNC_ERR_WORKSPACE;
      if (int rc = tnc_svd_rows_stage(dt, kmin, m, B.rbuf, B.wbuf, B.S, B.order, core_path ? kCoreFp32Sweeps : 0,
                                      core_path ? kCoreFp32Tol : 0.0, core_path ? kCoreStopTol : 0.0, block_rows,
                                      B.fact, factb, B.info, st))
        return rc;
    } else {  // the accumulating SVD of R: its VH rows are U^H of M
      if (tnc_svd_workspace_size(dt, kmin, m, &xb) != TNC_OK || xb > factb) return TNC_ERR_WORKSPACE;
      if (int rc = tnc_svd(dt, kmin, m, B.rbuf, m, B.svbuf, B.S, B.wbuf, 0, 0.0, B.fact, factb, B.info, st))
        return rc;
    }
    prof.end(2, st);
    // the FP64 finish of the core (rows up to the FP64 register limit)
    if (core_path) {
      // an FP32 stage that stopped at its sweep cap hands over to the FP64 stage
      if (cudaMemcpyAsync(s_host.data(), B.S, (size_t)kmin * sizeof(R), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return TNC_ERR_CUDA;
      if (int stq = device_status(B.info, st); stq && stq != TNC_ERR_NOT_CONVERGED) return stq;
      prof.add(2, svd_flops(kmin, m, cplx));
      // rows in FP32-norm order, widened; only the rows that can be retained
      // (the FP32 rank plus a margin) need FP64 orthogonality to every row
      sd.assign(s_host.begin(), s_host.begin() + kmin);
      const int64_t k32 = rank_rule<double>(sd, chi, threshold, eps);
      int64_t nkeep = ((k32 + kCoreKeepMargin + 7) / 8) * 8;
      if (nkeep > kmin) nkeep = kmin;
      const int cdt = core_dtype(dt);
      const int64_t kall = kmin;
      if (cudaMemcpyAsync(B.kdev, &kall, sizeof(int64_t), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return TNC_ERR_CUDA;
      if (int rc = tnc_gather_rows(dt, B.wbuf, m, B.order, B.kdev, kmin, nullptr, 0, B.ubuf, st)) return rc;
      if (tnc_svd_rows_workspace_size(cdt, kmin, m, &xb) != TNC_OK || xb > factb) return TNC_ERR_WORKSPACE;
      double fp64_flops = 0.0;
      const double tol64 = core_tol > 0 ? core_tol : kCoreTol;
      for (int attempt = 0; attempt < 2; ++attempt) {
        if (P.core_df) {
          prof.begin(3, st);
          if (int rc = tnc_svd_rows_df(dt, kmin, m, B.ubuf, B.w64b, B.S64, B.order64, 0, tol64, block_rows, nkeep,
                                       B.fact, factb, B.info, st))
            return rc;
          prof.end(3, st);
        } else {
          if (int rc = tnc_cast(dt, cdt, kmin * m, B.ubuf, B.w64a, st)) return rc;
          prof.begin(3, st);
          if (int rc = tnc_svd_rows_keep(cdt, kmin, m, B.w64a, B.w64b, B.S64, B.order64, 0, tol64, block_rows,
                                         nkeep, B.fact, factb, B.info, st))
            return rc;
          prof.end(3, st);
        }
        sd.resize((size_t)kmin);
        if (cudaMemcpyAsync(sd.data(), B.S64, (size_t)kmin * sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess)
          return TNC_ERR_CUDA;
        ord.resize((size_t)kmin);
        if (cudaMemcpyAsync(ord.data(), B.order64, (size_t)kmin * sizeof(int64_t), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess)
          return TNC_ERR_CUDA;
        int hinfo[4] = {0, 0, 0, 0};
        if (cudaMemcpyAsync(hinfo, B.info, sizeof(hinfo), cudaMemcpyDeviceToHost, st) != cudaSuccess)
          return TNC_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return TNC_ERR_CUDA;
        if (hinfo[0]) return hinfo[0];
        {  // executed arithmetic: rotating sweeps, then the checking one unless the finish
           // stopped without it (info[3]) (pairs of kept rows); FP64 flops, or the FP32
           // operations of the double-float finish
          const double pairs = (double)kmin * kmin - (double)(kmin - nkeep) * (kmin - nkeep);
          const double nn = pairs * m, sweeps = hinfo[1] > 0 ? hinfo[1] : 1;
          const double rotating = hinfo[3] ? sweeps : sweeps - 1.0, checking = hinfo[3] ? 0.0 : 1.0;
          if (P.core_df) fp64_flops += (rotating * (cplx ? 44.0 : 15.0) + checking * (cplx ? 24.0 : 6.0)) * nn;
          else fp64_flops += (rotating * 14.0 + checking * 4.0) * nn / (cplx ? 1.0 : 3.0);
        }
        // the FP64 decision must retain only rows the FP64 stage finished
        const int64_t k64 = rank_rule<double>(sd, chi, threshold, eps);
        bool inside = true;
        for (int64_t j = 0; j < k64; ++j) inside = inside && ord[(size_t)j] < nkeep;
        if (inside || nkeep >= kmin) break;
        nkeep = kmin;  // rerun the whole finish
      }
      prof.add(3, fp64_flops);
    } else {
      if (cudaMemcpyAsync(s_host.data(), B.S, (size_t)kmin * sizeof(R), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return TNC_ERR_CUDA;
      if (int stq = device_status(B.info, st)) return stq;
      prof.add(2, svd_flops(kmin, m, cplx));
      sd.assign(s_host.begin(), s_host.begin() + kmin);
    }
    // the truncation decision (FP64 values with the FP64 core), capped at the
    // storage type's rounding-noise floor
    const int64_t k = rank_rule<double>(sd, chi, threshold, eps);
    const double smax = sd.empty() ? 0.0 : sd[0];
    if (!(smax > 0.0) || k < 1) return TNC_ERR_ARG;  // zero state
    if (out_discarded) {
      double tot = 0.0, dis = 0.0;
      for (int64_t j = 0; j < kmin; ++j) {
        tot += sd[j] * sd[j];
        if (j >= k) dis += sd[j] * sd[j];
      }
      out_discarded[i - 1] = tot > 0 ? dis / tot : 0.0;
    }
    // U (m x k)
    if (core_path) {
      const int cdt = core_dtype(dt);
      if (cudaMemcpyAsync(B.kdev, &k, sizeof(int64_t), cudaMemcpyHostToDevice, st) != cudaSuccess) return TNC_ERR_CUDA;
      if (int rc = tnc_gather_rows(cdt, B.w64b, m, B.order64, B.kdev, k, B.S64, 1, B.w64a, st)) return rc;
      if (int rc = tnc_cast(cdt, dt, m * k, B.w64a, B.ubuf, st)) return rc;
      if (cudaStreamSynchronize(st) != cudaSuccess) return TNC_ERR_CUDA;  // k lives on this frame
    } else if (rows_path) {
      if (cudaMemcpyAsync(B.kdev, &k, sizeof(int64_t), cudaMemcpyHostToDevice, st) != cudaSuccess) return TNC_ERR_CUDA;
      if (int rc = tnc_gather_rows(dt, B.wbuf, m, B.order, B.kdev, k, B.S, 1, B.ubuf, st)) return rc;
      if (cudaStreamSynchronize(st) != cudaSuccess) return TNC_ERR_CUDA;  // k lives on this frame
    } else {
      const int64_t shp[2] = {k, m};
      const int perm[2] = {1, 0};
      if (int rc = tnc_permute(dt, B.wbuf, B.ubuf, 2, shp, perm, 1, st)) return rc;
    }
    // S V^H = U^H M (k x n)
    if (int rc = gemm_any(dt, TNC_OP_C, TNC_OP_N, k, n, m, 1.0, B.ubuf, k, 0, M, n, 0, B.svbuf, n, 0, 1, B.fact, factb,
                          st))
      return rc;
    const void* U = B.ubuf;
    if (rows_path) {  // U's rows back in M's order (wbuf is free once U is formed)
      if (int rc = tnc_permute_rows(dt, m, k, B.ubuf, B.prank, B.wbuf, st)) return rc;
      U = B.wbuf;
    }
    {  // P_i = U as (d, r, k) -> (d, k, r)
      const int64_t shp[3] = {d, r, k};
      const int perm[3] = {0, 2, 1};
      if (int rc = tnc_permute(dt, U, B.slot[i], 3, shp, perm, 0, st)) return rc;
    }
    sl[i] = k;
    // P_{i-1} <- P_{i-1} (S V^H)^T / s_max  ((d lp) x k)
    const int64_t lp = sl[i - 1], rp = sr[i - 1];  // rp == l
    if (int rc = gemm_any(dt, TNC_OP_N, TNC_OP_T, d * lp, k, rp, 1.0 / smax, B.slot[i - 1], rp, 0, B.svbuf, n, 0,
                          B.scratch, k, 0, 1, B.fact, factb, st))
      return rc;
    if (cudaMemcpyAsync(B.slot[i - 1], B.scratch, (size_t)d * lp * k * sizeof(T), cudaMemcpyDeviceToDevice, st) !=
        cudaSuccess)
      return TNC_ERR_CUDA;
    sr[i - 1] = k;
    norm_acc *= smax;
  }
  // 4. the norm: s_max products into the first site; the QR sweep's factor too
  //    when it is representable in the storage type
  if (int rc = scale(dt, d * sl[0] * sr[0], norm_acc, B.slot[0], st)) return rc;
  const double lim = fp32_class(dt) ? 60.0 : 600.0;
  *folded = std::fabs(lnorm) <= lim ? 1 : 0;
  if (*folded) {
    if (int rc = scale(dt, d * sl[0] * sr[0], std::exp(lnorm), B.slot[0], st)) return rc;
  }
  *log_norm = lnorm + (norm_acc > 0 ? std::log(norm_acc) : 0.0);
  out_bonds[0] = sl[0];
  for (int i = 0; i < n_sites; ++i) {
    out_bonds[i + 1] = sr[i];
    out_offsets[i] = (int64_t)((char*)B.slot[i] - (char*)work);
  }
  return launch_status(0);
}

}  // namespace
}  // namespace tnc

using namespace tnc;

extern "C" int tnc_sweep_workspace_size(int dtype, int n_sites, int64_t d, const int64_t* mps_bonds,
                                        const int64_t* mpo_bonds, int core, size_t* bytes) {
  if (!elem_size(dtype) || n_sites < 2 || d <= 0 || !mps_bonds || !mpo_bonds || !bytes) return TNC_ERR_ARG;
  Dims P;
  if (int rc = plan(dtype, n_sites, d, mps_bonds, mpo_bonds, core, P)) return rc;
  Carve c{nullptr, 0};
  Buffers B;
  const size_t rs = (dtype == TNC_F32 || dtype == TNC_C64) ? 4 : 8;
  *bytes = carve(c, n_sites, d, P, (size_t)elem_size(dtype), rs, B) + kAlign;
  return TNC_OK;
}

extern "C" int tnc_sweep_apply_compress(int dtype, int n_sites, int64_t d, const void* const* sites,
                                        const int64_t* mps_bonds, const void* const* mpo, const int64_t* mpo_bonds,
                                        int64_t chi, double threshold, int block_rows, int core, double core_tol,
                                        void* work, size_t work_bytes, int64_t* out_bonds, int64_t* out_offsets,
                                        double* out_discarded, double* log_norm, int* folded, double* profile,
                                        void* stream) {
  if (n_sites < 2 || d <= 0 || !sites || !mps_bonds || !mpo || !mpo_bonds || !work || !out_bonds || !out_offsets ||
      !log_norm || !folded || chi < 0)
    return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return sweep_impl<T>(dtype, n_sites, d, sites, mps_bonds, mpo, mpo_bonds, chi, threshold, block_rows,
                                    core, core_tol, work, work_bytes, out_bonds, out_offsets, out_discarded, log_norm,
                                    folded, profile, st));
  return TNC_ERR_ARG;
}
