// Thin SVD (np.linalg.svd(full_matrices=False) in tensor_svd,
// tncontract/tensor.py:915, and its scipy gesvd retry, :916-929).
//
// One-sided (Hestenes) Jacobi on the ROWS of a working matrix W (nr x nr):
// pairs of rows are rotated until all rows are mutually orthogonal to within
// tol.  The rotations are accumulated into J (nr x nr, rows), so
//   W0 = J^H W,  W = D Y  (D = row norms, Y orthonormal rows).
// W0 is the triangular factor of a QR preconditioning step (svd_impl below
// says how U and VH of A follow from Y, D, J and Q).
//
// Parallel ordering: round-robin tournament over the rows (nr-1 rounds of
// nr/2 disjoint pairs per sweep), one warp per pair, the whole iteration in
// ONE cooperative persistent launch with a bounded grid barrier between
// rounds.  A sweep with no rotation ends the iteration (convergence); the
// number of sweeps is capped and reported.  Finally the rows are sorted by
// norm (descending, stable) and U, S, VH are written.
//
// Rotation for rows x (=w_p), y (=w_q): a=|x|^2, b=|y|^2, g=<x,y>=sum x conj(y),
// h=|g|, e=g/h, tau=(b-a)/(2h), t=sign(tau)/(|tau|+sqrt(1+tau^2)),
// c=1/sqrt(1+t^2), s=c t:   x' = c x - s e y,   y' = s conj(e) x + c y.
// This is the 2x2 Hermitian Jacobi rotation of the Gram matrix [[a,g],[g*,b]]
// (Golub & Van Loan, sec. 8.5 and 8.6.3), applied to rows.
#include "tnc_persist.cuh"

namespace tnc {

constexpr int kSvdWarps = 2;  // warps per CTA (spreads the pairs over many SMs)

template <typename T>
__device__ __forceinline__ void pair_indices(int64_t np, int64_t r, int64_t i, int64_t& p, int64_t& q) {
  const int64_t mod = np - 1;
  if (i == 0) { p = r; q = mod; }
  else { p = (r + i) % mod; q = (r - i + mod) % mod; }
}

template <typename T>
__global__ void __launch_bounds__(kSvdWarps * 32)
jacobi_kernel(T* W, T* J, int64_t nr, int64_t L, int max_sweeps, double tol, const double* frob2,
              unsigned* counters, SyncWords* sw, int* info) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * kSvdWarps + (threadIdx.x >> 5);
  const int64_t nwarps = (int64_t)gridDim.x * kSvdWarps;
  const int64_t np = nr + (nr & 1);
  const int64_t npairs = np / 2;
  const R rtol = (R)tol;
  const R noise2 = noise_floor2<T>(frob2);
  int sweep = 0;
  bool converged = false;
  unsigned last_rot = 0;
  for (; sweep < max_sweeps; ++sweep) {
    unsigned rot = 0;
    for (int64_t r = 0; r < np - 1; ++r) {
      for (int64_t pi = gw; pi < npairs; pi += nwarps) {
        int64_t p, q;
        pair_indices<T>(np, r, pi, p, q);
        if (p >= nr || q >= nr) continue;
        T* x = W + p * L;
        T* y = W + q * L;
        R a, b;
        T g;
        warp_pair_dots(x, y, L, a, b, g);
        const R h = abs_(g);
        // also skips NaN rows, rows at the rounding-noise floor and rows whose squared norm underflowed
        if (!(a > noise2 && b > noise2 && a > 0 && b > 0 && h > rtol * sqrt(a) * sqrt(b))) continue;
        const R tau = (b - a) / (2 * h);
        R t;
        if (fabs(tau) > (R)1e15) t = (R)0.5 / tau;
        else t = (tau >= 0 ? R(1) : R(-1)) / (fabs(tau) + sqrt(R(1) + tau * tau));
        const R c = R(1) / sqrt(R(1) + t * t);
        const R s = c * t;
        const T e = div_real_(g, h);
        const T se = s * e, sec = s * conj_(e);
        warp_pair_rotate(x, y, L, c, se, sec);
        if (J != nullptr) warp_pair_rotate(J + p * nr, J + q * nr, nr, c, se, sec);
        ++rot;
      }
      if (!grid_barrier(sw, gridDim.x)) return;
    }
    if (lane == 0 && rot) atomicAdd(&counters[sweep], rot);
    if (!grid_barrier(sw, gridDim.x)) return;
    last_rot = ld_volatile(&counters[sweep]);
    if (last_rot == 0) { converged = true; ++sweep; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (!converged) info[0] = TNC_ERR_NOT_CONVERGED;  // else keep the QR's status (OK or its timeout)
    info[1] = sweep;
    info[2] = (int)last_rot;
  }
}

// J = identity, W <- W0 (already in place)
template <typename T>
__global__ void eye_kernel(T* J, int64_t n) {
  const int64_t total = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / n, j = e - i * n;
    J[e] = (i == j) ? one_<T>() : zero_<T>();
  }
}

template <typename T>
__global__ void row_norms_kernel(const T* W, int64_t nr, int64_t L, typename traits<T>::real* D, int* info) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < nr; i += nw) {
    double acc = 0.0;
    for (int64_t k = lane; k < L; k += 32) acc += (double)abs2_(W[i * L + k]);
    acc = warp_sum(acc);
    if (lane == 0) {
      D[i] = (R)sqrt(acc);
      if (!isfinite(acc)) atomicExch(info, TNC_ERR_NONFINITE);
    }
  }
}

// pos[i] = #{j: D_j > D_i} + #{j < i: D_j == D_i}  (stable descending order)
template <typename R>
__global__ void rank_kernel(const R* D, int64_t n, int64_t* pos) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    R di = D[i];
    int64_t c = 0;
    for (int64_t j = 0; j < n; ++j) {
      R dj = D[j];
      c += (dj > di) || (dj == di && j < i);
    }
    pos[i] = c;
  }
}

// wide (W0 = A, nr = m, L = n):  U[r][pos_i] = conj(J[i][r]); VH[pos_i][:] = W[i][:]/D_i
// tall (W0 = A^H, nr = n, L = m): U[r][pos_i] = conj(W[i][r])/D_i; VH[pos_i][:] = J[i][:]
template <typename T>
__global__ void svd_output_kernel(const T* W, const T* J, const typename traits<T>::real* D, const int64_t* pos,
                                  int64_t nr, int64_t L, int tall, T* U, typename traits<T>::real* S, T* VH) {
  typedef typename traits<T>::real R;
  // part 1: rows of length L of W -> (wide) VH rows / (tall) U columns
  const int64_t t1 = nr * L;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < t1; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / L, r = e - i * L;
    R d = D[i];
    T v = W[e];
    T o = (d > R(0)) ? v * (R(1) / d) : zero_<T>();
    if (tall) U[r * nr + pos[i]] = conj_(o);
    else VH[pos[i] * L + r] = o;
    if (r == 0) S[pos[i]] = d;
  }
  // part 2: rows of J -> (wide) U columns / (tall) VH rows
  const int64_t t2 = nr * nr;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < t2; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / nr, r = e - i * nr;
    T v = J[e];
    if (tall) VH[pos[i] * nr + r] = v;
    else U[r * nr + pos[i]] = conj_(v);
  }
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct SvdLayout {
  size_t qr, w, j, d, frob2, pos, counters, sync, total;
};
static const int kMaxSweepsCap = 100;
// [QR workspace of X (L x nr): its transposed copy, reused for the small
//  output factor once R is out; tau; flags; Q^T] [W = R, nr x nr] [J] ...
static SvdLayout svd_layout(int64_t m, int64_t n, int dt, size_t es, size_t rs) {
  int64_t nr = m < n ? m : n, L = m < n ? n : m;
  SvdLayout Ly;
  size_t off = 0;
  Ly.qr = off; off = align256(off + qr_qt_workspace(L, nr, dt));
  Ly.w = off; off = align256(off + (size_t)nr * nr * es);
  Ly.j = off; off = align256(off + (size_t)nr * nr * es);
  Ly.d = off; off = align256(off + (size_t)nr * rs);
  Ly.frob2 = off; off = align256(off + sizeof(double));
  Ly.pos = off; off = align256(off + (size_t)nr * sizeof(int64_t));
  Ly.counters = off; off = align256(off + kMaxSweepsCap * sizeof(unsigned));
  Ly.sync = off; off = align256(off + sizeof(SyncWords));
  Ly.total = off;
  return Ly;
}

template <typename T> static int dtype_of();
template <> int dtype_of<float>() { return TNC_F32; }
template <> int dtype_of<double>() { return TNC_F64; }
template <> int dtype_of<c64>() { return TNC_C64; }
template <> int dtype_of<c128>() { return TNC_C128; }

// QR-preconditioned one-sided Jacobi (Drmac & Veselic 2008).  X is the
// matrix whose columns the Jacobi would orthogonalise (X = A^H for a wide A,
// X = A for a tall one; L x nr).  X = Q R, and the rows of R (nr x nr) are
// rotated until orthogonal while the rotations accumulate in J:
//   J R = D Y   =>   X = Q J^H D Y.
// Wide A = X^H = Y^H D J Q^H:  U = Y^H, S = D, VH = J Q^H.
// Tall A = X  = (Q J^H) D Y:   U = Q J^H, S = D, VH = Y.
// Both factors come out orthonormal for every singular value (the normalised
// rows Y and the accumulated J are unitary by construction), the Jacobi
// works on nr x nr instead of nr x L rows, and the triangular start needs far
// fewer sweeps on graded matrices than A itself.
template <typename T>
static int svd_impl(int64_t m, int64_t n, const T* A, int64_t lda, T* U, typename traits<T>::real* S, T* VH,
                    int max_sweeps, double tol, void* work, size_t wb, int* info, cudaStream_t st) {
  typedef typename traits<T>::real R;
  if (m <= 0 || n <= 0 || lda != n || !A || !U || !S || !VH || !work || !info) return TNC_ERR_ARG;
  SvdLayout Ly = svd_layout(m, n, dtype_of<T>(), sizeof(T), sizeof(R));
  if (wb < Ly.total) return TNC_ERR_WORKSPACE;
  if (max_sweeps <= 0) max_sweeps = 40;
  if (max_sweeps > kMaxSweepsCap) max_sweeps = kMaxSweepsCap;
  const int tall = m > n;
  const int64_t nr = tall ? n : m, L = tall ? m : n;
  if (tol <= 0) {
    double sl = sqrt((double)(nr > 8 ? nr : 8));
    tol = sl * traits<T>::eps * (sizeof(R) == 4 ? 4.0 : 1.0);
  }
  char* w = (char*)work;
  T* W = (T*)(w + Ly.w);
  T* J = (T*)(w + Ly.j);
  R* D = (R*)(w + Ly.d);
  int64_t* pos = (int64_t*)(w + Ly.pos);
  unsigned* counters = (unsigned*)(w + Ly.counters);
  SyncWords* sw = (SyncWords*)(w + Ly.sync);
  double* frob2 = (double*)(w + Ly.frob2);
  T* Qt = nullptr;
  // X = A^H (wide) or A (tall); R of X into W, Q^T (nr x L) kept in the QR workspace
  int s = qr_qt<T>(L, nr, A, tall ? 0 : 1, true, W, w + Ly.qr, qr_qt_workspace(L, nr, dtype_of<T>()), info, st, &Qt);
  if (s) return s;
  T* small = (T*)(w + Ly.qr);  // the QR's transposed copy (nr * L >= nr * nr elements) is free now
  eye_kernel<T><<<grid1d(nr * nr, 256), 256, 0, st>>>(J, nr);
  if (cudaMemsetAsync(counters, 0, kMaxSweepsCap * sizeof(unsigned), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(sw, 0, sizeof(SyncWords), st) != cudaSuccess) return TNC_ERR_CUDA;
  // info[0] holds the QR's status (a wait timeout) until the Jacobi writes its own
  if (cudaMemsetAsync(info + 1, 0, 3 * sizeof(int), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(frob2, 0, sizeof(double), st) != cudaSuccess) return TNC_ERR_CUDA;
  frob2_kernel<T><<<grid1d(nr * nr, 256, 152 * 4), 256, 0, st>>>(nr * nr, W, frob2);
  if (launch_status(2)) return TNC_ERR_CUDA;  // eye, frob2
  if (nr > 1) {
    const int threads = kSvdWarps * 32;
    int cap = coop_capacity((const void*)jacobi_kernel<T>, threads, 0);
    if (cap <= 0) return TNC_ERR_CUDA;
    int64_t npairs = (nr + 1) / 2;
    int64_t want = (npairs + kSvdWarps - 1) / kSvdWarps;
    int grid = (int)(want < cap ? want : cap);
    int64_t nr_ = nr, L_ = nr;
    int ms = max_sweeps;
    double tl = tol;
    void* args[] = {(void*)&W, (void*)&J, (void*)&nr_, (void*)&L_, (void*)&ms, (void*)&tl,
                    (void*)&frob2, (void*)&counters, (void*)&sw, (void*)&info};
    if (cudaLaunchCooperativeKernel((const void*)jacobi_kernel<T>, dim3(grid), dim3(threads), args, 0, st) !=
        cudaSuccess)
      return TNC_ERR_CUDA;
  }
  copy_sync_error<<<1, 1, 0, st>>>(sw, info);
  row_norms_kernel<T><<<grid1d(nr * 32, 256), 256, 0, st>>>(W, nr, nr, D, info);
  rank_kernel<R><<<grid1d(nr, 128), 128, 0, st>>>(D, nr, pos);
  // the square problem's factors: wide -> U = Y^H (out), J -> small; tall -> VH = Y (out), J^H -> small
  if (tall) svd_output_kernel<T><<<grid1d(nr * nr, 256), 256, 0, st>>>(W, J, D, pos, nr, nr, 0, small, S, VH);
  else svd_output_kernel<T><<<grid1d(nr * nr, 256), 256, 0, st>>>(W, J, D, pos, nr, nr, 1, U, S, small);
  if (launch_status(nr > 1 ? 4 : 3)) return TNC_ERR_CUDA;  // [jacobi], error copy, row norms, rank, output
  const T one = one_<T>(), zero = zero_<T>();
  if (tall)  // U (m x n) = Q (small) = (Q^T)^T small
    return gemm_launch<T>(TNC_OP_T, TNC_OP_N, L, nr, nr, one, Qt, L, 0, small, nr, 0, zero, U, nr, 0, 1, st);
  // VH (m x n) = small Q^H = small conj(Q^T)
  return gemm_launch<T>(TNC_OP_N, TNC_OP_R, nr, L, nr, one, small, nr, 0, Qt, L, 0, zero, VH, L, 0, 1, st);
}

TNC_DEFINE_SPIN_SETTER(spin_limit_set_svd)

}  // namespace tnc

using namespace tnc;

extern "C" int tnc_svd_workspace_size(int dtype, int64_t m, int64_t n, size_t* bytes) {
  int es = elem_size(dtype);
  if (!es || m <= 0 || n <= 0 || !bytes) return TNC_ERR_ARG;
  size_t rs = (dtype == TNC_F32 || dtype == TNC_C64) ? 4 : 8;
  *bytes = svd_layout(m, n, dtype, es, rs).total;
  return TNC_OK;
}

extern "C" int tnc_svd(int dtype, int64_t m, int64_t n, const void* A, int64_t lda, void* U, void* S, void* VH,
                       int max_sweeps, double tol, void* work, size_t work_bytes, int* info, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return svd_impl<T>(m, n, (const T*)A, lda, (T*)U, (typename traits<T>::real*)S, (T*)VH, max_sweeps,
                                  tol, work, work_bytes, info, st));
  return TNC_ERR_ARG;
}

// ---------------------------------------------------------------------------
// SVD without any device allocation by the caller.
//
// Some callers cannot hand this library a workspace: a plugin hosted inside
// another framework's process that owns the whole device-memory budget
// through its own allocator, or a service that reserves all its memory at
// start-up and forbids allocations afterwards.  For them the SVD below uses a
// fixed scratch area that lives in the library image itself (a file-scope
// __device__ array): every GPU that loads the library holds these bytes until
// the process exits, and no call allocates or frees device memory.
//
// Limit: a problem is accepted when its workspace, tnc_svd_workspace_size(
// dtype, m, n), fits in kNoAllocScratchBytes = 16 MiB: e.g. complex128 up to
// 450 x 450 or 433 x 512, complex64 / float64 up to 647 x 647 or 531 x 1024,
// float32 up to 931 x 931 (either orientation).  Larger problems are rejected
// with TNC_ERR_TOO_LARGE before anything is launched or written.
//
// All calls on a device share the one scratch area and it keeps whatever the
// previous call left there; the SVD initialises every part it reads (working
// copy, rotation accumulator, counters, barrier words) at the start of each
// call.  Calls whose work overlaps on the GPU (different streams, or
// different host threads without ordering) race on the shared scratch: order
// them on one stream.
//
// The device address of the scratch is looked up with the device current
// (cudaGetSymbolAddress) on the first call made on a device, and looked up
// again when that device's context is no longer the one the address was
// taken in (after cudaDeviceReset, or a primary context released and
// re-created, the library image is loaded anew at another address); make the
// first call on a device, and the first after such a reset, before any
// stream capture.
// ---------------------------------------------------------------------------
#include <cuda.h>

#include <mutex>

namespace tnc {

static constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_svd_scratch[kNoAllocScratchBytes];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);

// cuCtxGetCurrent through the runtime's driver entry point (no link-time
// dependency on the driver library)
static CtxGetCurrentFn ctx_get_current() {
  static std::once_flag once;
  static CtxGetCurrentFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}

struct NoallocSlot {
  CUcontext ctx;  // the context the address was looked up in
  void* ptr;
};
static std::mutex g_noalloc_mu;
static NoallocSlot g_noalloc[128] = {};  // per device ordinal

static int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
  if (dev < 0 || dev >= 128) return TNC_ERR_ARG;
  CtxGetCurrentFn get = ctx_get_current();
  if (!get) return TNC_ERR_CUDA;
  CUcontext ctx = nullptr;
  if (get(&ctx) != CUDA_SUCCESS) return TNC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (ctx == nullptr || g_noalloc[dev].ptr == nullptr || g_noalloc[dev].ctx != ctx) {
    void* p = nullptr;  // the lookup also makes the device's primary context current
    if (cudaGetSymbolAddress(&p, g_noalloc_svd_scratch) != cudaSuccess || p == nullptr) return TNC_ERR_CUDA;
    if (get(&ctx) != CUDA_SUCCESS || ctx == nullptr) return TNC_ERR_CUDA;
    g_noalloc[dev] = NoallocSlot{ctx, p};
  }
  *out = g_noalloc[dev].ptr;
  return TNC_OK;
}

}  // namespace tnc

extern "C" int tnc_svd_noalloc(int dtype, int64_t m, int64_t n, const void* A, int64_t lda, void* U, void* S,
                               void* VH, int max_sweeps, double tol, int* info, void* stream) {
  size_t need = 0;
  int s = tnc_svd_workspace_size(dtype, m, n, &need);
  if (s != TNC_OK) return s;
  if (need > tnc::kNoAllocScratchBytes) return TNC_ERR_TOO_LARGE;
  void* scratch = nullptr;
  s = tnc::noalloc_scratch(&scratch);
  if (s != TNC_OK) return s;
  return tnc_svd(dtype, m, n, A, lda, U, S, VH, max_sweeps, tol, scratch, tnc::kNoAllocScratchBytes, info, stream);
}
