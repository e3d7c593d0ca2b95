// Data-movement and small reduction kernels of the tncontract_gb300 C ABI:
// permute, scale/axpby/cast, norms and dots, trace, diagonal absorption,
// the truncation-rank decision and the fused MPO-MPS site product.
// All of these are HBM-bound: the kernels read and write each element once,
// with coalesced accesses on both sides.
#include "tnc_common.cuh"

namespace tnc {

unsigned long long g_tnc_launches = 0;

// ------------------------------------------------------------------ permute
struct PermParams {
  int rank;             // after merging, >= 1
  int64_t out_dims[8];  // output shape
  int64_t in_stride_of_out[8];  // input stride of output axis i
};

// Generic gather: one thread per output element (coalesced writes).
template <typename T, bool CONJ>
__global__ void permute_gather(const T* __restrict__ src, T* __restrict__ dst,
                               PermParams p, int64_t total) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = o, off = 0;
#pragma unroll 8
    for (int i = p.rank - 1; i >= 0; --i) {
      int64_t d = p.out_dims[i];
      int64_t q = rem / d;
      off += (rem - q * d) * p.in_stride_of_out[i];
      rem = q;
    }
    T v = src[off];
    dst[o] = CONJ ? conj_(v) : v;
  }
}

// Tiled transpose for permutations that move the input's innermost axis:
// a 32x32 tile is read along the input's fastest axis and written along the
// output's fastest axis through shared memory (both sides coalesced).
struct TileParams {
  int64_t dimA;        // size of the output-innermost axis (input axis a)
  int64_t dimB;        // size of the input-innermost axis (input axis b)
  int64_t in_strideA;  // input stride of axis a (axis b has stride 1)
  int64_t out_strideB; // output stride of axis b (axis a has stride 1)
  int nother;
  int64_t other_dims[8];
  int64_t other_in_stride[8];
  int64_t other_out_stride[8];
  int64_t nbatch;
};

template <typename T, bool CONJ>
__global__ void __launch_bounds__(256) permute_tiled(const T* __restrict__ src, T* __restrict__ dst, TileParams p) {
  __shared__ T tile[32][33];
  const int64_t tilesA = (p.dimA + 31) / 32;
  const int64_t tilesB = (p.dimB + 31) / 32;
  const int64_t ntiles = tilesA * tilesB * p.nbatch;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int64_t bi = t / (tilesA * tilesB);
    int64_t tr = t - bi * tilesA * tilesB;
    int64_t ta = tr / tilesB, tb = tr - ta * tilesB;
    int64_t in_off = 0, out_off = 0, rem = bi;
    for (int i = p.nother - 1; i >= 0; --i) {
      int64_t d = p.other_dims[i];
      int64_t q = rem / d;
      int64_t c = rem - q * d;
      in_off += c * p.other_in_stride[i];
      out_off += c * p.other_out_stride[i];
      rem = q;
    }
    const int64_t a0 = ta * 32, b0 = tb * 32;
    // read: rows indexed by a, contiguous along b
    for (int r = threadIdx.y; r < 32; r += 8) {
      int64_t a = a0 + r, b = b0 + threadIdx.x;
      if (a < p.dimA && b < p.dimB) tile[r][threadIdx.x] = src[in_off + a * p.in_strideA + b];
    }
    __syncthreads();
    // write: rows indexed by b, contiguous along a
    for (int r = threadIdx.y; r < 32; r += 8) {
      int64_t b = b0 + r, a = a0 + threadIdx.x;
      if (a < p.dimA && b < p.dimB) {
        T v = tile[threadIdx.x][r];
        dst[out_off + b * p.out_strideB + a] = CONJ ? conj_(v) : v;
      }
    }
    __syncthreads();
  }
}

template <typename T>
static int permute_impl(const T* src, T* dst, int rank, const int64_t* shape,
                        const int* perm, int conj, cudaStream_t st) {
  if (rank < 0 || rank > 8) return TNC_ERR_ARG;
  int64_t total = 1;
  for (int i = 0; i < rank; ++i) {
    if (shape[i] < 0) return TNC_ERR_ARG;
    total *= shape[i];
  }
  {  // perm must be a permutation of 0..rank-1
    int seen[8] = {0};
    for (int i = 0; i < rank; ++i) {
      if (perm[i] < 0 || perm[i] >= rank || seen[perm[i]]) return TNC_ERR_ARG;
      seen[perm[i]] = 1;
    }
  }
  if (total == 0) return TNC_OK;
  // input strides
  int64_t istr[8];
  {
    int64_t s = 1;
    for (int i = rank - 1; i >= 0; --i) { istr[i] = s; s *= shape[i]; }
  }
  // drop size-1 axes and merge output-adjacent axes that are input-adjacent
  int64_t od[8], os[8];  // output dims, input stride per output axis
  int r = 0;
  for (int i = 0; i < rank; ++i) {
    int ax = perm[i];
    if (shape[ax] == 1) continue;
    if (r > 0 && os[r - 1] == istr[ax] * shape[ax]) {
      od[r - 1] *= shape[ax];
      os[r - 1] = istr[ax];
    } else {
      od[r] = shape[ax];
      os[r] = istr[ax];
      ++r;
    }
  }
  if (r == 0) { od[0] = 1; os[0] = 1; r = 1; }
  const bool inner_kept = (os[r - 1] == 1);
  if (inner_kept && r == 1) {
    if (!conj || !traits<T>::is_complex) {
      return cudaMemcpyAsync(dst, src, total * sizeof(T), cudaMemcpyDeviceToDevice, st) == cudaSuccess
                 ? TNC_OK : TNC_ERR_CUDA;
    }
  }
  if (inner_kept || r == 1) {
    PermParams p;
    p.rank = r;
    for (int i = 0; i < r; ++i) { p.out_dims[i] = od[i]; p.in_stride_of_out[i] = os[i]; }
    unsigned g = grid1d(total, 256);
    if (conj) permute_gather<T, true><<<g, 256, 0, st>>>(src, dst, p, total);
    else permute_gather<T, false><<<g, 256, 0, st>>>(src, dst, p, total);
    return launch_status();
  }
  // tiled transpose: output axis r-1 (input stride os[r-1]) and the output
  // axis whose input stride is 1
  int pb = -1;
  for (int i = 0; i < r; ++i) if (os[i] == 1) pb = i;
  if (pb < 0) return TNC_ERR_ARG;
  int64_t ostr[8];
  {
    int64_t s = 1;
    for (int i = r - 1; i >= 0; --i) { ostr[i] = s; s *= od[i]; }
  }
  TileParams tp;
  tp.dimA = od[r - 1];
  tp.in_strideA = os[r - 1];
  tp.dimB = od[pb];
  tp.out_strideB = ostr[pb];
  tp.nother = 0;
  tp.nbatch = 1;
  for (int i = 0; i < r; ++i) {
    if (i == pb || i == r - 1) continue;
    tp.other_dims[tp.nother] = od[i];
    tp.other_in_stride[tp.nother] = os[i];
    tp.other_out_stride[tp.nother] = ostr[i];
    tp.nbatch *= od[i];
    tp.nother++;
  }
  int64_t ntiles = ((tp.dimA + 31) / 32) * ((tp.dimB + 31) / 32) * tp.nbatch;
  unsigned g = (unsigned)(ntiles < 152 * 16 ? ntiles : 152 * 16);
  dim3 blk(32, 8);
  if (conj) permute_tiled<T, true><<<g, blk, 0, st>>>(src, dst, tp);
  else permute_tiled<T, false><<<g, blk, 0, st>>>(src, dst, tp);
  return launch_status();
}

// ------------------------------------------------------------------ elementwise
template <typename T, bool CONJ>
__global__ void scale_kernel(int64_t n, T alpha, const T* __restrict__ x, T* y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T v = x[i];
    y[i] = alpha * (CONJ ? conj_(v) : v);
  }
}

template <typename T>
__global__ void axpby_kernel(int64_t n, T alpha, const T* __restrict__ x, T beta, T* y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = alpha * x[i] + beta * y[i];
}

template <typename S, typename D> __device__ inline D cvt(S s);
template <> __device__ inline float cvt<float, float>(float s) { return s; }
template <> __device__ inline double cvt<float, double>(float s) { return s; }
template <> __device__ inline c64 cvt<float, c64>(float s) { return c64(s, 0.f); }
template <> __device__ inline c128 cvt<float, c128>(float s) { return c128(s, 0.0); }
template <> __device__ inline float cvt<double, float>(double s) { return (float)s; }
template <> __device__ inline double cvt<double, double>(double s) { return s; }
template <> __device__ inline c64 cvt<double, c64>(double s) { return c64((float)s, 0.f); }
template <> __device__ inline c128 cvt<double, c128>(double s) { return c128(s, 0.0); }
template <> __device__ inline float cvt<c64, float>(c64 s) { return s.re; }
template <> __device__ inline double cvt<c64, double>(c64 s) { return s.re; }
template <> __device__ inline c64 cvt<c64, c64>(c64 s) { return s; }
template <> __device__ inline c128 cvt<c64, c128>(c64 s) { return c128(s.re, s.im); }
template <> __device__ inline float cvt<c128, float>(c128 s) { return (float)s.re; }
template <> __device__ inline double cvt<c128, double>(c128 s) { return s.re; }
template <> __device__ inline c64 cvt<c128, c64>(c128 s) { return c64((float)s.re, (float)s.im); }
template <> __device__ inline c128 cvt<c128, c128>(c128 s) { return s; }

template <typename S, typename D>
__global__ void cast_kernel(int64_t n, const S* __restrict__ x, D* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = cvt<S, D>(x[i]);
}

// sum |x|^2 in double, one atomic per block
template <typename T>
__global__ void sumsq_kernel(int64_t n, const T* __restrict__ x, double* out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)abs2_(x[i]);
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) atomicAdd(out, acc);
}

__global__ void sqrt_inplace(double* v) { v[0] = sqrt(v[0]); }

template <typename T>
__global__ void dot_kernel(int64_t n, const T* __restrict__ x, const T* __restrict__ y, int conj_x, double* out) {
  __shared__ double red[32];
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T a = x[i];
    if (conj_x) a = conj_(a);
    T p = a * y[i];
    if constexpr (traits<T>::is_complex) { re += (double)p.re; im += (double)p.im; }
    else { re += (double)p; }
  }
  re = block_sum(re, red);
  im = block_sum(im, red);
  if (threadIdx.x == 0) { atomicAdd(out, re); atomicAdd(out + 1, im); }
}

struct TraceParams {
  int nrest;
  int64_t rest_dims[8];
  int64_t rest_stride[8];
  int64_t diag_len, diag_stride;
};

template <typename T>
__global__ void trace_kernel(const T* __restrict__ src, T* __restrict__ dst, TraceParams p, int64_t total) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = o, off = 0;
    for (int i = p.nrest - 1; i >= 0; --i) {
      int64_t d = p.rest_dims[i];
      int64_t q = rem / d;
      off += (rem - q * d) * p.rest_stride[i];
      rem = q;
    }
    T acc = zero_<T>();
    for (int64_t k = 0; k < p.diag_len; ++k) acc += src[off + k * p.diag_stride];
    dst[o] = acc;
  }
}

template <typename T, bool ROWS>
__global__ void scale_rc_kernel(int64_t rows, int64_t cols, const typename traits<T>::real* __restrict__ d,
                                int mode, T* A, int64_t lda) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / cols, j = e - i * cols;
    typename traits<T>::real f = d[ROWS ? i : j];
    if (mode == 1) f = sqrt(f);
    else if (mode == 2) f = (f > 0) ? 1 / f : 0;
    else if (mode == 3) f = (f > 0) ? 1 / (f * f) : 0;
    A[i * lda + j] = A[i * lda + j] * f;
  }
}

// k = #{s_i > t} capped at chi; discarded = sum_{i>=k} s_i^2 (single block)
template <typename R>
__global__ void trunc_rank_kernel(int64_t n, const R* __restrict__ s, int64_t chi, double threshold,
                                  int relative, int64_t* kout, double* disc) {
  __shared__ double red[32];
  __shared__ double redc[32];
  double t = threshold;
  if (relative) t = (n > 0) ? threshold * (double)s[0] : 0.0;
  double cnt = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) cnt += ((double)s[i] > t) ? 1.0 : 0.0;
  cnt = block_sum(cnt, redc);
  int64_t k = (int64_t)(cnt + 0.5);
  if (chi > 0 && k > chi) k = chi;
  double acc = 0.0;
  for (int64_t i = k + threadIdx.x; i < n; i += blockDim.x) acc += (double)s[i] * (double)s[i];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) { *kout = k; *disc = acc; }
}

// out = sum_p A[p][l][r] * W[po][p][wl][wr] with the fused bond layout
template <typename T>
__global__ void mps_mpo_site_kernel(int64_t din, int64_t dout, int64_t chl, int64_t chr, int64_t Dl,
                                    int64_t Dr, const T* __restrict__ A, const T* __restrict__ W,
                                    T* __restrict__ out, int layout) {
  const int64_t L = chl * Dl, Rr = chr * Dr;
  const int64_t total = dout * L * Rr;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t po, li, ri;
    if (layout == 1) {  // (phys, left, right)
      po = e / (L * Rr);
      int64_t rem = e - po * L * Rr;
      li = rem / Rr;
      ri = rem - li * Rr;
    } else {            // (left, physout, right)
      li = e / (dout * Rr);
      int64_t rem = e - li * dout * Rr;
      po = rem / Rr;
      ri = rem - po * Rr;
    }
    const int64_t l = li / Dl, wl = li - l * Dl;
    const int64_t r = ri / Dr, wr = ri - r * Dr;
    T acc = zero_<T>();
    for (int64_t p = 0; p < din; ++p)
      fma_(acc, A[(p * chl + l) * chr + r], W[((po * din + p) * Dl + wl) * Dr + wr]);
    out[e] = acc;
  }
}

template <typename T>
__global__ void copy2d_kernel(int64_t rows, int64_t cols, const T* __restrict__ src, int64_t lds,
                              T* __restrict__ dst, int64_t ldd) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / cols, j = e - i * cols;
    dst[i * ldd + j] = src[i * lds + j];
  }
}

template <typename T>
__global__ void diag_matrix_kernel(int64_t n, const typename traits<T>::real* __restrict__ d, T* __restrict__ out) {
  const int64_t total = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / n, j = e - i * n;
    out[e] = (i == j) ? from_real<T>(d[i]) : zero_<T>();
  }
}

}  // namespace tnc

using namespace tnc;

extern "C" {

int tnc_abi_version(void) { return 1; }

unsigned long long tnc_kernel_launches(void) { return __atomic_load_n(&g_tnc_launches, __ATOMIC_RELAXED); }

const char* tnc_status_string(int s) {
  switch (s) {
    case TNC_OK: return "ok";
    case TNC_ERR_ARG: return "invalid argument";
    case TNC_ERR_NOT_CONVERGED: return "Jacobi SVD did not converge within the sweep cap";
    case TNC_ERR_NONFINITE: return "non-finite value in the input";
    case TNC_ERR_CUDA: return "CUDA error";
    case TNC_ERR_WORKSPACE: return "workspace too small";
    case TNC_ERR_TIMEOUT: return "device-side wait timed out";
    case TNC_ERR_TOO_LARGE: return "problem needs more than the fixed scratch of tnc_svd_noalloc (16 MiB)";
    default: return "unknown status";
  }
}

int tnc_permute(int dtype, const void* src, void* dst, int rank, const int64_t* shape, const int* perm,
                int conj, void* stream) {
  if ((!src || !dst) || (rank > 0 && (!shape || !perm))) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, return permute_impl<T>((const T*)src, (T*)dst, rank, shape, perm, conj, st));
  return TNC_ERR_ARG;
}

int tnc_scale(int dtype, int64_t n, const double* alpha, const void* x, void* y, int conj, void* stream) {
  if (n < 0 || !alpha) return TNC_ERR_ARG;
  if (n == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, {
    T a = from_pair<T>(alpha);
    if (conj) scale_kernel<T, true><<<grid1d(n, 256), 256, 0, st>>>(n, a, (const T*)x, (T*)y);
    else scale_kernel<T, false><<<grid1d(n, 256), 256, 0, st>>>(n, a, (const T*)x, (T*)y);
  });
  return launch_status();
}

int tnc_axpby(int dtype, int64_t n, const double* alpha, const void* x, const double* beta, void* y, void* stream) {
  if (n < 0 || !alpha || !beta) return TNC_ERR_ARG;
  if (n == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, {
    axpby_kernel<T><<<grid1d(n, 256), 256, 0, st>>>(n, from_pair<T>(alpha), (const T*)x, from_pair<T>(beta), (T*)y);
  });
  return launch_status();
}

int tnc_cast(int sd, int dd, int64_t n, const void* src, void* dst, void* stream) {
  if (n < 0) return TNC_ERR_ARG;
  if (n == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned g = grid1d(n, 256);
  TNC_DISPATCH(sd, S, { TNC_DISPATCH(dd, D, cast_kernel<S, D><<<g, 256, 0, st>>>(n, (const S*)src, (D*)dst)); });
  return launch_status();
}

int tnc_nrm2(int dtype, int64_t n, const void* x, double* out, void* stream) {
  if (n < 0 || !out) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, sizeof(double), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (n > 0) {
    TNC_DISPATCH(dtype, T, sumsq_kernel<T><<<grid1d(n, 256, 152 * 4), 256, 0, st>>>(n, (const T*)x, out));
  }
  sqrt_inplace<<<1, 1, 0, st>>>(out);
  return launch_status(n > 0 ? 2 : 1);
}

int tnc_dot(int dtype, int64_t n, const void* x, const void* y, int conj_x, double* out, void* stream) {
  if (n < 0 || !out) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, 2 * sizeof(double), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (n == 0) return TNC_OK;
  TNC_DISPATCH(dtype, T, dot_kernel<T><<<grid1d(n, 256, 152 * 4), 256, 0, st>>>(n, (const T*)x, (const T*)y, conj_x, out));
  return launch_status();
}

int tnc_trace(int dtype, int rank, const int64_t* shape, int a1, int a2, const void* src, void* dst, void* stream) {
  if (rank < 2 || rank > 8 || a1 == a2 || a1 < 0 || a2 < 0 || a1 >= rank || a2 >= rank) return TNC_ERR_ARG;
  if (shape[a1] != shape[a2]) return TNC_ERR_ARG;
  int64_t str[8];
  int64_t s = 1;
  for (int i = rank - 1; i >= 0; --i) { str[i] = s; s *= shape[i]; }
  TraceParams p;
  p.nrest = 0;
  int64_t total = 1;
  for (int i = 0; i < rank; ++i) {
    if (i == a1 || i == a2) continue;
    p.rest_dims[p.nrest] = shape[i];
    p.rest_stride[p.nrest] = str[i];
    total *= shape[i];
    p.nrest++;
  }
  p.diag_len = shape[a1];
  p.diag_stride = str[a1] + str[a2];
  if (total == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, trace_kernel<T><<<grid1d(total, 256), 256, 0, st>>>((const T*)src, (T*)dst, p, total));
  return launch_status();
}

int tnc_scale_rows(int dtype, int64_t rows, int64_t cols, const void* d, int mode, void* A, int64_t lda, void* stream) {
  if (rows < 0 || cols < 0 || lda < cols) return TNC_ERR_ARG;
  if (rows * cols == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, scale_rc_kernel<T, true><<<grid1d(rows * cols, 256), 256, 0, st>>>(
                             rows, cols, (const typename traits<T>::real*)d, mode, (T*)A, lda));
  return launch_status();
}

int tnc_scale_cols(int dtype, int64_t rows, int64_t cols, const void* d, int mode, void* A, int64_t lda, void* stream) {
  if (rows < 0 || cols < 0 || lda < cols) return TNC_ERR_ARG;
  if (rows * cols == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, scale_rc_kernel<T, false><<<grid1d(rows * cols, 256), 256, 0, st>>>(
                             rows, cols, (const typename traits<T>::real*)d, mode, (T*)A, lda));
  return launch_status();
}

int tnc_truncation_rank(int dtype, int64_t n, const void* S, int64_t chi, double threshold, int relative,
                        int64_t* k, double* discarded, void* stream) {
  if (n < 0 || !k || !discarded) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TNC_F32 || dtype == TNC_C64)
    trunc_rank_kernel<float><<<1, 256, 0, st>>>(n, (const float*)S, chi, threshold, relative, k, discarded);
  else if (dtype == TNC_F64 || dtype == TNC_C128)
    trunc_rank_kernel<double><<<1, 256, 0, st>>>(n, (const double*)S, chi, threshold, relative, k, discarded);
  else
    return TNC_ERR_ARG;
  return launch_status();
}

int tnc_copy2d(int dtype, int64_t rows, int64_t cols, const void* src, int64_t lds, void* dst, int64_t ldd,
               void* stream) {
  if (rows < 0 || cols < 0 || lds < cols || ldd < cols || !src || !dst) return TNC_ERR_ARG;
  if (rows * cols == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, copy2d_kernel<T><<<grid1d(rows * cols, 256), 256, 0, st>>>(
                             rows, cols, (const T*)src, lds, (T*)dst, ldd));
  return launch_status();
}

int tnc_diag_matrix(int dtype, int64_t n, const void* d, void* out, void* stream) {
  if (n < 0 || !d || !out) return TNC_ERR_ARG;
  if (n == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, diag_matrix_kernel<T><<<grid1d(n * n, 256), 256, 0, st>>>(
                             n, (const typename traits<T>::real*)d, (T*)out));
  return launch_status();
}

int tnc_mps_mpo_site(int dtype, int64_t din, int64_t dout, int64_t chl, int64_t chr, int64_t Dl, int64_t Dr,
                     const void* A, const void* W, void* out, int layout, void* stream) {
  if (din <= 0 || dout <= 0 || chl <= 0 || chr <= 0 || Dl <= 0 || Dr <= 0 || (layout != 0 && layout != 1))
    return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t total = dout * chl * Dl * chr * Dr;
  TNC_DISPATCH(dtype, T, mps_mpo_site_kernel<T><<<grid1d(total, 256), 256, 0, st>>>(
                             din, dout, chl, chr, Dl, Dr, (const T*)A, (const T*)W, (T*)out, layout));
  return launch_status();
}

}  // extern "C"
