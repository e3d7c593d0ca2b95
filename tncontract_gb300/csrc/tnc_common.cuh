// Shared definitions for the tncontract_gb300 CUDA library (sm_103a).
//
// Element types mirror the dtypes the reference preserves end to end
// (float32, float64, complex64, complex128): a tensor keeps its dtype through
// every contraction and factorisation (tncontract/tensor.py:48-55, 735, 915).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/tncontract_gb300.h"

namespace tnc {

// Default poll count of every bounded device-side wait (tnc_persist.cuh and the
// tensor-core GEMM's mbarrier waits); tnc_set_spin_limit changes it at run time.
constexpr long long kSpinLimitDefault = 1LL << 24;
// Per-translation-unit setters of the wait limit on the current device (each
// unit that spins keeps its own device copy of the limit).
int spin_limit_set_qr(long long polls);
int spin_limit_set_svd(long long polls);
int spin_limit_set_rows(long long polls);
int spin_limit_set_tc(long long polls);

// ---------------------------------------------------------------- complex
template <typename R>
struct __align__(2 * sizeof(R)) cplx {
  R re, im;
  cplx() = default;
  __host__ __device__ cplx(R r, R i = 0) : re(r), im(i) {}
};

template <typename R> __host__ __device__ inline cplx<R> operator+(cplx<R> a, cplx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator-(cplx<R> a, cplx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator-(cplx<R> a) { return {-a.re, -a.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, cplx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R> __host__ __device__ inline cplx<R> operator*(R s, cplx<R> a) { return {s * a.re, s * a.im}; }
template <typename R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, R s) { return {s * a.re, s * a.im}; }
template <typename R> __host__ __device__ inline cplx<R>& operator+=(cplx<R>& a, cplx<R> b) { a.re += b.re; a.im += b.im; return a; }
template <typename R> __host__ __device__ inline cplx<R>& operator-=(cplx<R>& a, cplx<R> b) { a.re -= b.re; a.im -= b.im; return a; }

// ---------------------------------------------------------------- traits
template <typename T> struct traits;
template <> struct traits<float> {
  typedef float real; static const bool is_complex = false;
  static constexpr double eps = 1.1920928955078125e-07;
};
template <> struct traits<double> {
  typedef double real; static const bool is_complex = false;
  static constexpr double eps = 2.220446049250313e-16;
};
template <> struct traits<cplx<float>> {
  typedef float real; static const bool is_complex = true;
  static constexpr double eps = 1.1920928955078125e-07;
};
template <> struct traits<cplx<double>> {
  typedef double real; static const bool is_complex = true;
  static constexpr double eps = 2.220446049250313e-16;
};

typedef cplx<float> c64;
typedef cplx<double> c128;

// Uniform scalar helpers so kernels are written once for real and complex.
__host__ __device__ inline float conj_(float x) { return x; }
__host__ __device__ inline double conj_(double x) { return x; }
template <typename R> __host__ __device__ inline cplx<R> conj_(cplx<R> a) { return {a.re, -a.im}; }

__host__ __device__ inline float abs2_(float x) { return x * x; }
__host__ __device__ inline double abs2_(double x) { return x * x; }
template <typename R> __host__ __device__ inline R abs2_(cplx<R> a) { return a.re * a.re + a.im * a.im; }
// |x| without squaring (x*x underflows for |x| below ~1e-19 in FP32)
__device__ __forceinline__ float abs_(float x) { return fabsf(x); }
__device__ __forceinline__ double abs_(double x) { return fabs(x); }
__device__ __forceinline__ float abs_(cplx<float> a) { return hypotf(a.re, a.im); }
__device__ __forceinline__ double abs_(cplx<double> a) { return hypot(a.re, a.im); }
// x / h for real h (a division, so a denormal h does not overflow 1/h)
__device__ __forceinline__ float div_real_(float x, float h) { return x / h; }
__device__ __forceinline__ double div_real_(double x, double h) { return x / h; }
template <typename R> __device__ __forceinline__ cplx<R> div_real_(cplx<R> x, R h) { return {x.re / h, x.im / h}; }

__host__ __device__ inline float real_(float x) { return x; }
__host__ __device__ inline double real_(double x) { return x; }
template <typename R> __host__ __device__ inline R real_(cplx<R> a) { return a.re; }

template <typename T> __host__ __device__ inline T zero_() { return T(0); }
template <typename T> __host__ __device__ inline T one_() { return T(1); }

// fused multiply-add c += a*b (real: one FMA; complex: four)
__device__ __forceinline__ void fma_(float& c, float a, float b) { c = fmaf(a, b, c); }
__device__ __forceinline__ void fma_(double& c, double a, double b) { c = fma(a, b, c); }
template <typename R>
__device__ __forceinline__ void fma_(cplx<R>& c, cplx<R> a, cplx<R> b) {
  c.re = fma(a.re, b.re, c.re); c.re = fma(-a.im, b.im, c.re);
  c.im = fma(a.re, b.im, c.im); c.im = fma(a.im, b.re, c.im);
}

// scalar from the C-ABI's (re, im) double pair
template <typename T> __host__ __device__ inline T from_pair(const double* p);
template <> __host__ __device__ inline float from_pair<float>(const double* p) { return (float)p[0]; }
template <> __host__ __device__ inline double from_pair<double>(const double* p) { return p[0]; }
template <> __host__ __device__ inline c64 from_pair<c64>(const double* p) { return c64((float)p[0], (float)p[1]); }
template <> __host__ __device__ inline c128 from_pair<c128>(const double* p) { return c128(p[0], p[1]); }

template <typename T> __host__ __device__ inline T from_real(typename traits<T>::real r) { return T(r); }

// ---------------------------------------------------------------- warp/block reductions
template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename R>
__device__ __forceinline__ cplx<R> warp_sum(cplx<R> v) {
  v.re = warp_sum(v.re);
  v.im = warp_sum(v.im);
  return v;
}

// Block-wide sum; every thread gets the result.  `scratch` holds >= 32 R.
template <typename R>
__device__ __forceinline__ R block_sum(R v, R* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  R t = (threadIdx.x < nw) ? scratch[threadIdx.x] : R(0);
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  R r = scratch[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- dispatch
#define TNC_DISPATCH(dtype, T, ...)                              \
  switch (dtype) {                                               \
    case TNC_F32: { typedef float T; __VA_ARGS__; break; }       \
    case TNC_F64: { typedef double T; __VA_ARGS__; break; }      \
    case TNC_C64: { typedef tnc::c64 T; __VA_ARGS__; break; }    \
    case TNC_C128: { typedef tnc::c128 T; __VA_ARGS__; break; }  \
    default: return TNC_ERR_ARG;                                 \
  }

inline int elem_size(int dtype) {
  switch (dtype) {
    case TNC_F32: return 4;
    case TNC_F64: return 8;
    case TNC_C64: return 8;
    case TNC_C128: return 16;
    default: return 0;
  }
}

// Number of kernels this library has launched (tnc_kernel_launches()).
extern unsigned long long g_tnc_launches;

// Record `n` kernel launches just issued and report the launch status.
inline int launch_status(int n = 1) {
  __atomic_fetch_add(&g_tnc_launches, (unsigned long long)n, __ATOMIC_RELAXED);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TNC_OK : TNC_ERR_CUDA;
}

inline unsigned grid1d(int64_t n, int threads, int64_t cap = 152 * 32) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// -------- internal (C++) entry points shared between translation units
template <typename T>
int gemm_launch(int opA, int opB, int64_t m, int64_t n, int64_t k, T alpha,
                const T* A, int64_t lda, int64_t sA, const T* B, int64_t ldb,
                int64_t sB, T beta, T* C, int64_t ldc, int64_t sC,
                int64_t batch, cudaStream_t st);

// Householder QR of X (fm x fn): X = A (adjoint = 0, A dense fm x fn) or
// X = A^H (adjoint = 1, A dense fn x fm).  Writes R (min(fm,fn) x fn); with
// want_qt also forms Q^T (min(fm,fn) x fm, row-major) inside the workspace
// and returns its address in *qt.  Workspace: qr_qt_workspace(fm, fn, dtype).
size_t qr_qt_workspace(int64_t fm, int64_t fn, int dtype);
template <typename T>
int qr_qt(int64_t fm, int64_t fn, const T* A, int adjoint, bool want_qt, T* R, void* work, size_t wb, int* info,
          cudaStream_t st, T** qt);

}  // namespace tnc
