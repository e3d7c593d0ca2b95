// Helpers for the persistent (cooperatively launched) factorisation kernels:
// a grid barrier and flag waits whose spins are bounded.  A wait that gives
// up records TNC_ERR_TIMEOUT in the shared error word and returns false; all
// CTAs then leave the kernel at their next wait, so no launch can hang.
#pragma once
#include "tnc_common.cuh"

#include <mutex>

namespace tnc {

// Polls a bounded wait makes before it gives up.  The default, roughly 2-4 s of
// polling at ~150 ns per iteration, is orders of magnitude above any
// legitimate wait (one Jacobi round or one Householder column step).  The
// value is a device variable of every translation unit that includes this
// header, set for the current device by tnc_set_spin_limit (tests shorten it
// to make a wait run out on purpose).
static __device__ long long g_spin_limit = kSpinLimitDefault;
__device__ __forceinline__ long long spin_limit() { return *(volatile long long*)&g_spin_limit; }

// Host side: sets this translation unit's copy on the current device.
#define TNC_DEFINE_SPIN_SETTER(name)                                                         \
  int name(long long polls) {                                                                \
    return cudaMemcpyToSymbol(g_spin_limit, &polls, sizeof(polls)) == cudaSuccess ? TNC_OK \
                                                                                   : TNC_ERR_CUDA; \
  }

struct SyncWords {
  unsigned count;  // grid barrier arrivals; the top bit is the phase
  unsigned gen;    // unused (keeps the layout of the zeroed words)
  int err;         // first error recorded by any CTA (0 = none)
  int pad;
};

__device__ __forceinline__ int ld_volatile(const int* p) { return *(volatile const int*)p; }
__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) { return *(volatile const unsigned*)p; }

// All CTAs of the grid; returns false if any CTA recorded an error.
// One atomic per CTA and barrier: CTA 0 adds 0x80000000 - (nblocks - 1), the
// others 1, so the arrivals of one barrier add exactly 0x80000000 and flip the
// top bit of `count` while leaving its low bits unchanged (partial sums stay
// below the flip until the last arrival).  The value the atomic returns tells
// each CTA the phase it waits to see flipped; `count` needs no reset.  A CTA
// that records an error never arrives, so a completed barrier implies no error
// before it; waiters poll the error word while they spin.
__device__ __forceinline__ bool grid_barrier(SyncWords* sw, unsigned nblocks) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned add = blockIdx.x == 0 ? 0x80000000u - (nblocks - 1u) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(&sw->count, add);
    // the CTA whose arrival flips the phase bit completed the barrier
    const bool last = (((old + add) ^ old) & 0x80000000u) != 0;
    long long spins = 0;
    const long long limit = spin_limit();
    while (!last && ((ld_volatile(&sw->count) ^ old) & 0x80000000u) == 0) {
      if (ld_volatile(&sw->err)) { ok = 0; break; }
      if (++spins > limit) { atomicCAS(&sw->err, 0, TNC_ERR_TIMEOUT); ok = 0; break; }
      __nanosleep(32);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// One warp waits until *flag != 0; returns false on error / timeout.
__device__ __forceinline__ bool warp_wait_flag(const int* flag, SyncWords* sw) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    long long spins = 0;
    const long long limit = spin_limit();
    while (ld_volatile(flag) == 0) {
      if (ld_volatile(&sw->err)) { ok = 0; break; }
      if (++spins > limit) { atomicCAS(&sw->err, 0, TNC_ERR_TIMEOUT); ok = 0; break; }
      __nanosleep(32);
    }
    __threadfence();
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

// L2-only loads/stores for data other CTAs write during the same launch.
template <typename T> __device__ __forceinline__ T ldcg(const T* p);
template <> __device__ __forceinline__ float ldcg<float>(const float* p) { return __ldcg(p); }
template <> __device__ __forceinline__ double ldcg<double>(const double* p) { return __ldcg(p); }
template <> __device__ __forceinline__ c64 ldcg<c64>(const c64* p) {
  float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return c64(v.x, v.y);
}
template <> __device__ __forceinline__ c128 ldcg<c128>(const c128* p) {
  double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return c128(v.x, v.y);
}
template <typename T> __device__ __forceinline__ void stcg(T* p, T v);
template <> __device__ __forceinline__ void stcg<float>(float* p, float v) { __stcg(p, v); }
template <> __device__ __forceinline__ void stcg<double>(double* p, double v) { __stcg(p, v); }
template <> __device__ __forceinline__ void stcg<c64>(c64* p, c64 v) {
  __stcg(reinterpret_cast<float2*>(p), make_float2(v.re, v.im));
}
template <> __device__ __forceinline__ void stcg<c128>(c128* p, c128 v) {
  __stcg(reinterpret_cast<double2*>(p), make_double2(v.re, v.im));
}

// ---------------------------------------------------------------- warp vector ops
// Vectors live in L2 (other CTAs update them between steps).  Each lane
// issues kChunk independent loads before using any of them, so a pass over a
// vector costs a few L2 round trips instead of one per element.
template <typename T> struct chunk { static constexpr int U = sizeof(T) >= 16 ? 4 : 8; };

// a = |x|^2, b = |y|^2, g = sum_k x_k conj(y_k) over one warp (all lanes get them)
template <typename T>
__device__ __forceinline__ void warp_pair_dots(const T* x, const T* y, int64_t L,
                                               typename traits<T>::real& a, typename traits<T>::real& b, T& g) {
  typedef typename traits<T>::real R;
  constexpr int U = chunk<T>::U;
  const int lane = threadIdx.x & 31;
  R a_ = 0, b_ = 0;
  T g_ = zero_<T>();
  for (int64_t base = 0; base < L; base += 32 * U) {
    T xv[U], yv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = base + u * 32 + lane;
      xv[u] = (k < L) ? ldcg(x + k) : zero_<T>();
      yv[u] = (k < L) ? ldcg(y + k) : zero_<T>();
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      a_ += abs2_(xv[u]);
      b_ += abs2_(yv[u]);
      fma_(g_, xv[u], conj_(yv[u]));
    }
  }
  a = warp_sum(a_);
  b = warp_sum(b_);
  g = warp_sum(g_);
}

// x' = c x - se y, y' = sec x + c y over one warp
template <typename T>
__device__ __forceinline__ void warp_pair_rotate(T* x, T* y, int64_t L, typename traits<T>::real c, T se, T sec) {
  constexpr int U = chunk<T>::U;
  const int lane = threadIdx.x & 31;
  for (int64_t base = 0; base < L; base += 32 * U) {
    T xv[U], yv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = base + u * 32 + lane;
      if (k < L) { xv[u] = ldcg(x + k); yv[u] = ldcg(y + k); }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = base + u * 32 + lane;
      if (k < L) {
        stcg(x + k, c * xv[u] - se * yv[u]);
        stcg(y + k, sec * xv[u] + c * yv[u]);
      }
    }
  }
}

// w = sum_{k >= c} conj(v_k) col_k with v_c = 1 (v in L2, col owned by the warp)
template <typename T>
__device__ __forceinline__ T warp_reflector_dot(const T* v, const T* col, int64_t c, int64_t m) {
  constexpr int U = chunk<T>::U;
  const int lane = threadIdx.x & 31;
  T w = (lane == 0) ? col[c] : zero_<T>();
  for (int64_t base = c + 1; base < m; base += 32 * U) {
    T vv[U], cv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = base + u * 32 + lane;
      vv[u] = (k < m) ? ldcg(v + k) : zero_<T>();
      cv[u] = (k < m) ? col[k] : zero_<T>();
    }
#pragma unroll
    for (int u = 0; u < U; ++u) fma_(w, conj_(vv[u]), cv[u]);
  }
  return warp_sum(w);
}

// col_k -= f v_k for k >= c (v_c = 1)
template <typename T>
__device__ __forceinline__ void warp_reflector_axpy(const T* v, T* col, T f, int64_t c, int64_t m) {
  constexpr int U = chunk<T>::U;
  const int lane = threadIdx.x & 31;
  if (lane == 0) col[c] = col[c] - f;
  for (int64_t base = c + 1; base < m; base += 32 * U) {
    T vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = base + u * 32 + lane;
      vv[u] = (k < m) ? ldcg(v + k) : zero_<T>();
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = base + u * 32 + lane;
      if (k < m) col[k] = col[k] - f * vv[u];
    }
  }
}

// info[0] = first error recorded by the persistent launch (0 = none)
static __global__ void copy_sync_error(const SyncWords* sw, int* info) {
  int e = sw->err;
  if (e) info[0] = e;
}

// out[0] += sum |x|^2 over n elements (double accumulation, one atomic per
// block; out zeroed by the caller).  The Jacobi kernels read it as the
// squared Frobenius norm, which their rotations preserve.
template <typename T>
static __global__ void frob2_kernel(int64_t n, const T* __restrict__ x, double* out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)abs2_(x[i]);
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) atomicAdd(out, acc);
}

// Squared row norm at or below which a row is rounding noise of a matrix with
// squared Frobenius norm f2: (eps |W|_F)^2.  Such rows take part in no
// rotation (their directions carry no information, and in FP32 their
// products fall into the denormal range where they lose all precision).
template <typename T>
__device__ __forceinline__ typename traits<T>::real noise_floor2(const double* f2) {
  return (typename traits<T>::real)(traits<T>::eps * traits<T>::eps * f2[0]);
}

// Largest co-resident grid for a cooperative launch of `kernel`; the answer
// is cached per (device, kernel, block size, shared memory), the occupancy
// query being host work on the launch path of every call.
inline int coop_capacity(const void* kernel, int threads, size_t smem) {
  struct Entry { const void* k; int threads, dev; size_t smem; int cap; };
  static Entry cache[256];
  static int used = 0;
  static std::mutex mu;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < used; ++i)
      if (cache[i].k == kernel && cache[i].threads == threads && cache[i].smem == smem && cache[i].dev == dev)
        return cache[i].cap;
  }
  int sms = 0, per = 0, coop = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess) return 0;
  const int cap = per * sms;
  std::lock_guard<std::mutex> lock(mu);
  if (used < 256) cache[used++] = Entry{kernel, threads, dev, smem, cap};
  return cap;
}

}  // namespace tnc
