// Jacobi stage of the sweep SVD (the truncating SVD of left_canonise,
// tncontract/onedim/onedim_core.py:317-343, as used by svd_compress and
// svd_compress_mps).
//
// The rows of W (W = A for a wide A, A^H for a tall one) are made mutually
// orthogonal by one-sided Jacobi rotations; the rotations are NOT
// accumulated.  A truncating sweep only needs the leading rows of the result
// (S V^H for a wide A, U^H S for a tall one) and recovers the other factor
// with one GEMM against A, so the rotation accumulator (a second n x n
// matrix streamed through every rotation) is dropped.
//
// Block ordering.  The rows are cut into half-blocks of h rows (h = warps per
// CTA).  Each sweep is:
//   phase 0 -- every half-block is loaded into shared memory by one CTA and
//              all pairs inside it are rotated (an h-point round-robin);
//   rounds  -- a round-robin tournament over the half-blocks; in each round a
//              CTA takes a half-block pair (P, Q), keeps the rows of P in
//              registers (warp i owns row i of P) and the rows of Q in shared
//              memory, and rotates every (P_i, Q_j) pair in h steps (step s:
//              warp i pairs with Q_{(i+s) mod h}).
// A task of one step (phase 0 or a round) waits only for the tasks of the
// previous step that wrote its two half-blocks (a step counter per
// half-block); one grid barrier per sweep closes it for the convergence test.
// That is 2n/h dependent steps per sweep instead of n for a point ordering,
// and each rotation streams its rows through registers and shared memory
// instead of L2.  One cooperative launch runs all sweeps; every wait is
// bounded (tnc_persist.cuh).
#include "tnc_persist.cuh"

#include <atomic>

namespace tnc {

__device__ __forceinline__ void circle_pair(int64_t np, int64_t r, int64_t i, int64_t& p, int64_t& q) {
  const int64_t mod = np - 1;
  if (i == 0) { p = r; q = mod; }
  else { p = (r + i) % mod; q = (r - i + mod) % mod; }
}

template <typename T>
struct Rot {
  typename traits<T>::real c, th;  // th = t |g|: the norms move to a - th, b + th
  T se, sec;
  bool apply;
};

// Jacobi rotation from the 2x2 Gram entries (see tnc_svd.cu for the formula)
template <typename T>
__device__ __forceinline__ Rot<T> make_rot(typename traits<T>::real a, typename traits<T>::real b, T g,
                                           typename traits<T>::real rtol, typename traits<T>::real noise2) {
  typedef typename traits<T>::real R;
  Rot<T> r;
  const R h = abs_(g);
  // rows at the rounding-noise floor (or whose squared norm underflowed) count as converged
  r.apply = (a > noise2) && (b > noise2) && (a > 0) && (b > 0) && (h > rtol * sqrt(a) * sqrt(b));
  if (!r.apply) { r.c = 1; r.th = 0; r.se = zero_<T>(); r.sec = zero_<T>(); return r; }
  const R tau = (b - a) / (2 * h);
  R t;
  if (fabs(tau) > (R)1e15) t = (R)0.5 / tau;
  else t = (tau >= 0 ? R(1) : R(-1)) / (fabs(tau) + sqrt(R(1) + tau * tau));
  r.c = R(1) / sqrt(R(1) + t * t);
  r.th = t * h;
  const R s = r.c * t;
  const R inv_h = R(1) / h;  // one division for both parts of e = g / |g|
  const T e = isfinite(inv_h) ? g * inv_h : div_real_(g, h);
  r.se = s * e;
  r.sec = s * conj_(e);
  return r;
}

// rows x (registers, MAXE per lane) and y (shared memory), one warp.  The
// squared norms a (of x) and *b (of y) are carried, not recomputed: only
// g = <x, y> is reduced, and a rotation moves them to a - t|g|, b + t|g|
// (exact in exact arithmetic; recomputed from the rows once per sweep).
template <typename T, int MAXE>
__device__ __forceinline__ bool rotate_reg_smem(T (&x)[MAXE], T* y, int64_t L, typename traits<T>::real rtol,
                                                typename traits<T>::real noise2, typename traits<T>::real& a,
                                                typename traits<T>::real* b) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  const int Li = (int)L;  // row length <= 32 * MAXE
  T g0 = zero_<T>(), g1 = zero_<T>();
  T yr[MAXE];  // the partner row stays in registers between the two passes
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    const int k = lane + 32 * u;
    yr[u] = (k < Li) ? y[k] : zero_<T>();
  }
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    if (u & 1) fma_(g1, x[u], conj_(yr[u]));
    else fma_(g0, x[u], conj_(yr[u]));
  }
  const T g = warp_sum(g0 + g1);
  const R bb = *b;
  const Rot<T> r = make_rot<T>(a, bb, g, rtol, noise2);
  if (!r.apply) return false;
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    const int k = lane + 32 * u;
    const T xv = x[u];
    x[u] = r.c * xv - r.se * yr[u];
    if (k < Li) y[k] = r.sec * xv + r.c * yr[u];
  }
  a = a - r.th;
  if (lane == 0) *b = bb + r.th;
  return true;
}

// rows x and y both in shared memory, one warp; squared norms *a, *b carried
template <typename T>
__device__ __forceinline__ bool rotate_smem_smem(T* x, T* y, int64_t L, typename traits<T>::real rtol,
                                                 typename traits<T>::real noise2, typename traits<T>::real* a,
                                                 typename traits<T>::real* b) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  T g0 = zero_<T>(), g1 = zero_<T>();
  int64_t k = lane;
  for (; k + 32 < L; k += 64) {
    fma_(g0, x[k], conj_(y[k]));
    fma_(g1, x[k + 32], conj_(y[k + 32]));
  }
  if (k < L) fma_(g0, x[k], conj_(y[k]));
  const T g = warp_sum(g0 + g1);
  const R aa = *a, bb = *b;
  const Rot<T> r = make_rot<T>(aa, bb, g, rtol, noise2);
  if (!r.apply) return false;
  for (int64_t kk = lane; kk < L; kk += 32) {
    const T xv = x[kk], yv = y[kk];
    x[kk] = r.c * xv - r.se * yv;
    y[kk] = r.sec * xv + r.c * yv;
  }
  __syncwarp();
  if (lane == 0) { *a = aa - r.th; *b = bb + r.th; }
  __syncwarp();
  return true;
}

// squared norm of one row (length L) by one warp, every lane gets it
template <typename T>
__device__ __forceinline__ typename traits<T>::real warp_row_norm2(const T* x, int64_t L) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  R a0 = 0, a1 = 0;
  int64_t k = lane;
  for (; k + 32 < L; k += 64) { a0 += abs2_(x[k]); a1 += abs2_(x[k + 32]); }
  if (k < L) a0 += abs2_(x[k]);
  return warp_sum(a0 + a1);
}

// cooperative copy of rows [row0, row0 + cnt) of W (row length L) to/from smem
template <typename T>
__device__ __forceinline__ void rows_to_smem(const T* W, int64_t row0, int cnt, int64_t L, T* s) {
  // 8 independent loads in flight per thread before any is stored
  constexpr int U = 8;
  const int64_t total = (int64_t)cnt * L;
  const T* src = W + row0 * L;
  for (int64_t base = 0; base < total; base += (int64_t)blockDim.x * U) {
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t e = base + (int64_t)u * blockDim.x + threadIdx.x;
      if (e < total) v[u] = ldcg(src + e);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t e = base + (int64_t)u * blockDim.x + threadIdx.x;
      if (e < total) s[e] = v[u];
    }
  }
}
template <typename T>
__device__ __forceinline__ void rows_from_smem(T* W, int64_t row0, int cnt, int64_t L, const T* s) {
  const int64_t total = (int64_t)cnt * L;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x) stcg(W + row0 * L + e, s[e]);
}

// Step counters of the half-blocks: ver[b] = steps completed on half-block b
// (phase 0 and the rounds, counted across sweeps).  The CTA that finished a
// step on P and Q publishes after its rows are stored; the CTA that takes them
// next waits for that, not for the whole grid.  Both are called by every
// thread of the CTA.
__device__ __forceinline__ void publish_steps(unsigned* ver, int64_t P, int64_t Q, unsigned value) {
  __syncthreads();  // every thread's rows and norms stored
  if (threadIdx.x == 0) {
    __threadfence();
    *(volatile unsigned*)(ver + P) = value;
    if (Q != P) *(volatile unsigned*)(ver + Q) = value;
  }
}

// Wait until P and Q have completed `target` steps; false on error / timeout.
__device__ __forceinline__ bool wait_steps(const unsigned* ver, int64_t P, int64_t Q, unsigned target,
                                           SyncWords* sw) {
  __shared__ int ok_s;
  if (threadIdx.x == 0) {
    int ok = 1;
    long long spins = 0;
    const long long limit = spin_limit();
    for (;;) {
      const unsigned a = ld_volatile(ver + P), b = ld_volatile(ver + Q);
      if (a >= target && b >= target) break;
      if (ld_volatile(&sw->err)) { ok = 0; break; }
      if (++spins > limit) { atomicCAS(&sw->err, 0, TNC_ERR_TIMEOUT); ok = 0; break; }
      __nanosleep(32);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  const int ok = ok_s;
  __syncthreads();  // ok_s is free for the next wait
  return ok != 0;
}

// FP32 rows of up to 512 elements in 256-thread CTAs are held to 128 registers
// so two CTAs fit on one SM: the kernel is latency-bound (8 warps, dependent
// rotation steps), and concurrent factorisations on other streams fill the
// second slot.  The bound costs a few spilled registers.
// FP64 rows (PREG = false) keep both half-blocks in shared memory and the
// kernel at 128 registers: its rotations are bound by the FP64 pipe (1.6 FMA a
// clock per SM on GB300, measured), not by shared-memory traffic, and the other
// half of the register file stays free for an FP32 kernel of another instance
// on the same SM (a register-resident FP64 row took all 255 registers a
// thread, so nothing else could share the SM).
template <typename T, int MAXE, int MAXT, bool PREG>
constexpr int jacobi_min_blocks() {
  return (!PREG || (MAXT == 256 && MAXE <= 16 && sizeof(typename traits<T>::real) == 4)) ? 2 : 1;
}

template <typename T, int MAXE, int MAXT, bool PREG>
__global__ void __launch_bounds__(MAXT, jacobi_min_blocks<T, MAXE, MAXT, PREG>())
jacobi_block_kernel(T* W, int64_t nr, int64_t L, int h, int max_sweeps, double tol, const double* frob2,
                    typename traits<T>::real* Dn, unsigned* counters, unsigned* ver, SyncWords* sw, int* info) {
  typedef typename traits<T>::real R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sB = reinterpret_cast<T*>(smem_raw);
  __shared__ R sn[32];   // squared norms of the shared-memory rows
  __shared__ R snA[32];  // ... of the P half-block when it is in shared memory too
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nb = (nr + h - 1) / h;
  const int64_t nbp = nb + (nb & 1);
  const int64_t ntask = nbp / 2;
  const R rtol = (R)tol;
  const R noise2 = noise_floor2<T>(frob2);
  int sweep = 0;
  bool converged = false;
  unsigned last_rot = 0;
  T x[PREG ? MAXE : 1];
  for (; sweep < max_sweeps; ++sweep) {
    unsigned rot = 0;
    // step index of this sweep's phase 0; a sweep is nbp steps (phase 0 and
    // nbp - 1 rounds).  The grid barrier that ends the previous sweep has
    // ordered every earlier step, so phase 0 waits for nothing.
    const unsigned g0 = (unsigned)sweep * (unsigned)nbp;
    // phase 0: pairs inside each half-block
    for (int64_t hb = blockIdx.x; hb < nb; hb += gridDim.x) {
      const int64_t row0 = hb * h;
      const int cnt = (int)((nr - row0) < h ? (nr - row0) : h);
      rows_to_smem(W, row0, cnt, L, sB);
      __syncthreads();
      // exact squared norms once per sweep (the rounds carry them)
      if (warp < cnt) {
        const R a = warp_row_norm2(sB + (int64_t)warp * L, L);
        if (lane == 0) sn[warp] = a;
      }
      __syncthreads();
      const int hp = h + (h & 1);
      for (int rr = 0; rr < hp - 1; ++rr) {
        if (warp < hp / 2) {
          int64_t p, q;
          circle_pair(hp, rr, warp, p, q);
          if (p < cnt && q < cnt)
            rot += rotate_smem_smem(sB + p * L, sB + q * L, L, rtol, noise2, &sn[p], &sn[q]) ? 1u : 0u;
        }
        __syncthreads();
      }
      rows_from_smem(W, row0, cnt, L, sB);
      if (threadIdx.x < cnt) stcg(Dn + row0 + threadIdx.x, sn[threadIdx.x]);
      publish_steps(ver, hb, hb, g0 + 1u);
    }
    // rounds over half-block pairs; a task waits only for the two tasks of
    // the previous step that wrote its half-blocks
    for (int64_t r = 0; r < nbp - 1; ++r) {
      const unsigned g = g0 + 1u + (unsigned)r;
      for (int64_t t = blockIdx.x; t < ntask; t += gridDim.x) {
        int64_t P, Q;
        circle_pair(nbp, r, t, P, Q);
        if (P >= nb || Q >= nb) {  // paired with the padding block: pass the real one on
          const int64_t Pr = P < nb ? P : Q;
          if (!wait_steps(ver, Pr, Pr, g, sw)) return;
          publish_steps(ver, Pr, Pr, g + 1u);
          continue;
        }
        if (!wait_steps(ver, P, Q, g, sw)) return;
        const int64_t q0 = Q * h;
        const int cntB = (int)((nr - q0) < h ? (nr - q0) : h);
        if constexpr (PREG) {
          const int64_t rowA = P * h + warp;
          const bool hasA = rowA < nr;
          R an = 0;
          if (hasA) {
#pragma unroll
            for (int u = 0; u < MAXE; ++u) {
              const int64_t k = lane + 32 * u;
              x[u] = (k < L) ? ldcg(W + rowA * L + k) : zero_<T>();
            }
            an = ldcg(Dn + rowA);
          }
          rows_to_smem(W, q0, cntB, L, sB);
          if (threadIdx.x < cntB) sn[threadIdx.x] = ldcg(Dn + q0 + threadIdx.x);
          __syncthreads();
          for (int s = 0; s < h; ++s) {
            const int j = (warp + s) % h;
            if (hasA && j < cntB)
              rot += rotate_reg_smem<T, MAXE>(x, sB + (int64_t)j * L, L, rtol, noise2, an, &sn[j]) ? 1u : 0u;
            __syncthreads();
          }
          if (hasA) {
#pragma unroll
            for (int u = 0; u < MAXE; ++u) {
              const int64_t k = lane + 32 * u;
              if (k < L) stcg(W + rowA * L + k, x[u]);
            }
            if (lane == 0) stcg(Dn + rowA, an);
          }
          rows_from_smem(W, q0, cntB, L, sB);
          if (threadIdx.x < cntB) stcg(Dn + q0 + threadIdx.x, sn[threadIdx.x]);
        } else {
          T* sA = sB + (int64_t)h * L;
          const int64_t p0 = P * h;
          const int cntA = (int)((nr - p0) < h ? (nr - p0) : h);
          rows_to_smem(W, p0, cntA, L, sA);
          rows_to_smem(W, q0, cntB, L, sB);
          if (threadIdx.x < cntA) snA[threadIdx.x] = ldcg(Dn + p0 + threadIdx.x);
          if (threadIdx.x < cntB) sn[threadIdx.x] = ldcg(Dn + q0 + threadIdx.x);
          __syncthreads();
          for (int s = 0; s < h; ++s) {
            const int j = (warp + s) % h;
            if (warp < cntA && j < cntB)
              rot += rotate_smem_smem(sA + (int64_t)warp * L, sB + (int64_t)j * L, L, rtol, noise2, &snA[warp],
                                      &sn[j])
                         ? 1u
                         : 0u;
            __syncthreads();
          }
          rows_from_smem(W, p0, cntA, L, sA);
          if (threadIdx.x < cntA) stcg(Dn + p0 + threadIdx.x, snA[threadIdx.x]);
          rows_from_smem(W, q0, cntB, L, sB);
          if (threadIdx.x < cntB) stcg(Dn + q0 + threadIdx.x, sn[threadIdx.x]);
        }
        publish_steps(ver, P, Q, g + 1u);
      }
    }
    if (lane == 0 && rot) atomicAdd(&counters[sweep], rot);
    if (!grid_barrier(sw, gridDim.x)) return;
    last_rot = ld_volatile(&counters[sweep]);
    if (last_rot == 0) { converged = true; ++sweep; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    info[0] = converged ? TNC_OK : TNC_ERR_NOT_CONVERGED;
    info[1] = sweep;
    info[2] = (int)last_rot;
  }
}

// D_i = |W_i| (double accumulation), non-finite check
template <typename T>
__global__ void rows_norm_kernel(const T* W, int64_t nr, int64_t L, typename traits<T>::real* D, int* info) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < nr; i += nw) {
    double acc = 0.0;
    for (int64_t k = lane; k < L; k += 32) acc += (double)abs2_(W[i * L + k]);
    acc = warp_sum(acc);
    if (lane == 0) {
      D[i] = (typename traits<T>::real)sqrt(acc);
      if (!isfinite(acc)) atomicExch(info, TNC_ERR_NONFINITE);
    }
  }
}

// order[pos] = i with pos = #{j: D_j > D_i} + #{j < i: D_j == D_i}; S[pos] = D_i
template <typename R>
__global__ void sort_desc_kernel(const R* D, int64_t n, int64_t* order, R* S) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const R di = D[i];
    int64_t c = 0;
    for (int64_t j = 0; j < n; ++j) {
      const R dj = D[j];
      c += (dj > di) || (dj == di && j < i);
    }
    order[c] = i;
    S[c] = di;
  }
}

// dst[i][:] = f(src[order[i]][:]) for i < k (k read on the device, capped by kmax)
//   mode 0: copy rows (dst k x L, ld L)
//   mode 1: dst[c][i] = conj(src[order[i]][c]) / S[i]   (dst L x k, ld = k)
template <typename T>
__global__ void gather_rows_kernel(const T* src, int64_t L, const int64_t* order, const int64_t* kdev, int64_t kmax,
                                   const typename traits<T>::real* S, int mode, T* dst) {
  int64_t k = *kdev;
  if (k > kmax) k = kmax;
  const int64_t total = k * L;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / L, c = e - i * L;
    const T v = src[order[i] * L + c];
    if (mode == 0) dst[i * L + c] = v;
    else {
      const typename traits<T>::real s = S[i];
      dst[c * k + i] = (s > 0) ? conj_(v) * (typename traits<T>::real(1) / s) : zero_<T>();
    }
  }
}

// Self-test of the bounded waits: one CTA waits on something nothing will
// complete -- a grid barrier expecting two CTAs (kind 0), a half-block step
// counter nobody publishes (kind 1), a flag nobody sets (kind 2) -- until the
// wait limit runs out, then reports the error word (TNC_ERR_TIMEOUT).
__global__ void wait_selftest_kernel(int kind, SyncWords* sw, unsigned* ver, int* flag, int* info) {
  if (kind == 0) {
    grid_barrier(sw, 2u);
  } else if (kind == 1) {
    wait_steps(ver, 0, 1, 1u, sw);
  } else if (threadIdx.x < 32) {
    warp_wait_flag(flag, sw);
  }
  __syncthreads();
  if (threadIdx.x == 0) info[0] = ld_volatile(&sw->err);
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct RowsLayout { size_t d, dn, frob2, counters, sync, total; };
static const int kRowsMaxSweeps = 100;
static RowsLayout rows_layout(int64_t nr, size_t rs) {
  RowsLayout Ly;
  size_t off = 0;
  Ly.d = off; off = align256(off + (size_t)nr * rs);
  Ly.dn = off; off = align256(off + (size_t)nr * rs);
  Ly.frob2 = off; off = align256(off + sizeof(double));
  // sweep rotation counters, then one step counter per half-block (<= nr)
  Ly.counters = off; off = align256(off + (kRowsMaxSweeps + (size_t)nr) * sizeof(unsigned));
  Ly.sync = off; off = align256(off + sizeof(SyncWords));
  Ly.total = off;
  return Ly;
}

template <typename T> static int dtype_code();
template <> int dtype_code<float>() { return TNC_F32; }
template <> int dtype_code<double>() { return TNC_F64; }
template <> int dtype_code<c64>() { return TNC_C64; }
template <> int dtype_code<c128>() { return TNC_C128; }

// Largest dynamic shared memory a half block may use; the kernel attribute is
// raised to it once per device (never lowered: concurrent callers with
// different row lengths share the setting).
static const size_t kMaxHalfBlockBytes = 200 * 1024;

template <typename T, int MAXE, int MAXT, bool PREG>
static int ensure_smem_attr() {
  static std::atomic<unsigned long long> done_mask{0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done_mask.load() & bit) return TNC_OK;
  if (cudaFuncSetAttribute((const void*)jacobi_block_kernel<T, MAXE, MAXT, PREG>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxHalfBlockBytes) != cudaSuccess)
    return TNC_ERR_CUDA;
  done_mask.fetch_or(bit);
  return TNC_OK;
}

template <typename T, int MAXE, int MAXT, bool PREG = true>
static int launch_block(T* W, int64_t nr, int64_t L, int h, int ms, double tol, const double* frob2,
                        typename traits<T>::real* Dn, unsigned* counters, SyncWords* sw, int* info, cudaStream_t st) {
  const size_t smem = (size_t)(PREG ? 1 : 2) * h * L * sizeof(T);
  const void* fn = (const void*)jacobi_block_kernel<T, MAXE, MAXT, PREG>;
  if (smem > kMaxHalfBlockBytes || 32 * h > MAXT) return TNC_ERR_ARG;
  if (int rc = ensure_smem_attr<T, MAXE, MAXT, PREG>()) return rc;
  const int threads = 32 * h;
  int cap = coop_capacity(fn, threads, smem);
  if (cap <= 0) return TNC_ERR_CUDA;
  const int64_t nb = (nr + h - 1) / h;
  const int64_t ntask = (nb + (nb & 1)) / 2;
  // one CTA per half-block pair: every CTA works in every round (phase 0
  // takes two half-blocks per CTA)
  int64_t want = ntask;
  if (want < 1) want = 1;
  int grid = (int)(want < cap ? want : cap);
  unsigned* ver = counters + kRowsMaxSweeps;
  int64_t nr_ = nr, L_ = L;
  int h_ = h, ms_ = ms;
  double tol_ = tol;
  void* args[] = {(void*)&W, (void*)&nr_, (void*)&L_, (void*)&h_, (void*)&ms_, (void*)&tol_,
                  (void*)&frob2, (void*)&Dn, (void*)&counters, (void*)&ver, (void*)&sw, (void*)&info};
  if (cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, smem, st) != cudaSuccess) return TNC_ERR_CUDA;
  return TNC_OK;
}

template <typename T>
static int svd_rows_impl(int64_t m, int64_t n, const T* A, T* W, typename traits<T>::real* S, int64_t* order,
                         int max_sweeps, double tol, int block_rows, void* work, size_t wb, int* info,
                         cudaStream_t st) {
  typedef typename traits<T>::real R;
  if (m <= 0 || n <= 0 || !A || !W || !S || !order || !work || !info) return TNC_ERR_ARG;
  const int tall = m > n;
  const int64_t nr = tall ? n : m, L = tall ? m : n;
  RowsLayout Ly = rows_layout(nr, sizeof(R));
  if (wb < Ly.total) return TNC_ERR_WORKSPACE;
  if (max_sweeps <= 0) max_sweeps = 40;
  if (max_sweeps > kRowsMaxSweeps) max_sweeps = kRowsMaxSweeps;
  if (tol <= 0) tol = sqrt((double)(L > 8 ? L : 8)) * traits<T>::eps * (sizeof(R) == 4 ? 4.0 : 1.0);
  char* w = (char*)work;
  R* D = (R*)(w + Ly.d);
  unsigned* counters = (unsigned*)(w + Ly.counters);
  SyncWords* sw = (SyncWords*)(w + Ly.sync);
  double* frob2 = (double*)(w + Ly.frob2);
  R* Dn = (R*)(w + Ly.dn);
  int s;
  if (tall) {
    int64_t shp[2] = {m, n};
    int perm[2] = {1, 0};
    s = tnc_permute(dtype_code<T>(), A, W, 2, shp, perm, 1, st);
  } else {
    s = cudaMemcpyAsync(W, A, (size_t)m * n * sizeof(T), cudaMemcpyDeviceToDevice, st) == cudaSuccess ? TNC_OK
                                                                                                      : TNC_ERR_CUDA;
  }
  if (s) return s;
  if (cudaMemsetAsync(counters, 0, (kRowsMaxSweeps + (size_t)nr) * sizeof(unsigned), st) != cudaSuccess)
    return TNC_ERR_CUDA;
  if (cudaMemsetAsync(sw, 0, sizeof(SyncWords), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(info, 0, 4 * sizeof(int), st) != cudaSuccess) return TNC_ERR_CUDA;
  int launched = 0;
  if (nr > 1) {
    if (cudaMemsetAsync(frob2, 0, sizeof(double), st) != cudaSuccess) return TNC_ERR_CUDA;
    frob2_kernel<T><<<grid1d(nr * L, 256, 152 * 4), 256, 0, st>>>(nr * L, W, frob2);
    ++launched;
    // half-block height: 16 rows (fewest barriers) when the shared-memory half
    // block and the register row fit, else smaller
    // (16: 512-thread CTAs, rows up to 512 and element types up to 8 bytes)
    int h = 8;
    if (block_rows == 2 || block_rows == 4 || block_rows == 8) h = block_rows;
    if (block_rows == 16 && L <= 512 && sizeof(T) <= 8) h = 16;
    while (h > 2 && (size_t)h * L * sizeof(T) > kMaxHalfBlockBytes) h >>= 1;
    while (h > 2 && h / 2 >= nr) h >>= 1;
    const bool big = sizeof(T) >= 16;
    int rc;
    if (sizeof(typename traits<T>::real) == 8 && L <= 512) {
      // FP64 rows: both half-blocks in shared memory (2 h L elements)
      if (h > 8) h = 8;
      while (h > 2 && (size_t)2 * h * L * sizeof(T) > kMaxHalfBlockBytes) h >>= 1;
      rc = launch_block<T, 1, 256, false>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, st);
    } else if (h == 16) {
      if constexpr (sizeof(T) <= 8) {
        if (L <= 256) rc = launch_block<T, 8, 512>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, st);
        else rc = launch_block<T, 16, 512>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, st);
      } else {
        return TNC_ERR_ARG;
      }
    } else if (L <= 256) {
      rc = launch_block<T, 8, 256>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, st);
    } else if (L <= 512) {
      rc = launch_block<T, 16, 256>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, st);
    } else if (L <= 1024 && !big) {
      if constexpr (sizeof(T) < 16) rc = launch_block<T, 32, 256>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, st);
      else return TNC_ERR_ARG;
    } else {
      return TNC_ERR_ARG;  // rows too long for the register-resident half block
    }
    if (rc) return rc;
    ++launched;
  }
  copy_sync_error<<<1, 1, 0, st>>>(sw, info);
  rows_norm_kernel<T><<<grid1d(nr * 32, 256), 256, 0, st>>>(W, nr, L, D, info);
  sort_desc_kernel<R><<<grid1d(nr, 128), 128, 0, st>>>(D, nr, order, S);
  return launch_status(3 + launched);
}

template <typename T>
static int gather_impl(const T* src, int64_t L, const int64_t* order, const int64_t* kdev, int64_t kmax,
                       const typename traits<T>::real* S, int mode, T* dst, cudaStream_t st) {
  if (L <= 0 || kmax < 0 || !src || !order || !kdev || !dst || (mode == 1 && !S)) return TNC_ERR_ARG;
  if (kmax == 0) return TNC_OK;
  gather_rows_kernel<T><<<grid1d(kmax * L, 256), 256, 0, st>>>(src, L, order, kdev, kmax, S, mode, dst);
  return launch_status();
}

TNC_DEFINE_SPIN_SETTER(spin_limit_set_rows)

}  // namespace tnc

using namespace tnc;

extern "C" int tnc_svd_rows_workspace_size(int dtype, int64_t m, int64_t n, size_t* bytes) {
  if (!elem_size(dtype) || m <= 0 || n <= 0 || !bytes) return TNC_ERR_ARG;
  size_t rs = (dtype == TNC_F32 || dtype == TNC_C64) ? 4 : 8;
  *bytes = rows_layout(m < n ? m : n, rs).total;
  return TNC_OK;
}

extern "C" int tnc_svd_rows(int dtype, int64_t m, int64_t n, const void* A, void* W, void* S, int64_t* order,
                            int max_sweeps, double tol, int block_rows, void* work, size_t work_bytes, int* info,
                            void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return svd_rows_impl<T>(m, n, (const T*)A, (T*)W, (typename traits<T>::real*)S, order, max_sweeps,
                                       tol, block_rows, work, work_bytes, info, st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_gather_rows(int dtype, const void* src, int64_t L, const int64_t* order, const int64_t* k,
                               int64_t kmax, const void* S, int mode, void* dst, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return gather_impl<T>((const T*)src, L, order, k, kmax, (const typename traits<T>::real*)S, mode,
                                     (T*)dst, st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_set_spin_limit(long long polls) {
  if (polls <= 0) polls = kSpinLimitDefault;
  if (int rc = spin_limit_set_qr(polls)) return rc;
  if (int rc = spin_limit_set_svd(polls)) return rc;
  if (int rc = spin_limit_set_rows(polls)) return rc;
  return spin_limit_set_tc(polls);
}

extern "C" int tnc_wait_selftest(int kind, void* work, size_t work_bytes, int* info, void* stream) {
  if (kind < 0 || kind > 2 || !work || !info || work_bytes < 256) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = (char*)work;
  SyncWords* sw = (SyncWords*)w;
  unsigned* ver = (unsigned*)(w + 64);
  int* flag = (int*)(w + 128);
  if (cudaMemsetAsync(work, 0, 256, st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(info, 0, sizeof(int), st) != cudaSuccess) return TNC_ERR_CUDA;
  wait_selftest_kernel<<<1, 64, 0, st>>>(kind, sw, ver, flag, info);
  return launch_status(1);
}
