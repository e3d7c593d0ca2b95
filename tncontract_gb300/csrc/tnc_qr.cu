// Reduced QR (np.linalg.qr(mode="reduced") in tensor_qr, tncontract/tensor.py:1044).
//
// Householder QR in LAPACK's convention (geqrf + ungqr: Q = H_0 ... H_{k-1},
// H_c = I - tau_c v_c v_c^H, v_c[c] = 1, R's diagonal real for complex input),
// run as ONE cooperative persistent launch organised as a column-owner
// dataflow: every column of A is owned by one warp; reflector c is published
// (with a flag) by the owner of column c as soon as reflectors 0..c-1 have
// been applied to that column, and each warp applies the published
// reflectors to its own columns in order.  The owner of column c+1 applies
// reflector c to that column first and publishes reflector c+1 before
// touching its other columns (look-ahead), which keeps the critical path at
// one column update + one reflector per step.  No grid-wide barrier is needed.
//
// Working layout: Bt = A^T (row c of Bt is column c of A, contiguous), so
// every warp streams its own column and the published reflector with
// coalesced loads.  Q is formed by backward accumulation, each warp applying
// H_{min(j,k-1)} ... H_0 to its own column e_j -- independent across warps.
#include "tnc_persist.cuh"

#include <atomic>

namespace tnc {

constexpr int kQrWarps = 4;  // warps per CTA

template <typename T>
__device__ __forceinline__ T div_(T a, T b);
template <> __device__ __forceinline__ float div_(float a, float b) { return a / b; }
template <> __device__ __forceinline__ double div_(double a, double b) { return a / b; }
template <typename R>
__device__ __forceinline__ cplx<R> div_c(cplx<R> a, cplx<R> b) {
  R d = b.re * b.re + b.im * b.im;
  return cplx<R>((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
template <> __device__ __forceinline__ c64 div_(c64 a, c64 b) { return div_c(a, b); }
template <> __device__ __forceinline__ c128 div_(c128 a, c128 b) { return div_c(a, b); }

// CTA-local barrier over the first `count` threads' warps (count a multiple of
// 32), id 1..15 (0 is __syncthreads)
__device__ __forceinline__ void named_barrier(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

template <typename T> __device__ __forceinline__ typename traits<T>::real imag_(T v) {
  if constexpr (traits<T>::is_complex) return v.im; else return 0;
}

// Reflector for column c (row c of Bt), LAPACK larfg convention.
template <typename T>
__device__ void make_reflector(T* col, int64_t c, int64_t m, T* tau_out) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  R xn = 0;
  for (int64_t i = c + 1 + lane; i < m; i += 32) xn += abs2_(col[i]);
  xn = warp_sum(xn);
  T alpha = col[c];
  T tau = zero_<T>();
  if (!(xn == R(0) && imag_(alpha) == R(0))) {
    R ar = real_(alpha);
    R beta = -copysign(sqrt(abs2_(alpha) + xn), ar);
    T betaT = from_real<T>(beta);
    tau = div_(betaT - alpha, betaT);
    T scal = div_(one_<T>(), alpha - betaT);
    for (int64_t i = c + 1 + lane; i < m; i += 32) col[i] = scal * col[i];
    __syncwarp();
    if (lane == 0) col[c] = betaT;
  }
  if (lane == 0) *tau_out = tau;
  __syncwarp();
}

// col[i] -= conj(tau) * (v^H col) * v[i], i >= c  (applies H_c^H)
template <typename T>
__device__ __forceinline__ void apply_reflector_h(T* col, const T* v, T tau, int64_t c, int64_t m) {
  const T w = warp_reflector_dot(v, col, c, m);
  __syncwarp();
  warp_reflector_axpy(v, col, conj_(tau) * w, c, m);
  __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(kQrWarps * 32)
qr_factor_kernel(T* Bt, int64_t m, int64_t n, int64_t ld, T* tau, int* flags, SyncWords* sw) {
  const int64_t k = m < n ? m : n;
  const int64_t nwarps = (int64_t)gridDim.x * kQrWarps;
  const int64_t wid = (int64_t)blockIdx.x * kQrWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (wid >= n) return;
  // my columns: wid, wid + nwarps, ...
  if (wid == 0) {  // column 0 needs no earlier reflector
    make_reflector(Bt, 0, m, tau);
    __threadfence();
    if (lane == 0) atomicExch(&flags[0], 1);
  }
  int64_t first = wid;  // first own column not yet past all reflectors
  for (int64_t c = 0; c < k; ++c) {
    // skip own columns <= c: they are final (their reflector is published)
    while (first <= c) first += nwarps;
    if (first >= n) break;  // nothing left to update
    if (!warp_wait_flag(&flags[c], sw)) return;
    const T* v = Bt + c * ld;
    const T tc = ldcg(tau + c);
    for (int64_t j = first; j < n; j += nwarps) {
      apply_reflector_h(Bt + j * ld, v, tc, c, m);
      if (j == c + 1 && j < k) {  // look-ahead: publish the next reflector now
        make_reflector(Bt + j * ld, j, m, tau + j);
        __threadfence();
        if (lane == 0) atomicExch(&flags[j], 1);
      }
    }
  }
}

// Qt[j] = H_{min(j,k-1)} ... H_0 e_j  (row j of Qt = column j of Q)
template <typename T>
__global__ void __launch_bounds__(kQrWarps * 32)
qr_form_q_kernel(const T* __restrict__ Bt, int64_t m, int64_t k, const T* __restrict__ tau, T* __restrict__ Qt) {
  const int64_t nwarps = (int64_t)gridDim.x * kQrWarps;
  const int lane = threadIdx.x & 31;
  for (int64_t j = (int64_t)blockIdx.x * kQrWarps + (threadIdx.x >> 5); j < k; j += nwarps) {
    T* q = Qt + j * m;
    for (int64_t i = lane; i < m; i += 32) q[i] = (i == j) ? one_<T>() : zero_<T>();
    __syncwarp();
    for (int64_t c = j; c >= 0; --c) {
      const T* v = Bt + c * m;
      const T tc = tau[c];
      // q -= tau * (v^H q) * v  (H_c, not conjugated)
      const T w = warp_reflector_dot(v, q, c, m);
      __syncwarp();
      warp_reflector_axpy(v, q, tc * w, c, m);
      __syncwarp();
    }
  }
}

// R[i][j] = Bt[j][i] for i <= j, 0 below (R is k x n)
template <typename T>
__global__ void qr_extract_r(const T* __restrict__ Bt, int64_t m, int64_t n, int64_t k, T* __restrict__ R) {
  const int64_t total = k * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / n, j = e - i * n;
    R[e] = (i <= j) ? Bt[j * m + i] : zero_<T>();
  }
}

// ---------------------------------------------------------------------------
// Register-resident panel variant (columns of up to 32*E rows).
//
// Each warp keeps its column in registers (element i at lane i%32, slot i/32);
// a CTA of kPanel warps owns kPanel consecutive columns (a panel).  Inside a
// panel, reflector c is made by its owner warp, written to shared memory and
// applied by the panel's later columns after a CTA barrier -- no global
// round trip.  Each reflector is also published to global memory with a
// flag; warps of later panels wait on the flag (bounded) and apply it from
// registers loaded in one burst.  The critical path is the in-panel chain,
// one CTA barrier per column.
constexpr int kPanel = 8;

template <typename T>
__device__ __forceinline__ T shfl_T(T v, int src) {
  if constexpr (traits<T>::is_complex) {
    v.re = __shfl_sync(0xffffffffu, v.re, src);
    v.im = __shfl_sync(0xffffffffu, v.im, src);
    return v;
  } else {
    return __shfl_sync(0xffffffffu, v, src);
  }
}

// value at row i of a register-resident column, broadcast to the warp
template <typename T, int E>
__device__ __forceinline__ T reg_get(const T (&x)[E], int i) {
  const int slot = i >> 5;
  T a = zero_<T>();
#pragma unroll
  for (int u = 0; u < E; ++u)
    if (u == slot) a = x[u];
  return shfl_T(a, (int)(i & 31));
}

// larfg on the register column: entries > c scaled to v, entry c = beta.
// Norm with four independent partial sums (short dependency chains).
template <typename T, int E>
__device__ __forceinline__ T make_reflector_reg(T (&x)[E], int c, int m) {
  typedef typename traits<T>::real R;
  const int lane = threadIdx.x & 31;
  R xn0 = 0, xn1 = 0, xn2 = 0, xn3 = 0;
#pragma unroll
  for (int u = 0; u < E; ++u) {
    const int i = lane + 32 * u;
    const R a = (i > c && i < m) ? abs2_(x[u]) : R(0);
    if ((u & 3) == 0) xn0 += a; else if ((u & 3) == 1) xn1 += a; else if ((u & 3) == 2) xn2 += a; else xn3 += a;
  }
  const R xn = warp_sum((xn0 + xn1) + (xn2 + xn3));
  const T alpha = reg_get(x, c);
  T tau = zero_<T>();
  if (!(xn == R(0) && imag_(alpha) == R(0))) {
    const R beta = -copysign(sqrt(abs2_(alpha) + xn), real_(alpha));
    const T betaT = from_real<T>(beta);
    tau = div_(betaT - alpha, betaT);
    const T scal = div_(one_<T>(), alpha - betaT);
#pragma unroll
    for (int u = 0; u < E; ++u) {
      const int i = lane + 32 * u;
      if (i > c && i < m) x[u] = scal * x[u];
      else if (i == c) x[u] = betaT;
    }
  }
  return tau;
}

// x <- H_c^H x, v read twice from `v` (entries i > c; v_c = 1 implied):
// shared memory for the panel's own reflectors, L2 for earlier panels'.  Each
// pass fetches v in chunks of C independent loads before using them (keeps
// the L2 latency overlapped without a full register copy of v); the dot
// product runs four independent partial sums.
template <typename T, int E, bool GLOBAL>
__device__ __forceinline__ void apply_stream(T (&x)[E], const T* v, T tau, int c, int m) {
  constexpr int C = (E % 16 == 0 && E < 48) ? 16 : 8;
  const int lane = threadIdx.x & 31;
  T w0 = zero_<T>(), w1 = zero_<T>(), w2 = zero_<T>(), w3 = zero_<T>();
#pragma unroll
  for (int u0 = 0; u0 < E; u0 += C) {
    T vc[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int i = lane + 32 * (u0 + q);
      vc[q] = (i > c && i < m) ? (GLOBAL ? ldcg(v + i) : v[i]) : zero_<T>();
    }
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int u = u0 + q;
      const int i = lane + 32 * u;
      if (i == c) w0 += x[u];
      else if ((q & 3) == 0) fma_(w0, conj_(vc[q]), x[u]);
      else if ((q & 3) == 1) fma_(w1, conj_(vc[q]), x[u]);
      else if ((q & 3) == 2) fma_(w2, conj_(vc[q]), x[u]);
      else fma_(w3, conj_(vc[q]), x[u]);
    }
  }
  const T w = warp_sum((w0 + w1) + (w2 + w3));
  const T f = conj_(tau) * w;
#pragma unroll
  for (int u0 = 0; u0 < E; u0 += C) {
    T vc[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int i = lane + 32 * (u0 + q);
      vc[q] = (i > c && i < m) ? (GLOBAL ? ldcg(v + i) : v[i]) : zero_<T>();
    }
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int u = u0 + q;
      const int i = lane + 32 * u;
      if (i == c) x[u] = x[u] - f;
      else x[u] = x[u] - f * vc[q];  // vc is 0 outside (c, m)
    }
  }
}

// The look-ahead step of the owner of column c+1: x <- H_c^H x (v from shared
// memory) and then the reflector of x at row c+1, in three passes over the
// register column instead of six: (1) the dot product; (2) the update, the
// norm of rows > c+1 and row c+1 itself (one shuffle, no select chain);
// (3) the scaling, written straight to `out` (the next shared buffer).
template <typename T, int E>
__device__ __forceinline__ T apply_and_reflect(T (&x)[E], const T* v, T tau, int c, int m, T* out) {
  typedef typename traits<T>::real R;
  constexpr int C = (E % 16 == 0 && E < 48) ? 16 : 8;
  const int lane = threadIdx.x & 31;
  T w0 = zero_<T>(), w1 = zero_<T>(), w2 = zero_<T>(), w3 = zero_<T>();
#pragma unroll
  for (int u0 = 0; u0 < E; u0 += C) {
    T vc[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int i = lane + 32 * (u0 + q);
      vc[q] = (i > c && i < m) ? v[i] : zero_<T>();
    }
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int u = u0 + q;
      const int i = lane + 32 * u;
      if (i == c) w0 += x[u];
      else if ((q & 3) == 0) fma_(w0, conj_(vc[q]), x[u]);
      else if ((q & 3) == 1) fma_(w1, conj_(vc[q]), x[u]);
      else if ((q & 3) == 2) fma_(w2, conj_(vc[q]), x[u]);
      else fma_(w3, conj_(vc[q]), x[u]);
    }
  }
  const T f = conj_(tau) * warp_sum((w0 + w1) + (w2 + w3));
  const int c1 = c + 1;
  R n0 = 0, n1 = 0, n2 = 0, n3 = 0;
  T a_l = zero_<T>();
#pragma unroll
  for (int u0 = 0; u0 < E; u0 += C) {
    T vc[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int i = lane + 32 * (u0 + q);
      vc[q] = (i > c && i < m) ? v[i] : zero_<T>();
    }
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int u = u0 + q;
      const int i = lane + 32 * u;
      x[u] = (i == c) ? x[u] - f : x[u] - f * vc[q];
      const R a = (i > c1 && i < m) ? abs2_(x[u]) : R(0);
      if ((q & 3) == 0) n0 += a; else if ((q & 3) == 1) n1 += a; else if ((q & 3) == 2) n2 += a; else n3 += a;
      if (i == c1) a_l = x[u];
    }
  }
  const R xn = warp_sum((n0 + n1) + (n2 + n3));
  const T alpha = shfl_T(a_l, c1 & 31);
  T t = zero_<T>();
  T scal = one_<T>(), betaT = alpha;
  if (!(xn == R(0) && imag_(alpha) == R(0))) {
    const R beta = -copysign(sqrt(abs2_(alpha) + xn), real_(alpha));
    betaT = from_real<T>(beta);
    t = div_(betaT - alpha, betaT);
    scal = div_(one_<T>(), alpha - betaT);
  }
#pragma unroll
  for (int u = 0; u < E; ++u) {
    const int i = lane + 32 * u;
    if (i > c1 && i < m) x[u] = scal * x[u];
    else if (i == c1) x[u] = betaT;
    if (i < m) out[i] = x[u];
  }
  return t;
}

// x <- H_c^H x with v held in registers vv (v_c = 1 implied); used by the
// Q formation kernel below
template <typename T, int E>
__device__ __forceinline__ void apply_reg(T (&x)[E], const T (&vv)[E], T tau, int c, int m) {
  const int lane = threadIdx.x & 31;
  T w0 = zero_<T>(), w1 = zero_<T>();
#pragma unroll
  for (int u = 0; u < E; ++u) {
    const int i = lane + 32 * u;
    if (i == c) w0 += x[u];
    else if (i > c && i < m) {
      if (u & 1) fma_(w1, conj_(vv[u]), x[u]);
      else fma_(w0, conj_(vv[u]), x[u]);
    }
  }
  const T w = warp_sum(w0 + w1);
  const T f = conj_(tau) * w;
#pragma unroll
  for (int u = 0; u < E; ++u) {
    const int i = lane + 32 * u;
    if (i == c) x[u] = x[u] - f;
    else if (i > c && i < m) x[u] = x[u] - f * vv[u];
  }
}

template <typename T, int E>
__global__ void __launch_bounds__(kPanel * 32)
qr_panel_kernel(T* Bt, int64_t m, int64_t n, int64_t ld, T* tau, int* flags, SyncWords* sw) {
  __shared__ T sv[2 * 32 * E];
  __shared__ T stau[2];
  extern __shared__ __align__(16) unsigned char qr_panel_dyn[];  // kPanel staging rows of 32 * E
  const int64_t k = m < n ? m : n;
  const int mi = (int)m;  // rows <= 32 * E
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t p0 = (int64_t)blockIdx.x * kPanel;  // first column of the panel
  const int64_t j = p0 + warp;                      // my column
  const bool has = j < n;
  T x[E];
  if (has) {
#pragma unroll
    for (int u = 0; u < E; ++u) {
      const int i = lane + 32 * u;
      x[u] = (i < mi) ? Bt[j * ld + i] : zero_<T>();
    }
  }
  // reflectors of earlier panels, as they are published: each is staged from
  // L2 into this warp's shared-memory row (16 independent loads a lane in
  // flight), then applied from there in two passes
  const int64_t cend = p0 < k ? p0 : k;
  if (has) {
    T* stage = reinterpret_cast<T*>(qr_panel_dyn) + warp * (32 * E);
    for (int64_t c = 0; c < cend; ++c) {
      if (!warp_wait_flag(&flags[c], sw)) break;
      const T* src = Bt + c * ld;
      const int ci = (int)c;
      constexpr int CH = 16;
#pragma unroll
      for (int u0 = 0; u0 < E; u0 += CH) {
        T vc[CH];
#pragma unroll
        for (int q = 0; q < CH && u0 + q < E; ++q) {
          const int i = lane + 32 * (u0 + q);
          vc[q] = (i > ci && i < mi) ? ldcg(src + i) : zero_<T>();
        }
#pragma unroll
        for (int q = 0; q < CH && u0 + q < E; ++q) stage[lane + 32 * (u0 + q)] = vc[q];
      }
      __syncwarp();
      apply_stream<T, E, false>(x, stage, ldcg(tau + c), ci, mi);
      __syncwarp();
    }
  }
  __syncthreads();
  if (ld_volatile(&sw->err)) return;  // uniform: every warp sees the same error word after the barrier
  // this panel's reflectors.  Reflector c is written to shared memory buffer
  // (c & 1) by its owner; after one barrier the later columns apply it, and
  // the owner of column c+1 builds reflector c+1 into the other buffer right
  // after applying c (look-ahead).  The owner of c is then done: it
  // publishes c to global memory (stores, fence, flag) and leaves the loop,
  // so the barrier of step w counts only warps w..kPanel-1 (a named barrier
  // with a shrinking count) and no fence sits on the column chain.  The
  // owner keeps its tau in a register (the shared slot is reused two steps
  // later, possibly before a departed owner has read it).
  const int64_t nw = (k - p0) < kPanel ? (k - p0) : kPanel;
  T my_tau = zero_<T>();
  if (nw > 0 && warp == 0) {
    my_tau = make_reflector_reg(x, (int)p0, mi);
#pragma unroll
    for (int u = 0; u < E; ++u) {
      const int i = lane + 32 * u;
      if (i < mi) sv[i] = x[u];
    }
    if (lane == 0) stau[0] = my_tau;
  }
  for (int w = 0; w < nw; ++w) {
    const int64_t c = p0 + w;
    const int b = w & 1;
    named_barrier(1, (kPanel - w) * 32);
    if (warp == w) {
#pragma unroll
      for (int u = 0; u < E; ++u) {
        const int i = lane + 32 * u;
        if (i >= (int)c && i < mi) stcg(Bt + c * ld + i, x[u]);
      }
      if (lane == 0) stcg(tau + c, my_tau);
      __threadfence();
      __syncwarp();
      if (lane == 0) atomicExch(&flags[c], 1);
      break;
    }
    if (has) {  // warp > w
      if (warp == w + 1 && w + 1 < nw) {
        my_tau = apply_and_reflect<T, E>(x, sv + b * (32 * E), stau[b], (int)c, mi, sv + (b ^ 1) * (32 * E));
        if (lane == 0) stau[b ^ 1] = my_tau;
      } else {
        apply_stream<T, E, false>(x, sv + b * (32 * E), stau[b], (int)c, mi);
      }
    }
  }
  if (has) {
#pragma unroll
    for (int u = 0; u < E; ++u) {
      const int i = lane + 32 * u;
      if (i < mi) Bt[j * ld + i] = x[u];
    }
  }
}

// Qt[j] = H_{min(j,k-1)} ... H_0 e_j with the column in registers
template <typename T, int E>
__global__ void __launch_bounds__(kPanel * 32)
qr_form_q_reg_kernel(const T* __restrict__ Bt, int64_t m, int64_t k, const T* __restrict__ tau, T* __restrict__ Qt) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * kPanel;
  for (int64_t j = (int64_t)blockIdx.x * kPanel + (threadIdx.x >> 5); j < k; j += nwarps) {
    T x[E], vv[E];
#pragma unroll
    for (int u = 0; u < E; ++u) x[u] = (lane + 32 * u == j) ? one_<T>() : zero_<T>();
    for (int64_t c = j; c >= 0; --c) {
#pragma unroll
      for (int u = 0; u < E; ++u) {
        const int64_t i = lane + 32 * u;
        vv[u] = (i > c && i < m) ? Bt[c * m + i] : zero_<T>();
      }
      // H_c (not conjugated): x -= tau (v^H x) v
      apply_reg(x, vv, conj_(tau[c]), (int)c, (int)m);
    }
#pragma unroll
    for (int u = 0; u < E; ++u) {
      const int64_t i = lane + 32 * u;
      if (i < m) Qt[j * m + i] = x[u];
    }
  }
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// ---------------------------------------------------------------------------
// Blocked factorisation (the geqrf / ungqr structure with compact-WY block
// reflectors, Schreiber & Van Loan 1989).  Panels of kQrNB columns are factored
// by the dataflow kernels above on the panel's sub-matrix; then, with
//   H_c0 ... H_c0+nb-1 = I - V T V^H        (T upper triangular, larft),
// the trailing columns get A2 <- (I - V T^H V^H) A2 and Q is formed backwards,
// Q <- (I - V T V^H) Q for the panels in reverse order.  In the transposed
// working layout (rows of Bt / Qt are columns of A / Q) each update is
//   Wt = X2t conj(V) ,  W2t = Wt op(T) ,  X2t -= W2t Vt
// with the long dimension as GEMM rows, all on the CUDA-core GEMM (the
// products have K = 64 or a narrow output; FP32 rounding keeps the
// reflectors orthogonal to FP32 accuracy).
template <typename T>
static int dtype_of() {
  return sizeof(T) == 4 ? TNC_F32 : (sizeof(T) == 8 ? (traits<T>::is_complex ? TNC_C64 : TNC_F64) : TNC_C128);
}

constexpr int64_t kQrNB = 64;
constexpr int64_t kQrBlockedMin = 2 * kQrNB;  // k below this: unblocked dataflow only

constexpr int64_t kQrSplitK = 128;  // K chunk of the split-K products

struct QrLayout {
  size_t bt, tau, flags, sync, qt, vt, sm, wt, w2t, part, total;
  bool blocked;
};
static QrLayout qr_layout(int64_t m, int64_t n, int dt) {
  const size_t es = (size_t)elem_size(dt);
  int64_t k = m < n ? m : n;
  QrLayout L;
  size_t off = 0;
  L.blocked = k >= kQrBlockedMin;
  L.bt = off; off = align256(off + (size_t)n * m * es);
  L.tau = off; off = align256(off + (size_t)k * es);
  L.flags = off; off = align256(off + (size_t)k * sizeof(int));
  L.sync = off; off = align256(off + sizeof(SyncWords));
  L.qt = off; off = align256(off + (size_t)k * m * es);
  L.vt = L.sm = L.wt = L.w2t = L.part = off;
  if (L.blocked) {
    const int64_t nblk = (k + kQrNB - 1) / kQrNB;
    const int64_t rows = n > k ? n : k;
    L.vt = off; off = align256(off + (size_t)kQrNB * m * es);
    L.sm = off; off = align256(off + (size_t)nblk * kQrNB * kQrNB * es);
    L.wt = off; off = align256(off + (size_t)rows * kQrNB * es);
    L.w2t = off; off = align256(off + (size_t)rows * kQrNB * es);
    L.part = off; off = align256(off + (size_t)((m + kQrSplitK - 1) / kQrSplitK) * rows * kQrNB * es);
  }
  L.total = off;
  return L;
}

// Vt[j][i] = reflector j of a panel (i = row within the panel's sub-matrix):
// 0 above the diagonal, 1 on it, the stored entries below
template <typename T>
__global__ void qr_extract_vt(const T* __restrict__ Bt, int64_t ld, int64_t nbb, int64_t ms, T* __restrict__ Vt) {
  const int64_t total = nbb * ms;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / ms, i = e - j * ms;
    Vt[e] = (i < j) ? zero_<T>() : (i == j ? one_<T>() : Bt[j * ld + i]);
  }
}

template <typename T> __device__ __forceinline__ bool is_zero_(T v) {
  if constexpr (traits<T>::is_complex) return v.re == 0 && v.im == 0; else return v == 0;
}

// The block reflector's T enters only as T^H W (trailing update) and T W (Q
// formation).  For Householder blocks T^-1 = U = striu(S) + diag(1/tau) with
// S = V^H V (from Q = I - V T V^H unitary: T^-1 + T^-H = V^H V, T^-1 upper
// triangular), so both products are triangular solves against S:
//   adjoint: U^H W2 = W (forward),   else: U W2 = W (backward).
// A reflector with tau = 0 (H = I) drops out of the product: its component
// of W2 is 0 and it is skipped by the others.  Rows of Wt / W2t are columns
// of W / W2 (rows x nbb); one warp per row, lane l holding components l and
// l + 32, S and tau staged in shared memory (nbb * nbb + nbb elements).
template <typename T>
__global__ void qr_apply_tinv(const T* __restrict__ S, const T* __restrict__ tau, int64_t nbb, const T* __restrict__ Wt,
                              T* __restrict__ W2t, int64_t rows, int adjoint) {
  extern __shared__ __align__(16) unsigned char qr_t_smem[];
  T* sS = reinterpret_cast<T*>(qr_t_smem);
  T* st = sS + nbb * nbb;
  for (int64_t e = threadIdx.x; e < nbb * nbb; e += blockDim.x) sS[e] = S[e];
  for (int64_t e = threadIdx.x; e < nbb; e += blockDim.x) st[e] = tau[e];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int n = (int)nbb;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += nwarps) {
    const T* wr = Wt + r * nbb;
    T a0 = zero_<T>(), a1 = zero_<T>();
    if (adjoint) {
      for (int i = 0; i < n; ++i) {
        T p = zero_<T>();
        if (lane < i) p = conj_(sS[lane * n + i]) * a0;
        if (lane + 32 < i) p += conj_(sS[(lane + 32) * n + i]) * a1;
        p = warp_sum(p);
        const T ti = st[i];
        const T val = is_zero_(ti) ? zero_<T>() : (wr[i] - p) * conj_(ti);
        if (lane == i) a0 = val;
        if (lane + 32 == i) a1 = val;
      }
    } else {
      for (int i = n - 1; i >= 0; --i) {
        T p = zero_<T>();
        if (lane > i && lane < n) p = sS[i * n + lane] * a0;
        if (lane + 32 > i && lane + 32 < n) p += sS[i * n + lane + 32] * a1;
        p = warp_sum(p);
        const T ti = st[i];
        const T val = is_zero_(ti) ? zero_<T>() : (wr[i] - p) * ti;
        if (lane == i) a0 = val;
        if (lane + 32 == i) a1 = val;
      }
    }
    if (lane < n) W2t[r * nbb + lane] = a0;
    if (lane + 32 < n) W2t[r * nbb + lane + 32] = a1;
  }
}

// Dynamic shared memory of qr_apply_tinv beyond the 48 KB default
// (complex128): raised once per device.
template <typename T>
static int ensure_tinv_smem() {
  constexpr size_t bytes = (size_t)(kQrNB * kQrNB + kQrNB) * sizeof(T);
  if constexpr (bytes <= 48 * 1024) {
    return TNC_OK;
  } else {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return TNC_OK;
    if (cudaFuncSetAttribute((const void*)qr_apply_tinv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
      return TNC_ERR_CUDA;
    done.fetch_or(bit);
    return TNC_OK;
  }
}

// C (rows x cols, ld ldc) = sum over nparts of P[p] (rows x cols, dense)
template <typename T>
__global__ void qr_sum_parts(const T* __restrict__ P, int64_t nparts, int64_t rows, int64_t cols, T* __restrict__ C,
                             int64_t ldc) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    T acc = zero_<T>();
    for (int64_t p = 0; p < nparts; ++p) acc += P[p * total + e];
    const int64_t r = e / cols, c = e - r * cols;
    C[r * ldc + c] = acc;
  }
}

// Qt = the first k rows of the m x m identity
template <typename T>
__global__ void qr_eye_rows(T* Qt, int64_t k, int64_t m) {
  const int64_t total = k * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / m, i = e - j * m;
    Qt[e] = (i == j) ? one_<T>() : zero_<T>();
  }
}

// C (M x N, ld ldc) = op(A) op(B) with A (M x K, row-major, opA N or R) and B
// (N x K, row-major, opB T or C): the K range is cut into chunks of kQrSplitK,
// each chunk one member of a batched CUDA-core GEMM into P, then the partial
// products are summed -- enough CTAs for the long-K, narrow products of the
// blocked QR, at FP32 accuracy.
template <typename T>
static int qr_gemm_splitk(int opA, int opB, int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const T* B,
                          int64_t ldb, T* C, int64_t ldc, T* P, cudaStream_t st) {
  const int64_t nparts = (K + kQrSplitK - 1) / kQrSplitK;
  const int64_t full = K / kQrSplitK;  // chunks of full length
  const T one = one_<T>(), zero = zero_<T>();
  if (full > 0) {
    if (int rc = gemm_launch<T>(opA, opB, M, N, kQrSplitK, one, A, lda, kQrSplitK, B, ldb, kQrSplitK, zero, P, N, M * N,
                                full, st))
      return rc;
  }
  if (full < nparts) {  // the ragged last chunk
    const int64_t k0 = full * kQrSplitK;
    if (int rc = gemm_launch<T>(opA, opB, M, N, K - k0, one, A + k0, lda, 0, B + k0, ldb, 0, zero, P + full * M * N, N,
                                0, 1, st))
      return rc;
  }
  qr_sum_parts<T><<<grid1d(M * N, 256), 256, 0, st>>>(P, nparts, M, N, C, ldc);
  return launch_status(1);
}

// Dynamic shared memory of the panel kernel (kPanel staging rows of 32 * E
// elements, up to 96 KB): the attribute is raised once per device.
template <typename T, int E>
static int ensure_panel_smem() {
  constexpr size_t bytes = (size_t)kPanel * 32 * E * sizeof(T);
  if constexpr (bytes <= 48 * 1024) {
    return TNC_OK;
  } else {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return TNC_OK;
    if (cudaFuncSetAttribute((const void*)qr_panel_kernel<T, E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes) != cudaSuccess)
      return TNC_ERR_CUDA;
    done.fetch_or(bit);
    return TNC_OK;
  }
}

// Unblocked dataflow factorisation of the m x n matrix whose transpose is at
// Bt (row stride ld): reflectors in place, tau, per-column flags (zeroed by
// the caller), errors in sw.  Returns the register width E of the panel
// kernel used (0: the general kernel).
template <typename T>
static int qr_dataflow(int64_t m, int64_t n, int64_t ld, T* Bt, T* tau, int* flags, SyncWords* sw, cudaStream_t st,
                       int* E_used) {
  void* args[] = {(void*)&Bt, (void*)&m, (void*)&n, (void*)&ld, (void*)&tau, (void*)&flags, (void*)&sw};
  // register-resident panels when the column fits (E slots of 32 rows)
  const void* panel_fn = nullptr;
  int E = 0;
  int attr_rc = TNC_OK;
  const int64_t slots = (m + 31) / 32;
  const int64_t maxE = sizeof(T) >= 16 ? 16 : 48;
  if (slots <= 8) { panel_fn = (const void*)qr_panel_kernel<T, 8>; E = 8; attr_rc = ensure_panel_smem<T, 8>(); }
  else if (slots <= 16) { panel_fn = (const void*)qr_panel_kernel<T, 16>; E = 16; attr_rc = ensure_panel_smem<T, 16>(); }
  else if constexpr (sizeof(T) < 16) {
    if (slots <= 32 && maxE >= 32) {
      panel_fn = (const void*)qr_panel_kernel<T, 32>; E = 32; attr_rc = ensure_panel_smem<T, 32>();
    } else if (slots <= 48 && maxE >= 48) {
      panel_fn = (const void*)qr_panel_kernel<T, 48>; E = 48; attr_rc = ensure_panel_smem<T, 48>();
    }
  }
  if (attr_rc) return attr_rc;
  if (panel_fn != nullptr) {
    const int64_t want = (n + kPanel - 1) / kPanel;
    const size_t dyn = (size_t)kPanel * 32 * E * sizeof(T);
    const int cap = coop_capacity(panel_fn, kPanel * 32, dyn);
    if (cap > 0 && want <= cap) {
      if (cudaLaunchCooperativeKernel(panel_fn, dim3((unsigned)want), dim3(kPanel * 32), args, dyn, st) != cudaSuccess)
        return TNC_ERR_CUDA;
      *E_used = E;
      return launch_status(1);
    }
  }
  *E_used = 0;
  const int threads = kQrWarps * 32;
  int cap = coop_capacity((const void*)qr_factor_kernel<T>, threads, 0);
  if (cap <= 0) return TNC_ERR_CUDA;
  int64_t want = (n + kQrWarps - 1) / kQrWarps;
  int grid = (int)(want < cap ? want : cap);
  if (cudaLaunchCooperativeKernel((const void*)qr_factor_kernel<T>, dim3(grid), dim3(threads), args, 0, st) !=
      cudaSuccess)
    return TNC_ERR_CUDA;
  return launch_status(1);
}

// Householder factorisation of the m x n matrix X whose transpose is already
// in Bt (n x m, dense).  R (k x n) is always extracted; the rows of Q^T
// (k x m, in the workspace at L.qt) are formed when want_qt or Q is set, and
// Q = (Q^T)^T (m x k) is written when Q is not null.
template <typename T>
static int qr_factor_bt(int64_t m, int64_t n, T* Q, bool want_qt, T* R, const QrLayout& L, char* w, int* info,
                        cudaStream_t st) {
  const int64_t k = m < n ? m : n;
  T* Bt = (T*)(w + L.bt);
  T* tau = (T*)(w + L.tau);
  int* flags = (int*)(w + L.flags);
  SyncWords* sw = (SyncWords*)(w + L.sync);
  T* Qt = (T*)(w + L.qt);
  const bool form_q = (Q != nullptr || want_qt);
  if (cudaMemsetAsync(flags, 0, (size_t)k * sizeof(int), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(sw, 0, sizeof(SyncWords), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(info, 0, sizeof(int), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (!L.blocked) {
    int E = 0;
    if (int rc = qr_dataflow<T>(m, n, m, Bt, tau, flags, sw, st, &E)) return rc;
    copy_sync_error<<<1, 1, 0, st>>>(sw, info);
    int launches = 2;  // error copy, extract R
    if (form_q) {
      void (*formq_fn)(const T*, int64_t, int64_t, const T*, T*) = nullptr;
      if (E == 8) formq_fn = qr_form_q_reg_kernel<T, 8>;
      else if (E == 16) formq_fn = qr_form_q_reg_kernel<T, 16>;
      else if constexpr (sizeof(T) < 16) {
        if (E == 32) formq_fn = qr_form_q_reg_kernel<T, 32>;
        else if (E == 48) formq_fn = qr_form_q_reg_kernel<T, 48>;
      }
      if (formq_fn != nullptr) {
        int64_t gq = (k + kPanel - 1) / kPanel;
        formq_fn<<<(unsigned)gq, kPanel * 32, 0, st>>>(Bt, m, k, tau, Qt);
      } else {
        const int threads = kQrWarps * 32;
        int64_t gq = (k + kQrWarps - 1) / kQrWarps;
        if (gq > 152 * 16) gq = 152 * 16;
        qr_form_q_kernel<T><<<(unsigned)gq, threads, 0, st>>>(Bt, m, k, tau, Qt);
      }
      ++launches;
    }
    qr_extract_r<T><<<grid1d(k * n, 256), 256, 0, st>>>(Bt, m, n, k, R);
    if (launch_status(launches)) return TNC_ERR_CUDA;
  } else {
    T* Vt = (T*)(w + L.vt);
    T* Sall = (T*)(w + L.sm);  // S = V^H V of every panel
    T* Wt = (T*)(w + L.wt);
    T* W2t = (T*)(w + L.w2t);
    T* P = (T*)(w + L.part);
    const T one = one_<T>(), mone = zero_<T>() - one_<T>();
    const int64_t nblk = (k + kQrNB - 1) / kQrNB;
    if (int rc = ensure_tinv_smem<T>()) return rc;
    const size_t tinv_smem = (size_t)(kQrNB * kQrNB + kQrNB) * sizeof(T);
    for (int64_t b = 0; b < nblk; ++b) {
      const int64_t c0 = b * kQrNB;
      const int64_t nbb = (k - c0) < kQrNB ? (k - c0) : kQrNB;
      const int64_t ms = m - c0;
      T* panel = Bt + c0 * m + c0;
      int E = 0;
      if (int rc = qr_dataflow<T>(ms, nbb, m, panel, tau + c0, flags + c0, sw, st, &E)) return rc;
      const int64_t n2 = n - c0 - nbb;
      const bool need_t = form_q || n2 > 0;
      if (!need_t) continue;
      qr_extract_vt<T><<<grid1d(nbb * ms, 256), 256, 0, st>>>(panel, m, nbb, ms, Vt);
      // S = V^H V = conj(Vt) Vt^T, kept per panel for the Q formation
      T* Sb = Sall + b * kQrNB * kQrNB;
      if (int rc = qr_gemm_splitk<T>(TNC_OP_R, TNC_OP_T, nbb, nbb, ms, Vt, ms, Vt, ms, Sb, nbb, P, st)) return rc;
      if (launch_status(1)) return TNC_ERR_CUDA;
      if (n2 > 0) {
        T* X2t = Bt + (c0 + nbb) * m + c0;  // trailing columns, rows c0.. (n2 x ms, ld m)
        if (int rc = qr_gemm_splitk<T>(TNC_OP_N, TNC_OP_C, n2, nbb, ms, X2t, m, Vt, ms, Wt, nbb, P, st)) return rc;
        // W2 = T^H W
        qr_apply_tinv<T><<<grid1d(n2 * 32, 256, 152 * 8), 256, tinv_smem, st>>>(Sb, tau + c0, nbb, Wt, W2t, n2, 1);
        if (launch_status(1)) return TNC_ERR_CUDA;
        if (int rc = gemm_launch<T>(TNC_OP_N, TNC_OP_N, n2, ms, nbb, mone, W2t, nbb, 0, Vt, ms, 0, one, X2t, m, 0, 1,
                                    st))
          return rc;
      }
    }
    copy_sync_error<<<1, 1, 0, st>>>(sw, info);
    qr_extract_r<T><<<grid1d(k * n, 256), 256, 0, st>>>(Bt, m, n, k, R);
    if (launch_status(2)) return TNC_ERR_CUDA;
    if (form_q) {
      qr_eye_rows<T><<<grid1d(k * m, 256), 256, 0, st>>>(Qt, k, m);
      if (launch_status(1)) return TNC_ERR_CUDA;
      for (int64_t b = nblk - 1; b >= 0; --b) {
        const int64_t c0 = b * kQrNB;
        const int64_t nbb = (k - c0) < kQrNB ? (k - c0) : kQrNB;
        const int64_t ms = m - c0;
        const int64_t nq = k - c0;            // columns of Q touched
        T* Qs = Qt + c0 * m + c0;             // nq x ms, ld m
        const T* Sb = Sall + b * kQrNB * kQrNB;
        qr_extract_vt<T><<<grid1d(nbb * ms, 256), 256, 0, st>>>(Bt + c0 * m + c0, m, nbb, ms, Vt);
        if (launch_status(1)) return TNC_ERR_CUDA;
        if (int rc = qr_gemm_splitk<T>(TNC_OP_N, TNC_OP_C, nq, nbb, ms, Qs, m, Vt, ms, Wt, nbb, P, st)) return rc;
        // W2 = T W
        qr_apply_tinv<T><<<grid1d(nq * 32, 256, 152 * 8), 256, tinv_smem, st>>>(Sb, tau + c0, nbb, Wt, W2t, nq, 0);
        if (launch_status(1)) return TNC_ERR_CUDA;
        if (int rc = gemm_launch<T>(TNC_OP_N, TNC_OP_N, nq, ms, nbb, mone, W2t, nbb, 0, Vt, ms, 0, one, Qs, m, 0, 1, st))
          return rc;
      }
    }
  }
  if (Q == nullptr) return TNC_OK;
  // Q = Qt^T
  int64_t shp[2] = {k, m};
  int perm[2] = {1, 0};
  return tnc_permute(dtype_of<T>(), Qt, Q, 2, shp, perm, 0, st);
}

template <typename T>
static int qr_impl(int64_t m, int64_t n, const T* A, int64_t lda, T* Q, T* R, void* work, size_t wb,
                   int* info, cudaStream_t st) {
  if (m <= 0 || n <= 0 || lda < n || !A || !Q || !R || !work || !info) return TNC_ERR_ARG;
  if (lda != n) return TNC_ERR_ARG;
  QrLayout L = qr_layout(m, n, dtype_of<T>());
  if (wb < L.total) return TNC_ERR_WORKSPACE;
  char* w = (char*)work;
  // Bt = A^T
  int64_t shp[2] = {m, n};
  int perm[2] = {1, 0};
  if (int s = tnc_permute(dtype_of<T>(), A, (T*)(w + L.bt), 2, shp, perm, 0, st)) return s;
  return qr_factor_bt<T>(m, n, Q, false, R, L, w, info, st);
}

// R factor only, of A (m x n) or, with adjoint, of A^H (n x m).  For A^H the
// transposed copy the factorisation works on is conj(A) itself, so no
// transpose runs.
template <typename T>
static int qr_r_impl(int64_t m, int64_t n, const T* A, int adjoint, T* R, void* work, size_t wb, int* info,
                     cudaStream_t st) {
  if (m <= 0 || n <= 0 || !A || !R || !work || !info) return TNC_ERR_ARG;
  const int64_t fm = adjoint ? n : m, fn = adjoint ? m : n;  // the factorised matrix is fm x fn
  QrLayout L = qr_layout(fm, fn, dtype_of<T>());
  if (wb < L.total) return TNC_ERR_WORKSPACE;
  char* w = (char*)work;
  if (adjoint) {
    int64_t shp[2] = {m, n};
    int perm[2] = {0, 1};
    if (int s = tnc_permute(dtype_of<T>(), A, (T*)(w + L.bt), 2, shp, perm, traits<T>::is_complex ? 1 : 0, st))
      return s;
  } else {
    int64_t shp[2] = {m, n};
    int perm[2] = {1, 0};
    if (int s = tnc_permute(dtype_of<T>(), A, (T*)(w + L.bt), 2, shp, perm, 0, st)) return s;
  }
  return qr_factor_bt<T>(fm, fn, (T*)nullptr, false, R, L, w, info, st);
}

}  // namespace tnc

namespace tnc {

size_t qr_qt_workspace(int64_t fm, int64_t fn, int dt) { return qr_layout(fm, fn, dt).total; }

template <typename T>
int qr_qt(int64_t fm, int64_t fn, const T* A, int adjoint, bool want_qt, T* R, void* work, size_t wb, int* info,
          cudaStream_t st, T** qt) {
  if (fm <= 0 || fn <= 0 || !A || !R || !work || !info) return TNC_ERR_ARG;
  QrLayout L = qr_layout(fm, fn, dtype_of<T>());
  if (wb < L.total) return TNC_ERR_WORKSPACE;
  char* w = (char*)work;
  // Bt = X^T: for X = A^H that is conj(A) as stored (A is fn x fm)
  int64_t shp[2] = {adjoint ? fn : fm, adjoint ? fm : fn};
  int perm_id[2] = {0, 1}, perm_t[2] = {1, 0};
  if (int s = tnc_permute(dtype_of<T>(), A, (T*)(w + L.bt), 2, shp, adjoint ? perm_id : perm_t,
                          (adjoint && traits<T>::is_complex) ? 1 : 0, st))
    return s;
  if (qt) *qt = (T*)(w + L.qt);
  return qr_factor_bt<T>(fm, fn, (T*)nullptr, want_qt, R, L, w, info, st);
}

template int qr_qt<float>(int64_t, int64_t, const float*, int, bool, float*, void*, size_t, int*, cudaStream_t, float**);
template int qr_qt<double>(int64_t, int64_t, const double*, int, bool, double*, void*, size_t, int*, cudaStream_t,
                           double**);
template int qr_qt<c64>(int64_t, int64_t, const c64*, int, bool, c64*, void*, size_t, int*, cudaStream_t, c64**);
template int qr_qt<c128>(int64_t, int64_t, const c128*, int, bool, c128*, void*, size_t, int*, cudaStream_t, c128**);

TNC_DEFINE_SPIN_SETTER(spin_limit_set_qr)

}  // namespace tnc

using namespace tnc;

extern "C" int tnc_qr_workspace_size(int dtype, int64_t m, int64_t n, size_t* bytes) {
  if (!elem_size(dtype) || m <= 0 || n <= 0 || !bytes) return TNC_ERR_ARG;
  *bytes = qr_layout(m, n, dtype).total;
  return TNC_OK;
}

extern "C" int tnc_qr(int dtype, int64_t m, int64_t n, const void* A, int64_t lda, void* Q, void* R, void* work,
                      size_t work_bytes, int* info, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, return qr_impl<T>(m, n, (const T*)A, lda, (T*)Q, (T*)R, work, work_bytes, info, st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_qr_r_workspace_size(int dtype, int64_t m, int64_t n, int adjoint, size_t* bytes) {
  if (!elem_size(dtype) || m <= 0 || n <= 0 || !bytes) return TNC_ERR_ARG;
  *bytes = adjoint ? qr_layout(n, m, dtype).total : qr_layout(m, n, dtype).total;
  return TNC_OK;
}

extern "C" int tnc_qr_r(int dtype, int64_t m, int64_t n, const void* A, int adjoint, void* R, void* work,
                        size_t work_bytes, int* info, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, return qr_r_impl<T>(m, n, (const T*)A, adjoint, (T*)R, work, work_bytes, info, st));
  return TNC_ERR_ARG;
}
