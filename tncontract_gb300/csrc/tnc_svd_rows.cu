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
#include "tnc_df.cuh"
#include "tnc_persist.cuh"

#include <atomic>
#include <type_traits>

namespace tnc {

// sweep cap; the counter words hold a rotation count per sweep, then a count
// of the rotations above the stage-stop tolerance per sweep, then one step
// counter per half-block
constexpr int kRowsMaxSweeps = 100;

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
  bool big;  // |g| > stol sqrt(a b): above the stage-stop tolerance
};

// Jacobi rotation from the 2x2 Gram entries (see tnc_svd.cu for the formula)
template <typename T>
__device__ __forceinline__ Rot<T> make_rot_ieee(typename traits<T>::real a, typename traits<T>::real b, T g,
                                                typename traits<T>::real rtol, typename traits<T>::real noise2,
                                                typename traits<T>::real stol) {
  typedef typename traits<T>::real R;
  Rot<T> r;
  const R h = abs_(g);
  const R sab = sqrt(a) * sqrt(b);
  // rows at the rounding-noise floor (or whose squared norm underflowed) count as converged
  r.apply = (a > noise2) && (b > noise2) && (a > 0) && (b > 0) && (h > rtol * sab);
  r.big = r.apply && h > stol * sab;
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

// The same rotation for single-precision rows with a shorter dependency
// chain (the rotation parameters are on the critical path of every Jacobi
// step): the tests compare squares (|g|^2 > tol^2 a b, no square roots),
// |g| is one square root of |g|^2 instead of a hypot, and the divisions of
// 1/|g|, tau, t and c become a product and correctly rounded reciprocals.  Every rounding stays round-to-nearest, so
// the rotations carry no systematic bias (|e| = 1 and c^2 + s^2 = 1 to an
// ulp either side; a Newton-refined hardware estimate here drifted the FP32
// sweep's discarded weights by 1.5e-6).  Operands whose squares or products
// leave the comfortable FP32 range take the IEEE formula.
template <typename T>
__device__ __forceinline__ Rot<T> make_rot(typename traits<T>::real a, typename traits<T>::real b, T g,
                                           typename traits<T>::real rtol, typename traits<T>::real noise2,
                                           typename traits<T>::real stol = 0) {
  typedef typename traits<T>::real R;
  if constexpr (sizeof(R) != 4) {
    return make_rot_ieee<T>(a, b, g, rtol, noise2, stol);
  } else {
    const float h2 = abs2_(g), ab = a * b;
    if (!(h2 > 1e-30f && h2 < 1e30f && ab > 1e-30f && ab < 1e30f))
      return make_rot_ieee<T>(a, b, g, rtol, noise2, stol);
    Rot<T> r;
    r.apply = (a > noise2) && (b > noise2) && (h2 > (rtol * rtol) * ab);
    r.big = r.apply && h2 > (stol * stol) * ab;
    if (!r.apply) { r.c = 1; r.th = 0; r.se = zero_<T>(); r.sec = zero_<T>(); return r; }
    // |g| and 1/|g| by correctly rounded FP32 operations (sqrt.rn, rcp.rn):
    // a correctly rounded reciprocal square root has no FP32 instruction and
    // would be emulated on GB300's slow FP64 pipe
    const float hg = sqrtf(h2);
    const float ih = __frcp_rn(hg);
    const float tau = (b - a) * 0.5f * ih;
    const float at = fabsf(tau);
    float t;
    if (at > 1e15f) {
      t = 0.5f / tau;
    } else {
      t = copysignf(__frcp_rn(at + sqrtf(fmaf(tau, tau, 1.f))), tau);
    }
    const float c = __frcp_rn(sqrtf(fmaf(t, t, 1.f)));
    const float s = c * t;
    r.c = c;
    r.th = t * hg;
    const T e = g * ih;
    r.se = s * e;
    r.sec = s * conj_(e);
    return r;
  }
}

// rows x (registers, MAXE per lane) and y (shared memory), one warp.  The
// squared norms a (of x) and *b (of y) are carried, not recomputed: only
// g = <x, y> is reduced, and a rotation moves them to a - t|g|, b + t|g|
// (exact in exact arithmetic; recomputed from the rows once per sweep).
// Returns 0 (no rotation), 1 (a rotation) or 3 (a rotation above stol).
template <typename T, int MAXE>
__device__ __forceinline__ int rotate_reg_smem(T (&x)[MAXE], T* y, int64_t L, typename traits<T>::real rtol,
                                               typename traits<T>::real noise2, typename traits<T>::real& a,
                                               typename traits<T>::real* b, typename traits<T>::real stol) {
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
  const Rot<T> r = make_rot<T>(a, bb, g, rtol, noise2, stol);
  if (!r.apply) return 0;
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    const int k = lane + 32 * u;
    const T xv = x[u];
    x[u] = r.c * xv - r.se * yr[u];
    if (k < Li) y[k] = r.sec * xv + r.c * yr[u];
  }
  a = a - r.th;
  if (lane == 0) *b = bb + r.th;
  return r.big ? 3 : 1;
}

// rows x and y both in shared memory, one warp; squared norms *a, *b carried;
// returns as rotate_reg_smem
template <typename T>
__device__ __forceinline__ int rotate_smem_smem(T* x, T* y, int64_t L, typename traits<T>::real rtol,
                                                typename traits<T>::real noise2, typename traits<T>::real* a,
                                                typename traits<T>::real* b, typename traits<T>::real stol) {
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
  const Rot<T> r = make_rot<T>(aa, bb, g, rtol, noise2, stol);
  if (!r.apply) return 0;
  for (int64_t kk = lane; kk < L; kk += 32) {
    const T xv = x[kk], yv = y[kk];
    x[kk] = r.c * xv - r.se * yv;
    y[kk] = r.sec * xv + r.c * yv;
  }
  __syncwarp();
  if (lane == 0) { *a = aa - r.th; *b = bb + r.th; }
  __syncwarp();
  return r.big ? 3 : 1;
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

// ------------------------------------------------------------ DF rows
// The extended-precision finish (tnc_svd_rows_df) runs the same kernel on
// double-float rows (tnc_df.cuh); these overloads are its rotation and norm.

// Jacobi rotation of two DF rows from their carried squared norms a, b and
// g = <x, y>, same formula as make_rot.  A small angle (|t| < 2^-12, the
// finish's usual case: rows already orthogonal to FP32 level) is computed in
// FP32 and applied as x + ((c - 1) x - s e y): the FP32 rounding then falls on
// the small correction only, 2^-24 |t| relative to the row, and the
// transformation stays orthogonal to 4 eps t^2.  A larger angle (two rows
// of nearly equal norm) takes the FP64 formula on the DF inputs and a full DF
// product.
struct RotDF {
  bool apply, big;
  bool above;           // a large angle, or |g| above the stop tolerance
  float cm1, ser, sei;  // small angle: c - 1 and s e (e = g / |g|)
  dfr c, sr, si;        // large angle: c and s e
  dfr a, b;             // the rows' new squared norms
};

__device__ __forceinline__ RotDF make_rot_df(dfr a, dfr b, dfr gre, dfr gim, float rtol, float noise2, bool cplx,
                                             float stol) {
  RotDF r;
  r.apply = false;
  r.big = false;
  r.above = false;
  const float gabs = cplx ? hypotf(gre.h, gim.h) : fabsf(gre.h);
  const float sab = sqrtf(a.h) * sqrtf(b.h);
  // rows at the rounding-noise floor count as converged (as make_rot)
  if (!(a.h > noise2 && b.h > noise2 && gabs > rtol * sab)) return r;
  r.above = gabs > stol * sab;
  float ds, de;
  two_sum(b.h, -a.h, ds, de);
  de = __fadd_rn(de, __fsub_rn(b.l, a.l));
  const float tau = __fadd_rn(ds, de) / (2.f * gabs);
  if (fabsf(tau) >= 4096.f) {
    const float t = fabsf(tau) > 1e7f ? 0.5f / tau
                                      : (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.f)));
    if (t == 0.f) return r;  // below FP32 range: nothing to rotate
    const float q = sqrtf(fmaf(t, t, 1.f));
    const float s = t / q, inv = 1.f / gabs;
    r.apply = true;
    r.cm1 = -(t * t) / (q * (1.f + q));
    r.ser = s * (gre.h * inv);
    r.sei = cplx ? s * (gim.h * inv) : 0.f;
    const float th = t * gabs;
    r.a = df_add(a, dfr(-th, 0.f));
    r.b = df_add(b, dfr(th, 0.f));
    return r;
  }
  r.above = true;
  const double ad = to_double(a), bd = to_double(b);
  const double gr = to_double(gre), gi = cplx ? to_double(gim) : 0.0;
  const double h = cplx ? hypot(gr, gi) : fabs(gr);
  const double taud = (bd - ad) / (2.0 * h);
  const double t = (taud >= 0 ? 1.0 : -1.0) / (fabs(taud) + sqrt(1.0 + taud * taud));
  const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
  r.apply = true;
  r.big = true;
  r.c = dfr(c);
  r.sr = dfr(s * (gr / h));
  r.si = dfr(cplx ? s * (gi / h) : 0.0);
  const double th = t * h;
  r.a = dfr(ad - th);
  r.b = dfr(bd + th);
  return r;
}

__device__ __forceinline__ dfr df_neg(dfr v) { return dfr(-v.h, -v.l); }
// c u + p v + q w in DF
__device__ __forceinline__ dfr df_dot3(dfr c, dfr u, dfr p, dfr v, dfr q, dfr w) {
  return df_add(df_add(df_mul(c, u), df_mul(p, v)), df_mul(q, w));
}

// complex DF rows x, y in shared memory, one warp; squared norms carried
__device__ __forceinline__ int rotate_smem_smem(dfc* x, dfc* y, int64_t L, dfr rtol, dfr noise2, dfr* a, dfr* b,
                                                dfr stol) {
  const int lane = threadIdx.x & 31;
  // g = sum x conj(y): Re = xr yr + xi yi, Im = xi yr - xr yi, four Dot2 chains
  float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f, s3 = 0.f, c3 = 0.f;
  for (int64_t k = lane; k < L; k += 32) {
    const dfc xv = x[k], yv = y[k];
    dot2_acc(s0, c0, xv.re.h, xv.re.l, yv.re.h, yv.re.l);
    dot2_acc(s1, c1, xv.im.h, xv.im.l, yv.im.h, yv.im.l);
    dot2_acc(s2, c2, xv.im.h, xv.im.l, yv.re.h, yv.re.l);
    dot2_acc(s3, c3, -xv.re.h, -xv.re.l, yv.im.h, yv.im.l);
  }
  const dfr gre = warp_sum_df(df_add(df_norm(s0, c0), df_norm(s1, c1)));
  const dfr gim = warp_sum_df(df_add(df_norm(s2, c2), df_norm(s3, c3)));
  const RotDF r = make_rot_df(*a, *b, gre, gim, rtol.h, noise2.h, true, stol.h);
  if (!r.apply) return 0;
  if (!r.big) {
    // x += (c-1) x - se y, y += conj(se) x + (c-1) y, from the hi parts
    const float cm1 = r.cm1, ser = r.ser, sei = r.sei;
    for (int64_t k = lane; k < L; k += 32) {
      dfc xv = x[k], yv = y[k];
      const float xr = xv.re.h, xi = xv.im.h, yr = yv.re.h, yi = yv.im.h;
      const float syr = fmaf(ser, yr, -sei * yi), syi = fmaf(ser, yi, sei * yr);
      const float sxr = fmaf(ser, xr, sei * xi), sxi = fmaf(ser, xi, -sei * xr);
      df_acc(xv.re, fmaf(cm1, xr, -syr));
      df_acc(xv.im, fmaf(cm1, xi, -syi));
      df_acc(yv.re, fmaf(cm1, yr, sxr));
      df_acc(yv.im, fmaf(cm1, yi, sxi));
      x[k] = xv;
      y[k] = yv;
    }
  } else {
    // x' = c x - se y, y' = conj(se) x + c y in DF
    const dfr c = r.c, sr = r.sr, si = r.si, nsr = df_neg(r.sr), nsi = df_neg(r.si);
    for (int64_t k = lane; k < L; k += 32) {
      const dfc xv = x[k], yv = y[k];
      dfc nx, ny;
      nx.re = df_dot3(c, xv.re, nsr, yv.re, si, yv.im);
      nx.im = df_dot3(c, xv.im, nsr, yv.im, nsi, yv.re);
      ny.re = df_dot3(c, yv.re, sr, xv.re, si, xv.im);
      ny.im = df_dot3(c, yv.im, sr, xv.im, nsi, xv.re);
      x[k] = nx;
      y[k] = ny;
    }
  }
  __syncwarp();
  if (lane == 0) { *a = r.a; *b = r.b; }
  __syncwarp();
  return r.above ? 3 : 1;
}

// real DF rows
__device__ __forceinline__ int rotate_smem_smem(dfr* x, dfr* y, int64_t L, dfr rtol, dfr noise2, dfr* a, dfr* b,
                                                dfr stol) {
  const int lane = threadIdx.x & 31;
  float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
  int64_t k = lane;
  for (; k + 32 < L; k += 64) {
    const dfr x0 = x[k], y0 = y[k], x1 = x[k + 32], y1 = y[k + 32];
    dot2_acc(s0, c0, x0.h, x0.l, y0.h, y0.l);
    dot2_acc(s1, c1, x1.h, x1.l, y1.h, y1.l);
  }
  if (k < L) dot2_acc(s0, c0, x[k].h, x[k].l, y[k].h, y[k].l);
  const dfr g = warp_sum_df(df_add(df_norm(s0, c0), df_norm(s1, c1)));
  const RotDF r = make_rot_df(*a, *b, g, dfr(0.f, 0.f), rtol.h, noise2.h, false, stol.h);
  if (!r.apply) return 0;
  if (!r.big) {
    const float cm1 = r.cm1, se = r.ser;
    for (int64_t kk = lane; kk < L; kk += 32) {
      dfr xv = x[kk], yv = y[kk];
      const float xh = xv.h, yh = yv.h;
      df_acc(xv, fmaf(cm1, xh, -se * yh));
      df_acc(yv, fmaf(cm1, yh, se * xh));
      x[kk] = xv;
      y[kk] = yv;
    }
  } else {
    const dfr c = r.c, s = r.sr, ns = df_neg(r.sr), zero(0.f, 0.f);
    for (int64_t kk = lane; kk < L; kk += 32) {
      const dfr xv = x[kk], yv = y[kk];
      x[kk] = df_dot3(c, xv, ns, yv, zero, zero);
      y[kk] = df_dot3(c, yv, s, xv, zero, zero);
    }
  }
  __syncwarp();
  if (lane == 0) { *a = r.a; *b = r.b; }
  __syncwarp();
  return r.above ? 3 : 1;
}

__device__ __forceinline__ dfr warp_row_norm2(const dfc* x, int64_t L) {
  const int lane = threadIdx.x & 31;
  float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
  for (int64_t k = lane; k < L; k += 32) {
    const dfc v = x[k];
    dot2_acc(s0, c0, v.re.h, v.re.l, v.re.h, v.re.l);
    dot2_acc(s1, c1, v.im.h, v.im.l, v.im.h, v.im.l);
  }
  return warp_sum_df(df_add(df_norm(s0, c0), df_norm(s1, c1)));
}
__device__ __forceinline__ dfr warp_row_norm2(const dfr* x, int64_t L) {
  const int lane = threadIdx.x & 31;
  float s0 = 0.f, c0 = 0.f;
  for (int64_t k = lane; k < L; k += 32) dot2_acc(s0, c0, x[k].h, x[k].l, x[k].h, x[k].l);
  return warp_sum_df(df_norm(s0, c0));
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
// thread, so nothing else could share the SM).  Double-float rows fill the
// shared memory of an SM with one CTA (2 x 8 rows of 512 16-byte elements)
// and keep the registers of their Dot2 chains (held to 128 registers the
// complex kernel spills 144 bytes and took 6.8 against 4.8 ms at 512 x 512;
// the sweep fell from 4.98 to 4.54 sweeps/s although an FP32 CTA then fits
// beside it).
template <typename T, int MAXE, int MAXT, bool PREG>
constexpr int jacobi_min_blocks() {
  if (std::is_same<T, dfc>::value || std::is_same<T, dfr>::value) return 1;
  return (!PREG || (MAXT == 256 && MAXE <= 16 && sizeof(typename traits<T>::real) == 4)) ? 2 : 1;
}

template <typename T, int MAXE, int MAXT, bool PREG>
__global__ void __launch_bounds__(MAXT, jacobi_min_blocks<T, MAXE, MAXT, PREG>())
jacobi_block_kernel(T* W, int64_t nr, int64_t L, int h, int max_sweeps, double tol, const double* frob2,
                    typename traits<T>::real* Dn, unsigned* counters, unsigned* ver, SyncWords* sw, int* info,
                    int64_t nkeep, double stop_tol) {
  typedef typename traits<T>::real R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sB = reinterpret_cast<T*>(smem_raw);
  __shared__ R sn[32];   // squared norms of the shared-memory rows
  __shared__ R snA[32];  // ... of the P half-block when it is in shared memory too
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nb = (nr + h - 1) / h;
  const int64_t nbp = nb + (nb & 1);
  const int64_t ntask = nbp / 2;
  // half-blocks holding the first nkeep rows; pairs of two later half-blocks
  // take no rotation (their rows need only be orthogonal to the kept ones)
  const int64_t kb = (nkeep + h - 1) / h;
  const R rtol = (R)tol;
  const R stol = (R)stop_tol;
  const R noise2 = noise_floor2<T>(frob2);
  int sweep = 0;
  bool converged = false, staged = false;
  unsigned last_rot = 0;
  T x[PREG ? MAXE : 1];
  for (; sweep < max_sweeps; ++sweep) {
    unsigned rot = 0, rotb = 0;
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
      for (int rr = 0; hb < kb && rr < hp - 1; ++rr) {
        if (warp < hp / 2) {
          int64_t p, q;
          circle_pair(hp, rr, warp, p, q);
          if (p < cnt && q < cnt) {
            const int rr = rotate_smem_smem(sB + p * L, sB + q * L, L, rtol, noise2, &sn[p], &sn[q], stol);
            rot += (unsigned)(rr & 1);
            rotb += (unsigned)(rr >> 1);
          }
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
        if (P >= kb && Q >= kb) {  // two discarded half-blocks: pass them on
          publish_steps(ver, P, Q, g + 1u);
          continue;
        }
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
            if (hasA && j < cntB) {
              const int rr = rotate_reg_smem<T, MAXE>(x, sB + (int64_t)j * L, L, rtol, noise2, an, &sn[j], stol);
              rot += (unsigned)(rr & 1);
              rotb += (unsigned)(rr >> 1);
            }
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
            if (warp < cntA && j < cntB) {
              const int rr = rotate_smem_smem(sA + (int64_t)warp * L, sB + (int64_t)j * L, L, rtol, noise2,
                                              &snA[warp], &sn[j], stol);
              rot += (unsigned)(rr & 1);
              rotb += (unsigned)(rr >> 1);
            }
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
    if (lane == 0 && rotb) atomicAdd(&counters[kRowsMaxSweeps + sweep], rotb);
    if (!grid_barrier(sw, gridDim.x)) return;
    last_rot = ld_volatile(&counters[sweep]);
    if (last_rot == 0) { converged = true; ++sweep; break; }
    // stage stop: no rotation of this sweep was above stop_tol (a later
    // stage finishes the rows)
    if (stop_tol > 0 && ld_volatile(&counters[kRowsMaxSweeps + sweep]) == 0) { staged = true; ++sweep; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    info[0] = (converged || staged) ? TNC_OK : TNC_ERR_NOT_CONVERGED;
    info[1] = sweep;
    info[2] = (int)last_rot;
    info[3] = staged ? 1 : 0;
  }
}

// ------------------------------------------------------------ Gram-form block update
// The same rotation sequence as jacobi_block_kernel, with every task's
// rotations accumulated before they touch the rows.  A task (a half-block
// pair, or one half-block in phase 0) loads its 2h rows X into shared memory
// and forms their Gram matrix G = X X^H (2h x 2h, one register-tiled product
// over the row length); its h rotation steps then run on G (two-sided, all h
// disjoint pairs of a step at once: G <- J G J^H) and are accumulated into a
// 2h x 2h unitary U (U <- J U), and the rows are replaced by U X, written
// straight back to global memory.  The 2 x 2 rotations are the ones the
// row-by-row kernel computes (same formula, order and tolerance test, fed by
// G's entries instead of fresh inner products), so the sweep count is the
// same; what changes is the work a step waits on: O(h) arithmetic on G
// instead of an O(L) inner product, reduction and row update, and the
// O(h^2 L) products are GEMM-shaped (FMA-pipe bound, not latency bound).
// Single-precision rows (FP32, complex64), half-blocks of 8 rows, 256
// threads, both tiles of the product in shared memory with a row stride
// padded so the 16 rows fall in distinct banks.  Measured against the
// row-by-row kernel on a 512 x 512 complex64 core (same 11-12 sweeps): 14.5
// against 9.7 ms -- the products are 2.7x the row-by-row kernel's FMAs (Gram
// plus application against inner products plus updates) and every task
// still moves its rows through L2, so it is an option (TNC_ROWS_GRAM, an
// autotuner candidate), not the default.
constexpr int kGramH = 8;
constexpr int kGramRows = 2 * kGramH;  // rows of a task
constexpr int kGramWarps = 8;          // 256 threads = one per Gram entry

template <typename T>
struct GramState {
  T G[2][kGramRows * kGramRows];  // the task's Gram matrix (double buffer)
  T U[2][kGramRows * kGramRows];  // its accumulated rotations
  T jo[kGramRows];                // this step's rotation: row a <- jc[a] a + jo[a] pa[a]
  typename traits<T>::real jc[kGramRows];
  int pa[kGramRows];
};

// row stride of the shared-memory tile: consecutive rows start 4 bytes x
// (element words) apart modulo 128 bytes, so the 16 rows of a column are in
// distinct banks
template <typename T>
__host__ __device__ inline int64_t gram_stride(int64_t L) {
  const int64_t q = 32 / (int64_t)(sizeof(T) / 4);
  return (L + q - 1) / q * q + 1;
}
template <typename T>
inline size_t gram_smem_bytes(int64_t L) {
  return ((size_t)kGramRows * gram_stride<T>(L) + (size_t)kGramWarps * kGramRows * kGramRows) * sizeof(T);
}

// One task: half-blocks P and Q (Q < 0: phase 0, the pairs inside P).
// Returns the number of rotations applied.  Called by every thread.
template <typename T>
__device__ unsigned gram_task(T* W, int64_t nr, int64_t L, int64_t LP, T* X, T* part, GramState<T>& gs,
                              int64_t P, int64_t Q, typename traits<T>::real rtol, typename traits<T>::real noise2,
                              typename traits<T>::real stol, unsigned& rotb) {
  typedef typename traits<T>::real R;
  constexpr int H = kGramH, H2 = kGramRows, NE = H2 * H2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool ph0 = Q < 0;
  const int64_t p0 = P * H, q0 = ph0 ? 0 : Q * H;
  const int cntA = (int)((nr - p0) < H ? (nr - p0) : H);
  const int cntB = ph0 ? 0 : (int)((nr - q0) < H ? (nr - q0) : H);
  // 1. the rows (absent ones zero): P in tile rows 0..H-1, Q in H..2H-1
  for (int a = warp; a < H2; a += kGramWarps) {
    const int ia = a < H ? a : a - H;
    const bool live = a < H ? ia < cntA : ia < cntB;
    const T* src = W + ((a < H ? p0 : q0) + ia) * L;
    T* dst = X + a * LP;
#pragma unroll 4
    for (int64_t k = lane; k < L; k += 32) dst[k] = live ? ldcg(src + k) : zero_<T>();
  }
  __syncthreads();
  // 2. G = X X^H: warp w sums the columns [w kc, (w+1) kc), lane (g, j) the
  //    4 x 2 tile rows 4g..4g+3, columns 2j, 2j+1; then the warps' partials
  {
    const int ar = (lane >> 3) * 4, bc = (lane & 7) * 2;
    const int64_t kc = (L + kGramWarps - 1) / kGramWarps;
    const int64_t k0 = warp * kc, k1 = (k0 + kc) < L ? (k0 + kc) : L;
    T acc[4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      acc[i][0] = zero_<T>();
      acc[i][1] = zero_<T>();
    }
    for (int64_t k = k0; k < k1; ++k) {
      T xa[4], xb[2];
#pragma unroll
      for (int i = 0; i < 4; ++i) xa[i] = X[(ar + i) * LP + k];
#pragma unroll
      for (int j = 0; j < 2; ++j) xb[j] = conj_(X[(bc + j) * LP + k]);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        fma_(acc[i][0], xa[i], xb[0]);
        fma_(acc[i][1], xa[i], xb[1]);
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      part[warp * NE + (ar + i) * H2 + bc] = acc[i][0];
      part[warp * NE + (ar + i) * H2 + bc + 1] = acc[i][1];
    }
  }
  __syncthreads();
  {
    const int t = threadIdx.x;
    T v = zero_<T>();
#pragma unroll
    for (int w = 0; w < kGramWarps; ++w) v += part[w * NE + t];
    gs.G[0][t] = v;
    gs.U[0][t] = (t / H2 == t % H2) ? one_<T>() : zero_<T>();
  }
  __syncthreads();
  // 3. the rotation steps on G (the row-by-row kernel's order: phase 0 an
  //    h-point round-robin inside P, a round step s the pairs (P_i, Q_(i+s)%h))
  const int nsteps = ph0 ? H - 1 : H;
  int cur = 0;
  unsigned rot = 0;
  for (int s = 0; s < nsteps; ++s) {
    int applied = 0;
    if (warp == 0) {
      if (lane < H2) {
        gs.jc[lane] = R(1);
        gs.jo[lane] = zero_<T>();
        gs.pa[lane] = lane;
      }
      __syncwarp();
      int x = 0, y = 0;
      bool ok = false;
      if (ph0) {
        if (lane < H / 2) {
          int64_t p, q;
          circle_pair(H, s, lane, p, q);
          x = (int)p;
          y = (int)q;
          ok = x < cntA && y < cntA;
        }
      } else if (lane < H) {
        x = lane;
        y = H + (lane + s) % H;
        ok = x < cntA && (y - H) < cntB;
      }
      if (ok) {
        const T* Gc = gs.G[cur];
        const Rot<T> r =
            make_rot<T>(real_(Gc[x * H2 + x]), real_(Gc[y * H2 + y]), Gc[x * H2 + y], rtol, noise2, stol);
        if (r.apply) {
          applied = r.big ? 3 : 1;
          gs.jc[x] = r.c;
          gs.jc[y] = r.c;
          gs.jo[x] = -r.se;
          gs.jo[y] = r.sec;
          gs.pa[x] = y;
          gs.pa[y] = x;
        }
      }
      const unsigned nrot = __popc(__ballot_sync(0xffffffffu, applied != 0));
      const unsigned nbig = __popc(__ballot_sync(0xffffffffu, applied == 3));
      rot += lane == 0 ? nrot : 0u;
      rotb += lane == 0 ? nbig : 0u;
    }
    // one barrier that also tells every thread whether anything rotated (a
    // step without rotations leaves G and U as they are; the next step's
    // rotation parameters are written only after the update's barrier)
    if (!__syncthreads_or(applied)) continue;
    {
      const int t = threadIdx.x, a = t / H2, b = t % H2;
      const int pa_ = gs.pa[a], pb_ = gs.pa[b];
      const T* Gc = gs.G[cur];
      const R ca = gs.jc[a], cb = gs.jc[b];
      const T oa = gs.jo[a], ob = conj_(gs.jo[b]);
      // (J G J^H)[a][b] = J[a][a] (G J^H)[a][b] + J[a][pa] (G J^H)[pa][b]
      const T v = Gc[a * H2 + b] * cb + Gc[a * H2 + pb_] * ob;
      const T w = Gc[pa_ * H2 + b] * cb + Gc[pa_ * H2 + pb_] * ob;
      gs.G[cur ^ 1][t] = ca * v + oa * w;
      const T* Uc = gs.U[cur];
      gs.U[cur ^ 1][t] = ca * Uc[a * H2 + b] + oa * Uc[pa_ * H2 + b];
    }
    __syncthreads();
    cur ^= 1;
  }
  // 4. the rows <- U X, warp w writing rows 2w and 2w + 1 to global memory
  {
    const T* Uc = gs.U[cur];
    const int a0 = 2 * warp, a1 = a0 + 1;
    T u0[H2], u1[H2];
#pragma unroll
    for (int c = 0; c < H2; ++c) {
      u0[c] = Uc[a0 * H2 + c];
      u1[c] = Uc[a1 * H2 + c];
    }
    const bool live0 = a0 < H ? a0 < cntA : (a0 - H) < cntB;
    const bool live1 = a1 < H ? a1 < cntA : (a1 - H) < cntB;
    T* d0 = W + (a0 < H ? p0 + a0 : q0 + a0 - H) * L;
    T* d1 = W + (a1 < H ? p0 + a1 : q0 + a1 - H) * L;
    for (int64_t k = lane; k < L; k += 32) {
      T o0 = zero_<T>(), o1 = zero_<T>();
#pragma unroll
      for (int c = 0; c < H2; ++c) {
        const T xv = X[c * LP + k];
        fma_(o0, u0[c], xv);
        fma_(o1, u1[c], xv);
      }
      if (live0) stcg(d0 + k, o0);
      if (live1) stcg(d1 + k, o1);
    }
  }
  return rot;
}

template <typename T>
__global__ void __launch_bounds__(kGramWarps * 32, 2)
jacobi_gram_kernel(T* W, int64_t nr, int64_t L, int max_sweeps, double tol, const double* frob2, unsigned* counters,
                   unsigned* ver, SyncWords* sw, int* info, int64_t nkeep, double stop_tol) {
  typedef typename traits<T>::real R;
  constexpr int H = kGramH;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ GramState<T> gs;
  const int64_t LP = gram_stride<T>(L);
  T* X = reinterpret_cast<T*>(smem_raw);
  T* part = X + kGramRows * LP;
  const int64_t nb = (nr + H - 1) / H;
  const int64_t nbp = nb + (nb & 1);
  const int64_t ntask = nbp / 2;
  const int64_t kb = (nkeep + H - 1) / H;
  const R rtol = (R)tol;
  const R stol = (R)stop_tol;
  const R noise2 = noise_floor2<T>(frob2);
  int sweep = 0;
  bool converged = false, staged = false;
  unsigned last_rot = 0;
  for (; sweep < max_sweeps; ++sweep) {
    unsigned rot = 0, rotb = 0;
    const unsigned g0 = (unsigned)sweep * (unsigned)nbp;
    for (int64_t hb = blockIdx.x; hb < nb; hb += gridDim.x) {
      if (hb < kb) rot += gram_task<T>(W, nr, L, LP, X, part, gs, hb, -1, rtol, noise2, stol, rotb);
      publish_steps(ver, hb, hb, g0 + 1u);
    }
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
        if (!(P >= kb && Q >= kb)) rot += gram_task<T>(W, nr, L, LP, X, part, gs, P, Q, rtol, noise2, stol, rotb);
        publish_steps(ver, P, Q, g + 1u);
      }
    }
    if (threadIdx.x == 0 && rot) atomicAdd(&counters[sweep], rot);
    if (threadIdx.x == 0 && rotb) atomicAdd(&counters[kRowsMaxSweeps + sweep], rotb);
    if (!grid_barrier(sw, gridDim.x)) return;
    last_rot = ld_volatile(&counters[sweep]);
    if (last_rot == 0) { converged = true; ++sweep; break; }
    if (stop_tol > 0 && ld_volatile(&counters[kRowsMaxSweeps + sweep]) == 0) { staged = true; ++sweep; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    info[0] = (converged || staged) ? TNC_OK : TNC_ERR_NOT_CONVERGED;
    info[1] = sweep;
    info[2] = (int)last_rot;
    info[3] = staged ? 1 : 0;
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
static RowsLayout rows_layout(int64_t nr, size_t rs) {
  RowsLayout Ly;
  size_t off = 0;
  Ly.d = off; off = align256(off + (size_t)nr * rs);
  Ly.dn = off; off = align256(off + (size_t)nr * rs);
  Ly.frob2 = off; off = align256(off + sizeof(double));
  // sweep rotation counters, then one step counter per half-block (<= nr)
  Ly.counters = off; off = align256(off + (2 * kRowsMaxSweeps + (size_t)nr) * sizeof(unsigned));
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
                        typename traits<T>::real* Dn, unsigned* counters, SyncWords* sw, int* info, int64_t nkeep,
                        cudaStream_t st, double stop_tol = 0.0) {
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
  unsigned* ver = counters + 2 * kRowsMaxSweeps;
  int64_t nr_ = nr, L_ = L;
  int h_ = h, ms_ = ms;
  double tol_ = tol;
  int64_t nkeep_ = nkeep;
  double stop_ = stop_tol;
  void* args[] = {(void*)&W,  (void*)&nr_,      (void*)&L_,  (void*)&h_,  (void*)&ms_,   (void*)&tol_,    (void*)&frob2,
                  (void*)&Dn, (void*)&counters, (void*)&ver, (void*)&sw,  (void*)&info,  (void*)&nkeep_,  (void*)&stop_};
  if (cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, smem, st) != cudaSuccess) return TNC_ERR_CUDA;
  return TNC_OK;
}

template <typename T>
static int launch_gram(T* W, int64_t nr, int64_t L, int ms, double tol, const double* frob2, unsigned* counters,
                       SyncWords* sw, int* info, int64_t nkeep, cudaStream_t st, double stop_tol) {
  const size_t smem = gram_smem_bytes<T>(L);
  const void* fn = (const void*)jacobi_gram_kernel<T>;
  if (smem > kMaxHalfBlockBytes) return TNC_ERR_ARG;
  {  // the shared-memory attribute, once per device (as ensure_smem_attr)
    static std::atomic<unsigned long long> done_mask{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(done_mask.load() & bit)) {
      if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxHalfBlockBytes) !=
          cudaSuccess)
        return TNC_ERR_CUDA;
      done_mask.fetch_or(bit);
    }
  }
  const int threads = kGramWarps * 32;
  const int cap = coop_capacity(fn, threads, smem);
  if (cap <= 0) return TNC_ERR_CUDA;
  const int64_t nb = (nr + kGramH - 1) / kGramH;
  const int64_t ntask = (nb + (nb & 1)) / 2;
  const int grid = (int)(ntask < cap ? (ntask < 1 ? 1 : ntask) : cap);
  unsigned* ver = counters + 2 * kRowsMaxSweeps;
  int64_t nr_ = nr, L_ = L, nkeep_ = nkeep;
  int ms_ = ms;
  double tol_ = tol, stop_ = stop_tol;
  void* args[] = {(void*)&W,        (void*)&nr_, (void*)&L_,  (void*)&ms_,  (void*)&tol_,   (void*)&frob2,
                  (void*)&counters, (void*)&ver, (void*)&sw,  (void*)&info, (void*)&nkeep_, (void*)&stop_};
  if (cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, smem, st) != cudaSuccess) return TNC_ERR_CUDA;
  return TNC_OK;
}

template <typename T>
static int svd_rows_impl(int64_t m, int64_t n, const T* A, T* W, typename traits<T>::real* S, int64_t* order,
                         int max_sweeps, double tol, int block_rows, int64_t nkeep, void* work, size_t wb, int* info,
                         cudaStream_t st, double stop_tol = 0.0) {
  typedef typename traits<T>::real R;
  if (m <= 0 || n <= 0 || !A || !W || !S || !order || !work || !info) return TNC_ERR_ARG;
  const int tall = m > n;
  const int64_t nr = tall ? n : m, L = tall ? m : n;
  RowsLayout Ly = rows_layout(nr, sizeof(R));
  if (wb < Ly.total) return TNC_ERR_WORKSPACE;
  if (nkeep > nr) nkeep = nr;  // every row kept (the kernel rounds nkeep up to half-blocks)
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
  if (cudaMemsetAsync(counters, 0, (2 * kRowsMaxSweeps + (size_t)nr) * sizeof(unsigned), st) != cudaSuccess)
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
    // single-precision rows: the Gram-form block update on request (measured
    // slower than the row-by-row kernel at 512 x 512 complex64: 14.5 against
    // 9.7 ms; it executes 2.7x the FMAs and keeps the per-task L2 round trip)
    const bool gram = sizeof(R) == 4 && block_rows == TNC_ROWS_GRAM && h == kGramH &&
                      gram_smem_bytes<T>(L) <= kMaxHalfBlockBytes;
    int rc;
    if (gram) {
      if constexpr (sizeof(R) == 4)
        rc = launch_gram<T>(W, nr, L, max_sweeps, tol, frob2, counters, sw, info, nkeep, st, stop_tol);
      else return TNC_ERR_ARG;
    } else if (sizeof(typename traits<T>::real) == 8 && L <= 512) {
      // FP64 rows: both half-blocks in shared memory (2 h L elements)
      if (h > 8) h = 8;
      while (h > 2 && (size_t)2 * h * L * sizeof(T) > kMaxHalfBlockBytes) h >>= 1;
      rc = launch_block<T, 1, 256, false>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, nkeep, st, stop_tol);
    } else if (h == 16) {
      if constexpr (sizeof(T) <= 8) {
        if (L <= 256) rc = launch_block<T, 8, 512>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, nkeep, st, stop_tol);
        else rc = launch_block<T, 16, 512>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, nkeep, st, stop_tol);
      } else {
        return TNC_ERR_ARG;
      }
    } else if (L <= 256) {
      rc = launch_block<T, 8, 256>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, nkeep, st, stop_tol);
    } else if (L <= 512) {
      rc = launch_block<T, 16, 256>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, nkeep, st, stop_tol);
    } else if (L <= 1024 && !big) {
      if constexpr (sizeof(T) < 16) rc = launch_block<T, 32, 256>(W, nr, L, h, max_sweeps, tol, frob2, Dn, counters, sw, info, nkeep, st, stop_tol);
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

// ------------------------------------------------------------ row pivoting
// The truncating sweep's QR preconditioner with its rows in decreasing-norm
// order: the R-only QR of M^H then sees M's rows (its columns) sorted, a
// static version of column pivoting, and the Jacobi on R's rows needs far
// fewer sweeps on graded matrices (Drmac and Veselic, "New fast and
// accurate Jacobi SVD algorithm I", SIAM J. Matrix Anal. Appl. 29 (2008)).
// A bond matrix of the right sweep has rows graded by the previous bond's
// singular values, one descending run per physical index.

// squared row norms, one warp a row (double accumulation)
template <typename T>
__global__ void row_norm2_kernel(const T* W, int64_t nr, int64_t L, double* D) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < nr; i += nw) {
    double acc = 0.0;
    for (int64_t k = lane; k < L; k += 32) acc += (double)abs2_(W[i * L + k]);
    acc = warp_sum(acc);
    if (lane == 0) D[i] = acc;
  }
}

// order[c] = i and rank[i] = c for the stable descending ranking of D (a
// NaN ranks below every number, so the ranking is a permutation)
__global__ void rank_desc_kernel(const double* D, int64_t n, int64_t* order, int64_t* rank) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double di = isnan(D[i]) ? -1.0 : D[i];
    int64_t c = 0;
    for (int64_t j = 0; j < n; ++j) {
      const double dj = isnan(D[j]) ? -1.0 : D[j];
      c += (dj > di) || (dj == di && j < i);
    }
    order[c] = i;
    rank[i] = c;
  }
}

// dst[i] = src[idx[i]] (rows of length L), i < n
template <typename T>
__global__ void permute_rows_kernel(const T* src, int64_t L, const int64_t* idx, int64_t n, T* dst) {
  const int64_t total = n * L;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / L, c = e - i * L;
    dst[e] = src[idx[i] * L + c];
  }
}

// The ranking compares every pair of rows (m threads, m comparisons each):
// bond matrices have at most a few thousand rows.
constexpr int64_t kSortRowsMax = 1 << 16;

template <typename T>
static int sort_rows_impl(int64_t m, int64_t L, const T* src, T* dst, int64_t* order, int64_t* rank, double* norms2,
                          cudaStream_t st) {
  if (m <= 0 || m > kSortRowsMax || L <= 0 || !src || !dst || !order || !rank || !norms2 ||
      (const void*)src == (void*)dst)
    return TNC_ERR_ARG;
  row_norm2_kernel<T><<<grid1d(m * 32, 256), 256, 0, st>>>(src, m, L, norms2);
  rank_desc_kernel<<<grid1d(m, 128), 128, 0, st>>>(norms2, m, order, rank);
  permute_rows_kernel<T><<<grid1d(m * L, 256), 256, 0, st>>>(src, L, order, m, dst);
  return launch_status(3);
}

// ------------------------------------------------------------ DF finish
// The finish ends after a rotating sweep whose rotations were all small
// angles (|t| < 2^-12) below kDfStopTol relative, without a checking sweep:
// every rotation zeroes its pair's inner product to DF precision, and a later
// rotation of the same sweep puts back at most |t| eps <= 2^-12 1e-5 ~ 2.4e-9
// (|<x, z>| / |x||z| <= eps) of it -- a residual of order 1e-8 after the ~2n
// later rotations of the two rows, below the 1e-7 tolerance and the FP32
// rounding of the stored result.  A sweep with a large angle (two rows of
// nearly equal norm) is followed by a checking sweep as before.
constexpr double kDfStopTol = 1e-5;

// Exponent k with |A|_F about 2^k: the DF rows are A 2^-k, inside FP32's range.
__device__ __forceinline__ int df_scale_exp(const double* f2) {
  const double f = f2[0];
  return (f > 0.0 && isfinite(f)) ? ilogb(sqrt(f)) : 0;
}
__device__ __forceinline__ dfr df_widen(float v, int k) { return dfr(ldexpf(v, -k), 0.f); }
__device__ __forceinline__ dfc df_widen(c64 v, int k) {
  dfc r;
  r.re = dfr(ldexpf(v.re, -k), 0.f);
  r.im = dfr(ldexpf(v.im, -k), 0.f);
  return r;
}
__device__ __forceinline__ double df_narrow(dfr v, int k) { return ldexp(to_double(v), k); }
__device__ __forceinline__ c128 df_narrow(dfc v, int k) { return c128(ldexp(to_double(v.re), k), ldexp(to_double(v.im), k)); }

// W = A 2^-k as DF; frob2[1] = frob2[0] 2^-2k (the scaled rows' squared norm)
template <typename Tin, typename Tdf>
__global__ void df_widen_kernel(int64_t n, const Tin* A, Tdf* W, double* frob2) {
  const int k = df_scale_exp(frob2);
  if (blockIdx.x == 0 && threadIdx.x == 0) frob2[1] = ldexp(frob2[0], -2 * k);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    W[i] = df_widen(A[i], k);
}
// in place: the DF element i becomes the FP64 element i (same size) times 2^k
template <typename Tdf, typename Tout>
__global__ void df_narrow_kernel(int64_t n, Tdf* W, const double* frob2) {
  static_assert(sizeof(Tdf) == sizeof(Tout), "in-place narrowing keeps the element size");
  const int k = df_scale_exp(frob2);
  Tout* out = reinterpret_cast<Tout*>(W);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const Tdf v = W[i];
    out[i] = df_narrow(v, k);
  }
}

// The finish of single-precision rows in double-float: A (m x n, m <= n,
// FP32 or complex64) -> W (m x n, FP64 / complex128 elements), S (FP64), order.
template <typename Tin, typename Tdf, typename Tout>
static int svd_rows_df_impl(int64_t m, int64_t n, const Tin* A, void* Wv, double* S, int64_t* order, int max_sweeps,
                            double tol, int block_rows, int64_t nkeep, void* work, size_t wb, int* info,
                            cudaStream_t st) {
  if (m <= 0 || n <= 0 || m > n || !A || !Wv || !S || !order || !work || !info || nkeep < 0) return TNC_ERR_ARG;
  const int64_t nr = m, L = n;
  RowsLayout Ly = rows_layout(nr, sizeof(double));
  if (wb < Ly.total) return TNC_ERR_WORKSPACE;
  if (nkeep > nr) nkeep = nr;
  if (max_sweeps <= 0) max_sweeps = 40;
  if (max_sweeps > kRowsMaxSweeps) max_sweeps = kRowsMaxSweeps;
  if (tol <= 0) tol = 1e-7;
  char* w = (char*)work;
  double* D = (double*)(w + Ly.d);
  dfr* Dn = (dfr*)(w + Ly.dn);
  unsigned* counters = (unsigned*)(w + Ly.counters);
  SyncWords* sw = (SyncWords*)(w + Ly.sync);
  double* frob2 = (double*)(w + Ly.frob2);  // [0] of A, [1] of the scaled rows
  Tdf* W = (Tdf*)Wv;
  if (cudaMemsetAsync(counters, 0, (2 * kRowsMaxSweeps + (size_t)nr) * sizeof(unsigned), st) != cudaSuccess)
    return TNC_ERR_CUDA;
  if (cudaMemsetAsync(sw, 0, sizeof(SyncWords), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(info, 0, 4 * sizeof(int), st) != cudaSuccess) return TNC_ERR_CUDA;
  if (cudaMemsetAsync(frob2, 0, 2 * sizeof(double), st) != cudaSuccess) return TNC_ERR_CUDA;
  frob2_kernel<Tin><<<grid1d(nr * L, 256, 152 * 4), 256, 0, st>>>(nr * L, A, frob2);
  df_widen_kernel<Tin, Tdf><<<grid1d(nr * L, 256), 256, 0, st>>>(nr * L, A, W, frob2);
  int launched = 2;
  if (nr > 1) {
    int h = 8;
    if (block_rows == 2 || block_rows == 4) h = block_rows;
    while (h > 2 && (size_t)2 * h * L * sizeof(Tdf) > kMaxHalfBlockBytes) h >>= 1;
    while (h > 2 && h / 2 >= nr) h >>= 1;
    if ((size_t)2 * h * L * sizeof(Tdf) > kMaxHalfBlockBytes) return TNC_ERR_ARG;  // rows too long
    if (int rc = launch_block<Tdf, 1, 256, false>(W, nr, L, h, max_sweeps, tol, frob2 + 1, Dn, counters, sw, info,
                                                 nkeep, st, kDfStopTol))
      return rc;
    ++launched;
  }
  copy_sync_error<<<1, 1, 0, st>>>(sw, info);
  df_narrow_kernel<Tdf, Tout><<<grid1d(nr * L, 256), 256, 0, st>>>(nr * L, W, frob2);
  rows_norm_kernel<Tout><<<grid1d(nr * 32, 256), 256, 0, st>>>((const Tout*)Wv, nr, L, D, info);
  sort_desc_kernel<double><<<grid1d(nr, 128), 128, 0, st>>>(D, nr, order, S);
  return launch_status(4 + launched);
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
                                       tol, block_rows, INT64_MAX, work, work_bytes, info, st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_svd_rows_keep(int dtype, int64_t m, int64_t n, const void* A, void* W, void* S, int64_t* order,
                                 int max_sweeps, double tol, int block_rows, int64_t nkeep, void* work,
                                 size_t work_bytes, int* info, void* stream) {
  if (nkeep < 0) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return svd_rows_impl<T>(m, n, (const T*)A, (T*)W, (typename traits<T>::real*)S, order, max_sweeps,
                                       tol, block_rows, nkeep, work, work_bytes, info, st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_svd_rows_stage(int dtype, int64_t m, int64_t n, const void* A, void* W, void* S, int64_t* order,
                                  int max_sweeps, double tol, double stop_tol, int block_rows, void* work,
                                  size_t work_bytes, int* info, void* stream) {
  if (!(stop_tol >= 0.0)) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return svd_rows_impl<T>(m, n, (const T*)A, (T*)W, (typename traits<T>::real*)S, order, max_sweeps,
                                       tol, block_rows, INT64_MAX, work, work_bytes, info, st, stop_tol));
  return TNC_ERR_ARG;
}

extern "C" int tnc_sort_rows(int dtype, int64_t m, int64_t L, const void* src, void* dst, int64_t* order,
                             int64_t* rank, double* norms2, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return sort_rows_impl<T>(m, L, (const T*)src, (T*)dst, order, rank, norms2, st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_permute_rows(int dtype, int64_t n, int64_t L, const void* src, const int64_t* idx, void* dst,
                                void* stream) {
  if (n < 0 || L <= 0 || !src || !idx || !dst || src == dst) return TNC_ERR_ARG;
  if (n == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, {
    permute_rows_kernel<T><<<grid1d(n * L, 256), 256, 0, st>>>((const T*)src, L, idx, n, (T*)dst);
    return launch_status();
  });
  return TNC_ERR_ARG;
}

extern "C" int tnc_svd_rows_df(int dtype, int64_t m, int64_t n, const void* A, void* W, void* S, int64_t* order,
                               int max_sweeps, double tol, int block_rows, int64_t nkeep, void* work,
                               size_t work_bytes, int* info, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TNC_C64)
    return svd_rows_df_impl<c64, dfc, c128>(m, n, (const c64*)A, W, (double*)S, order, max_sweeps, tol, block_rows,
                                            nkeep, work, work_bytes, info, st);
  if (dtype == TNC_F32)
    return svd_rows_df_impl<float, dfr, double>(m, n, (const float*)A, W, (double*)S, order, max_sweeps, tol,
                                                block_rows, nkeep, work, work_bytes, info, st);
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
