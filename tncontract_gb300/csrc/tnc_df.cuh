// Double-float ("DF") arithmetic for the extended-precision finish of the
// sweep's bond cores.
//
// GB300's FP64 pipe issues about 1.6 fused multiply-adds a clock per SM
// against about 116 for FP32 (both measured), so the finish that brings
// FP32-Jacobi rows to FP64-level orthogonality runs on the FP32 pipe instead:
// a real number is the unevaluated sum hi + lo of two floats (about 48
// significant bits), and every operation is built from the error-free
// transformations of floating-point arithmetic:
//   TwoSum  (Knuth, TAOCP vol. 2 4.2.2): s + e == a + b exactly, s = fl(a + b);
//   TwoProd (by FMA): p + e == a * b exactly, p = fl(a * b), e = fma(a, b, -p);
//   Dot2    (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J.
//            Sci. Comput. 26 (2005)): a dot product accumulated as a float
//            sum s plus a float compensation c of the TwoSum / TwoProd
//            errors, as accurate as if computed in twice the precision.
// Every primitive uses the _rn intrinsics so the compiler neither contracts
// nor reorders them.  The exponent range is FP32's: callers scale their data
// by a power of two to unit Frobenius norm first.
#pragma once

#include "tnc_persist.cuh"

namespace tnc {

struct __align__(8) dfr {
  float h, l;
  dfr() = default;
  __host__ __device__ dfr(float hh, float ll) : h(hh), l(ll) {}
  __host__ __device__ explicit dfr(double v) : h((float)v), l((float)(v - (double)(float)v)) {}
};
struct __align__(16) dfc {
  dfr re, im;
};

// rounding level of the DF data (2^-46: the Dot2 sums' error bound with
// margin), used for the rounding-noise floor of the rows
template <> struct traits<dfr> {
  typedef dfr real; static const bool is_complex = false;
  static constexpr double eps = 1.4210854715202004e-14;
};
template <> struct traits<dfc> {
  typedef dfr real; static const bool is_complex = true;
  static constexpr double eps = 1.4210854715202004e-14;
};

template <> __device__ __forceinline__ dfr ldcg<dfr>(const dfr* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return dfr(v.x, v.y);
}
template <> __device__ __forceinline__ dfc ldcg<dfc>(const dfc* p) {
  const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
  dfc r;
  r.re = dfr(v.x, v.y);
  r.im = dfr(v.z, v.w);
  return r;
}
template <> __device__ __forceinline__ void stcg<dfr>(dfr* p, dfr v) {
  __stcg(reinterpret_cast<float2*>(p), make_float2(v.h, v.l));
}
template <> __device__ __forceinline__ void stcg<dfc>(dfc* p, dfc v) {
  __stcg(reinterpret_cast<float4*>(p), make_float4(v.re.h, v.re.l, v.im.h, v.im.l));
}

__device__ __forceinline__ double to_double(dfr v) { return (double)v.h + (double)v.l; }

// TwoSum: s = fl(a + b), e = a + b - s exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (h, l) with h = fl(s + c): the normalised pair of an unevaluated sum
// (FastTwoSum: exact when |s| >= |c|, as for a compensated sum and its
// compensation; after a cancellation in df_add it is off by a few ulps of l)
__device__ __forceinline__ dfr df_norm(float s, float c) {
  const float h = __fadd_rn(s, c);
  return dfr(h, __fsub_rn(c, __fsub_rn(h, s)));
}

__device__ __forceinline__ dfr df_add(dfr a, dfr b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return df_norm(s, e);
}

// a * b for DF a, b (to about 2^-46 relative), unnormalised
__device__ __forceinline__ dfr df_mul(dfr a, dfr b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return dfr(p, e);
}

// Dot2 step: (s, c) += a * b with a = ah + al, b = bh + bl.  The hi product
// and the running sum are error-free transformed; the lo cross terms (about
// 2^-24 of the product) go into the compensation.
__device__ __forceinline__ void dot2_acc(float& s, float& c, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  const float e = __fmaf_rn(ah, bh, -p);
  float t;
  two_sum(s, p, s, t);
  c = __fadd_rn(c, __fadd_rn(t, e));
  c = __fmaf_rn(ah, bl, c);
  c = __fmaf_rn(al, bh, c);
}

// x += d for a DF x and a float d: the sum's rounding error joins the lo part
// (left unnormalised; lo stays a few ulps of hi over a finish)
__device__ __forceinline__ void df_acc(dfr& x, float d) {
  float s, e;
  two_sum(x.h, d, s, e);
  x.h = s;
  x.l = __fadd_rn(x.l, e);
}

// warp sum; every lane gets lane 0's result (identical on every lane)
__device__ __forceinline__ dfr warp_sum_df(dfr v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const dfr w(__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o));
    v = df_add(v, w);
  }
  return dfr(__shfl_sync(0xffffffffu, v.h, 0), __shfl_sync(0xffffffffu, v.l, 0));
}

}  // namespace tnc
