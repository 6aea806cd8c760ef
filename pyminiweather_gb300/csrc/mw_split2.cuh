// mw_split2.cuh -- pairs of double-FP32 values in packed FP32 instructions.
//
// sm_100-class SMs execute FP32 add / multiply / FMA on register pairs
// (f32x2): one issued instruction performs the same operation on two
// independent values.  dw2 holds two independent double-words,
// (h.x + l.x) and (h.y + l.y), and applies the algorithms of mw_split.cuh to
// both at once.  The direction-stage kernels pair the state variables as
// (DENS, UMOM) and (WMOM, RHOT), which halves the instruction count of the
// per-variable work (interpolation, hyperviscosity, flux differences).
#pragma once

#include <cuda_runtime.h>

#include "mw_split.cuh"

namespace mw {
namespace split {

struct dw2 {
  float2 h, l;
};

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b = RN(b * -1 + a): a packed FMA rounds once, exactly like a subtraction
// (there is no packed subtract intrinsic).
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 f2splat(float v) { return make_float2(v, v); }

__device__ __forceinline__ dw2 two_sum2(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  const float2 bb = f2sub(s, a);
  const float2 e = f2add(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
  return {s, e};
}
// a - b exactly as s + e
__device__ __forceinline__ dw2 two_diff2(float2 a, float2 b) {
  const float2 s = f2sub(a, b);
  const float2 bb = f2sub(s, a);  // -b as rounded
  const float2 e = f2sub(f2sub(a, f2sub(s, bb)), f2add(b, bb));
  return {s, e};
}
// requires |a| >= |b| (or a == 0) in each lane
__device__ __forceinline__ dw2 fast_two_sum2(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  return {s, f2sub(b, f2sub(s, a))};
}

__device__ __forceinline__ dw2 add2(dw2 x, dw2 y) {
  const dw2 s = two_sum2(x.h, y.h);
  return fast_two_sum2(s.h, f2add(s.l, f2add(x.l, y.l)));
}
__device__ __forceinline__ dw2 sub2(dw2 x, dw2 y) {
  const dw2 s = two_diff2(x.h, y.h);
  return fast_two_sum2(s.h, f2add(s.l, f2sub(x.l, y.l)));
}
// x * y; ny_h = -y.h (callers multiplying by a constant pass it precomputed)
// The leading product is formed only negated, pn = x.h * (-y.h) = -p exactly
// (rounding is symmetric), so FastTwoSum(p, e) is written with pn:
// s = RN(e - pn) = RN(p + e), err = e - RN(s + pn) = e - RN(s - p).
__device__ __forceinline__ dw2 mul2n(dw2 x, dw2 y, float2 ny_h) {
  const float2 pn = f2mul(x.h, ny_h);
  float2 e = f2fma(x.h, y.h, pn);  // exact product error: x.h*y.h - p
  e = f2fma(x.h, y.l, e);
  e = f2fma(x.l, y.h, e);
  const float2 sum = f2sub(e, pn);
  return {sum, f2sub(e, f2add(sum, pn))};
}
__device__ __forceinline__ dw2 mul2(dw2 x, dw2 y) {
  return mul2n(x, y, f2mul(y.h, make_float2(-1.f, -1.f)));
}

__device__ __forceinline__ dw2 pack(dw a, dw b) { return {make_float2(a.h, b.h), make_float2(a.l, b.l)}; }
__device__ __forceinline__ dw lo_of(dw2 p) { return {p.h.x, p.l.x}; }
__device__ __forceinline__ dw hi_of(dw2 p) { return {p.h.y, p.l.y}; }
__device__ __forceinline__ dw2 splat(dw a) { return {f2splat(a.h), f2splat(a.l)}; }

}  // namespace split
}  // namespace mw
