// mw_split.cuh -- double-FP32 ("split") arithmetic for sm_103.
//
// On GB300 the FP64 pipe retires about 1.9 FMA per clock per SM against
// about 118 for FP32, and FP64<->FP32 conversions (F2F) run on the FP64 pipe
// too.  A value is therefore carried as an unevaluated sum h + l of two
// floats (about 47 significant bits), built from the FP64 bit pattern with
// integer instructions, and combined with error-free transformations:
//   TwoSum (Knuth), FastTwoSum (Dekker), TwoProd via FMA (Dekker/Kahan),
// and the double-word algorithms analysed in M. Joldes, J.-M. Muller,
// V. Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017.  The addition used here is
// their "sloppy" double-word sum: its ABSOLUTE error is bounded by about
// 2^-47 (|x| + |y|), which is the quantity the per-variable normwise error
// of the time step depends on.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mw {
namespace split {

struct dw {
  float h, l;
};

__device__ __forceinline__ dw two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dw fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}

__device__ __forceinline__ dw two_prod(float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  return {p, e};
}

__device__ __forceinline__ dw neg(dw x) { return {-x.h, -x.l}; }

__device__ __forceinline__ dw add(dw x, dw y) {
  dw s = two_sum(x.h, y.h);
  float e = s.l + (x.l + y.l);
  return fast_two_sum(s.h, e);
}

__device__ __forceinline__ dw sub(dw x, dw y) { return add(x, neg(y)); }

// c + x when the exponent of c.h is at least that of x.h (a series coefficient
// plus a smaller Horner term): FastTwoSum replaces TwoSum for the leading parts.
__device__ __forceinline__ dw add_big(dw c, dw x) {
  const float s = c.h + x.h;
  const float e = ((c.h - s) + x.h) + (c.l + x.l);
  return fast_two_sum(s, e);
}

__device__ __forceinline__ dw mul(dw x, dw y) {
  float p = x.h * y.h;
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, e);
  e = fmaf(x.l, y.h, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ dw mulf(dw x, float y) {
  float p = x.h * y;
  float e = fmaf(x.h, y, -p);
  e = fmaf(x.l, y, e);
  return fast_two_sum(p, e);
}

// x*y + z for double-word x, y, z.
__device__ __forceinline__ dw fma_dw(dw x, dw y, dw z) { return add(mul(x, y), z); }

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// 1/y: hardware reciprocal estimate (relative error about 2^-23) refined by
// one Newton step r' = r + r (1 - y r) evaluated in double-word arithmetic.
__device__ __forceinline__ dw rcp(dw y) {
  float r = rcp_approx(y.h);
  float p = y.h * r;
  float pe = fmaf(y.h, r, -p);
  float e = ((1.0f - p) - pe) - y.l * r;
  return fast_two_sum(r, r * e);
}

// ---------------------------------------------------------------------------
// Conversions by integer operations on the IEEE-754 bit patterns.

// FP64 -> double-word.  h takes the leading 24 significand bits (truncated),
// l the other 29 rounded to 24 significant bits, so |x - (h + l)| <= 2^-47 |x|.
//   h: the float bit pattern is bits 60..29 of the double (one funnel shift)
//      with the exponent rebiased from 1023 to 127: adding 0x40000000 modulo
//      2^32 turns the low 8 exponent bits into the float exponent for every
//      exponent in float range; the sign is put back with one LOP3.
//   l: the 29 remaining significand bits as an integer, converted to float
//      (rounded to nearest) and scaled by sign * 2^(E - 52), E the exponent
//      of x, a float built from the bits of h.
// |x| < 2^-74 (zero included) gives (0, 0), absolute error < 6e-23; NaN, Inf
// and |x| >= 2^128 give NaN.
__device__ __forceinline__ dw from_f64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned ex = hi & 0x7ff00000u;
  const unsigned sh = __funnelshift_l(lo, hi, 3);
  const unsigned hb = ((sh + 0x40000000u) & 0x7fffffffu) | (hi & 0x80000000u);
  const float scale = __uint_as_float((hb & 0xff800000u) - (52u << 23));
  float h = __uint_as_float(hb);
  float l = __uint2float_rn(lo & 0x1fffffffu) * scale;
  // one unsigned range test; the rare out-of-range values take a branch
  if (ex - ((1023u - 74u) << 20) > ((74u + 127u) << 20)) {
    h = ex < ((1023u - 74u) << 20) ? 0.0f : __uint_as_float(0x7fc00000u);
    l = 0.0f;
  }
  return {h, l};
}

// FP32 -> FP64, exact (subnormal floats become 0, Inf/NaN stay Inf/NaN).
__device__ __forceinline__ double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = u & 0x7f800000u;
  unsigned hi = (((u >> 3) & 0x0fffffffu) + (896u << 20)) | (u & 0x80000000u);
  unsigned lo = u << 29;
  if (ex == 0u) {
    hi = u & 0x80000000u;
    lo = 0u;
  }
  if (ex == 0x7f800000u) hi |= 0x7ff00000u;
  return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

// double-word -> FP64: h + l on the FP64 pipe (one add, exact whenever the two
// parts span at most 53 bits, which holds for normalised pairs).
__device__ __forceinline__ double to_f64(dw x) { return f2d(x.h) + f2d(x.l); }

// The float's sign, exponent field and significand placed in a double without
// rebiasing the exponent: the double's value is exactly f * 2^-896 for every
// normal float, and 0 for zero (subnormal floats become values below 2^-1022,
// i.e. negligible).  Three integer operations; callers fold 2^896 into an FP64
// constant.  Inf / NaN are not preserved (see to_f64_scaled).
__device__ __forceinline__ double f2d_scaled(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned hi = ((u >> 3) & 0x0fffffffu) | (u & 0x80000000u);
  return __longlong_as_double((long long)(((unsigned long long)hi << 32) | (u << 29)));
}

// (h + l) * 2^-896 as an FP64 value (one FP64 add), for finite h.
__device__ __forceinline__ double to_f64_scaled_finite(dw x) { return f2d_scaled(x.h) + f2d_scaled(x.l); }

// (h + l) * 2^-896 as an FP64 value (one FP64 add); NaN when h is Inf or NaN.
__device__ __forceinline__ double to_f64_scaled(dw x) {
  const double v = f2d_scaled(x.h) + f2d_scaled(x.l);
  return (__float_as_uint(x.h) & 0x7f800000u) == 0x7f800000u ? __longlong_as_double(0x7ff8000000000000LL) : v;
}
constexpr double kTwoPow896 = 5.28294531135665246352339629e+269;  // 2^896

// FP64 -> FP32 rounded to nearest (ties away), by integer operations.
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const int ef = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  unsigned f = sign | ((unsigned)ef << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  f += (lo >> 28) & 1u;
  float r = __uint_as_float(f);
  const bool is_nan = ((hi & 0x7ff00000u) == 0x7ff00000u) && (((hi & 0xfffffu) | lo) != 0u);
  if (ef <= 0) r = __uint_as_float(sign);
  if (ef >= 255) r = __uint_as_float(is_nan ? 0x7fc00000u : (sign | 0x7f800000u));
  return r;
}

// Host-side split of an FP64 constant.
struct dwc {
  float h, l;
};
inline dwc split_host(double v) {
  dwc r;
  r.h = (float)v;
  r.l = (float)(v - (double)r.h);
  return r;
}
__device__ __forceinline__ dw ld(const dwc& c) { return {c.h, c.l}; }

// Device-side split of a per-launch constant, rounded exactly as split_host
// rounds it (two FP64->FP32 conversions; used once per work item, not per cell).
__device__ __forceinline__ dwc split_rn(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

}  // namespace split
}  // namespace mw
