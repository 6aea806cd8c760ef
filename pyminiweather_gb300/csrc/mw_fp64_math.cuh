// mw_fp64_math.cuh -- IEEE-FP64 building blocks of the fewest-operation form
// (f64_mode MW_F64_IEEE), shared by its direction-stage kernels
// (mw_fp64_stage.cu) and its adjoint (mw_adjoint.cu).  Every floating-point
// operation on state values is an FP64 add, multiply or FMA; integer
// instructions (bit conversions, table look-ups) are nearly free beside them
// on GB300, whose FP64 pipe retires 2 operations per clock per SM.
#pragma once

#include "mw_common.cuh"

namespace mw {
namespace ieee {

constexpr double binom(double e, int n) {  // C(e, n)
  double c = 1.0;
  for (int k = 0; k < n; ++k) c = c * (e - k) / (k + 1);
  return c;
}
constexpr double cabs(double v) { return v < 0 ? -v : v; }

// The binomial series (1 + d)^e = sum_n C(e, n) d^n: coefficients c[n] and,
// for |d| < 2^-s (s >= 3), the Horner degree deg[s] -- the smallest n with
// |C(e, n+1) / C(e, 1)| 2^(-s n) <= 2^-54, a truncation below half an FP64
// ulp of the first-order term.  |d| >= 1/8 is left to expm1 / log1p.
constexpr int kMaxDeg = 15;
struct Series {
  double c[kMaxDeg + 1];
  unsigned char deg[65];
};
constexpr Series make_series(double e) {
  Series t{};
  for (int n = 0; n <= kMaxDeg; ++n) t.c[n] = binom(e, n);
  for (int s = 0; s <= 64; ++s) {
    int n = kMaxDeg;
    if (s >= 3) {
      for (n = 1; n < kMaxDeg; ++n) {
        double b = cabs(binom(e, n + 1) / binom(e, 1));
        for (int j = 0; j < s * n && b > 0.0; ++j) b *= 0.5;
        if (b <= 5.551115123125783e-17) break;  // 2^-54
      }
    }
    t.deg[s] = (unsigned char)n;
  }
  return t;
}

// 1/y for the lanes in `mask`, which call it together: an FP32 estimate
// (operand and result converted by integer operations) refined by one cubic
// Newton step in FP64, r = r0 (1 + e + e^2), e = 1 - y r0, whose relative
// error e^3 <= 2^-66 lies below FP64 rounding: 3 FP64 operations.  |y|
// outside [2^-125, 2^126) (and Inf, NaN, 0) takes the FP64 division, behind
// a warp-uniform branch so that it is never evaluated speculatively on the
// other lanes.
__device__ __forceinline__ double rcp(double y, unsigned mask) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(y);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned ex = (hi >> 20) & 0x7ffu;
  // float with y's sign, rebiased exponent and leading 23 significand bits
  const unsigned fb = ((__funnelshift_l(lo, hi, 3) + 0x40000000u) & 0x7fffffffu) | (hi & 0x80000000u);
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(fb)));
  const unsigned rb = __float_as_uint(rf);
  const unsigned rhi = (((rb >> 3) & 0x0fffffffu) + (896u << 20)) | (rb & 0x80000000u);
  const double r0 = __longlong_as_double((long long)(((unsigned long long)rhi << 32) | (rb << 29)));
  const double e = fma(-y, r0, 1.0);
  const double t = fma(e, e, e);
  double r = fma(r0, t, r0);
  const bool out = ex - (1023u - 125u) > 250u;
  if (__any_sync(mask, out)) {
    if (out) r = 1.0 / y;
  }
  return r;
}

// The Horner degree of series S that the largest |d| among the lanes in
// `mask` (which call it together) needs; big: this lane's |d| >= 1/8 (or
// Inf / NaN), left out of the degree and to be evaluated otherwise.
__device__ __forceinline__ int series_degree(double d, unsigned mask, const Series& S, bool& big) {
  const unsigned ex = ((unsigned)((unsigned long long)__double_as_longlong(d) >> 52)) & 0x7ffu;
  big = ex >= 1020u;  // |d| >= 2^-3
  const unsigned exm = __reduce_max_sync(mask, big ? 0u : ex);
  const int s = min(1022 - (int)exm, 64);  // |d| < 2^-s for every series lane
  return S.deg[s];
}

// g with (1 + d)^e - 1 = d g: Horner's rule over c[n] .. c[1] (n - 1 FMAs).
__device__ __forceinline__ double series_g(double d, int n, const Series& S) {
  double g = S.c[n];
  for (int k = n - 1; k >= 1; --k) g = fma(g, d, S.c[k]);
  return g;
}

// 12 x the 4-point interpolation (the stencil of interpolate.py:33-43 and
// 69-79 with its division by 12 folded into the scaling).
__device__ __forceinline__ double interp12(double s0, double s1, double s2, double s3) {
  return fma(7.0, s1 + s2, -(s0 + s3));
}

}  // namespace ieee
}  // namespace mw
