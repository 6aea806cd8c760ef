// mw_split_flux.cuh -- the double-FP32 flux arithmetic shared by the split
// direction-stage kernels (mw_split_stage.cu) and their adjoint
// (mw_adjoint_split.cu).  Quantities are carried scaled by 12 so that the
// 4-point interpolation (-s0 + 7 s1 + 7 s2 - s3)/12 needs no division.
// Pressure: P_row ((1 + delta)^gamma - 1), delta = (rho theta)' / (rho theta)_bg,
// evaluated by its binomial series (pow_m1).
#pragma once

#include "mw_common.cuh"
#include "mw_split.cuh"
#include "mw_split2.cuh"

namespace mw {
namespace {
using namespace split;

constexpr double binom(double e, int n) {
  double c = e;
  for (int k = 1; k < n; ++k) c = c * (e - k) / (k + 1);
  return c;
}
constexpr float f_hi(double v) { return (float)v; }
constexpr float f_lo(double v) { return (float)(v - (double)(float)v); }

// Binomial series coefficients C(e, n): n = 1..6 as double-FP32 pairs, n = 1..16 in FP32.
struct PowTab {
  float h[7], l[7], f[17];
};
#define MW_POWTAB(e)                                                                                            \
  {{0.f, f_hi(binom(e, 1)), f_hi(binom(e, 2)), f_hi(binom(e, 3)), f_hi(binom(e, 4)), f_hi(binom(e, 5)),        \
    f_hi(binom(e, 6))},                                                                                         \
   {0.f, f_lo(binom(e, 1)), f_lo(binom(e, 2)), f_lo(binom(e, 3)), f_lo(binom(e, 4)), f_lo(binom(e, 5)),        \
    f_lo(binom(e, 6))},                                                                                         \
   {0.f, (float)binom(e, 1), (float)binom(e, 2), (float)binom(e, 3), (float)binom(e, 4), (float)binom(e, 5),    \
    (float)binom(e, 6), (float)binom(e, 7), (float)binom(e, 8), (float)binom(e, 9), (float)binom(e, 10),         \
    (float)binom(e, 11), (float)binom(e, 12), (float)binom(e, 13), (float)binom(e, 14), (float)binom(e, 15),     \
    (float)binom(e, 16)}}
__constant__ PowTab c_pow_g = MW_POWTAB(kGamma);          // pressure
__constant__ PowTab c_pow_gm1 = MW_POWTAB(kGamma - 1.0);  // its derivative
#undef MW_POWTAB

struct RowS {
  dw R;    // 12 * background rho
  dw RT;   // 12 * background rho*theta
  dw IRT;  // 1 / (12 * background rho*theta)
  dw P12;  // 12 * background pressure
};


// (1 + d)^e - 1 for the binomial series table T of exponent e: sum_n C(e, n) d^n.
// For |d| <= 1/64 (most cells) degree 8 leaves a tail below 2^-56 relative;
// terms 4..8 are summed in FP32, 1..3 in double-FP32 (the FP32 rounding of a
// Horner partial sum y_k reaches the result scaled by |d|^(k-1)).  For
// |d| <= 1/8, degree 16 with terms 7..16 in FP32; beyond that,
// expm1(e log1p(d)) in FP64.  Each coefficient exceeds the Horner term added
// to it (|C(e, n+1) d| < |C(e, n)| for these |d|), so the additions use
// FastTwoSum.
//
// Where the largest |d| of the warp's active lanes is small, fewer terms are
// evaluated (a warp-uniform choice, so no lane diverges): below 2^-49 the
// first-order term C(e, 1) d alone (the next is under 2^-48 of it), below
// 2^-24 degree 2, below 2^-16 degree 3, all in double-FP32.
__device__ __forceinline__ dw pow_m1(const PowTab& T, double e, dw d) {
  const float ad = fabsf(d.h);
  const float df = d.h;
  {
    const unsigned am = __activemask();
    // |d| as unsigned bits orders like the value (NaN above every finite |d|)
    const float mx = __uint_as_float(__reduce_max_sync(am, __float_as_uint(ad)));
    if (mx < 0x1p-16f) {
      const dw c1{T.h[1], T.l[1]};
      if (mx < 0x1p-49f) return mul(c1, d);
      if (mx < 0x1p-24f) return mul(add_big(c1, mulf(d, T.f[2])), d);
      const dw y = add_big(dw{T.h[2], T.l[2]}, mulf(d, T.f[3]));
      return mul(add_big(c1, mul(y, d)), d);
    }
  }
  // degree 8, computed for every cell so that it schedules with the
  // surrounding flux work; the rare larger |d| redo it below
  float t = fmaf(T.f[8], df, T.f[7]);
  t = fmaf(t, df, T.f[6]);
  t = fmaf(t, df, T.f[5]);
  t = fmaf(t, df, T.f[4]);
  dw y = add_big(dw{T.h[3], T.l[3]}, mulf(d, t));
  y = add_big(dw{T.h[2], T.l[2]}, mul(y, d));
  y = add_big(dw{T.h[1], T.l[1]}, mul(y, d));
  dw r = mul(y, d);
  if (ad > 0.015625f) {
    if (ad <= 0.125f) {
      float t16 = T.f[16];
#pragma unroll
      for (int n = 15; n >= 7; --n) t16 = fmaf(t16, df, T.f[n]);
      dw y16 = add_big(dw{T.h[6], T.l[6]}, mulf(d, t16));
#pragma unroll
      for (int n = 5; n >= 1; --n) y16 = add_big(dw{T.h[n], T.l[n]}, mul(y16, d));
      r = mul(y16, d);
    } else {
      r = from_f64(expm1(e * log1p(to_f64(d))));
    }
  }
  return r;
}

// (1 + d)^gamma - 1
__device__ __forceinline__ dw pgm1(dw d) { return pow_m1(c_pow_g, kGamma, d); }

// 12 * (4-point interpolation) = 7 (s1 + s2) - (s0 + s3) and the third
// difference (s3 - s0) - 3 (s2 - s1), for a pair of variables at once.  The
// leading floats are combined with error-free transformations (exact), the
// trailing floats and the rounding errors are summed in FP32 (error about
// 2^-48 of the operands), and each result is renormalised once.
// The products 7 a.h and 3 q.h are formed only negated (a7n = -a7 and q3n =
// -q3 exactly, rounding being symmetric), and the error-free steps that take
// them are written for the negated value, giving the same bits as the plain
// form: TwoSum(a7n, b.h) = -TwoDiff(a7, b.h), TwoSum(p.h, q3n) =
// TwoDiff(p.h, q3), and FastTwoSum(r.h, lo) = (RN(lo - rn.h), lo - RN(s + rn.h))
// with rn = -r.
__device__ __forceinline__ void interp2(dw2 s0, dw2 s1, dw2 s2, dw2 s3, dw2& A, dw2& D) {
  const float2 c7 = f2splat(7.0f), m7 = f2splat(-7.0f), c3 = f2splat(3.0f), m3 = f2splat(-3.0f);
  const dw2 a = two_sum2(s1.h, s2.h);
  const dw2 b = two_sum2(s0.h, s3.h);
  const float2 a7n = f2mul(a.h, m7);                  // -RN(7 a.h)
  const float2 a7e = f2fma(a.h, c7, a7n);             // exact: 7 a.h - RN(7 a.h)
  const dw2 rn = two_sum2(a7n, b.h);                  // -(7 a.h - b.h) exactly
  const float2 lo = f2sub(f2sub(f2fma(c7, f2add(f2add(s1.l, s2.l), a.l), a7e), f2add(f2add(s0.l, s3.l), b.l)), rn.l);
  const float2 Ah = f2sub(lo, rn.h);
  A = {Ah, f2sub(lo, f2add(Ah, rn.h))};
  const dw2 p = two_diff2(s3.h, s0.h);
  const dw2 q = two_diff2(s2.h, s1.h);
  const float2 q3n = f2mul(q.h, m3);                  // -RN(3 q.h)
  const float2 q3e = f2fma(q.h, c3, q3n);
  const dw2 t = two_sum2(p.h, q3n);
  const float2 lo2 =
      f2add(f2sub(f2add(f2sub(s3.l, s0.l), p.l), f2fma(c3, f2add(f2sub(s2.l, s1.l), q.l), q3e)), t.l);
  D = fast_two_sum2(t.h, lo2);
}

// The two halves of interp2 on their own: 7 (s1 + s2) - (s0 + s3) and
// (s3 - s0) - 3 (s2 - s1).
__device__ __forceinline__ dw2 acombo2(dw2 s0, dw2 s1, dw2 s2, dw2 s3) {
  const float2 c7 = f2splat(7.0f), m7 = f2splat(-7.0f);
  const dw2 a = two_sum2(s1.h, s2.h);
  const dw2 b = two_sum2(s0.h, s3.h);
  const float2 a7n = f2mul(a.h, m7);
  const float2 a7e = f2fma(a.h, c7, a7n);
  const dw2 rn = two_sum2(a7n, b.h);
  const float2 lo = f2sub(f2sub(f2fma(c7, f2add(f2add(s1.l, s2.l), a.l), a7e), f2add(f2add(s0.l, s3.l), b.l)), rn.l);
  const float2 Ah = f2sub(lo, rn.h);
  return {Ah, f2sub(lo, f2add(Ah, rn.h))};
}
__device__ __forceinline__ dw2 dcombo2(dw2 s0, dw2 s1, dw2 s2, dw2 s3) {
  const float2 c3 = f2splat(3.0f), m3 = f2splat(-3.0f);
  const dw2 p = two_diff2(s3.h, s0.h);
  const dw2 q = two_diff2(s2.h, s1.h);
  const float2 q3n = f2mul(q.h, m3);
  const float2 q3e = f2fma(q.h, c3, q3n);
  const dw2 t = two_sum2(p.h, q3n);
  const float2 lo2 =
      f2add(f2sub(f2add(f2sub(s3.l, s0.l), p.l), f2fma(c3, f2add(f2sub(s2.l, s1.l), q.l), q3e)), t.l);
  return fast_two_sum2(t.h, lo2);
}

// Hyperviscosity constant in paired form: HV = 12 hv in both lanes, nHV its negated leading float.
struct Hv2 {
  dw2 v;
  float2 nh;
};
__device__ __forceinline__ Hv2 make_hv2(dw hv12) { return {splat(hv12), f2splat(-hv12.h)}; }

// x flux times 12 (interpolate.py:105-129) for the taps s[pair][j], pairs
// (DENS, UMOM) and (WMOM, RHOT).  With u = (rho u)'/rho:
// F = ((rho u)', u (rho u)' + p', u (rho w)', u (rho theta)) - hv d3.
__device__ __forceinline__ void flux_x2(const dw2 s[2][4], const RowS& r, const Hv2& hv, dw2 F[2]) {
  dw2 A[2], D[2];
  interp2(s[0][0], s[0][1], s[0][2], s[0][3], A[0], D[0]);
  interp2(s[1][0], s[1][1], s[1][2], s[1][3], A[1], D[1]);
  const dw AD = lo_of(A[0]), AU = hi_of(A[0]), AW = lo_of(A[1]), AT = hi_of(A[1]);
  const dw ri = rcp(add(AD, r.R));
  const dw u = mul(AU, ri);
  const dw pp = mul(r.P12, pgm1(mul(AT, r.IRT)));
  const dw2 uu = mul2(splat(u), pack(AU, AW));
  const dw X1 = add(lo_of(uu), pp);
  const dw X3 = mul(u, add(AT, r.RT));
  F[0] = sub2(pack(AU, X1), mul2n(D[0], hv.v, hv.nh));
  F[1] = sub2(pack(hi_of(uu), X3), mul2n(D[1], hv.v, hv.nh));
}

// z flux times 12 (interpolate.py:153-186); w and d3[DENS] vanish at the walls.
__device__ __forceinline__ void flux_z2(const dw2 s[2][4], const RowS& r, const Hv2& hv, bool wall, dw2 F[2]) {
  dw2 A[2], D[2];
  interp2(s[0][0], s[0][1], s[0][2], s[0][3], A[0], D[0]);
  interp2(s[1][0], s[1][1], s[1][2], s[1][3], A[1], D[1]);
  const dw AD = lo_of(A[0]), AU = hi_of(A[0]), AT = hi_of(A[1]);
  dw rw = lo_of(A[1]);
  if (wall) {
    rw = dw{0.f, 0.f};
    D[0].h.x = 0.f;
    D[0].l.x = 0.f;
  }
  const dw ri = rcp(add(AD, r.R));
  const dw pp = mul(r.P12, pgm1(mul(AT, r.IRT)));
  const dw w = mul(rw, ri);
  const dw2 ww = mul2(splat(w), pack(AU, rw));
  const dw X2 = add(hi_of(ww), pp);
  const dw X3 = mul(w, add(AT, r.RT));
  F[0] = sub2(pack(rw, lo_of(ww)), mul2n(D[0], hv.v, hv.nh));
  F[1] = sub2(pack(X2, X3), mul2n(D[1], hv.v, hv.nh));
}

__device__ __forceinline__ RowS row_consts(double hy_r, double hy_rt, double P) {
  RowS r;
  r.R = from_f64(12.0 * hy_r);
  r.RT = from_f64(12.0 * hy_rt);
  r.IRT = from_f64(1.0 / (12.0 * hy_rt));
  r.P12 = from_f64(12.0 * P);
  return r;
}

__device__ __forceinline__ int wrap_x(int j, int nx) { return j < 0 ? j + nx : (j >= nx ? j - nx : j); }

__device__ __forceinline__ void pack4(const double v[4], dw2 out[2]) {
  out[0] = pack(from_f64(v[DENS]), from_f64(v[UMOM]));
  out[1] = pack(from_f64(v[WMOM]), from_f64(v[RHOT]));
}

}  // namespace
}  // namespace mw
