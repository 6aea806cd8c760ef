// mw_fp64_stage.cu -- direction-stage kernels in IEEE FP64 arithmetic with
// the fewest FP64 operations (f64_mode MW_F64_IEEE): the FP64 form of
// discrete_step (pyminiweather/solve/step.py:21-82).
//
// Every floating-point operation on state values is an FP64 add, multiply or
// FMA (no FP32 arithmetic on them, no double-FP32 pairs).  On GB300 the FP64
// pipe retires 2 operations per clock per SM, so one FP64 warp-instruction
// occupies it for 16 SM clocks, in which the SM can issue 64 other
// warp-instructions: the kernels are bound by their FP64 operation count, and
// integer work (conversions, index arithmetic, table look-ups) is nearly free.
// Against the reference's formulas (one pow, three divides and ~50 operations
// per interface, interpolate.py:82-186) each interface costs ~37 + n FP64
// operations and each cell update 8 (ncu: 47.6 per cell-stage in x, 49.3 in
// z on the collision case):
//   - quantities are carried scaled by 12, so the 4-point interpolation is
//     A = 7 (s1 + s2) - (s0 + s3) and needs no division; the third
//     difference is D = (s3 - s0) + 3 (s1 - s2): 6 operations per variable;
//   - one reciprocal per interface, 3 FP64 operations (ieee::rcp);
//   - pressure enters as the perturbation P_row ((1 + delta)^gamma - 1),
//     delta = (rho theta)' / (rho theta)_bg, P_row = C0 (rho theta)_bg^gamma:
//     exactly the reference's p - hy_pressure_int in z (hy_pressure_int is
//     C0 hy_dens_theta_int^gamma, ics/initial.py:105); in x the row constant
//     cancels in the flux difference.  (1 + delta)^gamma - 1 is its binomial
//     series summed by Horner's rule to the degree n that the warp's largest
//     |delta| needs for a truncation below 2^-54 relative (one FMA in a
//     region at rest, up to 15 terms for |delta| < 1/8), and
//     expm1(gamma log1p(delta)) beyond; the single-grid kernels evaluate it
//     as a polynomial in 12 (rho theta)' with per-row coefficients (RowP), n
//     operations in all;
//   - the stage update is out = init + c (F(i) - F(i+1)), c = dt / (12 d):
//     2 operations per value.
//
// x pass: warps walk 63-cell segments of the rows with no CTA barrier, lane l
// evaluating the fluxes at interfaces x0+l and x0+32+l (two independent FP64
// chains) from values staged in the warp's shared-memory slice.  z pass: one
// thread per column marching a tile of rows with a rolling 4-row window, so
// each interface flux is evaluated once.  Halo cells are never read: the
// periodic-x and wall-z rules of ics/bcs.py are applied to the indices and
// values as they are loaded.  Every global access goes through MW_AT
// (bounds-checked in the debug library).
#include <algorithm>
#include <atomic>

#include "mw_common.cuh"
#include "mw_ensemble.cuh"
#include "mw_fp64_math.cuh"

namespace mw {
namespace ieee {

constexpr int kXT = 256;            // threads per x CTA
constexpr int kZT = 128;            // columns per z CTA
constexpr int kZTileMax = 64;       // rows per z CTA
#ifndef MW_IEEE_X_SEGS_PER_WARP
#define MW_IEEE_X_SEGS_PER_WARP 16
#endif

// (1 + d)^gamma: the pressure perturbation.
__constant__ Series c_pow_g = make_series(kGamma);

// Row constants, scaled by 12 like the interpolated values.
struct RowD {
  double R12;    // 12 background rho
  double RT12;   // 12 background rho theta
  double IRT12;  // 1 / (12 background rho theta)
  double P12;    // 12 background pressure C0 (rho theta)^gamma
  double PC1;    // P12 C(gamma, 1) IRT12: the pressure perturbation per unit of 12 (rho theta)' to first order
};
__device__ __forceinline__ RowD row_consts(double r, double rt, double P) {
  const double irt = 1.0 / (12.0 * rt);
  return {12.0 * r, 12.0 * rt, irt, 12.0 * P, 12.0 * P * c_pow_g.c[1] * irt};
}

// P12 ((1 + d)^gamma - 1) + add, d = AT IRT12, for the lanes in `mask`, which
// call it together: the binomial series to the degree the largest |d| among
// them needs (a warp-uniform loop), or expm1(gamma log1p(d)) for |d| >= 1/8,
// Inf and NaN.  At degree 1 (|d| < 2^-52 on every lane, e.g. a region at
// rest) the series is P12 C1 d = AT PC1: one FMA in all.
__device__ __forceinline__ double pressure(double AT, const RowD& r, double add, unsigned mask) {
  const double d = AT * r.IRT12;
  bool big;
  const int n = series_degree(d, mask, c_pow_g, big);
  if (n == 1 && !__any_sync(mask, big)) return fma(AT, r.PC1, add);
  double f = d * series_g(d, n, c_pow_g);
  if (__any_sync(mask, big)) {
    if (big) f = expm1(kGamma * log1p(d));
  }
  return fma(r.P12, f, add);
}

// Row constants with the pressure series as a polynomial in the interpolated
// 12 (rho theta)' itself: b[n] = P12 C(gamma, n) IRT12^n, so that
// P12 ((1 + d)^gamma - 1) = sum_n b[n] AT^n (d = AT IRT12) is Horner's rule in
// AT with no multiplication by IRT12 before it and none by P12 after it: two
// FP64 operations fewer per interface wherever the degree exceeds one.
struct RowP {
  RowD d;
  double b[kMaxDeg + 1];  // b[0] unused
  int eI;                 // biased exponent of IRT12; 4096 where the b[n] would leave the normal range
  unsigned mI;            // an upper bound of 2^16 x IRT12's significand (in [1, 2)): top 16 fraction bits + 1
};
__device__ __forceinline__ RowP row_consts_p(double r, double rt, double P) {
  RowP o;
  o.d = row_consts(r, rt, P);
  double pw = o.d.IRT12;
  o.b[0] = 0.0;
#pragma unroll
  for (int n = 1; n <= kMaxDeg; ++n) {
    o.b[n] = o.d.P12 * c_pow_g.c[n] * pw;
    pw *= o.d.IRT12;
  }
  const double lo = fabs(o.b[kMaxDeg]), hi = fabs(o.b[1]);
  const bool normal = lo >= 0x1p-1000 && hi <= 0x1p1000 && pw >= 0x1p-1000;
  const unsigned long long bI = (unsigned long long)__double_as_longlong(o.d.IRT12);
  o.eI = normal ? (int)(bI >> 52 & 0x7ffu) : 4096;
  o.mI = (unsigned)(bI >> 36 & 0xffffu) + 0x10001u;
  return o;
}

// The same as pressure(AT, r.d, add, mask), evaluated in AT: the degree comes
// from an upper bound on the exponent of d = AT IRT12 (the sum of the exponents
// of AT and IRT12, plus one where the product of upper bounds of their leading
// 17 significand bits reaches 2), found by integer operations and never below
// the degree d itself needs; warps where the bound reaches 1/8 (and Inf, NaN,
// rows with eI = 4096) take the series in d.
__device__ __forceinline__ double pressure(double AT, const RowP& r, double add, unsigned mask) {
  const unsigned long long bA = (unsigned long long)__double_as_longlong(AT);
  const int exA = (int)(bA >> 52 & 0x7ffu);
  const unsigned mA = (unsigned)(bA >> 36 & 0xffffu) + 0x10001u;
  const int carry = (unsigned long long)mA * r.mI >= (1ull << 33) ? 1 : 0;
  const int eu = exA == 0 ? 0 : exA + r.eI - 1023 + carry;  // biased exponent of d is at most eu
  if (__any_sync(mask, eu >= 1020)) return pressure(AT, r.d, add, mask);
  const int exm = (int)__reduce_max_sync(mask, (unsigned)max(eu, 0));
  const int n = c_pow_g.deg[min(1022 - exm, 64)];
  double g = r.b[n];
  for (int k = n - 1; k >= 1; --k) g = fma(g, AT, r.b[k]);
  return fma(g, AT, add);
}

__device__ __forceinline__ const RowD& rowd(const RowD& r) { return r; }
__device__ __forceinline__ const RowD& rowd(const RowP& r) { return r.d; }

// 12 x the 4-point interpolation and the third difference of one variable
// (the stencils of interpolate.py:33-43 and 69-79).
__device__ __forceinline__ void interp(double s0, double s1, double s2, double s3, double& A, double& D) {
  A = interp12(s0, s1, s2, s3);
  D = fma(3.0, s1 - s2, s3 - s0);
}

// x flux times 12 (interpolate.py:82-129): with u = (rho u)' / rho,
// F = ((rho u)', u (rho u)' + p', u (rho w)', u (rho theta)) - hv d3, HV = -12 hv.
template <typename Row>
__device__ __forceinline__ void flux_x(const double s[4][4], const Row& r, double HV, unsigned mask, double F[4]) {
  double A[4], D[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) interp(s[q][0], s[q][1], s[q][2], s[q][3], A[q], D[q]);
  const double ri = rcp(A[DENS] + rowd(r).R12, mask);
  const double u = A[UMOM] * ri;
  F[0] = fma(HV, D[DENS], A[UMOM]);
  F[1] = fma(A[UMOM], u, pressure(A[RHOT], r, HV * D[UMOM], mask));
  F[2] = fma(u, A[WMOM], HV * D[WMOM]);
  F[3] = fma(u, A[RHOT] + rowd(r).RT12, HV * D[RHOT]);
}

// z flux times 12 (interpolate.py:132-186); w and d3[DENS] vanish at the walls.
template <typename Row>
__device__ __forceinline__ void flux_z(const double s[4][4], const Row& r, double HV, bool wall, unsigned mask,
                                       double F[4]) {
  double A[4], D[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) interp(s[q][0], s[q][1], s[q][2], s[q][3], A[q], D[q]);
  double AW = A[WMOM];
  if (wall) {
    AW = 0.0;
    D[DENS] = 0.0;
  }
  const double ri = rcp(A[DENS] + rowd(r).R12, mask);
  const double w = AW * ri;
  F[0] = fma(HV, D[DENS], AW);
  F[1] = fma(w, A[UMOM], HV * D[UMOM]);
  F[2] = fma(AW, w, pressure(A[RHOT], r, HV * D[WMOM], mask));
  F[3] = fma(w, A[RHOT] + rowd(r).RT12, HV * D[RHOT]);
}

// ---- arguments -------------------------------------------------------------
struct Args {
  int nx, nz, pitch;
  long long plane;
  const double* hyc;
  const double* hytc;
  const double* hyi;
  const double* hyti;
  const double* hypi;
  const double* srcw;
  const double* init;
  double* forcing;
  double* out;
  unsigned flags;
  double HV;    // -12 hv, hv = -hv_beta d / (16 dt_full) (interpolate.py:101,149)
  double c;     // dt_stage / (12 d)
  double dt;    // dt_stage (source terms)
  double gdt;   // -dt_stage grav (z)
  int z_tile;
  int r0, r1;   // output rows [r0, r1)
};

__device__ __forceinline__ int wrap_x(int j, int nx) { return j < 0 ? j + nx : (j >= nx ? j - nx : j); }

#define MW_F(a, off) MW_AT((a).forcing, (off), 4 * (a).plane)

// Forcing value of variable q at interior row k in [-2, nz+1] of the
// halo-indexed column col, with the wall rule of ics/bcs.py:92-148 in the halo rows.
__device__ __forceinline__ double zval(const Args& a, int q, int k, int col) {
  if (k >= 0 && k < a.nz) return MW_F(a, q * a.plane + (long long)(k + kHs) * a.pitch + col);
  if (q == WMOM) return 0.0;
  const int src = k < 0 ? kHs : a.nz + kHs - 1;
  const double s = MW_F(a, q * a.plane + (long long)src * a.pitch + col);
  if (q == UMOM) return s / MW_AT(a.hyc, src, a.nz + 2 * kHs) * MW_AT(a.hyc, k + kHs, a.nz + 2 * kHs);
  return s;
}

// Wall halo rows of one column of the forcing array: -2, -1 (bottom) from
// row 0, nz and nz+1 (top) from row nz-1.
__device__ __forceinline__ void write_z_halo_column(const Args& a, int col, bool bottom, bool top) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    if (!(h == 0 ? bottom : top)) continue;
    const int r0 = h == 0 ? -2 : a.nz;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double v0 = zval(a, q, r0, col), v1 = zval(a, q, r0 + 1, col);
      MW_F(a, q * a.plane + (long long)(r0 + kHs) * a.pitch + col) = v0;
      MW_F(a, q * a.plane + (long long)(r0 + 1 + kHs) * a.pitch + col) = v1;
    }
  }
}

// ---- x ---------------------------------------------------------------------
// x, warp segments: the CTA owns the contiguous range [g0, g1) of the
// row-major list of 63-cell segments (nseg per row) and splits it evenly over
// its eight warps, which walk their segments with no CTA barrier.  Lane l
// evaluates the fluxes at interfaces x0+l and x0+32+l (two independent FP64
// chains) from the segment's values staged in the warp's shared-memory slice,
// and updates cells x0+l and x0+32+l (l < 31) from its own and the next
// lane's fluxes.  The next segment's values are loaded one segment ahead; the
// row constants (an FP64 pow per row) are tabled once per CTA.
constexpr int kWI = 64;             // interfaces per warp segment
constexpr int kWCells = kWI - 1;    // cells per warp segment
constexpr int kXWarps = kXT / 32;
constexpr int kXRowsMax = 64;       // rows of one CTA's range
struct SmemXW {
  double sS[kXWarps][4][kWI + 4];   // [warp][variable][cell x0-2 .. x0+64]
};

// Walks the segments [g0, g1) of the row-major list of kWCells-cell segments
// (nseg per row); row_at(k) gives the constants of row k.  Every lane of the
// warp calls it; prologue() runs once, after the first segment's loads are
// issued (so that their latency overlaps it), also when the range is empty
// (it may contain a CTA barrier).  sS is the warp's shared-memory slice.
template <typename RowAt, typename Prologue>
__device__ __forceinline__ void x_warp_walk(const Args& a, int nseg, long long g0, long long g1, RowAt row_at,
                                            bool halo, double (*sS)[kWI + 4], Prologue prologue) {
  const int lane = threadIdx.x & 31;
  // values of the segment in row k at x0: cells x0-2+lane, x0+30+lane and (lanes 0..2) x0+62+lane
  auto load = [&](int k, int x0, double v[3][4]) {
    const long long row = (long long)(k + kHs) * a.pitch;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int c = x0 - 2 + 32 * j + lane;
      if ((j < 2 || lane < 3) && c <= a.nx + 1) {
        const long long col = wrap_x(c, a.nx) + kHs;
#pragma unroll
        for (int q = 0; q < 4; ++q) v[j][q] = __ldg(&MW_F(a, q * a.plane + row + col));
      }
    }
  };
  // (row, segment in row) of the current segment, advanced incrementally (one
  // 64-bit division per walk, not per segment)
  int k = (int)(g0 / nseg), sg = (int)(g0 - (long long)k * nseg);
  double v[3][4] = {};
  if (g0 < g1) load(k, sg * kWCells, v);
  prologue();
  for (long long g = g0; g < g1; ++g) {
    const int x0 = sg * kWCells;
    const int kn = sg + 1 == nseg ? k + 1 : k, sgn = sg + 1 == nseg ? 0 : sg + 1;  // the next segment
    const long long row = (long long)(k + kHs) * a.pitch;
    __syncwarp();  // the previous segment's taps are read
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (j < 2 || lane < 3)
#pragma unroll
        for (int q = 0; q < 4; ++q) sS[q][32 * j + lane] = v[j][q];
    if (halo && sg == 0 && lane < 4) {  // columns 0, 1 <- nx, nx+1; nx+2, nx+3 <- 2, 3 (ics/bcs.py:35-39)
      const int dst = lane < 2 ? lane : a.nx + lane, src = lane < 2 ? a.nx + lane : lane;
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_F(a, q * a.plane + row + dst) = MW_F(a, q * a.plane + row + src);
    }
    if (g + 1 < g1) load(kn, sgn * kWCells, v);
    const int ia = x0 + lane, ib = x0 + 32 + lane;  // interfaces (and cells) of this lane
    const bool ua = ia < a.nx, ub = lane < 31 && ib < a.nx;
    double iva[4], ivb[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (ua) iva[q] = MW_AT(a.init, q * a.plane + row + ia + kHs, 4 * a.plane);
      if (ub) ivb[q] = MW_AT(a.init, q * a.plane + row + ib + kHs, 4 * a.plane);
    }
    __syncwarp();
    const auto& rc = row_at(k);
    double Fa[4] = {0, 0, 0, 0}, Fb[4] = {0, 0, 0, 0};
    const unsigned ma = __ballot_sync(0xffffffffu, ia <= a.nx), mb = __ballot_sync(0xffffffffu, ib <= a.nx);
    if (ia <= a.nx) {
      double s[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int j = 0; j < 4; ++j) s[q][j] = sS[q][lane + j];
      flux_x(s, rc, a.HV, ma, Fa);
    }
    if (ib <= a.nx) {
      double s[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int j = 0; j < 4; ++j) s[q][j] = sS[q][32 + lane + j];
      flux_x(s, rc, a.HV, mb, Fb);
    }
    // lane l needs the flux at interface x0+l+1: lane l+1's Fa, or for l = 31 lane 0's Fb
    double Fa1[4], Fb1[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      Fa1[q] = __shfl_sync(0xffffffffu, lane == 0 ? Fb[q] : Fa[q], (lane + 1) & 31);
      Fb1[q] = __shfl_down_sync(0xffffffffu, Fb[q], 1);
    }
    if (ua) {
      double o[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) o[q] = fma(a.c, Fa[q] - Fa1[q], iva[q]);
      if (a.srcw) o[WMOM] = fma(a.dt, MW_AT(a.srcw, (long long)k * a.nx + ia, (long long)a.nx * a.nz), o[WMOM]);
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_AT(a.out, q * a.plane + row + ia + kHs, 4 * a.plane) = o[q];
    }
    if (ub) {
      double o[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) o[q] = fma(a.c, Fb[q] - Fb1[q], ivb[q]);
      if (a.srcw) o[WMOM] = fma(a.dt, MW_AT(a.srcw, (long long)k * a.nx + ib, (long long)a.nx * a.nz), o[WMOM]);
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_AT(a.out, q * a.plane + row + ib + kHs, 4 * a.plane) = o[q];
    }
    k = kn;
    sg = sgn;
  }
}

#ifndef MW_IEEE_X_MIN_BLOCKS
#define MW_IEEE_X_MIN_BLOCKS 2
#endif
// Single grid: the CTA owns the contiguous range [g0, g1) of segments of rows
// [r0, r1) and splits it evenly over its warps; the row constants (an FP64 pow
// per row) are tabled once per CTA while the warps' first loads are in flight.
__global__ void __launch_bounds__(kXT, MW_IEEE_X_MIN_BLOCKS) k_stage_x_ieee_w(Args a, int nseg, long long total,
                                                                               long long gbase) {
  __shared__ SmemXW sm;
  __shared__ RowP rows[kXRowsMax];
  const long long g0 = gbase + total * blockIdx.x / gridDim.x, g1 = gbase + total * (blockIdx.x + 1) / gridDim.x;
  if (g0 >= g1) return;
  const int row0 = (int)(g0 / nseg), nrows = (int)((g1 - 1) / nseg) - row0 + 1;  // nrows <= kXRowsMax (host)
  const int w = threadIdx.x >> 5;
  const long long n = g1 - g0;
  x_warp_walk(a, nseg, g0 + n * w / kXWarps, g0 + n * (w + 1) / kXWarps,
              [&](int k) -> const RowP& { return rows[k - row0]; },
              a.flags & MW_FLAG_WRITE_HALO, sm.sS[w], [&]() {
                for (int r = threadIdx.x; r < nrows; r += kXT) {
                  const double rt = MW_AT(a.hytc, row0 + r + kHs, a.nz + 2 * kHs);
                  rows[r] = row_consts_p(MW_AT(a.hyc, row0 + r + kHs, a.nz + 2 * kHs), rt, kC0 * pow(rt, kGamma));
                }
                __syncthreads();
              });
}

// ---- z ---------------------------------------------------------------------
struct SmemZ {
  RowP row[kZTileMax + 1];
};

// Columns [cb*NC, cb*NC+NC), rows [z0, z1), z1 - z0 <= kZTileMax; every
// thread of the CTA calls it.  hbot / htop: write the bottom / top wall halo
// rows of these columns (cb == 0 also of the four x-halo columns).
template <int NC>
__device__ __forceinline__ void z_tile(const Args& a, int cb, int z0, int z1, bool hbot, bool htop, SmemZ& sm) {
  for (int rr = threadIdx.x; rr <= z1 - z0; rr += NC) {
    const int k = z0 + rr;
    sm.row[rr] = row_consts_p(MW_AT(a.hyi, k, a.nz + 1), MW_AT(a.hyti, k, a.nz + 1), MW_AT(a.hypi, k, a.nz + 1));
  }
  __syncthreads();
  const int c = cb * NC + threadIdx.x;  // interior column
  if ((hbot || htop) && cb == 0 && threadIdx.x < 4)
    write_z_halo_column(a, threadIdx.x < 2 ? threadIdx.x : a.nx + threadIdx.x, hbot, htop);
  const unsigned mask = __ballot_sync(0xffffffffu, c < a.nx);
  if (c < a.nx) {
    const int col = c + kHs;
    if (hbot || htop) write_z_halo_column(a, col, hbot, htop);
    double w[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q][j] = zval(a, q, z0 - 2 + j, col);
    double nxt[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) nxt[q] = zval(a, q, z0 + 2, col);
    double Fp[4];
    flux_z(w, sm.row[0], a.HV, z0 == 0, mask, Fp);
    for (int k = z0; k < z1; ++k) {
      const long long o = (long long)(k + kHs) * a.pitch + col;
      double iv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) iv[q] = MW_AT(a.init, q * a.plane + o, 4 * a.plane);
      const double rho_k = w[DENS][2];  // forcing rho' at cell k (interpolate.py:248-250)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        w[q][0] = w[q][1];
        w[q][1] = w[q][2];
        w[q][2] = w[q][3];
        w[q][3] = nxt[q];
      }
      if (k + 1 < z1) {  // the row the next iteration needs, loaded one step ahead
#pragma unroll
        for (int q = 0; q < 4; ++q) nxt[q] = zval(a, q, k + 3, col);
      }
      double Fn[4];
      flux_z(w, sm.row[k + 1 - z0], a.HV, k + 1 == a.nz, mask, Fn);
      double v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = fma(a.c, Fp[q] - Fn[q], iv[q]);
      v[WMOM] = fma(a.gdt, rho_k, v[WMOM]);
      if (a.srcw) v[WMOM] = fma(a.dt, MW_AT(a.srcw, (long long)k * a.nx + c, (long long)a.nx * a.nz), v[WMOM]);
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_AT(a.out, q * a.plane + o, 4 * a.plane) = v[q];
#pragma unroll
      for (int q = 0; q < 4; ++q) Fp[q] = Fn[q];
    }
  }
  __syncthreads();  // the row table is rewritten by the next tile
}

// Tiles of a.z_tile rows of [a.r0, a.r1), one per CTA row.
__global__ void __launch_bounds__(kZT) k_stage_z_ieee(Args a, int tile0) {
  __shared__ SmemZ sm;
  const int tile = tile0 + blockIdx.y;  // grid.y is capped at 65535: one launch per 65535 tiles
  const int z0 = a.r0 + tile * a.z_tile, z1 = min(z0 + a.z_tile, a.r1);
  const bool halo = a.flags & MW_FLAG_WRITE_HALO;
  z_tile<kZT>(a, blockIdx.x, z0, z1, halo && z0 == 0, halo && z1 == a.nz, sm);
}

// ---- ensembles -------------------------------------------------------------
// One persistent launch per direction-stage walks a work list over all members
// (x items: member rows; z items: member column-block tiles).  Each member's
// stage constants were formed on the host with the plan, exactly as
// launch_stage_ieee forms them for a single grid, and the x row constants
// come from a table the step call writes once (no FP64 pow per row).
__device__ __forceinline__ Args member_args(const EnsStage& es, int e) {
  const mw_ens_member m = MW_AT(es.members, e, es.n_members);
  Args a;
  a.nx = m.nx;
  a.nz = m.nz;
  a.pitch = m.nx + 2 * kHs;
  a.plane = (long long)(m.nz + 2 * kHs) * a.pitch;
  a.hyc = es.hyc + m.cell_off;
  a.hytc = es.hytc + m.cell_off;
  a.hyi = es.hyi + m.int_off;
  a.hyti = es.hyti + m.int_off;
  a.hypi = es.hypi + m.int_off;
  a.srcw = nullptr;
  a.init = es.init + m.state_off;
  a.forcing = es.forcing + m.state_off;
  a.out = es.out + m.state_off;
  a.flags = es.flags;
  const EnsMemberConsts& c = MW_AT(reinterpret_cast<const EnsMemberConsts*>(es.mconsts), mconsts_index(es, e),
                                   (long long)kEnsConstsPerMember * es.n_members);
  a.HV = c.HV;
  a.c = c.c;
  a.dt = c.dt;
  a.gdt = c.gdt;
  a.z_tile = es.z_tile;
  a.r0 = 0;
  a.r1 = m.nz;
  return a;
}

static_assert(sizeof(RowD) <= kEnsRowBytes, "row-constant table entry size");

__global__ void k_ens_row_table_ieee(const double* hyc, const double* hytc, long long n, RowD* table) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
    const double rt = MW_AT(hytc, j, n);
    MW_AT(table, j, n) = row_consts(MW_AT(hyc, j, n), rt, kC0 * pow(rt, kGamma));
  }
}

// x items are rows (member, row), one per warp: the warp walks the row's
// segments as the single-grid kernel does.
__global__ void __launch_bounds__(kXT, MW_IEEE_X_MIN_BLOCKS) k_ens_x_ieee(EnsStage es) {
  __shared__ SmemXW sm;
  const int w = threadIdx.x >> 5;
  for (unsigned it = ens_take_warp(es.cursor); it < (unsigned)es.n_items; it = ens_take_warp(es.cursor)) {
    const int2 item = MW_AT(es.items, it, es.n_items);  // (member, row)
    const Args a = member_args(es, item.x);
    const int nseg = (a.nx + kWCells - 1) / kWCells;
    const RowD r = MW_AT(reinterpret_cast<const RowD*>(es.xrows),
                         MW_AT(es.members, item.x, es.n_members).cell_off + item.y + kHs, es.n_xrows);
    x_warp_walk(a, nseg, (long long)item.y * nseg, (long long)(item.y + 1) * nseg,
                [&](int) -> const RowD& { return r; },
                a.flags & MW_FLAG_WRITE_HALO, sm.sS[w], []() {});
  }
  ens_finish(es.cursor);
}

__global__ void __launch_bounds__(kEnsZCols) k_ens_z_ieee(EnsStage es) {
  __shared__ SmemZ sm;
  __shared__ unsigned slot[2];
  int parity = 0;
  for (unsigned it = ens_take_cta(es.cursor, slot, parity); it < (unsigned)es.n_items;
       it = ens_take_cta(es.cursor, slot, parity)) {
    const int2 item = MW_AT(es.items, it, es.n_items);  // (member, column block + ncb * tile)
    const Args a = member_args(es, item.x);
    const int ncb = (a.nx + kEnsZCols - 1) / kEnsZCols;
    const int cb = item.y % ncb, tile = item.y / ncb;
    const int z0 = tile * es.z_tile, z1 = min(z0 + es.z_tile, a.nz);
    const bool halo = a.flags & MW_FLAG_WRITE_HALO;
    z_tile<kEnsZCols>(a, cb, z0, z1, halo && z0 == 0, halo && z1 == a.nz, sm);
  }
  ens_finish(es.cursor);
}

// CTAs of k_stage_x_ieee_w (which 0) / k_stage_z_ieee (which 1) resident on
// the current device, cached per device.
int resident_ctas(int which, int* out) {
  static std::atomic<int> cache[2][64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(MW_ERR_CUDA, "cudaGetDevice failed");
  const bool cached = dev >= 0 && dev < 64;
  if (cached && (*out = cache[which][dev].load(std::memory_order_relaxed)) > 0) return MW_OK;
  int per_sm = 0, sms = 0;
  cudaError_t e = which == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_x_ieee_w, kXT, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_z_ieee, kZT, 0);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  *out = std::max(1, per_sm) * sms;
  if (cached) cache[which][dev].store(*out, std::memory_order_relaxed);
  return MW_OK;
}

}  // namespace ieee

int launch_ens_ieee(const EnsStage& es, int grid) {
  using namespace ieee;
  if (es.n_items == 0) return MW_OK;
  if (es.direction == MW_DIR_X)
    k_ens_x_ieee<<<grid, kXT, 0, es.stream>>>(es);
  else
    k_ens_z_ieee<<<grid, kEnsZCols, 0, es.stream>>>(es);
  return check_launch("ensemble IEEE-FP64 stage launch");
}

int ens_ieee_occupancy(int direction, int* blocks_per_sm) {
  using namespace ieee;
  cudaError_t e = direction == MW_DIR_X
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_ens_x_ieee, kXT, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_ens_z_ieee, kEnsZCols, 0);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  return MW_OK;
}

int launch_ens_ieee_rowtable(const double* hyc, const double* hytc, long long n, void* table, cudaStream_t stream) {
  using namespace ieee;
  if (n <= 0) return MW_OK;
  MW_REQUIRE(((uintptr_t)table % 16) == 0, MW_ERR_ALIGN, "row table misaligned");
  const long long blocks = std::min<long long>((n + 127) / 128, 4096);
  k_ens_row_table_ieee<<<(unsigned)blocks, 128, 0, stream>>>(hyc, hytc, n, (RowD*)table);
  return check_launch("ensemble row-table launch");
}

// One direction-stage in the IEEE-FP64 form over output rows [r0, r1) (the
// whole grid: 0, nz); arguments validated by the caller.
int launch_stage_ieee(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                      const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                      const double* init, double* forcing, double* out, double dt_stage, int direction,
                      unsigned flags, int r0, int r1, cudaStream_t stream) {
  using namespace ieee;
  MW_REQUIRE(0 <= r0 && r0 < r1 && r1 <= nz, MW_ERR_INVALID_ARG, "row range [%d, %d) outside [0, %d)", r0, r1, nz);
  const Geom g = make_geom(nx, nz);
  Args a;
  a.nx = nx;
  a.nz = nz;
  a.pitch = g.pitch;
  a.plane = g.plane;
  a.hyc = hyc;
  a.hytc = hytc;
  a.hyi = hyi;
  a.hyti = hyti;
  a.hypi = hypi;
  a.srcw = srcw;
  a.init = init;
  a.forcing = forcing;
  a.out = out;
  a.flags = flags;
  const double d = direction == MW_DIR_X ? dx : dz;
  a.HV = 12.0 * kHvBeta * d / (16 * dt_full);  // -12 hv
  a.c = dt_stage / (12.0 * d);
  a.dt = dt_stage;
  a.gdt = -dt_stage * kGrav;
  a.r0 = r0;
  a.r1 = r1;
  const int rows = r1 - r0;
  if (direction == MW_DIR_Z) {
    // rows per z CTA: at most kZTileMax and at least 8 (each tile re-reads 4
    // window rows), chosen so that the launch is a whole number of resident
    // waves or just under (CTAs cost about the same, so a partly filled last
    // wave would idle SMs; one wave for the bands of the host-buffer step)
    int resident = 0, st = resident_ctas(1, &resident);
    if (st) return st;
    const long long ncb = (nx + kZT - 1) / kZT;
    const long long waves = std::max(1LL, ((long long)rows * ncb + (long long)kZTileMax * resident - 1) /
                                              ((long long)kZTileMax * resident));
    const long long tiles = std::max(1LL, waves * resident / ncb);
    a.z_tile = (int)std::max(8LL, std::min<long long>(kZTileMax, (rows + tiles - 1) / tiles));
  } else {
    a.z_tile = kZTileMax;
  }
  if (direction == MW_DIR_X) {
    // About MW_IEEE_X_SEGS_PER_WARP segments per warp in a whole number of
    // resident waves of equal ranges (one wave, at least one segment per warp,
    // for small grids); at most kXRowsMax rows per CTA range.
    const int nseg = (nx + kWCells - 1) / kWCells;
    const long long total = (long long)nseg * rows;
    int resident = 0, st = resident_ctas(0, &resident);
    if (st) return st;
    long long grid = std::min<long long>(resident, (total + kXWarps - 1) / kXWarps);
    grid = std::max<long long>(grid, total / (kXWarps * MW_IEEE_X_SEGS_PER_WARP));
    if (grid > resident) grid = (grid + resident - 1) / resident * resident;
    grid = std::max<long long>(grid, (rows + kXRowsMax - 3) / (kXRowsMax - 2));
    MW_REQUIRE(grid <= 0x7fffffffLL, MW_ERR_SHAPE, "grid too large for the x direction-stage launch");
    k_stage_x_ieee_w<<<(unsigned)grid, kXT, 0, stream>>>(a, nseg, total, (long long)r0 * nseg);
  } else {
    const int ntiles = (rows + a.z_tile - 1) / a.z_tile;
    for (int t0 = 0; t0 < ntiles; t0 += 65535) {
      dim3 grid((nx + kZT - 1) / kZT, (unsigned)std::min(ntiles - t0, 65535));
      k_stage_z_ieee<<<grid, kZT, 0, stream>>>(a, t0);
      if (t0 + 65535 < ntiles) {
        const int st = check_launch("z IEEE-FP64 direction-stage launch");
        if (st) return st;
      }
    }
  }
  return check_launch(direction == MW_DIR_X ? "x IEEE-FP64 direction-stage launch"
                                            : "z IEEE-FP64 direction-stage launch");
}

#if MW_CHECK
MW_OOB_COUNTER(oob_count_ieee_stage)
#endif

}  // namespace mw
