// mw_adjoint_split.cu -- the direction-stage adjoint (vector-Jacobian product)
// with the interior arithmetic in double-FP32, the split counterpart of
// mw_adjoint.cu.  Storage, the adjoint inputs and outputs stay FP64.
//
// For one direction-stage out = init + (dt/(12 d)) (F12(i) - F12(i+1)), with
// F12 the flux scaled by 12 (mw_split_flux.cuh), and g = dJ/d(out):
//   G(f)   = g(f) - g(f-1)                       (interface f; g = 0 beyond the walls in z,
//                                                  periodic in x, where interfaces 0 and nx coincide)
//   AbG(f) = J(f)^T G(f)                         (J = dF/dA, scale-free)
//   S(t)   = acombo(AbG[t-1..t+2]) + 12 hv dcombo(Gd[t-1..t+2])
//   g_dst(t) = bases + dt/(12 d) S(t)  [- dt grav g_w(t) on rho' in z]
// acombo / dcombo are the interpolation and third-difference combinations of
// the forward (the taps' weights transposed), Gd = G with the rho' component
// zeroed at the z walls (where d3[DENS] is held at zero, interpolate.py:167-173).
// With u = (rho u)'/rho, w = (rho w)'/rho, theta = rho theta/rho and
// dp = gamma p/(rho theta) = gamma P_bg/(rho theta)_bg (1 + delta)^(gamma-1),
// X = G_U u + G_W w + G_T theta:
//   x: AbG = (-u X, G_D + G_U u + X, G_W u, G_U dp + G_T u)
//   z: AbG = (-w X, G_U w, G_D + G_W w + X, G_W dp + G_T w); at the walls only (0, 0, 0, G_W dp).
// In z, taps in the halo rows map back to rows 0 and nz-1 through the wall
// rule (bcs.py:92-148): rho', (rho theta)' copied, (rho u)' scaled by the
// background ratio, (rho w)' zero.
//
// One kernel per stage: a warp walks 29-cell segments of a line (a row in x,
// a column in z); lane l owns interface p0-1+l and, for l < 29, cell p0+l.
// In x the warps read their rows directly; in z (k_vjp_split_zt) a CTA stages
// a tile of a few columns x one segment through shared memory so that every
// global access is row-contiguous.  Interface background constants come from
// a table that k_vjp_row_table writes into the caller's workspace.
#include <algorithm>

#include "mw_common.cuh"
#include "mw_split_flux.cuh"

namespace mw {
namespace {
using namespace split;

constexpr int kVThreads = 256;
constexpr int kVWarps = kVThreads / 32;
constexpr int kVCells = 29;            // cells per warp segment
constexpr int kVVals = kVCells + 6;    // staged forcing positions p0-3 .. p0+31

// Interface (z) or row (x) background constants, all scaled by 12 like the flux.
struct RowV {
  dw R;    // 12 rho_bg
  dw RT;   // 12 (rho theta)_bg
  dw IRT;  // 1 / (12 (rho theta)_bg)
  dw GPI;  // gamma P_bg / (rho theta)_bg
};

struct VjpSplitArgs {
  int nx, nz, pitch;
  long long plane;
  const double* hyc;
  const RowV* rows;      // x: nz rows; z: nz + 1 interfaces
  const double* forcing;
  const double* gout;
  const double* base_a;
  const double* base_b;
  int add_gout;
  double* gdst;
  dwc hv12;              // 12 hv
  double cs;             // 2^896 dt_stage / (12 d)
  double dtg;            // dt_stage grav (z)
};

__global__ void k_vjp_row_table(const double* hyc, const double* hytc, const double* hyi, const double* hyti,
                                const double* hypi, int nx, int nz, RowV* tx, RowV* tz) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= 2 * nz; r += gridDim.x * blockDim.x) {
    double rho, rt, P;
    RowV* dst;
    if (r < nz) {  // x rows: cell-centre background, P = C0 (rho theta)^gamma
      rho = MW_AT(hyc, r + kHs, nz + 2 * kHs);
      rt = MW_AT(hytc, r + kHs, nz + 2 * kHs);
      P = kC0 * pow(rt, kGamma);
      dst = tx + r;
    } else {       // z interfaces
      const int k = r - nz;
      rho = MW_AT(hyi, k, nz + 1);
      rt = MW_AT(hyti, k, nz + 1);
      P = MW_AT(hypi, k, nz + 1);
      dst = tz + k;
    }
    RowV v;
    v.R = from_f64(12.0 * rho);
    v.RT = from_f64(12.0 * rt);
    v.IRT = from_f64(1.0 / (12.0 * rt));
    v.GPI = from_f64(kGamma * P / rt);
    *dst = v;
  }
}

struct SmemV {
  dw2 sS[kVWarps][2][kVVals + 1];  // forcing, [warp][pair][position]
  dw2 sG[kVWarps][2][33];          // g at positions p0-2 .. p0+30
  dw2 sH[kVWarps][2][32];          // AbG at interfaces p0-1 .. p0+30
  dw2 sD[kVWarps][2][32];          // Gd
};

// J(f)^T G for the taps s (pairs (DENS, UMOM), (WMOM, RHOT)) of one interface.
template <int DIR>
__device__ __forceinline__ void jt_g(const dw2 s[2][4], const RowV& rv, const dw2 Gv[2], bool wall, dw2 Ab[2]) {
  const dw2 A0 = acombo2(s[0][0], s[0][1], s[0][2], s[0][3]);
  const dw2 A1 = acombo2(s[1][0], s[1][1], s[1][2], s[1][3]);
  const dw AD = lo_of(A0), AU = hi_of(A0), AW = lo_of(A1), AT = hi_of(A1);
  const dw GD = lo_of(Gv[0]), GU = hi_of(Gv[0]), GW = lo_of(Gv[1]), GT = hi_of(Gv[1]);
  const dw ri = rcp(add(AD, rv.R));
  const dw dp = add(rv.GPI, mul(rv.GPI, pow_m1(c_pow_gm1, kGamma - 1.0, mul(AT, rv.IRT))));
  if (DIR == MW_DIR_Z && wall) {
    Ab[0] = pack(dw{0.f, 0.f}, dw{0.f, 0.f});
    Ab[1] = pack(dw{0.f, 0.f}, mul(GW, dp));
    return;
  }
  const dw2 uw = mul2(splat(ri), pack(AU, AW));  // (u, w)
  const dw u = lo_of(uw), w = hi_of(uw);
  const dw th = mul(add(AT, rv.RT), ri);
  const dw2 p1 = mul2(pack(GU, GW), uw);          // (G_U u, G_W w)
  const dw X = add(add(lo_of(p1), hi_of(p1)), mul(GT, th));
  if (DIR == MW_DIR_X) {
    const dw2 q = mul2(splat(u), pack(X, GW));             // (u X, G_W u)
    const dw2 r = mul2(pack(GU, GT), pack(dp, u));         // (G_U dp, G_T u)
    Ab[0] = pack(neg(lo_of(q)), add(GD, add(lo_of(p1), X)));
    Ab[1] = pack(hi_of(q), add(lo_of(r), hi_of(r)));
  } else {
    const dw2 q = mul2(splat(w), pack(X, GU));             // (w X, G_U w)
    const dw2 r = mul2(pack(GW, GT), pack(dp, w));         // (G_W dp, G_T w)
    Ab[0] = pack(neg(lo_of(q)), hi_of(q));
    Ab[1] = pack(add(GD, add(hi_of(p1), X)), add(lo_of(r), hi_of(r)));
  }
}

// Forcing value at position p of line `line` (x: row, periodic column; z:
// column, wall rule in the halo rows).
template <int DIR>
__device__ __forceinline__ double fval(const VjpSplitArgs& a, int q, int line, int p) {
  if (DIR == MW_DIR_X) {
    const int c = ((p % a.nx) + a.nx) % a.nx;
    return MW_AT(a.forcing, q * a.plane + (long long)(line + kHs) * a.pitch + c + kHs, 4 * a.plane);
  }
  const int col = line + kHs;
  if (p >= 0 && p < a.nz) return MW_AT(a.forcing, q * a.plane + (long long)(p + kHs) * a.pitch + col, 4 * a.plane);
  if (q == WMOM) return 0.0;
  const int src = p < 0 ? kHs : a.nz + kHs - 1;
  const double s = MW_AT(a.forcing, q * a.plane + (long long)src * a.pitch + col, 4 * a.plane);
  if (q == UMOM) return s / MW_AT(a.hyc, src, a.nz + 2 * kHs) * MW_AT(a.hyc, p + kHs, a.nz + 2 * kHs);
  return s;
}

template <int DIR>
__device__ __forceinline__ long long cell_off(const VjpSplitArgs& a, int line, int p) {
  return DIR == MW_DIR_X ? (long long)(line + kHs) * a.pitch + p + kHs : (long long)(p + kHs) * a.pitch + line + kHs;
}

// g at position p (0 outside the walls in z, periodic in x)
template <int DIR>
__device__ __forceinline__ void gload(const VjpSplitArgs& a, int line, int p, double v[4]) {
  const int len = DIR == MW_DIR_X ? a.nx : a.nz;
  if (DIR == MW_DIR_X) {
    p = ((p % len) + len) % len;
  } else if (p < 0 || p >= len) {
    v[0] = v[1] = v[2] = v[3] = 0.0;
    return;
  }
  const long long o = cell_off<DIR>(a, line, p);
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = MW_AT(a.gout, q * a.plane + o, 4 * a.plane);
}

// Weight of a halo-row tap (row h) on its source row in z, for UMOM.
__device__ __forceinline__ dw halo_umom_weight(const VjpSplitArgs& a, int h) {
  const int src = h < 0 ? kHs : a.nz + kHs - 1;
  return from_f64(MW_AT(a.hyc, h + kHs, a.nz + 2 * kHs) / MW_AT(a.hyc, src, a.nz + 2 * kHs));
}

// T_j(f) = c12_j AbG(f) - e_j 12hv Gd(f) for one (AbG, Gd) pair of a variable pair.
__device__ __forceinline__ dw2 tap_term(int j, const dw2& ab, const dw2& gd, const dw2& hv, const float2& nhv) {
  const float c = (j == 1 || j == 2) ? 7.f : -1.f;
  const float e = j == 0 ? -1.f : (j == 1 ? 3.f : (j == 2 ? -3.f : 1.f));
  const dw2 abc = mul2(ab, splat(dw{c, 0.f}));
  const dw2 gde = mul2n(gd, hv, nhv);
  return sub2(abc, mul2(gde, splat(dw{e, 0.f})));
}

template <int DIR>
__device__ __forceinline__ void vjp_segments(const VjpSplitArgs& a, int nseg, long long g0, long long g1, SmemV& sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (g0 >= g1) return;
  const int len = DIR == MW_DIR_X ? a.nx : a.nz;
  const dw hv12 = ld(a.hv12);
  const dw2 hv = splat(hv12);
  const float2 nhv = f2splat(-hv12.h);
  for (long long g = g0; g < g1; ++g) {
    const int line = (int)(g / nseg), p0 = (int)(g - (long long)line * nseg) * kVCells;
    // stage forcing positions p0-3+l and (lanes 0..2) p0+29+l
    {
      const int pA = p0 - 3 + lane, pB = p0 + 29 + lane;
      const bool okA = DIR == MW_DIR_X || (pA >= -2 && pA <= a.nz + 1);
      const bool okB = lane < 3 && (DIR == MW_DIR_X || pB <= a.nz + 1);
      double v[4] = {0, 0, 0, 0};
      if (okA) {
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = fval<DIR>(a, q, line, pA);
      }
      dw2 pk[2];
      pack4(v, pk);
      sm.sS[w][0][lane] = pk[0];
      sm.sS[w][1][lane] = pk[1];
      if (okB) {
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = fval<DIR>(a, q, line, pB);
        pack4(v, pk);
        sm.sS[w][0][32 + lane] = pk[0];
        sm.sS[w][1][32 + lane] = pk[1];
      }
    }
    // stage g at positions p0-1+l (index l+1) and p0-2 (index 0)
    {
      double v[4];
      gload<DIR>(a, line, p0 - 1 + lane, v);
      dw2 pk[2];
      pack4(v, pk);
      sm.sG[w][0][lane + 1] = pk[0];
      sm.sG[w][1][lane + 1] = pk[1];
      if (lane == 0) {
        gload<DIR>(a, line, p0 - 2, v);
        pack4(v, pk);
        sm.sG[w][0][0] = pk[0];
        sm.sG[w][1][0] = pk[1];
      }
    }
    __syncwarp();
    // interface f = p0 - 1 + lane
    {
      const int f = p0 - 1 + lane;
      dw2 Ab[2], Gd[2];
      const bool exists = DIR == MW_DIR_X || (f >= 0 && f <= a.nz);
      if (exists) {
        Gd[0] = sub2(sm.sG[w][0][lane + 1], sm.sG[w][0][lane]);
        Gd[1] = sub2(sm.sG[w][1][lane + 1], sm.sG[w][1][lane]);
        dw2 s[2][4];
#pragma unroll
        for (int pr = 0; pr < 2; ++pr)
#pragma unroll
          for (int j = 0; j < 4; ++j) s[pr][j] = sm.sS[w][pr][lane + j];
        const int ri = DIR == MW_DIR_X ? line : f;
        const RowV rv = MW_AT(a.rows, ri, DIR == MW_DIR_X ? a.nz : a.nz + 1);
        const bool wall = DIR == MW_DIR_Z && (f == 0 || f == a.nz);
        jt_g<DIR>(s, rv, Gd, wall, Ab);
        if (wall) {
          Gd[0].h.x = 0.f;
          Gd[0].l.x = 0.f;
        }
      } else {
        Ab[0] = Ab[1] = Gd[0] = Gd[1] = pack(dw{0.f, 0.f}, dw{0.f, 0.f});
      }
      sm.sH[w][0][lane] = Ab[0];
      sm.sH[w][1][lane] = Ab[1];
      sm.sD[w][0][lane] = Gd[0];
      sm.sD[w][1][lane] = Gd[1];
    }
    __syncwarp();
    // cell t = p0 + lane
    const int t = p0 + lane;
    if (lane < kVCells && t < len) {
      dw2 S[2];
#pragma unroll
      for (int pr = 0; pr < 2; ++pr) {
        const dw2 Ac = acombo2(sm.sH[w][pr][lane], sm.sH[w][pr][lane + 1], sm.sH[w][pr][lane + 2], sm.sH[w][pr][lane + 3]);
        const dw2 Dc = dcombo2(sm.sD[w][pr][lane], sm.sD[w][pr][lane + 1], sm.sD[w][pr][lane + 2], sm.sD[w][pr][lane + 3]);
        S[pr] = add2(Ac, mul2n(Dc, hv, nhv));
      }
      if (DIR == MW_DIR_Z && (t == 0 || t == a.nz - 1)) {
        // halo-row taps (halo row h, interface f, tap j): rows -2, -1 return to
        // row 0, rows nz, nz+1 to row nz-1
        const int hs[6] = {-2, -1, -1, a.nz, a.nz, a.nz + 1};
        const int fs[6] = {0, 0, 1, a.nz - 1, a.nz, a.nz};
        const int js[6] = {0, 1, 0, 3, 2, 3};
        for (int m = (t == 0 ? 0 : 3); m < (t == a.nz - 1 ? 6 : 3); ++m) {
          const int li = fs[m] - p0 + 1;  // lane of interface fs[m]
          dw2 T0 = tap_term(js[m], sm.sH[w][0][li], sm.sD[w][0][li], hv, nhv);
          dw2 T1 = tap_term(js[m], sm.sH[w][1][li], sm.sD[w][1][li], hv, nhv);
          T0 = pack(lo_of(T0), mul(hi_of(T0), halo_umom_weight(a, hs[m])));
          T1 = pack(dw{0.f, 0.f}, hi_of(T1));
          S[0] = add2(S[0], T0);
          S[1] = add2(S[1], T1);
        }
      }
      const long long o = cell_off<DIR>(a, line, t);
      const dw d[4] = {lo_of(S[0]), hi_of(S[0]), lo_of(S[1]), hi_of(S[1])};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long long oq = q * a.plane + o;
        double base = 0.0;
        if (a.add_gout) base += MW_AT(a.gout, oq, 4 * a.plane);
        if (a.base_a) base += MW_AT(a.base_a, oq, 4 * a.plane);
        if (a.base_b) base += MW_AT(a.base_b, oq, 4 * a.plane);
        double v = fma(a.cs, to_f64_scaled(d[q]), base);
        if (DIR == MW_DIR_Z && q == DENS) v = fma(-a.dtg, MW_AT(a.gout, WMOM * a.plane + o, 4 * a.plane), v);
        MW_AT(a.gdst, oq, 4 * a.plane) = v;
      }
    }
    __syncwarp();
  }
}

// g_dst's halo cells: zero (the frame, strided over every thread of the launch).
__device__ __forceinline__ void zero_frame(const VjpSplitArgs& a) {
  const int rows = a.nz + 2 * kHs;
  const long long hrow = 2LL * kHs * a.pitch;               // the halo rows' cells
  const long long frame = hrow + 2LL * kHs * a.nz;          // + the halo columns of the interior rows
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < frame; e += step) {
    long long o;
    if (e < hrow) {
      const int r = (int)(e / a.pitch), c = (int)(e % a.pitch);
      o = (long long)(r < kHs ? r : rows - 2 * kHs + r) * a.pitch + c;
    } else {
      const long long e2 = e - hrow;
      const int k = (int)(e2 / (2 * kHs)), h = (int)(e2 % (2 * kHs));
      o = (long long)(k + kHs) * a.pitch + (h < kHs ? h : a.nx + h);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) MW_AT(a.gdst, q * a.plane + o, 4 * a.plane) = 0.0;
  }
}

// Launched for the x direction (rows are contiguous); the z direction runs
// k_vjp_split_zt below, which applies the same per-line computation to
// shared-memory tiles.
template <int DIR>
__global__ void __launch_bounds__(kVThreads) k_vjp_split(VjpSplitArgs a, int nseg, long long total) {
  __shared__ SmemV sm;
  zero_frame(a);
  const long long g0 = total * blockIdx.x / gridDim.x, g1 = total * (blockIdx.x + 1) / gridDim.x;
  const int w = threadIdx.x >> 5;
  const long long n = g1 - g0;
  vjp_segments<DIR>(a, nseg, g0 + n * w / kVWarps, g0 + n * (w + 1) / kVWarps, sm);
}

// z, tiled: the z lines are columns, so a warp walking one column directly
// would read 32 different rows per access.  Here a CTA takes a tile of kZTCols
// columns x one 29-row segment: the forcing (rows p0-3 .. p0+31) and g (rows
// p0-2 .. p0+30) of its columns are staged into shared memory by row-contiguous
// loads (consecutive threads, consecutive columns); each warp then runs the
// per-column computation of vjp_segments on its column from shared memory, and
// the results are written back row-contiguously by the whole CTA.
#ifndef MW_VJP_ZT_COLS
#define MW_VJP_ZT_COLS 4
#endif
constexpr int kZTCols = MW_VJP_ZT_COLS;  // columns per tile = warps per CTA (one column each)
constexpr int kZTThreads = 32 * kZTCols;
constexpr int kZTPos = kVCells + 6;  // staged forcing positions
constexpr int kZTG = kVCells + 4;    // staged g positions
struct SmemVZ {
  dw2 sF[2][kZTCols][kZTPos];     // forcing pairs [pair][column][position p0-3+j]
  dw2 sG[2][kZTCols][kZTG];       // g pairs [pair][column][position p0-2+i]
  dw2 sO[2][kZTCols][kVCells];    // S (the scaled increment) [pair][column][cell p0+t]
  dw2 sH[kZTCols][2][32];         // AbG at interfaces p0-1 .. p0+30 (per warp)
  dw2 sD[kZTCols][2][32];         // Gd
};

__global__ void __launch_bounds__(kZTThreads) k_vjp_split_zt(VjpSplitArgs a, int nseg, int ncb, long long total) {
  extern __shared__ __align__(16) unsigned char vz_raw[];
  SmemVZ& sm = *reinterpret_cast<SmemVZ*>(vz_raw);
  zero_frame(a);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const dw hv12 = ld(a.hv12);
  const dw2 hv = splat(hv12);
  const float2 nhv = f2splat(-hv12.h);
  for (long long it = blockIdx.x; it < total; it += gridDim.x) {
    const int cb = (int)(it % ncb), sg = (int)(it / ncb);
    const int c0 = cb * kZTCols, p0 = sg * kVCells;
    // stage forcing and g (column fastest over the threads)
    for (int e = threadIdx.x; e < kZTCols * kZTPos; e += kZTThreads) {
      const int cl = e % kZTCols, j = e / kZTCols, c = c0 + cl, pp = p0 - 3 + j;
      double v[4] = {0, 0, 0, 0};
      if (c < a.nx && pp >= -2 && pp <= a.nz + 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = fval<MW_DIR_Z>(a, q, c, pp);
      }
      dw2 pk[2];
      pack4(v, pk);
      sm.sF[0][cl][j] = pk[0];
      sm.sF[1][cl][j] = pk[1];
    }
    for (int e = threadIdx.x; e < kZTCols * kZTG; e += kZTThreads) {
      const int cl = e % kZTCols, i = e / kZTCols, c = c0 + cl;
      double v[4] = {0, 0, 0, 0};
      if (c < a.nx) gload<MW_DIR_Z>(a, c, p0 - 2 + i, v);
      dw2 pk[2];
      pack4(v, pk);
      sm.sG[0][cl][i] = pk[0];
      sm.sG[1][cl][i] = pk[1];
    }
    __syncthreads();
    for (int cl = w; cl < kZTCols; cl += kZTCols) {
      if (c0 + cl >= a.nx) break;  // warp-uniform; columns beyond nx are skipped by every later warp too
      // interface f = p0 - 1 + lane
      {
        const int f = p0 - 1 + lane;
        dw2 Ab[2], Gd[2];
        if (f >= 0 && f <= a.nz) {
          Gd[0] = sub2(sm.sG[0][cl][lane + 1], sm.sG[0][cl][lane]);
          Gd[1] = sub2(sm.sG[1][cl][lane + 1], sm.sG[1][cl][lane]);
          dw2 s[2][4];
#pragma unroll
          for (int pr = 0; pr < 2; ++pr)
#pragma unroll
            for (int j = 0; j < 4; ++j) s[pr][j] = sm.sF[pr][cl][lane + j];
          const RowV rv = MW_AT(a.rows, f, a.nz + 1);
          const bool wall = f == 0 || f == a.nz;
          jt_g<MW_DIR_Z>(s, rv, Gd, wall, Ab);
          if (wall) {
            Gd[0].h.x = 0.f;
            Gd[0].l.x = 0.f;
          }
        } else {
          Ab[0] = Ab[1] = Gd[0] = Gd[1] = pack(dw{0.f, 0.f}, dw{0.f, 0.f});
        }
        sm.sH[w][0][lane] = Ab[0];
        sm.sH[w][1][lane] = Ab[1];
        sm.sD[w][0][lane] = Gd[0];
        sm.sD[w][1][lane] = Gd[1];
      }
      __syncwarp();
      // cell t = p0 + lane
      const int t = p0 + lane;
      if (lane < kVCells && t < a.nz) {
        dw2 S[2];
#pragma unroll
        for (int pr = 0; pr < 2; ++pr) {
          const dw2 Ac = acombo2(sm.sH[w][pr][lane], sm.sH[w][pr][lane + 1], sm.sH[w][pr][lane + 2], sm.sH[w][pr][lane + 3]);
          const dw2 Dc = dcombo2(sm.sD[w][pr][lane], sm.sD[w][pr][lane + 1], sm.sD[w][pr][lane + 2], sm.sD[w][pr][lane + 3]);
          S[pr] = add2(Ac, mul2n(Dc, hv, nhv));
        }
        if (t == 0 || t == a.nz - 1) {  // halo-row taps, as in vjp_segments
          const int hs[6] = {-2, -1, -1, a.nz, a.nz, a.nz + 1};
          const int fs[6] = {0, 0, 1, a.nz - 1, a.nz, a.nz};
          const int js[6] = {0, 1, 0, 3, 2, 3};
          for (int m = (t == 0 ? 0 : 3); m < (t == a.nz - 1 ? 6 : 3); ++m) {
            const int li = fs[m] - p0 + 1;
            dw2 T0 = tap_term(js[m], sm.sH[w][0][li], sm.sD[w][0][li], hv, nhv);
            dw2 T1 = tap_term(js[m], sm.sH[w][1][li], sm.sD[w][1][li], hv, nhv);
            T0 = pack(lo_of(T0), mul(hi_of(T0), halo_umom_weight(a, hs[m])));
            T1 = pack(dw{0.f, 0.f}, hi_of(T1));
            S[0] = add2(S[0], T0);
            S[1] = add2(S[1], T1);
          }
        }
        sm.sO[0][cl][lane] = S[0];
        sm.sO[1][cl][lane] = S[1];
      }
      __syncwarp();
    }
    __syncthreads();
    // g_dst = bases + dt/(12 dz) S [- dt grav g_w on rho'], row-contiguous
    for (int e = threadIdx.x; e < kZTCols * kVCells; e += kZTThreads) {
      const int cl = e % kZTCols, j = e / kZTCols, c = c0 + cl, t = p0 + j;
      if (c >= a.nx || t >= a.nz) continue;
      const dw2 S0 = sm.sO[0][cl][j], S1 = sm.sO[1][cl][j];
      const dw d[4] = {lo_of(S0), hi_of(S0), lo_of(S1), hi_of(S1)};
      const long long o = cell_off<MW_DIR_Z>(a, c, t);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long long oq = q * a.plane + o;
        double base = 0.0;
        if (a.add_gout) base += MW_AT(a.gout, oq, 4 * a.plane);
        if (a.base_a) base += MW_AT(a.base_a, oq, 4 * a.plane);
        if (a.base_b) base += MW_AT(a.base_b, oq, 4 * a.plane);
        double v = fma(a.cs, to_f64_scaled(d[q]), base);
        if (q == DENS) v = fma(-a.dtg, MW_AT(a.gout, WMOM * a.plane + o, 4 * a.plane), v);
        MW_AT(a.gdst, oq, 4 * a.plane) = v;
      }
    }
    __syncthreads();  // the tiles are rewritten by the next item
  }
}

int vjp_resident_ctas(int* out) {
  int per_sm = 0, sms = 0, dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vjp_split<MW_DIR_X>, kVThreads, 0);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  *out = std::max(1, per_sm) * sms;
  return MW_OK;
}

}  // namespace

#if MW_CHECK
MW_OOB_COUNTER(oob_count_adjoint_split)
#endif

size_t vjp_split_table_bytes(int nz) { return sizeof(RowV) * (size_t)(2 * nz + 1); }

// Row / interface constants into the workspace (x rows then z interfaces).
int launch_vjp_row_table(int nx, int nz, const double* hyc, const double* hytc, const double* hyi, const double* hyti,
                         const double* hypi, void* workspace, cudaStream_t stream) {
  RowV* tx = (RowV*)workspace;
  k_vjp_row_table<<<(2 * nz + 1 + 127) / 128, 128, 0, stream>>>(hyc, hytc, hyi, hyti, hypi, nx, nz, tx, tx + nz);
  return check_launch("vjp row-table launch");
}

// One split direction-stage VJP; the table must have been written by launch_vjp_row_table.
int launch_vjp_split(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const void* table,
                     const double* forcing, const double* g_out, const double* g_base_a, const double* g_base_b,
                     int add_g_out, double* g_dst, double dt_stage, int direction, cudaStream_t stream) {
  const Geom g = make_geom(nx, nz);
  VjpSplitArgs a;
  a.nx = nx;
  a.nz = nz;
  a.pitch = g.pitch;
  a.plane = g.plane;
  a.hyc = hyc;
  a.rows = (const RowV*)table + (direction == MW_DIR_X ? 0 : nz);
  a.forcing = forcing;
  a.gout = g_out;
  a.base_a = g_base_a;
  a.base_b = g_base_b;
  a.add_gout = add_g_out;
  a.gdst = g_dst;
  const double d = direction == MW_DIR_X ? dx : dz;
  a.hv12 = split_host(12.0 * (-kHvBeta * d / (16 * dt_full)));
  a.cs = dt_stage / (12.0 * d) * kTwoPow896;
  MW_REQUIRE(std::isfinite(a.cs), MW_ERR_INVALID_ARG, "dt_stage / (12 d) is above the split form's range");
  a.dtg = dt_stage * kGrav;
  const int len = direction == MW_DIR_X ? nx : nz;
  const int lines = direction == MW_DIR_X ? nz : nx;
  const int nseg = (len + kVCells - 1) / kVCells;
  const long long total = (long long)nseg * lines;
  int resident = 0, st = vjp_resident_ctas(&resident);
  if (st) return st;
  long long grid = std::min<long long>(resident, (total + kVWarps - 1) / kVWarps);
  grid = std::max<long long>(grid, total / (kVWarps * 32));
  grid = std::max<long long>(1, std::min<long long>(grid, 0x7fffffffLL));
  if (direction == MW_DIR_X) {
    k_vjp_split<MW_DIR_X><<<(unsigned)grid, kVThreads, 0, stream>>>(a, nseg, total);
  } else {  // tiles of kZTCols columns x one segment, a grid of resident CTAs
    const int ncb = (nx + kZTCols - 1) / kZTCols;
    const long long tiles = (long long)ncb * nseg;
    int per_sm = 0, sms = 0, dev = 0;
    const size_t smem = sizeof(SmemVZ);
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_vjp_split_zt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vjp_split_zt, kZTThreads, smem);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(MW_ERR_CUDA, "z vjp setup: %s", cudaGetErrorString(e));
    const long long gz = std::max<long long>(1, std::min<long long>(tiles, (long long)std::max(1, per_sm) * sms));
    k_vjp_split_zt<<<(unsigned)gz, kZTThreads, smem, stream>>>(a, nseg, ncb, tiles);
  }
  return check_launch("split vjp launch");
}

}  // namespace mw
