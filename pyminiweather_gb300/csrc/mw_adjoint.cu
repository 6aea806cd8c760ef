// mw_adjoint.cu -- adjoint (vector-Jacobian product) of one direction-stage.
//
// Forward (pyminiweather/solve/step.py:21-82, interpolate.py:82-250):
//   out = init + dt * L(forcing),  L = -(F(i+1) - F(i)) / d  [- rho' g on w in z],
//   F(i) = f(A(i), D(i)),  A = sum_j c_j s(i-2+j),  D = sum_j e_j s(i-2+j),
//   c = (-1, 7, 7, -1)/12, e = (-1, 3, -3, 1), s read through the halo rules
//   (periodic in x, ics/bcs.py:35-39; wall in z, bcs.py:92-148).
// Adjoint, given g = dJ/d(out) on the interior cells:
//   dJ/d(init)    += g
//   dJ/d(forcing) += dt * (dL/d forcing)^T g:
//     Fbar(i) = (dt/d) (g(i) - g(i-1))      (g = 0 outside the interior)
//     (Abar, Dbar)(i) = (df/dA, df/dD)^T Fbar(i)
//     sbar(t) += c_j Abar(i) + e_j Dbar(i)  for the taps t = i-2+j, mapped
//     back through the halo rules (a halo value's adjoint goes to the cell it
//     was copied or scaled from), and sbar_rho(k) -= dt g_w(k) grav in z.
// The flux Jacobian uses rho theta = A3 + (rho theta)_bg and p = C0 (rho theta)^gamma,
// so dp/dA3 = gamma p / (rho theta); at the z walls w and d3[DENS] are held at
// zero (interpolate.py:167-173), so those paths carry no adjoint.
//
// f64_mode MW_F64_NATIVE (the reference's formulas: a pow and three divides
// per interface) runs two kernels per call: one thread per interface writes
// (Abar, Dbar) to a caller-provided workspace; one thread per cell gathers its
// taps.  MW_F64_IEEE (the fewest FP64 operations: values scaled by 12, 1/rho
// by a Newton step, dp/d(rho theta) = gamma P_row (1 + delta)^(gamma-1) /
// (rho theta)_bg by its binomial series, per-row constants from a table in the
// workspace) runs the same two kernels in z and, in x, one kernel that computes
// each warp segment's interface adjoints into shared memory and gathers them
// there.
#include <algorithm>

#include "mw_common.cuh"
#include "mw_fp64_math.cuh"

namespace mw {
namespace {

struct VjpArgs {
  int nx, nz, pitch;
  long long plane;
  double d;         // dx or dz
  double hv;        // -hv_beta d / (16 dt_full)
  double dt_stage;
  const double *hyc, *hytc, *hyi, *hyti, *hypi;
  const double* forcing;
  const double* gout;
  const double* base_a;
  const double* base_b;
  int add_gout;
  double* gdst;
  double* ws;       // 8 x n_interfaces: Abar[4], Dbar[4]
  long long nif;    // interfaces per variable plane of ws
};

__device__ __forceinline__ int wrap_x(int j, int nx) { return j < 0 ? j + nx : (j >= nx ? j - nx : j); }

// Bounds-checked element access (MW_AT) to the arrays of one stage adjoint.
#define MW_VF(a, off) MW_AT((a).forcing, (off), 4 * (a).plane)
#define MW_VC(a, p, k) MW_AT((a).p, (k), (a).nz + 2 * kHs)  // cell-centre background
#define MW_VI(a, p, k) MW_AT((a).p, (k), (a).nz + 1)        // interface background
#define MW_WS(a, off) MW_AT((a).ws, (off), 8 * (a).nif)

__device__ __forceinline__ double zval(const VjpArgs& a, int q, int k, int col) {
  if (k >= 0 && k < a.nz) return MW_VF(a, q * a.plane + (long long)(k + kHs) * a.pitch + col);
  if (q == WMOM) return 0.0;
  const int src = k < 0 ? kHs : a.nz + kHs - 1;
  const double s = MW_VF(a, q * a.plane + (long long)src * a.pitch + col);
  if (q == UMOM) return s / MW_VC(a, hyc, src) * MW_VC(a, hyc, k + kHs);
  return s;
}

__device__ __forceinline__ double gval(const VjpArgs& a, int q, int k, int i) {
  return MW_AT(a.gout, q * a.plane + (long long)(k + kHs) * a.pitch + i + kHs, 4 * a.plane);
}

// tap weights of the interpolation (data/fields.py:94-97, convolution order
// reversed) and of the third difference
__constant__ double kC[4] = {-1.0 / 12, 7.0 / 12, 7.0 / 12, -1.0 / 12};
__constant__ double kE[4] = {-1.0, 3.0, -3.0, 1.0};

// Interface adjoints.  x: interface (k, i), i in [0, nx]; z: (k, c), k in [0, nz].
template <int DIR>
__global__ void k_vjp_iface(VjpArgs a) {
  const long long n = a.nif;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    double s[4][4];
    double Fb[4];
    bool wall = false;
    double hy_r, hy_rt;
    if (DIR == MW_DIR_X) {
      const int k = (int)(idx / (a.nx + 1)), i = (int)(idx % (a.nx + 1));
      const long long row = (long long)(k + kHs) * a.pitch;
      for (int j = 0; j < 4; ++j) {
        const long long col = wrap_x(i - 2 + j, a.nx) + kHs;
        for (int q = 0; q < 4; ++q) s[q][j] = MW_VF(a, q * a.plane + row + col);
      }
      for (int q = 0; q < 4; ++q) {
        const double gr = i < a.nx ? gval(a, q, k, i) : 0.0;
        const double gl = i > 0 ? gval(a, q, k, i - 1) : 0.0;
        Fb[q] = a.dt_stage / a.d * (gr - gl);
      }
      hy_r = MW_VC(a, hyc, k + kHs);
      hy_rt = MW_VC(a, hytc, k + kHs);
    } else {
      const int k = (int)(idx / a.nx), c = (int)(idx % a.nx);
      for (int j = 0; j < 4; ++j)
        for (int q = 0; q < 4; ++q) s[q][j] = zval(a, q, k - 2 + j, c + kHs);
      for (int q = 0; q < 4; ++q) {
        const double gr = k < a.nz ? gval(a, q, k, c) : 0.0;
        const double gl = k > 0 ? gval(a, q, k - 1, c) : 0.0;
        Fb[q] = a.dt_stage / a.d * (gr - gl);
      }
      hy_r = MW_VI(a, hyi, k);
      hy_rt = MW_VI(a, hyti, k);
      wall = (k == 0) || (k == a.nz);
    }
    double A[4];
    for (int q = 0; q < 4; ++q) A[q] = ((s[q][0] * kC[0] + s[q][1] * kC[1]) + s[q][2] * kC[2]) + s[q][3] * kC[3];
    const double rho = A[DENS] + hy_r;
    const double rt = A[RHOT] + hy_rt;
    const double u = A[UMOM] / rho, w = A[WMOM] / rho, th = rt / rho;
    const double dpdA3 = kGamma * kC0 * pow(rt, kGamma) / rt;
    double Ab[4], Db[4];
    for (int q = 0; q < 4; ++q) Db[q] = -a.hv * Fb[q];
    if (DIR == MW_DIR_X) {
      Ab[DENS] = -(Fb[1] * u * u + Fb[2] * u * w + Fb[3] * u * th);
      Ab[UMOM] = Fb[0] + 2.0 * Fb[1] * u + Fb[2] * w + Fb[3] * th;
      Ab[WMOM] = Fb[2] * u;
      Ab[RHOT] = Fb[1] * dpdA3 + Fb[3] * u;
    } else if (!wall) {
      Ab[DENS] = -(Fb[1] * w * u + Fb[2] * w * w + Fb[3] * w * th);
      Ab[UMOM] = Fb[1] * w;
      Ab[WMOM] = Fb[0] + Fb[1] * u + 2.0 * Fb[2] * w + Fb[3] * th;
      Ab[RHOT] = Fb[2] * dpdA3 + Fb[3] * w;
    } else {
      Ab[DENS] = 0.0;
      Ab[UMOM] = 0.0;
      Ab[WMOM] = 0.0;
      Ab[RHOT] = Fb[2] * dpdA3;
      Db[DENS] = 0.0;
    }
    for (int q = 0; q < 4; ++q) {
      MW_WS(a, q * n + idx) = Ab[q];
      MW_WS(a, (4 + q) * n + idx) = Db[q];
    }
  }
}

// Cell gather: gdst = base_a + base_b + add_gout * gout + sbar (interior); halo cells of gdst = 0.
// The adjoint of interior cell (k, i) gathered from the interface adjoints
// of its taps by the general rule: periodic wrap in x, the wall rule's halo
// taps in z (any cell).
template <int DIR>
__device__ __forceinline__ void gather_general(const VjpArgs& a, int k, int i, double acc[4]) {
  const long long n = a.nif;
  if (DIR == MW_DIR_X) {
    for (int j = 0; j < 4; ++j)
      for (int m = -1; m <= 1; ++m) {
        const int f = i + 2 - j + m * a.nx;  // interface whose tap j is cell i
        if (f < 0 || f > a.nx) continue;
        const long long o = (long long)k * (a.nx + 1) + f;
        for (int q = 0; q < 4; ++q) acc[q] += kC[j] * MW_WS(a, q * n + o) + kE[j] * MW_WS(a, (4 + q) * n + o);
      }
  } else {
    // taps t = f - 2 + j of interface f in [0, nz]; t maps to row k directly,
    // or through the wall rule from halo rows -2,-1 (-> 0) and nz, nz+1 (-> nz-1)
    for (int f = k - 1; f <= k + 2; ++f) {  // interfaces with an interior tap at row k
      if (f < 0 || f > a.nz) continue;
      const int j = k - f + 2;
      const long long o = (long long)f * a.nx + i;
      for (int q = 0; q < 4; ++q) acc[q] += kC[j] * MW_WS(a, q * n + o) + kE[j] * MW_WS(a, (4 + q) * n + o);
    }
    auto halo_taps = [&](int t, double wq[4]) {  // weight of halo row t on row k
      const int src = t < 0 ? 0 : a.nz - 1;
      wq[DENS] = wq[RHOT] = (k == src) ? 1.0 : 0.0;
      wq[WMOM] = 0.0;
      wq[UMOM] = (k == src) ? MW_VC(a, hyc, t + kHs) / MW_VC(a, hyc, src + kHs) : 0.0;
    };
    const int halo_rows[4] = {-2, -1, a.nz, a.nz + 1};
    for (int h = 0; h < 4; ++h) {
      const int t = halo_rows[h];
      double wq[4];
      halo_taps(t, wq);
      if (wq[DENS] == 0.0 && wq[UMOM] == 0.0) continue;
      for (int j = 0; j < 4; ++j) {
        const int f = t + 2 - j;
        if (f < 0 || f > a.nz) continue;
        const long long o = (long long)f * a.nx + i;
        for (int q = 0; q < 4; ++q)
          acc[q] += wq[q] * (kC[j] * MW_WS(a, q * n + o) + kE[j] * MW_WS(a, (4 + q) * n + o));
      }
    }
  }
}

// One thread per cell of a row (grid.y strides over the rows): halo cells get
// zero; an interior cell whose four interfaces are all interior and none of
// whose taps wrap or come through the wall rule (x: 2 <= i <= nx - 3, z:
// 1 <= k <= nz - 2) reads them as a row (x) or column (z) of four, A0 .. A3
// and D0 .. D3 at interfaces i - 1 .. i + 2, and sums the transposed taps in
// the symmetric forms (7 (A1 + A2) - (A0 + A3)) / 12 and (D0 - D3) + 3 (D2 - D1);
// the others take the general rule.  In z the gravity term follows.
template <int DIR>
__global__ void __launch_bounds__(128) k_vjp_gather(VjpArgs a) {
  const long long n = a.nif;
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= a.pitch) return;
  const int i = ii - kHs;
  for (int kk = blockIdx.y; kk < a.nz + 2 * kHs; kk += gridDim.y) {
    const long long idx = (long long)kk * a.pitch + ii;
    const int k = kk - kHs;
    if (k < 0 || k >= a.nz || i < 0 || i >= a.nx) {
      for (int q = 0; q < 4; ++q) MW_AT(a.gdst, q * a.plane + idx, 4 * a.plane) = 0.0;
      continue;
    }
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const bool fast = DIR == MW_DIR_X ? (i >= 2 && i + 3 <= a.nx) : (k >= 1 && k + 2 <= a.nz);
    if (fast) {
      // interfaces i - 1 .. i + 2 (x: row k of nx + 1; z: rows k - 1 .. k + 2 of column i)
      const long long o0 = DIR == MW_DIR_X ? (long long)k * (a.nx + 1) + (i - 1) : (long long)(k - 1) * a.nx + i;
      const long long st = DIR == MW_DIR_X ? 1 : a.nx;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double A0 = MW_WS(a, q * n + o0), A1 = MW_WS(a, q * n + o0 + st);
        const double A2 = MW_WS(a, q * n + o0 + 2 * st), A3 = MW_WS(a, q * n + o0 + 3 * st);
        const double D0 = MW_WS(a, (4 + q) * n + o0), D1 = MW_WS(a, (4 + q) * n + o0 + st);
        const double D2 = MW_WS(a, (4 + q) * n + o0 + 2 * st), D3 = MW_WS(a, (4 + q) * n + o0 + 3 * st);
        // cell i is tap j of interface f = i + 2 - j, so kC = (-1, 7, 7, -1) / 12 and
        // kE = (-1, 3, -3, 1) act on the interfaces i + 2, i + 1, i, i - 1 = (A3, A2, A1, A0)
        const double ca = fma(7.0, A1 + A2, -(A0 + A3)) * (1.0 / 12.0);
        const double ce = fma(3.0, D2 - D1, D0 - D3);
        acc[q] = ca + ce;
      }
    } else {
      gather_general<DIR>(a, k, i, acc);
    }
    if (DIR == MW_DIR_Z) acc[DENS] -= a.dt_stage * kGrav * gval(a, WMOM, k, i);
    for (int q = 0; q < 4; ++q) {
      const long long o = q * a.plane + idx;
      double v = acc[q];
      if (a.add_gout) v += MW_AT(a.gout, o, 4 * a.plane);
      if (a.base_a) v += MW_AT(a.base_a, o, 4 * a.plane);
      if (a.base_b) v += MW_AT(a.base_b, o, 4 * a.plane);
      MW_AT(a.gdst, o, 4 * a.plane) = v;
    }
  }
}

// ---- IEEE-FP64 interface adjoint (f64_mode MW_F64_IEEE) --------------------
__constant__ ieee::Series c_pow_gm1 = ieee::make_series(kGamma - 1.0);  // (1 + d)^(gamma - 1)

// Row constants of the IEEE interface adjoint, scaled by 12 like the
// interpolated values: the x rows (cell centres, nz + 4 entries), then the z
// interface rows (nz + 1), in the workspace after the interface adjoints.
struct RowV {
  double R12;    // 12 background rho
  double RT12;   // 12 background rho theta
  double IRT12;  // 1 / (12 background rho theta)
  double Q;      // dp/d(rho theta) at the background, gamma C0 (rho theta)^(gamma - 1)
  double QC1;    // Q C(gamma - 1, 1) IRT12: its change per unit of 12 (rho theta)' to first order
};

__global__ void k_vjp_rows_ieee(int nz, const double* hyc, const double* hytc, const double* hyi, const double* hyti,
                                const double* hypi, RowV* t) {
  const int n = 2 * nz + 5;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double r, rt, Q;
    if (j < nz + 2 * kHs) {
      r = MW_AT(hyc, j, nz + 2 * kHs);
      rt = MW_AT(hytc, j, nz + 2 * kHs);
      Q = kGamma * kC0 * pow(rt, kGamma - 1.0);
    } else {  // hy_pressure_int = C0 hy_dens_theta_int^gamma (ics/initial.py:105)
      const int k = j - (nz + 2 * kHs);
      r = MW_AT(hyi, k, nz + 1);
      rt = MW_AT(hyti, k, nz + 1);
      Q = kGamma * MW_AT(hypi, k, nz + 1) / rt;
    }
    const double irt = 1.0 / (12.0 * rt);
    MW_AT(t, j, n) = {12.0 * r, 12.0 * rt, irt, Q, Q * c_pow_gm1.c[1] * irt};
  }
}

// J(f)^T of one interface in the fewest FP64 operations (~43 against ~300
// for k_vjp_iface, the same Jacobian): taps s, G = g(f) - g(f-1), the row
// constants rv; Ab = J^T (cd G) and Db = hvcd G, with (rho w)' and d3[DENS]
// held at zero at the z walls.  The lanes in `mask` call it together.
template <int DIR>
__device__ __forceinline__ void jt_ieee(const double s[4][4], const double dg[4], const RowV& rv, double cd,
                                        double hvcd, bool wall, unsigned mask, double Ab[4], double Db[4]) {
  double A[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) A[q] = ieee::interp12(s[q][0], s[q][1], s[q][2], s[q][3]);
  const double ri = ieee::rcp(A[DENS] + rv.R12, mask);
  const double u = A[UMOM] * ri, w = A[WMOM] * ri, th = (A[RHOT] + rv.RT12) * ri;
  // dp/dA3 = Q (1 + d)^(gamma - 1), d = (rho theta)' / (rho theta)_bg
  const double d = A[RHOT] * rv.IRT12;
  bool big;
  const int deg = ieee::series_degree(d, mask, c_pow_gm1, big);
  double dp;
  if (deg == 1 && !__any_sync(mask, big)) {
    dp = fma(A[RHOT], rv.QC1, rv.Q);
  } else {
    dp = fma(rv.Q * d, ieee::series_g(d, deg, c_pow_gm1), rv.Q);
    if (__any_sync(mask, big)) {
      if (big) dp = rv.Q * exp((kGamma - 1.0) * log1p(d));
    }
  }
  double Fb[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    Fb[q] = cd * dg[q];
    Db[q] = hvcd * dg[q];
  }
  if (DIR == MW_DIR_X) {
    const double y = fma(Fb[1], u, fma(Fb[2], w, Fb[3] * th));  // Fb1 u + Fb2 w + Fb3 th
    Ab[DENS] = -(u * y);
    Ab[UMOM] = fma(Fb[1], u, Fb[0]) + y;
    Ab[WMOM] = Fb[2] * u;
    Ab[RHOT] = fma(Fb[1], dp, Fb[3] * u);
  } else if (!wall) {
    const double y = fma(Fb[1], u, fma(Fb[2], w, Fb[3] * th));
    Ab[DENS] = -(w * y);
    Ab[UMOM] = Fb[1] * w;
    Ab[WMOM] = fma(Fb[2], w, Fb[0]) + y;
    Ab[RHOT] = fma(Fb[2], dp, Fb[3] * w);
  } else {
    Ab[DENS] = 0.0;
    Ab[UMOM] = 0.0;
    Ab[WMOM] = 0.0;
    Ab[RHOT] = Fb[2] * dp;
    Db[DENS] = 0.0;
  }
}

// ---- IEEE-FP64 stage adjoint, x: one kernel ---------------------------------
// The interface adjoints (jt_ieee) and the gather of their transposed taps in
// one pass, with no round trip through the workspace: a warp walks 29-cell
// segments of a row; lane l computes interface f = p0-1+l into shared memory
// and, for l < 29, gathers cell p0+l from interfaces p0-1+l .. p0+2+l in the
// symmetric forms of k_vjp_gather.  The row is periodic: interface f takes its
// taps and G = g(f) - g(f-1) with the periodic rule, so the reference's
// interfaces 0 and nx, which share their taps, enter as one.
constexpr int kFVCells = 29;
constexpr int kFVPos = kFVCells + 6;  // forcing positions p0-3 .. p0+31
constexpr int kFXThreads = 256;
constexpr int kFXWarps = kFXThreads / 32;

struct SmemFX {
  double s[kFXWarps][4][kFVPos];  // forcing at positions p0-3 .. p0+31
  double g[kFXWarps][4][33];      // g at positions p0-2 .. p0+30
  double ab[kFXWarps][4][32];     // Ab at interfaces p0-1 .. p0+30
  double db[kFXWarps][4][32];     // Db
};

// g_dst's halo cells: zero (the frame, strided over every thread of the launch).
__device__ __forceinline__ void zero_frame(const VjpArgs& a) {
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

// g_dst of one cell from its gathered adjoints acc: + g_out (add_gout), + the bases.
__device__ __forceinline__ void store_cell(const VjpArgs& a, long long o, const double acc[4]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const long long oq = q * a.plane + o;
    double v = acc[q];
    if (a.add_gout) v += MW_AT(a.gout, oq, 4 * a.plane);
    if (a.base_a) v += MW_AT(a.base_a, oq, 4 * a.plane);
    if (a.base_b) v += MW_AT(a.base_b, oq, 4 * a.plane);
    MW_AT(a.gdst, oq, 4 * a.plane) = v;
  }
}

// The transposed taps of interfaces p0-1+l .. p0+2+l (slots l .. l+3) on their cell.
__device__ __forceinline__ double gather4(const double* ab, const double* db, int l) {
  const double ca = fma(7.0, ab[l + 1] + ab[l + 2], -(ab[l] + ab[l + 3])) * (1.0 / 12.0);
  const double ce = fma(3.0, db[l + 2] - db[l + 1], db[l] - db[l + 3]);
  return ca + ce;
}

__global__ void __launch_bounds__(kFXThreads) k_vjp_ieee_x(VjpArgs a, const RowV* rows, int nseg, long long total) {
  __shared__ SmemFX sm;
  zero_frame(a);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long b0 = total * blockIdx.x / gridDim.x, b1 = total * (blockIdx.x + 1) / gridDim.x;
  const long long g0 = b0 + (b1 - b0) * w / kFXWarps, g1 = b0 + (b1 - b0) * (w + 1) / kFXWarps;
  const double cd = a.dt_stage / a.d, hvcd = -a.hv * cd;
  auto col = [&](int p) { return ((p % a.nx) + a.nx) % a.nx + kHs; };  // periodic
  for (long long g = g0; g < g1; ++g) {
    const int k = (int)(g / nseg), p0 = (int)(g - (long long)k * nseg) * kFVCells;
    const long long row = (long long)(k + kHs) * a.pitch;
    {
      const int cA = col(p0 - 3 + lane), cB = col(p0 + 29 + lane), cG = col(p0 - 1 + lane), cH = col(p0 - 2);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        sm.s[w][q][lane] = MW_VF(a, q * a.plane + row + cA);
        if (lane < 3) sm.s[w][q][32 + lane] = MW_VF(a, q * a.plane + row + cB);
        sm.g[w][q][lane + 1] = MW_AT(a.gout, q * a.plane + row + cG, 4 * a.plane);
        if (lane == 0) sm.g[w][q][0] = MW_AT(a.gout, q * a.plane + row + cH, 4 * a.plane);
      }
    }
    __syncwarp();
    {  // interface f = p0 - 1 + lane
      double s[4][4], dg[4], Ab[4], Db[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int j = 0; j < 4; ++j) s[q][j] = sm.s[w][q][lane + j];
        dg[q] = sm.g[w][q][lane + 1] - sm.g[w][q][lane];
      }
      const RowV rv = MW_AT(rows, k + kHs, 2 * a.nz + 5);
      jt_ieee<MW_DIR_X>(s, dg, rv, cd, hvcd, false, 0xffffffffu, Ab, Db);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        sm.ab[w][q][lane] = Ab[q];
        sm.db[w][q][lane] = Db[q];
      }
    }
    __syncwarp();
    const int t = p0 + lane;  // cell
    if (lane < kFVCells && t < a.nx) {
      double acc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = gather4(sm.ab[w][q], sm.db[w][q], lane);
      store_cell(a, row + t + kHs, acc);
    }
    __syncwarp();
  }
}

// z: the interface adjoints of k_vjp_iface (same Jacobian, same workspace
// layout) by jt_ieee, one thread per interface; k_vjp_gather follows.  (A
// fused z kernel over tiles of 4 columns x 29 rows staged through shared
// memory was slower at 512 x 256: 39.6 against 18.8 + 17.7 us per call.)
__global__ void k_vjp_iface_ieee_z(VjpArgs a, const RowV* rows) {
  const long long n = a.nif;
  const double cd = a.dt_stage / a.d, hvcd = -a.hv * cd;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
    const long long idx = base + threadIdx.x;
    const unsigned mask = __ballot_sync(0xffffffffu, idx < n);  // base is uniform over the block
    if (idx >= n) continue;
    const int k = (int)(idx / a.nx), c = (int)(idx % a.nx);
    double s[4][4], dg[4], Ab[4], Db[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q][j] = zval(a, q, k - 2 + j, c + kHs);
#pragma unroll
    for (int q = 0; q < 4; ++q) dg[q] = (k < a.nz ? gval(a, q, k, c) : 0.0) - (k > 0 ? gval(a, q, k - 1, c) : 0.0);
    const RowV rv = MW_AT(rows, a.nz + 2 * kHs + k, 2 * a.nz + 5);
    jt_ieee<MW_DIR_Z>(s, dg, rv, cd, hvcd, k == 0 || k == a.nz, mask, Ab, Db);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      MW_WS(a, q * n + idx) = Ab[q];
      MW_WS(a, (4 + q) * n + idx) = Db[q];
    }
  }
}

// k_vjp_gather: 128 columns per CTA, the rows strided over grid.y.
inline dim3 gather_grid(const Geom& g) {
  return dim3((unsigned)((g.pitch + 127) / 128), (unsigned)std::min<long long>(g.plane / g.pitch, 65535));
}

inline unsigned grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 65535LL * 32) b = 65535LL * 32;
  return (unsigned)b;
}

long long n_interfaces(int nx, int nz, int dir) {
  return dir == MW_DIR_X ? (long long)nz * (nx + 1) : (long long)(nz + 1) * nx;
}

// Doubles of the workspace before the IEEE row table: the interface adjoints
// of either direction (8 values per interface).
long long ieee_rows_off(int nx, int nz) {
  return 8 * std::max(n_interfaces(nx, nz, MW_DIR_X), n_interfaces(nx, nz, MW_DIR_Z));
}

}  // namespace

#if MW_CHECK
MW_OOB_COUNTER(oob_count_adjoint)
#endif

// mw_adjoint_split.cu
int launch_vjp_row_table(int nx, int nz, const double* hyc, const double* hytc, const double* hyi, const double* hyti,
                         const double* hypi, void* workspace, cudaStream_t stream);
int launch_vjp_split(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const void* table,
                     const double* forcing, const double* g_out, const double* g_base_a, const double* g_base_b,
                     int add_g_out, double* g_dst, double dt_stage, int direction, cudaStream_t stream);
size_t vjp_split_table_bytes(int nz);

}  // namespace mw

using namespace mw;

extern "C" size_t mw_dirstage_vjp_workspace_bytes(int nx, int nz) {
  if (nx < 1 || nz < 1) return 0;
  const size_t ieee = sizeof(double) * (size_t)ieee_rows_off(nx, nz) + sizeof(RowV) * (size_t)(2 * nz + 5);
  return std::max(ieee, vjp_split_table_bytes(nz));
}

// Checks and launches one stage VJP; split mode expects the background table
// (launch_vjp_row_table) in the workspace when table_ready, else writes it.
static int vjp_stage(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                     const double* hyi, const double* hyti, const double* hypi, const double* forcing,
                     const double* g_out, const double* g_base_a, const double* g_base_b, int add_g_out,
                     double* g_dst, double dt_stage, int direction, int f64_mode, bool table_ready, void* workspace,
                     size_t workspace_bytes, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(finite_pos(dx) && finite_pos(dz) && finite_pos(dt_full), MW_ERR_INVALID_ARG,
             "dx, dz, dt_full must be finite and positive");
  MW_REQUIRE(std::isfinite(dt_stage), MW_ERR_INVALID_ARG, "dt_stage must be finite");
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 or 1");
  MW_REQUIRE(hyc && hytc && hyi && hyti && hypi && forcing && g_out && g_dst && workspace, MW_ERR_INVALID_ARG,
             "NULL pointer argument");
  MW_REQUIRE(aligned(forcing) && aligned(g_out) && aligned(g_dst) && ((uintptr_t)workspace % 8) == 0, MW_ERR_ALIGN,
             "misaligned pointer");
  const size_t bytes = sizeof(double) * 4 * (size_t)make_geom(nx, nz).plane;
  MW_REQUIRE(!ranges_overlap(g_dst, bytes, g_out, bytes), MW_ERR_ALIAS, "g_dst must not overlap g_out");
  MW_REQUIRE(!ranges_overlap(g_dst, bytes, forcing, bytes), MW_ERR_ALIAS, "g_dst must not overlap forcing");
  MW_REQUIRE((!g_base_a || g_base_a == g_dst || !ranges_overlap(g_dst, bytes, g_base_a, bytes)) &&
                 (!g_base_b || g_base_b == g_dst || !ranges_overlap(g_dst, bytes, g_base_b, bytes)),
             MW_ERR_ALIAS, "a base array must equal g_dst or not overlap it");
  MW_REQUIRE(valid_f64_mode(f64_mode), MW_ERR_INVALID_ARG, "f64_mode must be MW_F64_NATIVE, _SPLIT or _IEEE");
  const size_t need = mw_dirstage_vjp_workspace_bytes(nx, nz);
  MW_REQUIRE(workspace_bytes >= need, MW_ERR_WORKSPACE, "vjp workspace needs %zu bytes, got %zu", need,
             workspace_bytes);
  if (f64_mode == MW_F64_SPLIT) {
    if (!table_ready && (st = launch_vjp_row_table(nx, nz, hyc, hytc, hyi, hyti, hypi, workspace, (cudaStream_t)stream)))
      return st;
    return launch_vjp_split(nx, nz, dx, dz, dt_full, hyc, workspace, forcing, g_out, g_base_a, g_base_b, add_g_out,
                            g_dst, dt_stage, direction, (cudaStream_t)stream);
  }
  const Geom g = make_geom(nx, nz);
  VjpArgs a;
  a.nx = nx;
  a.nz = nz;
  a.pitch = g.pitch;
  a.plane = g.plane;
  a.d = direction == MW_DIR_X ? dx : dz;
  a.hv = -kHvBeta * a.d / (16 * dt_full);
  a.dt_stage = dt_stage;
  a.hyc = hyc;
  a.hytc = hytc;
  a.hyi = hyi;
  a.hyti = hyti;
  a.hypi = hypi;
  a.forcing = forcing;
  a.gout = g_out;
  a.base_a = g_base_a;
  a.base_b = g_base_b;
  a.add_gout = add_g_out;
  a.gdst = g_dst;
  a.ws = (double*)workspace;
  a.nif = n_interfaces(nx, nz, direction);
  cudaStream_t s = (cudaStream_t)stream;
  RowV* rows = (RowV*)((double*)workspace + ieee_rows_off(nx, nz));
  if (f64_mode == MW_F64_IEEE && !table_ready) {
    k_vjp_rows_ieee<<<grid_for(2 * nz + 5, 128), 128, 0, s>>>(nz, hyc, hytc, hyi, hyti, hypi, rows);
    if ((st = check_launch("vjp row-table launch"))) return st;
  }
  if (f64_mode == MW_F64_IEEE && direction == MW_DIR_X) {  // one fused launch, a grid of resident CTAs at most
    int per_sm = 0, sms = 0, dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vjp_ieee_x, kFXThreads, 0);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(MW_ERR_CUDA, "vjp occupancy query: %s", cudaGetErrorString(e));
    const long long resident = (long long)std::max(1, per_sm) * sms;
    const int nseg = (nx + kFVCells - 1) / kFVCells;
    const long long total = (long long)nseg * nz;
    const long long grid = std::max(1LL, std::min(resident, (total + kFXWarps - 1) / kFXWarps));
    k_vjp_ieee_x<<<(unsigned)grid, kFXThreads, 0, s>>>(a, rows, nseg, total);
    return check_launch("vjp launch");
  }
  if (f64_mode == MW_F64_IEEE) {
    k_vjp_iface_ieee_z<<<grid_for(a.nif, 128), 128, 0, s>>>(a, rows);
    if ((st = check_launch("vjp interface launch"))) return st;
    k_vjp_gather<MW_DIR_Z><<<gather_grid(g), 128, 0, s>>>(a);
    return check_launch("vjp gather launch");
  }
  if (direction == MW_DIR_X) {
    k_vjp_iface<MW_DIR_X><<<grid_for(a.nif, 128), 128, 0, s>>>(a);
    if ((st = check_launch("vjp interface launch"))) return st;
    k_vjp_gather<MW_DIR_X><<<gather_grid(g), 128, 0, s>>>(a);
  } else {
    k_vjp_iface<MW_DIR_Z><<<grid_for(a.nif, 128), 128, 0, s>>>(a);
    if ((st = check_launch("vjp interface launch"))) return st;
    k_vjp_gather<MW_DIR_Z><<<gather_grid(g), 128, 0, s>>>(a);
  }
  return check_launch("vjp gather launch");
}

extern "C" int mw_dirstage_vjp_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hyc,
                                   const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                                   const double* forcing, const double* g_out, const double* g_base_a,
                                   const double* g_base_b, int add_g_out, double* g_dst, double dt_stage,
                                   int direction, int f64_mode, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  return vjp_stage(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, forcing, g_out, g_base_a, g_base_b, add_g_out,
                   g_dst, dt_stage, direction, f64_mode, false, workspace, workspace_bytes, stream);
}

// ---------------------------------------------------------------------------
// Adjoint of one recorded time step (stages from mw_step_record_f64).  Per
// direction, in reverse (RK3 of solve/step.py:112-141):
//   s2bar = VJP(s2; g),  s1bar = VJP(s1; s2bar),  Sbar = g + s2bar + s1bar + VJP(S; s1bar).
extern "C" int mw_step_vjp_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                               const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                               const double* stages, const double* g_out, double* g_in, double* gbuf, int reverse,
                               int f64_mode, void* workspace, size_t workspace_bytes, void* stream) {
  MW_REQUIRE(stages && g_out && g_in && gbuf, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(finite_pos(dt), MW_ERR_INVALID_ARG, "dt must be finite and positive");
  const size_t n = 4 * (size_t)make_geom(nx, nz).plane;
  MW_REQUIRE(!ranges_overlap(gbuf, 3 * n * sizeof(double), g_in, n * sizeof(double)) &&
                 !ranges_overlap(gbuf, 3 * n * sizeof(double), g_out, n * sizeof(double)),
             MW_ERR_ALIAS, "gbuf must not overlap g_in or g_out");
  double* gA = gbuf;
  double* gB = gbuf + n;
  double* gC = gbuf + 2 * n;
  const int dirs[2] = {reverse ? MW_DIR_X : MW_DIR_Z, reverse ? MW_DIR_Z : MW_DIR_X};
  const double* cur = g_out;
  int st;
  bool ready = false;  // split / IEEE modes: the background table is written by the first stage call
  for (int d = 1; d >= 0; --d) {
    const double* S = stages + (3 * d) * n;
    const double* s1 = S + n;
    const double* s2 = S + 2 * n;
    double* out = d == 1 ? gC : g_in;
    if ((st = vjp_stage(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, s2, cur, nullptr, nullptr, 0, gA, dt,
                        dirs[d], f64_mode, ready, workspace, workspace_bytes, stream)))
      return st;
    ready = true;
    if ((st = vjp_stage(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, s1, gA, nullptr, nullptr, 0, gB, dt / 2,
                        dirs[d], f64_mode, ready, workspace, workspace_bytes, stream)))
      return st;
    if ((st = vjp_stage(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, S, gB, cur, gA, 1, out, dt / 3, dirs[d],
                        f64_mode, ready, workspace, workspace_bytes, stream)))
      return st;
    cur = out;
  }
  return MW_OK;
}
