// mw_dirstage.cu -- fused direction-stage kernels and the RK3 step driver.
//
// One kernel launch performs one discrete_step of the reference
// (pyminiweather/solve/step.py:21-82): halo rule, 4-point interpolation,
// flux with hyperviscosity, flux divergence, gravity term, forcing, stage
// update.  Halo cells are never read: the periodic (x) and wall (z) rules of
// ics/bcs.py are applied to the indices / values as they are loaded.
//
// Native FP64 and FP32 forms (the IEEE-FP64 form with the fewest operations
// is in mw_fp64_stage.cu, the split form in mw_split_stage.cu); this file
// also holds the stage and step entry points of every form.
// x pass (plain loads): a CTA walks a run of 255-cell chunks of one row.
// Thread t evaluates the flux at interface x0+t into shared memory; after one
// barrier thread t updates cell x0+t from interfaces t and t+1.  Interface
// loads are coalesced rows; the four taps hit L1.  Row constants are formed
// once per CTA and row.
// z pass (plain loads): one thread per column marching down a tile of kZTile
// rows with a rolling 4-row register window, so every forcing value is loaded
// once per tile and every interface flux is evaluated once; rows are
// coalesced across the warp.
// FP32 on 16-byte-aligned rows (nx % 4 == 0, nx >= 128): both passes are fed
// by tensor copies instead (k_stage_x_f32_bulk, k_stage_z_f32_bulk below).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

#include "mw_common.cuh"
#include "mw_ensemble.cuh"
#include "mw_split.cuh"

namespace mw {

constexpr int kXThreads = 256;          // interfaces per x chunk
constexpr int kXCells = kXThreads - 1;  // cells updated per x chunk
constexpr int kXBlocksPerRow = 4;       // x CTAs per row; each walks a run of chunks
constexpr int kZThreads = 128;          // columns per z CTA
constexpr int kZTile = 64;              // rows marched per z thread

enum Mode { MODE_NATIVE64 = 0, MODE_SPLIT64 = 1, MODE_F32 = 2 };

template <typename T>
struct StageArgs {
  int nx, nz, pitch;
  long long plane;
  double dx, dz;
  double hv;        // -hv_beta * d / (16 dt_full), d = dx or dz (interpolate.py:101,149)
  double dt_stage;
  const double* hyc;
  const double* hytc;
  const double* hyi;
  const double* hyti;
  const double* hypi;
  const double* srcw;
  const T* init;
  T* forcing;
  T* out;
  unsigned flags;
  int chunks_per_block;
  int z_tile;
  // FP32 form: the stage constants rounded once (FP64 arithmetic in the
  // kernels would occupy the FP64 pipe per cell)
  float hv_f;       // hv
  float c_f;        // dt_stage / d
  float dt_f;       // dt_stage
};

// Bounds-checked element access (MW_AT) to the arrays of one stage.
#define MW_SF(a, off) MW_AT((a).forcing, (off), 4 * (a).plane)
#define MW_SI(a, off) MW_AT((a).init, (off), 4 * (a).plane)
#define MW_SO(a, off) MW_AT((a).out, (off), 4 * (a).plane)
#define MW_BC(a, p, k) MW_AT((a).p, (k), (a).nz + 2 * kHs)  // cell-centre background
#define MW_BI(a, p, k) MW_AT((a).p, (k), (a).nz + 1)        // interface background
#define MW_SW(a, off) MW_AT((a).srcw, (off), (long long)(a).nx * (a).nz)

template <typename T>
__host__ __device__ inline void set_f32_constants(StageArgs<T>& a, int direction) {
  a.hv_f = float(a.hv);
  a.c_f = float(a.dt_stage / (direction == MW_DIR_X ? a.dx : a.dz));
  a.dt_f = float(a.dt_stage);
}

// ---- interpolation in the accumulation order of scipy.signal.convolve ----
template <typename T>
__device__ __forceinline__ T interp4(T s0, T s1, T s2, T s3) {
  const T k0 = T(-1.0 / 12), k1 = T(7.0 / 12);
  return ((s0 * k0 + s1 * k1) + s2 * k1) + s3 * k0;
}
template <typename T>
__device__ __forceinline__ T diff3(T s0, T s1, T s2, T s3) {
  return ((s0 * T(-1) + s1 * T(3)) + s2 * T(-3)) + s3;
}

// ---- fluxes: the reference's formulas on the FP64 pipe ----
__device__ __forceinline__ void flux_x_native(const double s[4][4], double hyc, double hytc, double hv, double F[4]) {
  double v[4], d3[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = interp4(s[q][0], s[q][1], s[q][2], s[q][3]);
    d3[q] = diff3(s[q][0], s[q][1], s[q][2], s[q][3]);
  }
  double rho = v[DENS] + hyc;
  double u = v[UMOM] / rho;
  double w = v[WMOM] / rho;
  double t = (v[RHOT] + hytc) / rho;
  double p = kC0 * pow(rho * t, kGamma);
  F[0] = rho * u - hv * d3[DENS];
  F[1] = rho * (u * u) + p - hv * d3[UMOM];
  F[2] = rho * u * w - hv * d3[WMOM];
  F[3] = rho * u * t - hv * d3[RHOT];
}

__device__ __forceinline__ void flux_z_native(const double s[4][4], double hyi, double hyti, double hypi, double hv,
                                              bool wall, double F[4]) {
  double v[4], d3[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = interp4(s[q][0], s[q][1], s[q][2], s[q][3]);
    d3[q] = diff3(s[q][0], s[q][1], s[q][2], s[q][3]);
  }
  double rho = v[DENS] + hyi;
  double u = v[UMOM] / rho;
  double w = v[WMOM] / rho;
  double t = (v[RHOT] + hyti) / rho;
  double p = kC0 * pow(rho * t, kGamma) - hypi;
  if (wall) {
    w = 0.0;
    d3[DENS] = 0.0;
  }
  F[0] = rho * w - hv * d3[DENS];
  F[1] = rho * w * u - hv * d3[UMOM];
  F[2] = rho * (w * w) + p - hv * d3[WMOM];
  F[3] = rho * w * t - hv * d3[RHOT];
}

// ---- FP32 fluxes (precision form) ----
// Pressure enters as the perturbation P_row * ((1 + delta)^gamma - 1),
// delta = (rho theta)' / (rho theta)_background.  In z this is exactly the
// reference's p - hy_pressure_int; in x the row constant C0 (rho theta)_bg^gamma
// cancels in the flux difference, so the tendency is unchanged while FP32 no
// longer differences two values near 1e5.  rho*u is formed as (rho u)' itself.
// (1+d)^gamma - 1: the binomial series to degree 6 for |d| <= 1/8 (tail below
// 2^-26 relative), else expm1f(gamma log1pf(d)).
__device__ __forceinline__ float pgm1f(float d) {
  constexpr float c1 = float(kGamma);
  constexpr float c2 = float(kGamma * (kGamma - 1) / 2);
  constexpr float c3 = float(kGamma * (kGamma - 1) * (kGamma - 2) / 6);
  constexpr float c4 = float(kGamma * (kGamma - 1) * (kGamma - 2) * (kGamma - 3) / 24);
  constexpr float c5 = float(kGamma * (kGamma - 1) * (kGamma - 2) * (kGamma - 3) * (kGamma - 4) / 120);
  constexpr float c6 = float(kGamma * (kGamma - 1) * (kGamma - 2) * (kGamma - 3) * (kGamma - 4) * (kGamma - 5) / 720);
  if (fabsf(d) <= 0.125f) {
    float y = fmaf(c6, d, c5);
    y = fmaf(y, d, c4);
    y = fmaf(y, d, c3);
    y = fmaf(y, d, c2);
    y = fmaf(y, d, c1);
    return y * d;
  }
  return expm1f(float(kGamma) * log1pf(d));
}

struct RowF {
  float hy_r, hy_rt, inv_hy_rt, P;
};

__device__ __forceinline__ void flux_x_f32(const float s[4][4], const RowF& r, float hv, float F[4]) {
  float v[4], d3[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = interp4(s[q][0], s[q][1], s[q][2], s[q][3]);
    d3[q] = diff3(s[q][0], s[q][1], s[q][2], s[q][3]);
  }
  float rho = v[DENS] + r.hy_r;
  float ri = 1.0f / rho;
  float u = v[UMOM] * ri;
  float w = v[WMOM] * ri;
  float th = (v[RHOT] + r.hy_rt) * ri;
  float pp = r.P * pgm1f(v[RHOT] * r.inv_hy_rt);
  F[0] = v[UMOM] - hv * d3[DENS];
  F[1] = v[UMOM] * u + pp - hv * d3[UMOM];
  F[2] = v[UMOM] * w - hv * d3[WMOM];
  F[3] = v[UMOM] * th - hv * d3[RHOT];
}

__device__ __forceinline__ void flux_z_f32(const float s[4][4], const RowF& r, float hv, bool wall, float F[4]) {
  float v[4], d3[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = interp4(s[q][0], s[q][1], s[q][2], s[q][3]);
    d3[q] = diff3(s[q][0], s[q][1], s[q][2], s[q][3]);
  }
  float rho = v[DENS] + r.hy_r;
  float ri = 1.0f / rho;
  float u = v[UMOM] * ri;
  float w = v[WMOM] * ri;
  float th = (v[RHOT] + r.hy_rt) * ri;
  float pp = r.P * pgm1f(v[RHOT] * r.inv_hy_rt);
  float rw = v[WMOM];
  if (wall) {
    w = 0.0f;
    rw = 0.0f;
    d3[DENS] = 0.0f;
  }
  F[0] = rw - hv * d3[DENS];
  F[1] = rw * u - hv * d3[UMOM];
  F[2] = rw * w + pp - hv * d3[WMOM];
  F[3] = rw * th - hv * d3[RHOT];
}

// ---- halo rules -----------------------------------------------------------
// Periodic x (ics/bcs.py:35-39): interior column j in [-2, nx+1] maps to j mod nx.
__device__ __forceinline__ int wrap_x(int j, int nx) { return j < 0 ? j + nx : (j >= nx ? j - nx : j); }

// Wall z (ics/bcs.py:92-148): value of variable q at interior row k in
// [-2, nz+1] of the halo-indexed column col.
template <typename T>
__device__ __forceinline__ T zval(const StageArgs<T>& a, int q, int k, int col) {
  if (k >= 0 && k < a.nz) return MW_SF(a, q * a.plane + (long long)(k + kHs) * a.pitch + col);
  if (q == WMOM) return T(0);
  const int src = k < 0 ? kHs : a.nz + kHs - 1;  // halo-indexed source row
  T s = MW_SF(a, q * a.plane + (long long)src * a.pitch + col);
  if (q == UMOM) return T((double)s / MW_BC(a, hyc, src) * MW_BC(a, hyc, k + kHs));
  return s;
}

template <typename T>
__device__ __forceinline__ void write_z_halo_column(const StageArgs<T>& a, int col) {
  const int rows[4] = {-2, -1, a.nz, a.nz + 1};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    T vals[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) vals[r] = zval(a, q, rows[r], col);
#pragma unroll
    for (int r = 0; r < 4; ++r) MW_SF(a, q * a.plane + (long long)(rows[r] + kHs) * a.pitch + col) = vals[r];
  }
}

// ---------------------------------------------------------------------------
// Tiles, called by the single-grid kernels and the persistent ensemble
// kernels alike; every thread of the CTA must call them (they contain barriers).
template <typename T>
struct SmemXT {
  T sF[4][kXThreads];
  RowF row;
};
struct SmemZT {
  RowF row[kEnsZTileMax + 1];
};

__device__ __forceinline__ RowF rowf_x(double hy_r, double hy_rt) {
  RowF r;
  r.hy_r = split::d2f(hy_r);
  r.hy_rt = split::d2f(hy_rt);
  r.inv_hy_rt = 1.0f / r.hy_rt;
  r.P = float(kC0) * powf(r.hy_rt, float(kGamma));
  return r;
}

__device__ __forceinline__ RowF rowf_z(double hy_r, double hy_rt, double hy_p) {
  RowF r;
  r.hy_r = split::d2f(hy_r);
  r.hy_rt = split::d2f(hy_rt);
  r.inv_hy_rt = 1.0f / r.hy_rt;
  r.P = split::d2f(hy_p);
  return r;
}

// x: row k, chunks [cbeg, cend) of kXCells cells.  Thread t evaluates the
// flux at interface x0+t into shared memory; after one barrier thread t
// updates cell x0+t.  halo: write this row's periodic halo into forcing.
template <typename T, int MODE>
__device__ __forceinline__ void x_rowrun_t(const StageArgs<T>& a, int k, int cbeg, int cend, bool halo,
                                           SmemXT<T>& sm) {
  const int t = threadIdx.x;
  const long long row = (long long)(k + kHs) * a.pitch;
  if constexpr (MODE != MODE_NATIVE64) {
    if (t == 0) sm.row = rowf_x(MW_BC(a, hyc, k + kHs), MW_BC(a, hytc, k + kHs));
  }
  if (halo && t < 4) {
    const int dst[4] = {0, 1, a.nx + kHs, a.nx + kHs + 1};
    const int src[4] = {a.nx, a.nx + 1, kHs, kHs + 1};
#pragma unroll
    for (int q = 0; q < 4; ++q) MW_SF(a, q * a.plane + row + dst[t]) = MW_SF(a, q * a.plane + row + src[t]);
  }
  __syncthreads();
  for (int chunk = cbeg; chunk < cend; ++chunk) {
    const int x0 = chunk * kXCells;
    const int i = x0 + t;  // interface index 0..nx (between cells i-1 and i)
    const bool upd = t < kXCells && i < a.nx;
    const long long o = row + i + kHs;
    T iv[4];
    if (upd) {  // issued before the flux so the load latency is covered
#pragma unroll
      for (int q = 0; q < 4; ++q) iv[q] = MW_SI(a, q * a.plane + o);
    }
    if (i <= a.nx) {
      T s[4][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const long long col = wrap_x(i - 2 + j, a.nx) + kHs;
#pragma unroll
        for (int q = 0; q < 4; ++q) s[q][j] = __ldg(&MW_SF(a, q * a.plane + row + col));
      }
      T F[4];
      if constexpr (MODE == MODE_NATIVE64) {
        flux_x_native(s, MW_BC(a, hyc, k + kHs), MW_BC(a, hytc, k + kHs), a.hv, F);
      } else {
        flux_x_f32(s, sm.row, a.hv_f, F);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) sm.sF[q][t] = F[q];
    }
    __syncthreads();
    if (upd) {
      if constexpr (MODE == MODE_NATIVE64) {
        double tend[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) tend[q] = -(sm.sF[q][t + 1] - sm.sF[q][t]) / a.dx;
        if (a.srcw) tend[WMOM] = tend[WMOM] + MW_SW(a, (long long)k * a.nx + i);
#pragma unroll
        for (int q = 0; q < 4; ++q) MW_SO(a, q * a.plane + o) = iv[q] + a.dt_stage * tend[q];
      } else {
        const float c = a.c_f, dt = a.dt_f;
        float inc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) inc[q] = (sm.sF[q][t] - sm.sF[q][t + 1]) * c;
        if (a.srcw) inc[WMOM] += dt * split::d2f(MW_SW(a, (long long)k * a.nx + i));
#pragma unroll
        for (int q = 0; q < 4; ++q) MW_SO(a, q * a.plane + o) = iv[q] + inc[q];
      }
    }
    __syncthreads();
  }
}

// The plain-load FP32 passes wait on memory (one row or segment of loads in
// flight per thread, no registers to spare for more): prefetch instructions
// bring later rows / segments into L2 without holding registers.  Measured on
// the 256-member thermal ensemble (ms per step): none 1.474, z 2 rows ahead
// 1.410 (1, 3, 4, 8: 1.40-1.44 with x), x 1 segment 1.453, both (x 2, z 2) 1.393;
// x 3 segments ahead 1.406, x prefetched into L1 instead of L2 1.391; the next
// row taken one row early and its first lines prefetched 1.430.
#ifndef MW_F32_PF_Z
#define MW_F32_PF_Z 2  // FP32 z march: L2 prefetch of the rows this many steps ahead (0: none)
#endif
#ifndef MW_F32_PF_X
#define MW_F32_PF_X 2  // FP32 ensemble x rows: L2 prefetch of the segment this many ahead (0: none)
#endif
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// z: columns [cb*NC, cb*NC+NC) (NC threads), rows [z0, z0+zt), zt <= kEnsZTileMax; one
// thread per column marching the rows with a rolling 4-row window, the next
// row loaded one step ahead.  halo: write the wall halo rows of these columns
// (cb == 0 also does the four x-halo columns).
template <typename T, int MODE, int NC = kZThreads>
__device__ __forceinline__ void z_tile_t(const StageArgs<T>& a, int cb, int z0, int zt, bool halo, SmemZT& sm) {
  const int z1 = min(z0 + zt, a.nz);
  if constexpr (MODE != MODE_NATIVE64) {
    for (int r = threadIdx.x; r <= z1 - z0; r += NC) {
      const int k = z0 + r;
      sm.row[r] = rowf_z(MW_BI(a, hyi, k), MW_BI(a, hyti, k), MW_BI(a, hypi, k));
    }
    __syncthreads();
  }
  const int c = cb * NC + threadIdx.x;  // interior column
  if (halo && cb == 0 && threadIdx.x < 4) {
    const int hcol[4] = {0, 1, a.nx + kHs, a.nx + kHs + 1};
    write_z_halo_column(a, hcol[threadIdx.x]);
  }
  if (c < a.nx) {
    const int col = c + kHs;
    if (halo) write_z_halo_column(a, col);
    T w[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q][j] = zval(a, q, z0 - 2 + j, col);
    auto flux_at = [&](int k, T F[4]) {
      const bool wall = (k == 0) || (k == a.nz);
      if constexpr (MODE == MODE_NATIVE64) {
        flux_z_native(w, MW_BI(a, hyi, k), MW_BI(a, hyti, k), MW_BI(a, hypi, k), a.hv, wall, F);
      } else {
        flux_z_f32(w, sm.row[k - z0], a.hv_f, wall, F);
      }
    };
    T nxt[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) nxt[q] = zval(a, q, z0 + 2, col);
    T Fp[4];
    flux_at(z0, Fp);
    for (int k = z0; k < z1; ++k) {
      const long long o = (long long)(k + kHs) * a.pitch + col;
      T iv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) iv[q] = MW_SI(a, q * a.plane + o);
      const T rho_k = w[DENS][2];  // forcing rho' at cell k (interpolate.py:248-250)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        w[q][0] = w[q][1];
        w[q][1] = w[q][2];
        w[q][2] = w[q][3];
        w[q][3] = nxt[q];
      }
      if (k + 1 < z1) {  // load the row needed by the next iteration now
#pragma unroll
        for (int q = 0; q < 4; ++q) nxt[q] = zval(a, q, k + 3, col);
      }
      if constexpr (MODE == MODE_F32 && MW_F32_PF_Z > 0) {  // rows MW_F32_PF_Z steps ahead into L2
        const int kf = k + 3 + MW_F32_PF_Z, ki = k + MW_F32_PF_Z;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (kf < a.nz) prefetch_l2(&MW_SF(a, q * a.plane + (long long)(kf + kHs) * a.pitch + col));
          if (ki < z1) prefetch_l2(&MW_SI(a, q * a.plane + (long long)(ki + kHs) * a.pitch + col));
        }
      }
      T Fn[4];
      flux_at(k + 1, Fn);
      if constexpr (MODE == MODE_NATIVE64) {
        double tend[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) tend[q] = -(Fn[q] - Fp[q]) / a.dz;
        tend[WMOM] = tend[WMOM] - rho_k * kGrav;
        if (a.srcw) tend[WMOM] = tend[WMOM] + MW_SW(a, (long long)k * a.nx + c);
#pragma unroll
        for (int q = 0; q < 4; ++q) MW_SO(a, q * a.plane + o) = iv[q] + a.dt_stage * tend[q];
      } else {
        const float cz = a.c_f, dt = a.dt_f;
        float inc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) inc[q] = (Fp[q] - Fn[q]) * cz;
        inc[WMOM] -= dt * (rho_k * float(kGrav));
        if (a.srcw) inc[WMOM] += dt * split::d2f(MW_SW(a, (long long)k * a.nx + c));
#pragma unroll
        for (int q = 0; q < 4; ++q) MW_SO(a, q * a.plane + o) = iv[q] + inc[q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) Fp[q] = Fn[q];
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Single grid: x CTA (blockIdx.x, row) walks a run of chunks; z CTA is one tile.
template <typename T, int MODE>
__global__ void __launch_bounds__(kXThreads) k_stage_x(StageArgs<T> a) {
  __shared__ SmemXT<T> sm;
  const int nchunks = (a.nx + kXCells - 1) / kXCells;
  const int cbeg = blockIdx.x * a.chunks_per_block;
  const int cend = min(cbeg + a.chunks_per_block, nchunks);
  const bool halo = (a.flags & MW_FLAG_WRITE_HALO) && blockIdx.x == 0;
  for (int k = blockIdx.y; k < a.nz; k += gridDim.y) x_rowrun_t<T, MODE>(a, k, cbeg, cend, halo, sm);
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kZThreads) k_stage_z(StageArgs<T> a, int tile0) {
  __shared__ SmemZT sm;
  const int tile = tile0 + blockIdx.y;  // row tile (grid.y is capped at 65535: one launch per 65535 tiles)
  z_tile_t<T, MODE>(a, blockIdx.x, tile * a.z_tile, a.z_tile, (a.flags & MW_FLAG_WRITE_HALO) && tile == 0, sm);
}

// ---------------------------------------------------------------------------
// FP32 z pass fed by the tensor memory accelerator (cp.async.bulk.tensor +
// mbarrier).  The same march as k_stage_z<float, MODE_F32>, but the forcing
// and init rows reach shared memory through a ring of kBulkStages blocks of
// kBulkRows rows: per block and array one 3-D tensor copy of the CTA's
// 132-column segment of kBulkRows rows of the four variables (halo-indexed
// columns [128 cb, 128 cb + 132): a 16-byte-aligned start, so the grid needs
// nx % 4 == 0, nx >= 128 and 16-byte-aligned arrays).  Thread 0 issues a
// block's copies and their byte count on the block's mbarrier; the consumers
// wait on it (bounded: a copy that never lands counts a timeout and the tile
// is abandoned, never a hang) and, once every thread has finished a block,
// thread 0 refills its slot with the block kBulkStages further on.  Forcing
// rows outside [0, nz) are never copied: the wall rule builds them from the
// register window.
#ifndef MW_BZ_STAGES
#define MW_BZ_STAGES 3
#endif
constexpr int kBulkRows = 4;  // >= 4: the window's next row (4 rows ahead) then lies in block b + 1
constexpr int kBulkStages = MW_BZ_STAGES;  // ring slots (3: 51.7 KB of shared memory, 4 CTAs per SM;
                                           // 4 slots, 3 CTAs per SM, measured 5 % slower)
static_assert(kBulkStages >= 3, "the march waits for block b + 1 before refilling block b - 1's slot");
constexpr int kBulkCols = kZThreads + 4;  // 132 floats = 528 bytes, a multiple of 16
constexpr long long kBulkSpin = 1LL << 20;  // try_wait rounds before a wait gives up
constexpr unsigned kBulkBoxBytes = 4u * kBulkRows * kBulkCols * 4;  // one array's box: 4 variables x rows x columns

static __device__ unsigned long long g_bulk_timeouts;

struct SmemZBulk {
  float f[kBulkStages][4][kBulkRows][kBulkCols];  // forcing rows
  float i[kBulkStages][4][kBulkRows][kBulkCols];  // init rows
  RowF row[kEnsZTileMax + 1];
  unsigned long long full[kBulkStages];
};

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of the given parity to complete, at most kBulkSpin rounds.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  for (long long it = 0; it < kBulkSpin; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__global__ void __launch_bounds__(kZThreads) k_stage_z_f32_bulk(StageArgs<float> a, int tile0,
                                                                 const __grid_constant__ CUtensorMap tmf,
                                                                 const __grid_constant__ CUtensorMap tmi) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemZBulk& sm = *reinterpret_cast<SmemZBulk*>(smem_raw);
  const int tile = tile0 + blockIdx.y;
  const int z0 = tile * a.z_tile, z1 = min(z0 + a.z_tile, a.nz), zt = z1 - z0;
  const int cb = blockIdx.x, t = threadIdx.x;
  const int c = cb * kZThreads + t;                 // interior column of this thread
  const long long col0 = (long long)cb * kZThreads;  // first halo-indexed column of the segments
  const int nblk = (zt + 4 + kBulkRows - 1) / kBulkRows;  // forcing rows z0-2 .. z1+1
  for (int r = t; r <= zt; r += kZThreads) {
    const int k = z0 + r;
    sm.row[r] = rowf_z(MW_BI(a, hyi, k), MW_BI(a, hyti, k), MW_BI(a, hypi, k));
  }
  if (t == 0) {
    for (int s = 0; s < kBulkStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&sm.full[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // block b: forcing rows j = z0 - 2 + 4b + r and init rows k = z0 + 4b + r, r < kBulkRows, each a
  // 132-column x 4-row x 4-variable box of one tensor copy (rows beyond the array read as zero;
  // forcing rows outside [0, nz) are never used)
  auto issue = [&](int b) {
    const int s = b % kBulkStages;
    const unsigned bar = smem_addr(&sm.full[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(2u * kBulkBoxBytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(&sm.f[s][0][0][0])),
        "l"(reinterpret_cast<unsigned long long>(&tmf)), "r"((int)col0), "r"(z0 + kBulkRows * b), "r"(0), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(&sm.i[s][0][0][0])),
        "l"(reinterpret_cast<unsigned long long>(&tmi)), "r"((int)col0), "r"(z0 + kHs + kBulkRows * b), "r"(0),
        "r"(bar)
        : "memory");
  };
  int issued = 0, waited = 0;  // thread 0: blocks issued; every thread: blocks whose copies it saw land
  if (t == 0)
    for (; issued < min(kBulkStages, nblk); ++issued) issue(issued);
  auto wait_block = [&](int b) {
    const bool ok = mbar_wait_bounded(&sm.full[b % kBulkStages], (b / kBulkStages) & 1);
    if (ok) waited = b + 1;
    return ok;
  };
  bool ok = __syncthreads_and(wait_block(0));
  if (ok && (a.flags & MW_FLAG_WRITE_HALO) && tile == 0 && cb == 0 && t < 4) {
    const int hcol[4] = {0, 1, a.nx + kHs, a.nx + kHs + 1};
    write_z_halo_column(a, hcol[t]);
  }
  const bool act = c < a.nx;
  if (ok && act && (a.flags & MW_FLAG_WRITE_HALO) && tile == 0) write_z_halo_column(a, c + kHs);
  // forcing value of variable q at relative row rel (row z0 - 2 + rel), the
  // wall rule applied from the last interior row value `edge` outside [0, nz)
  auto fsm = [&](int q, int rel) {
    return sm.f[(rel / kBulkRows) % kBulkStages][q][rel % kBulkRows][t + 2];
  };
  auto wall = [&](int q, int k, float edge) {  // k outside [0, nz); edge = value of the nearest interior row
    if (q == WMOM) return 0.0f;
    if (q == UMOM) {
      const int src = k < 0 ? kHs : a.nz + kHs - 1;
      return float((double)edge / MW_BC(a, hyc, src) * MW_BC(a, hyc, k + kHs));
    }
    return edge;
  };
  float w[4][4], last[4];  // window rows z0-2 .. z0+1; last: the latest interior row loaded
  if (ok) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float e0 = fsm(q, max(0, 2 - z0));  // row max(0, z0 - 2)... the bottom row when z0 < 2
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = z0 - 2 + j;
        w[q][j] = (k >= 0 && k < a.nz) ? fsm(q, j) : wall(q, k, k < 0 ? e0 : fsm(q, a.nz - 1 - (z0 - 2)));
      }
      last[q] = fsm(q, min(3, a.nz - 1 - (z0 - 2)));
    }
  }
  float Fp[4] = {0.f, 0.f, 0.f, 0.f};
  if (ok) flux_z_f32(w, sm.row[0], a.hv_f, z0 == 0, Fp);
  for (int i = 0; ok && i < zt; ++i) {
    if (i % kBulkRows == 0) {
      const int b = i / kBulkRows;
      ok = __syncthreads_and(b + 1 < nblk ? wait_block(b + 1) : true);  // also: block b - 1 is done
      if (!ok) break;
      if (t == 0 && b >= 1 && issued < nblk) issue(issued++);
    }
    const int k = z0 + i;
    float iv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) iv[q] = sm.i[(i / kBulkRows) % kBulkStages][q][i % kBulkRows][t + 2];
    const float rho_k = w[DENS][2];
    const int kn = k + 2;  // the row entering the window
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float v;
      if (kn < a.nz) {
        v = fsm(q, i + 4);
        last[q] = v;
      } else {
        v = wall(q, kn, last[q]);
      }
      w[q][0] = w[q][1];
      w[q][1] = w[q][2];
      w[q][2] = w[q][3];
      w[q][3] = v;
    }
    float Fn[4];
    flux_z_f32(w, sm.row[i + 1], a.hv_f, k + 1 == a.nz, Fn);
    if (act) {
      const long long o = (long long)(k + kHs) * a.pitch + c + kHs;
      float inc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) inc[q] = (Fp[q] - Fn[q]) * a.c_f;
      inc[WMOM] -= a.dt_f * (rho_k * float(kGrav));
      if (a.srcw) inc[WMOM] += a.dt_f * split::d2f(MW_SW(a, (long long)k * a.nx + c));
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_SO(a, q * a.plane + o) = iv[q] + inc[q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) Fp[q] = Fn[q];
  }
  if (!ok) {
    // a copy never completed: count it, and let no copy of this CTA land after
    // it exits (each remaining wait again bounded)
    if (t == 0) {
      atomicAdd(&g_bulk_timeouts, 1ULL);
      for (int b = waited; b < issued; ++b) mbar_wait_bounded(&sm.full[b % kBulkStages], (b / kBulkStages) & 1);
    }
  }
}

// FP32 x pass fed by the tensor memory accelerator.  The row-major list of
// kBXCells-cell chunks is split into equal ranges, one per CTA of kBXThreads
// threads; per chunk one 3-D tensor copy per array of kBXCols columns x 1 row
// x 4 variables (halo-indexed columns [x0, x0 + kBXCols): cells x0 - 2 ..
// x0 + kBXCells + 1, starting at a 16-byte boundary since x0 is a multiple of
// 4) lands in a ring of kBXStages slots.  Thread t owns cells x0 + 4t ..
// x0 + 4t + 3: it reads their taps (cells x0 + 4t - 2 .. x0 + 4t + 5) as two
// 16-byte words per variable, evaluates the fluxes at its five interfaces
// x0 + 4t .. x0 + 4t + 4 (the last one again by thread t + 1: no flux
// exchange, no flux array) and updates its four cells.  Taps beyond a row end
// come from global memory with the periodic rule (halo columns are never
// trusted).  One CTA barrier per chunk, after which thread 0 refills the
// previous chunk's slot; waits are bounded as in the z pass.
constexpr int kBXCells = 252;
constexpr int kBXCols = kBXCells + 4;    // 256 floats = 1 KB per variable
constexpr int kBXThreads = 64;           // 63 own four cells each; the last is idle
#ifndef MW_BX_STAGES
#define MW_BX_STAGES 2
#endif
constexpr int kBXStages = MW_BX_STAGES;  // ring slots (2: 16.4 KB of shared memory per CTA; 3 or 4
                                         // slots, fewer CTAs per SM, measured 3-6 % slower; at most 5,
                                         // within the 48 KB a launch gets without an attribute)
static_assert(kBXStages >= 2, "chunk b's copies are issued before chunk b - 1's slot is refilled");
static_assert(kBXStages <= 5, "the x kernel's shared memory must stay within the default 48 KB");
constexpr unsigned kBXBoxBytes = 4u * kBXCols * 4;  // one array's box: 4 variables x 256 floats
static_assert(kBXCells % 4 == 0 && kBXCells / 4 <= kBXThreads, "x chunk layout");

struct SmemXBulk {
  float4 f[kBXStages][4][kBXCols / 4];  // forcing
  float4 i[kBXStages][4][kBXCols / 4];  // init
  unsigned long long full[kBXStages];
};

__global__ void __launch_bounds__(kBXThreads) k_stage_x_f32_bulk(StageArgs<float> a, long long total, int cpr,
                                                                  const __grid_constant__ CUtensorMap tmf,
                                                                  const __grid_constant__ CUtensorMap tmi) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemXBulk& sm = *reinterpret_cast<SmemXBulk*>(smem_raw);
  const int t = threadIdx.x;
  const long long j0 = total * blockIdx.x / gridDim.x, j1 = total * (blockIdx.x + 1) / gridDim.x;
  const int n = (int)(j1 - j0);  // chunks of this CTA (uniform)
  if (n <= 0) return;
  if (t == 0) {
    for (int s = 0; s < kBXStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&sm.full[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // (row, chunk in row) of the next chunk to issue (thread 0) and of the chunk being computed,
  // advanced incrementally (no 64-bit division per chunk)
  int ik = (int)(j0 / cpr), ic = (int)(j0 % cpr);
  int k = ik, cc = ic;
  auto issue = [&](int b) {  // chunk j0 + b into slot b % kBXStages (thread 0, in order of b)
    const int x0 = ic * kBXCells, kk = ik;
    if (++ic == cpr) {
      ic = 0;
      ++ik;
    }
    const int s = b % kBXStages;
    const unsigned bar = smem_addr(&sm.full[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(2u * kBXBoxBytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(&sm.f[s][0][0])),
        "l"(reinterpret_cast<unsigned long long>(&tmf)), "r"(x0), "r"(kk + kHs), "r"(0), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(&sm.i[s][0][0])),
        "l"(reinterpret_cast<unsigned long long>(&tmi)), "r"(x0), "r"(kk + kHs), "r"(0), "r"(bar)
        : "memory");
  };
  int issued = 0, waited = 0;  // thread 0: chunks issued / chunks whose copies have landed
  if (t == 0)
    for (; issued < min(kBXStages, n); ++issued) issue(issued);
  const bool halo = a.flags & MW_FLAG_WRITE_HALO;
  const float c = a.c_f, dt = a.dt_f;
  int rk = -1;
  RowF rc;
  bool ok = true;
  for (int b = 0; b < n; ++b) {
    if (b > 0 && ++cc == cpr) {
      cc = 0;
      ++k;
    }
    const int x0 = cc * kBXCells;
    const int s = b % kBXStages;
    const long long row = (long long)(k + kHs) * a.pitch;
    if (k != rk) {
      rk = k;
      rc = rowf_x(MW_BC(a, hyc, k + kHs), MW_BC(a, hytc, k + kHs));
    }
    const bool w_ok = mbar_wait_bounded(&sm.full[s], (b / kBXStages) & 1);
    if (w_ok) waited = b + 1;
    ok = __syncthreads_and(w_ok);  // every thread is done with chunk b - 1
    if (!ok) break;
    if (t == 0 && b >= 1 && issued < n) issue(issued++);  // refill chunk b - 1's slot
    if (halo && x0 == 0 && t < 4) {  // this row's periodic halo of the forcing array (ics/bcs.py:35-39)
      const int dst = t < 2 ? t : a.nx + t;  // columns 0, 1, nx+2, nx+3
      const int src = t < 2 ? a.nx + t : t;  // columns nx, nx+1, 2, 3
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_SF(a, q * a.plane + row + dst) = MW_SF(a, q * a.plane + row + src);
    }
    const int c0 = x0 + 4 * t;  // first cell of this thread (nx and x0 are multiples of 4: all four or none)
    if (t < kBXCells / 4 && c0 < a.nx) {
      float tap[4][8];  // cells c0 - 2 .. c0 + 5
      if (c0 >= 2 && c0 + 5 < a.nx) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 lo = sm.f[s][q][t], hi = sm.f[s][q][t + 1];
          tap[q][0] = lo.x, tap[q][1] = lo.y, tap[q][2] = lo.z, tap[q][3] = lo.w;
          tap[q][4] = hi.x, tap[q][5] = hi.y, tap[q][6] = hi.z, tap[q][7] = hi.w;
        }
      } else {  // a tap beyond a row end: the periodic rule, from global memory
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const long long col = wrap_x(c0 - 2 + jj, a.nx) + kHs;
#pragma unroll
          for (int q = 0; q < 4; ++q) tap[q][jj] = __ldg(&MW_SF(a, q * a.plane + row + col));
        }
      }
      float F[5][4];  // fluxes at interfaces c0 .. c0 + 4
#pragma unroll
      for (int f = 0; f < 5; ++f) {
        float sv[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) sv[q][jj] = tap[q][f + jj];
        flux_x_f32(sv, rc, a.hv_f, F[f]);
      }
      float iv[4][4];  // init of cells c0 .. c0 + 3 (halo-indexed columns 4t + 2 .. 4t + 5 of the box)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 lo = sm.i[s][q][t], hi = sm.i[s][q][t + 1];
        iv[q][0] = lo.z, iv[q][1] = lo.w, iv[q][2] = hi.x, iv[q][3] = hi.y;
      }
      const long long o = row + c0 + kHs;  // 8-byte aligned: two floats per store
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        float inc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) inc[q] = (F[m][q] - F[m + 1][q]) * c;
        if (a.srcw) inc[WMOM] += dt * split::d2f(MW_SW(a, (long long)k * a.nx + c0 + m));
#pragma unroll
        for (int q = 0; q < 4; ++q) iv[q][m] = iv[q][m] + inc[q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float2* dst = reinterpret_cast<float2*>(&MW_SO(a, q * a.plane + o));
        float2* dst2 = reinterpret_cast<float2*>(&MW_SO(a, q * a.plane + o + 2));
        *dst = make_float2(iv[q][0], iv[q][1]);
        *dst2 = make_float2(iv[q][2], iv[q][3]);
      }
    }
  }
  if (!ok && t == 0) {  // a copy never completed: count it, and let none land after the CTA exits
    atomicAdd(&g_bulk_timeouts, 1ULL);
    for (int b = waited; b < issued; ++b) mbar_wait_bounded(&sm.full[b % kBXStages], (b / kBXStages) & 1);
  }
}

__device__ StageArgs<float> member_args_f32(const EnsStageT<float>& es, int e) {
  const mw_ens_member m = MW_AT(es.members, e, es.n_members);
  StageArgs<float> a;
  a.nx = m.nx;
  a.nz = m.nz;
  a.pitch = m.nx + 2 * kHs;
  a.plane = (long long)(m.nz + 2 * kHs) * a.pitch;
  a.dx = m.dx;
  a.dz = m.dz;
  a.hv = 0.0;        // the FP32 kernels read hv_f, c_f, dt_f (below)
  a.dt_stage = 0.0;
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
  a.chunks_per_block = 0;
  a.z_tile = es.z_tile;
  // hv_f, c_f, dt_f from the plan (formed on the host as set_f32_constants forms them)
  const EnsMemberConsts& c = MW_AT(reinterpret_cast<const EnsMemberConsts*>(es.mconsts), mconsts_index(es, e),
                                   (long long)kEnsConstsPerMember * es.n_members);
  a.hv_f = c.hv_f;
  a.c_f = c.c_f;
  a.dt_f = c.dt_f;
  return a;
}

// x items are rows (member, row), one per warp: lane l evaluates the flux at
// interface x0+l of a 31-cell segment from its four taps (L1-resident loads)
// and takes the flux of interface x0+l+1 from lane l+1 by a shuffle, so rows
// of 64..1024 cells keep most lanes busy.
constexpr int kF32WCells = 31;

__device__ __forceinline__ void x_row_warp_f32(const StageArgs<float>& a, int k, bool halo) {
  const int lane = threadIdx.x & 31;
  const RowF r = rowf_x(MW_BC(a, hyc, k + kHs), MW_BC(a, hytc, k + kHs));
  const long long row = (long long)(k + kHs) * a.pitch;
  if (halo && lane < 4) {  // columns 0, 1 <- nx, nx+1; nx+2, nx+3 <- 2, 3
    const int dst = lane < 2 ? lane : a.nx + lane, src = lane < 2 ? a.nx + lane : lane;
#pragma unroll
    for (int q = 0; q < 4; ++q) MW_SF(a, q * a.plane + row + dst) = MW_SF(a, q * a.plane + row + src);
  }
  for (int x0 = 0; x0 < a.nx; x0 += kF32WCells) {
    if (MW_F32_PF_X && x0 + MW_F32_PF_X * kF32WCells < a.nx && lane < 16) {  // a later segment's lines into L2
      const int q = lane & 3;
      const float* base = (lane & 4) ? a.init : a.forcing;
      const int col = min(x0 + MW_F32_PF_X * kF32WCells + (lane >> 3) * 32, a.nx + 2 * kHs - 1);
      prefetch_l2(base + q * a.plane + row + col);
    }
    const int i = x0 + lane;
    const bool upd = lane < kF32WCells && i < a.nx;
    const long long o = row + i + kHs;
    float iv[4];
    if (upd) {
#pragma unroll
      for (int q = 0; q < 4; ++q) iv[q] = MW_SI(a, q * a.plane + o);
    }
    float F[4] = {0.f, 0.f, 0.f, 0.f};
    if (i <= a.nx) {
      float s4[4][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const long long col = wrap_x(i - 2 + j, a.nx) + kHs;
#pragma unroll
        for (int q = 0; q < 4; ++q) s4[q][j] = __ldg(&MW_SF(a, q * a.plane + row + col));
      }
      flux_x_f32(s4, r, a.hv_f, F);
    }
    float Fn[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) Fn[q] = __shfl_down_sync(0xffffffffu, F[q], 1);
    if (upd) {
#pragma unroll
      for (int q = 0; q < 4; ++q) MW_SO(a, q * a.plane + o) = iv[q] + (F[q] - Fn[q]) * a.c_f;
    }
  }
}

__global__ void __launch_bounds__(kXThreads) k_ens_x_f32(EnsStageT<float> es) {
  for (unsigned it = ens_take_warp(es.cursor); it < (unsigned)es.n_items; it = ens_take_warp(es.cursor)) {
    const int2 item = MW_AT(es.items, it, es.n_items);  // (member, row)
    const StageArgs<float> a = member_args_f32(es, item.x);
    x_row_warp_f32(a, item.y, a.flags & MW_FLAG_WRITE_HALO);
  }
  ens_finish(es.cursor);
}

__global__ void __launch_bounds__(kEnsZCols) k_ens_z_f32(EnsStageT<float> es) {
  __shared__ SmemZT sm;
  __shared__ unsigned slot[2];
  int parity = 0;
  for (unsigned it = ens_take_cta(es.cursor, slot, parity); it < (unsigned)es.n_items;
       it = ens_take_cta(es.cursor, slot, parity)) {
    const int2 item = MW_AT(es.items, it, es.n_items);
    const StageArgs<float> a = member_args_f32(es, item.x);
    const int ncb = (a.nx + kEnsZCols - 1) / kEnsZCols;
    const int cb = item.y % ncb, tile = item.y / ncb;
    z_tile_t<float, MODE_F32, kEnsZCols>(a, cb, tile * es.z_tile, es.z_tile,
                                         (a.flags & MW_FLAG_WRITE_HALO) && tile == 0, sm);
  }
  ens_finish(es.cursor);
}

int launch_ens_f32(const EnsStageT<float>& es, int grid) {
  if (es.n_items == 0) return MW_OK;
  if (es.direction == MW_DIR_X)
    k_ens_x_f32<<<grid, kXThreads, 0, es.stream>>>(es);
  else
    k_ens_z_f32<<<grid, kEnsZCols, 0, es.stream>>>(es);
  return check_launch("ensemble FP32 stage launch");
}

int ens_f32_occupancy(int direction, int* blocks_per_sm) {
  cudaError_t e = direction == MW_DIR_X
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_ens_x_f32, kXThreads, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_ens_z_f32, kEnsZCols, 0);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  return MW_OK;
}

// ---------------------------------------------------------------------------
// host side
#ifndef MW_F32_BULK
#define MW_F32_BULK 1  // FP32 passes: tiles staged by tensor copies where the layout allows (0: plain loads)
#endif

// cuTensorMapEncodeTiled, from the driver through the runtime (no link-time
// dependency on the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::atomic<void*> fn{nullptr};
  void* f = fn.load(std::memory_order_relaxed);
  if (f) return (PFN_cuTensorMapEncodeTiled_v12000)f;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  fn.store(f, std::memory_order_relaxed);
  return (PFN_cuTensorMapEncodeTiled_v12000)f;
}

// The (4, nz+4, nx+4) FP32 array as a 3-D tensor (columns, rows, variables)
// read in boxes of 132 columns x kBulkRows rows x 4 variables.
static int bulk_tensor_map(const float* p, int nx, int nz, int box_cols, int box_rows, CUtensorMap* tm) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return fail(MW_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t pitch = (cuuint64_t)nx + 2 * kHs, rows = (cuuint64_t)nz + 2 * kHs;
  const cuuint64_t dims[3] = {pitch, rows, 4};
  const cuuint64_t strides[2] = {pitch * sizeof(float), pitch * rows * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 4};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)p, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MW_ERR_CUDA, "tensor map encoding failed (%d)", (int)r);
  return MW_OK;
}

// The bulk kernel's shared memory exceeds the 48 KB default: raise its limit
// once per device.
static int bulk_z_setup() {
  static std::atomic<int> done[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(MW_ERR_CUDA, "cudaGetDevice failed");
  if (dev >= 0 && dev < 64 && done[dev].load(std::memory_order_relaxed)) return MW_OK;
  const cudaError_t e = cudaFuncSetAttribute(k_stage_z_f32_bulk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(SmemZBulk));
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "bulk z kernel shared memory: %s", cudaGetErrorString(e));
  if (dev >= 0 && dev < 64) done[dev].store(1, std::memory_order_relaxed);
  return MW_OK;
}

// Resident CTAs of the FP32 x bulk kernel on the current device, cached per device.
static int bulk_x_resident(int* out) {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(MW_ERR_CUDA, "cudaGetDevice failed");
  const bool cached = dev >= 0 && dev < 64;
  if (cached && (*out = cache[dev].load(std::memory_order_relaxed)) > 0) return MW_OK;
  int per_sm = 0, sms = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_x_f32_bulk, kBXThreads,
                                                                sizeof(SmemXBulk));
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  *out = std::max(1, per_sm) * sms;
  if (cached) cache[dev].store(*out, std::memory_order_relaxed);
  return MW_OK;
}

int bulk_wait_timeouts(unsigned long long* out, bool reset) {
  unsigned long long v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_bulk_timeouts, sizeof(v));
  if (e == cudaSuccess && reset) {
    const unsigned long long z = 0;
    e = cudaMemcpyToSymbol(g_bulk_timeouts, &z, sizeof(z));
  }
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "wait-timeout counter: %s", cudaGetErrorString(e));
  *out = v;
  return MW_OK;
}

template <typename T>
static int validate_stage(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                          const double* hyi, const double* hyti, const double* hypi, const T* init, const T* forcing,
                          const T* out, int direction) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(finite_pos(dx) && finite_pos(dz) && finite_pos(dt_full), MW_ERR_INVALID_ARG,
             "dx, dz and dt_full must be finite and positive (got %g, %g, %g)", dx, dz, dt_full);
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 (x) or 1 (z)");
  MW_REQUIRE(hyc && hytc && hyi && hyti && hypi, MW_ERR_INVALID_ARG, "background arrays must not be NULL");
  MW_REQUIRE(init && forcing && out, MW_ERR_INVALID_ARG, "state arrays must not be NULL");
  MW_REQUIRE(aligned(hyc) && aligned(hytc) && aligned(hyi) && aligned(hyti) && aligned(hypi), MW_ERR_ALIGN,
             "background arrays must be 8-byte aligned");
  MW_REQUIRE(aligned(init) && aligned(forcing) && aligned(out), MW_ERR_ALIGN, "state arrays misaligned");
  const size_t bytes = sizeof(T) * 4 * (size_t)make_geom(nx, nz).plane;
  MW_REQUIRE(!ranges_overlap(out, bytes, forcing, bytes), MW_ERR_ALIAS,
             "out must not overlap forcing (the fused kernel reads forcing neighbours while writing out)");
  MW_REQUIRE(out == init || !ranges_overlap(out, bytes, init, bytes), MW_ERR_ALIAS,
             "out must either equal init or not overlap it");
  return MW_OK;
}

template <typename T, int MODE>
static int launch_stage(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                        const double* hyi, const double* hyti, const double* hypi, const double* srcw, const T* init,
                        T* forcing, T* out, double dt_stage, int direction, unsigned flags, cudaStream_t stream) {
  const Geom g = make_geom(nx, nz);
  StageArgs<T> a;
  a.nx = nx;
  a.nz = nz;
  a.pitch = g.pitch;
  a.plane = g.plane;
  a.dx = dx;
  a.dz = dz;
  a.hv = -kHvBeta * (direction == MW_DIR_X ? dx : dz) / (16 * dt_full);
  a.dt_stage = dt_stage;
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
  const int nchunks = (nx + kXCells - 1) / kXCells;
  a.chunks_per_block = (nchunks + kXBlocksPerRow - 1) / kXBlocksPerRow;
  a.z_tile = z_tile_rows(nx, nz, kZThreads, kZTile);
  set_f32_constants(a, direction);
  // FP32: tiles staged by tensor copies, which start at 16-byte boundaries of
  // 4-float-aligned rows (the x pass also stores pairs of floats)
  const bool bulk = MODE == MODE_F32 && MW_F32_BULK && nx % 4 == 0 && nx >= kZThreads &&
                    ((uintptr_t)init % 16) == 0 && ((uintptr_t)forcing % 16) == 0 && ((uintptr_t)out % 16) == 0;
  if (direction == MW_DIR_X) {
    if constexpr (MODE == MODE_F32) {
      if (bulk) {
        // one wave of CTAs, each an equal range of the row-major chunk list
        CUtensorMap tmf, tmi;
        int resident = 0, st = bulk_x_resident(&resident);
        if (!st) st = bulk_tensor_map((const float*)forcing, nx, nz, kBXCols, 1, &tmf);
        if (!st) st = bulk_tensor_map((const float*)init, nx, nz, kBXCols, 1, &tmi);
        if (st) return st;
        const int cpr = (nx + kBXCells - 1) / kBXCells;
        const long long total = (long long)cpr * nz;
        const long long grid = std::min<long long>(total, resident);
        k_stage_x_f32_bulk<<<(unsigned)grid, kBXThreads, sizeof(SmemXBulk), stream>>>(a, total, cpr, tmf, tmi);
        return check_launch("x direction-stage launch");
      }
    }
    dim3 grid((nchunks + a.chunks_per_block - 1) / a.chunks_per_block, (unsigned)min(nz, 65535));
    k_stage_x<T, MODE><<<grid, kXThreads, 0, stream>>>(a);
  } else {
    const int ntiles = (nz + a.z_tile - 1) / a.z_tile;
    CUtensorMap tmf, tmi;
    if constexpr (MODE == MODE_F32) {
      if (bulk) {
        int st = bulk_z_setup();
        if (!st) st = bulk_tensor_map((const float*)forcing, nx, nz, kBulkCols, kBulkRows, &tmf);
        if (!st) st = bulk_tensor_map((const float*)init, nx, nz, kBulkCols, kBulkRows, &tmi);
        if (st) return st;
      }
    }
    for (int t0 = 0; t0 < ntiles; t0 += 65535) {
      dim3 grid((nx + kZThreads - 1) / kZThreads, (unsigned)min(ntiles - t0, 65535));
      if constexpr (MODE == MODE_F32) {
        if (bulk)
          k_stage_z_f32_bulk<<<grid, kZThreads, sizeof(SmemZBulk), stream>>>(a, t0, tmf, tmi);
        else
          k_stage_z<T, MODE><<<grid, kZThreads, 0, stream>>>(a, t0);
      } else {
        k_stage_z<T, MODE><<<grid, kZThreads, 0, stream>>>(a, t0);
      }
      if (t0 + 65535 < ntiles) {
        const int st = check_launch("z direction-stage launch");
        if (st) return st;
      }
    }
  }
  return check_launch(direction == MW_DIR_X ? "x direction-stage launch" : "z direction-stage launch");
}

// MW_FLAG_CHECK_FINITE: count non-finite interior values, blocking (mw_aux.cu);
// counter8 is 8 bytes of the step's scratch array (nothing is allocated).
template <typename T>
int check_finite_blocking(int nx, int nz, const T* state, void* counter8, cudaStream_t stream);

// Split-arithmetic launches live in mw_split_stage.cu.
int launch_stage_split(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                       const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                       const double* init, double* forcing, double* out, double dt_stage, int direction,
                       unsigned flags, int r0, int r1, int fmt, cudaStream_t stream);

// IEEE-FP64 launches live in mw_fp64_stage.cu.
int launch_stage_ieee(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                      const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                      const double* init, double* forcing, double* out, double dt_stage, int direction,
                      unsigned flags, int r0, int r1, cudaStream_t stream);

// Storage format of the split form's RK3 stage k (0, 1, 2) inside a whole
// step: the first stage's result s1 is read only by the second stage of the
// same direction, so it stays in the scratch array as double-FP32 pairs
// (format 1 writes them, format 2 reads them); everything else is FP64.
inline int split_step_fmt(int k) { return k == 0 ? 1 : (k == 1 ? 2 : 0); }

static int stage_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                     const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                     const double* init, double* forcing, double* out, double dt_stage, int direction, int mode,
                     unsigned flags, cudaStream_t stream, int fmt = 0) {
  if (mode == MW_F64_SPLIT)
    return launch_stage_split(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, srcw, init, forcing, out,
                              dt_stage, direction, flags, 0, nz, fmt, stream);
  if (mode == MW_F64_IEEE)
    return launch_stage_ieee(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, srcw, init, forcing, out, dt_stage,
                             direction, flags, 0, nz, stream);
  return launch_stage<double, MODE_NATIVE64>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, srcw, init, forcing,
                                             out, dt_stage, direction, flags, stream);
}

template <typename T, typename StageFn>
static int run_steps(double dt, T* S, T* Tmp, T* A, int nsteps, int* reverse, StageFn stage) {
  for (int n = 0; n < nsteps; ++n) {
    const int dirs[2] = {*reverse ? MW_DIR_X : MW_DIR_Z, *reverse ? MW_DIR_Z : MW_DIR_X};
    for (int d = 0; d < 2; ++d) {
      int st;
      if ((st = stage(S, S, A, dt / 3, dirs[d], 0))) return st;
      if ((st = stage(S, A, Tmp, dt / 2, dirs[d], 1))) return st;
      if ((st = stage(S, Tmp, S, dt / 1, dirs[d], 2))) return st;
    }
    *reverse = *reverse ? 0 : 1;
  }
  return MW_OK;
}

template <typename T>
static int validate_step(int nx, int nz, double dx, double dz, double dt, const double* hyc, const double* hytc,
                         const double* hyi, const double* hyti, const double* hypi, const T* S, const T* Tmp,
                         const T* A, int nsteps, const int* reverse) {
  int st = validate_stage<T>(nx, nz, dx, dz, dt, hyc, hytc, hyi, hyti, hypi, S, A, Tmp, MW_DIR_X);
  if (st) return st;
  MW_REQUIRE(reverse != nullptr, MW_ERR_INVALID_ARG, "reverse flag pointer must not be NULL");
  MW_REQUIRE(nsteps >= 0, MW_ERR_INVALID_ARG, "nsteps must be >= 0");
  const size_t bytes = sizeof(T) * 4 * (size_t)make_geom(nx, nz).plane;
  MW_REQUIRE(!ranges_overlap(S, bytes, Tmp, bytes) && !ranges_overlap(S, bytes, A, bytes) &&
                 !ranges_overlap(Tmp, bytes, A, bytes),
             MW_ERR_ALIAS, "state, state_tmp and scratch must be three separate arrays");
  return MW_OK;
}

#if MW_CHECK
MW_OOB_COUNTER(oob_count_dirstage)
#endif

}  // namespace mw

using namespace mw;

extern "C" int mw_debug_wait_timeouts(unsigned long long* count, int reset) {
  MW_REQUIRE(count != nullptr, MW_ERR_INVALID_ARG, "count must not be NULL");
  return mw::bulk_wait_timeouts(count, reset != 0);
}

extern "C" int mw_dirstage_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hyc,
                               const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                               const double* src_w, const double* init, double* forcing, double* out,
                               double dt_stage, int direction, int f64_mode, unsigned flags, void* stream) {
  int st = validate_stage<double>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, init, forcing, out, direction);
  if (st) return st;
  MW_REQUIRE(valid_f64_mode(f64_mode), MW_ERR_INVALID_ARG, "unknown f64_mode %d",
             f64_mode);
  MW_REQUIRE(std::isfinite(dt_stage), MW_ERR_INVALID_ARG, "dt_stage must be finite");
  const unsigned pairs = flags & (MW_FLAG_PAIRS_OUT | MW_FLAG_PAIRS_IN);
  MW_REQUIRE(!pairs || (f64_mode == MW_F64_SPLIT && pairs != (MW_FLAG_PAIRS_OUT | MW_FLAG_PAIRS_IN)),
             MW_ERR_INVALID_ARG, "MW_FLAG_PAIRS_OUT / _IN: split form only, one of the two");
  MW_REQUIRE(!(flags & MW_FLAG_PAIRS_OUT) || init == forcing, MW_ERR_INVALID_ARG,
             "MW_FLAG_PAIRS_OUT needs init == forcing (the first RK stage)");
  const int fmt = (flags & MW_FLAG_PAIRS_OUT) ? 1 : ((flags & MW_FLAG_PAIRS_IN) ? 2 : 0);
  return stage_f64(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, init, forcing, out, dt_stage,
                   direction, f64_mode, flags & ~pairs, (cudaStream_t)stream, fmt);
}

extern "C" int mw_dirstage_f32(int nx, int nz, double dx, double dz, double dt_full, const double* hyc,
                               const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                               const double* src_w, const float* init, float* forcing, float* out, double dt_stage,
                               int direction, unsigned flags, void* stream) {
  int st = validate_stage<float>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, init, forcing, out, direction);
  if (st) return st;
  MW_REQUIRE(std::isfinite(dt_stage), MW_ERR_INVALID_ARG, "dt_stage must be finite");
  return launch_stage<float, MODE_F32>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, init, forcing, out,
                                       dt_stage, direction, flags, (cudaStream_t)stream);
}

extern "C" int mw_step_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                           const double* hytc,
                           const double* hyi, const double* hyti, const double* hypi, const double* src_w,
                           double* state, double* state_tmp, double* scratch, int nsteps, int* reverse, int f64_mode,
                           unsigned flags, void* stream) {
  int st = validate_step<double>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, state, state_tmp, scratch,
                                 nsteps, reverse);
  if (st) return st;
  MW_REQUIRE(finite_pos(dt), MW_ERR_INVALID_ARG, "dt must be finite and positive");
  if (st) return st;
  MW_REQUIRE(valid_f64_mode(f64_mode), MW_ERR_INVALID_ARG, "unknown f64_mode %d",
             f64_mode);
  cudaStream_t s = (cudaStream_t)stream;
  st = run_steps<double>(dt, state, state_tmp, scratch, nsteps, reverse,
                         [&](const double* init, double* forcing, double* out, double dts, int dir, int k) {
                           return stage_f64(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, init, forcing,
                                            out, dts, dir, f64_mode, flags, s, split_step_fmt(k));
                         });
  if (st == MW_OK && nsteps > 0 && (flags & MW_FLAG_CHECK_FINITE)) st = check_finite_blocking(nx, nz, (const double*)state, scratch, s);
  return st;
}

extern "C" int mw_step_f32(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                           const double* hytc,
                           const double* hyi, const double* hyti, const double* hypi, const double* src_w, float* state,
                           float* state_tmp, float* scratch, int nsteps, int* reverse, unsigned flags, void* stream) {
  int st = validate_step<float>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, state, state_tmp, scratch,
                                nsteps, reverse);
  if (st) return st;
  MW_REQUIRE(finite_pos(dt), MW_ERR_INVALID_ARG, "dt must be finite and positive");
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  st = run_steps<float>(dt, state, state_tmp, scratch, nsteps, reverse,
                        [&](const float* init, float* forcing, float* out, double dts, int dir, int) {
                          return launch_stage<float, MODE_F32>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi,
                                                               src_w, init, forcing, out, dts, dir, flags, s);
                        });
  if (st == MW_OK && nsteps > 0 && (flags & MW_FLAG_CHECK_FINITE)) st = check_finite_blocking(nx, nz, (const float*)state, scratch, s);
  return st;
}

// ---------------------------------------------------------------------------
// Time step that allocates nothing.
//
// Some callers cannot hand this library a third state-sized array: a host
// model that keeps its fields in buffers it allocated itself and passes only
// those (a Fortran or C weather code embedding this solver), a custom call in
// a framework that pre-allocates every buffer it gives out, or a real-time
// loop whose rules forbid allocation once it is running.  For them the array
// the fused step ping-pongs through (see mw_step_f64) is this fixed device
// array, sized for grids up to 512 x 256 cells; every GPU that loads the
// library keeps it (4.3 MB) until the process exits.
namespace mw {
namespace {

constexpr int kNoAllocMaxNx = 512, kNoAllocMaxNz = 256;
constexpr long long kNoAllocValues = 4LL * (kNoAllocMaxNx + 2 * kHs) * (kNoAllocMaxNz + 2 * kHs);
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocValues];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  The host-side
// name is only a stand-in for the symbol, so the address is asked of the
// runtime once per device, with that device current, and kept for the life of
// the process: a device must not be reset (cudaDeviceReset) while this entry
// point is in use, since the array is loaded again at a new address.
int noalloc_scratch(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(MW_ERR_INVALID_ARG, "device %d beyond the %d devices this entry point supports", dev,
                kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      return fail(MW_ERR_CUDA, "cudaGetSymbolAddress of the built-in scratch array: %s", cudaGetErrorString(e));
    g_noalloc_addr[dev] = (double*)p;
  }
  *out = g_noalloc_addr[dev];
  return MW_OK;
}

}  // namespace
}  // namespace mw

extern "C" int mw_step_f64_noalloc(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                                   const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                                   const double* src_w, double* state, double* state_tmp, int nsteps, int* reverse,
                                   int f64_mode, unsigned flags, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  const long long need = 4LL * (nx + 2 * kHs) * (nz + 2 * kHs);
  MW_REQUIRE(need <= kNoAllocValues, MW_ERR_WORKSPACE,
             "grid %d x %d needs %lld scratch values; the built-in array holds %lld (grids up to %d x %d cells, "
             "or any shape with (nx+4)(nz+4) <= %lld); use mw_step_f64 with a caller-provided scratch array",
             nx, nz, need, kNoAllocValues, kNoAllocMaxNx, kNoAllocMaxNz, kNoAllocValues / 4);
  double* scratch = nullptr;
  st = noalloc_scratch(&scratch);
  if (st) return st;
  st = validate_step<double>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, state, state_tmp, scratch, nsteps,
                             reverse);
  if (st) return st;
  MW_REQUIRE(finite_pos(dt), MW_ERR_INVALID_ARG, "dt must be finite and positive");
  MW_REQUIRE(valid_f64_mode(f64_mode), MW_ERR_INVALID_ARG, "unknown f64_mode %d",
             f64_mode);
  cudaStream_t s = (cudaStream_t)stream;
  st = run_steps<double>(dt, state, state_tmp, scratch, nsteps, reverse,
                         [&](const double* init, double* forcing, double* out, double dts, int dir, int k) {
                           return stage_f64(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, init,
                                            forcing, out, dts, dir, f64_mode, flags, s, split_step_fmt(k));
                         });
  // the finite check counts into the first 8 bytes of the built-in array (no allocation)
  if (st == MW_OK && nsteps > 0 && (flags & MW_FLAG_CHECK_FINITE)) st = check_finite_blocking(nx, nz, (const double*)state, scratch, s);
  return st;
}

// ---------------------------------------------------------------------------
// One time step that keeps its six stage forcing states (for the adjoint).
extern "C" int mw_step_record_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                                  const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                                  const double* src_w, const double* state_in, double* stages, double* state_out,
                                  int reverse, int f64_mode, void* stream) {
  MW_REQUIRE(state_in && stages && state_out, MW_ERR_INVALID_ARG, "NULL pointer argument");
  const size_t n = 4 * (size_t)make_geom(nx, nz).plane;
  int st = validate_stage<double>(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, stages, stages + n, state_out,
                                  MW_DIR_X);
  if (st) return st;
  MW_REQUIRE(finite_pos(dt), MW_ERR_INVALID_ARG, "dt must be finite and positive");
  MW_REQUIRE(valid_f64_mode(f64_mode), MW_ERR_INVALID_ARG, "unknown f64_mode %d",
             f64_mode);
  MW_REQUIRE(!ranges_overlap(stages, 6 * n * sizeof(double), state_out, n * sizeof(double)) &&
                 !ranges_overlap(stages, 6 * n * sizeof(double), state_in, n * sizeof(double)),
             MW_ERR_ALIAS, "stages must not overlap state_in or state_out");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(stages, state_in, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "stage copy: %s", cudaGetErrorString(e));
  const int dirs[2] = {reverse ? MW_DIR_X : MW_DIR_Z, reverse ? MW_DIR_Z : MW_DIR_X};
  for (int d = 0; d < 2; ++d) {
    double* S = stages + (3 * d) * n;
    double* s1 = S + n;
    double* s2 = S + 2 * n;
    double* out = d == 0 ? stages + 3 * n : state_out;
    if ((st = stage_f64(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, S, S, s1, dt / 3, dirs[d], f64_mode,
                        0, s)))
      return st;
    if ((st = stage_f64(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, S, s1, s2, dt / 2, dirs[d], f64_mode,
                        0, s)))
      return st;
    if ((st = stage_f64(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, S, s2, out, dt, dirs[d], f64_mode, 0,
                        s)))
      return st;
  }
  return MW_OK;
}
