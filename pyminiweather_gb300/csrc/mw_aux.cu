// mw_aux.cu -- initial condition, diagnostics and the unfused pieces of one
// direction-stage.  Everything here is FP64 (the precision form keeps the
// initial condition, backgrounds and reductions in FP64 too).
//
// The unfused kernels follow the reference's NumPy expressions operation by
// operation with explicitly rounded intrinsics (__dadd_rn, __dmul_rn, ...),
// so that no multiply-add is contracted and results round exactly as NumPy's
// do, pow and cos aside.
#include <algorithm>
#include <cmath>

#include "mw_common.cuh"
#include "mw_fp64_math.cuh"
#include "mw_split.cuh"

namespace mw {

namespace {

__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div_(double a, double b) { return __ddiv_rn(a, b); }

// numpy.linspace(start, stop, num, endpoint=False)[k]
__device__ __forceinline__ double linspace_at(double start, double stop, int num, int k) {
  const double step = div_(sub_(stop, start), (double)num);
  return add_(mul_((double)k, step), start);
}

// pyminiweather/data/quadrature.py:15-30
__constant__ double c_qp[3] = {0.112701665379258311482073460022, 0.500000000000000000000000000000,
                               0.887298334620741688517926539980};
__constant__ double c_qw[3] = {0.277777777777777777777777777779, 0.444444444444444444444444444444,
                               0.277777777777777777777777777779};

// hydro_const_theta / hydro_const_bvfreq, ics/initial_conditions.py:26-81
__device__ void hydro(int bg, double z, double* hr, double* ht) {
  if (bg == MW_BG_BVFREQ) {
    const double bv0 = 0.02;
    const double t = mul_(kTheta0, exp(mul_(div_(mul_(bv0, bv0), kGrav), z)));
    const double exner =
        sub_(kExner0, div_(mul_(div_(mul_(kGrav, kGrav), mul_(mul_(kCp, bv0), bv0)), sub_(t, kTheta0)),
                           mul_(t, kTheta0)));
    const double p = mul_(kP0, pow(exner, kCp / kRd));
    *ht = t;
    *hr = div_(pow(div_(p, kC0), 1.0 / kGamma), t);
  } else {
    const double exner = sub_(kExner0, div_(mul_(kGrav, z), mul_(kCp, kTheta0)));
    const double p = mul_(kP0, pow(exner, kCp / kRd));
    *ht = kTheta0;
    *hr = div_(pow(div_(p, kC0), 1.0 / kGamma), kTheta0);
  }
}

struct Bubbles {
  int n;
  double b[MW_MAX_BUBBLES][5];  // amplitude, x0, z0, xrad, zrad
};

// sample_ellipse_cosine, utils/utils.py:5-51
__device__ __forceinline__ double ellipse_cos2(double x, double z, const double* B) {
  const double a = div_(sub_(x, B[1]), B[3]);
  const double b = div_(sub_(z, B[2]), B[4]);
  const double dist = div_(mul_(sqrt(add_(mul_(a, a), mul_(b, b))), kPi), 2.0);
  if (dist <= kPi / 2.0) {
    const double c = cos(dist);
    return mul_(B[0], mul_(c, c));
  }
  return 0.0;
}

// init(), ics/initial.py:57-77: one CTA per halo-indexed row.
template <typename T>
__global__ void k_init_state(int nx, int nz, double dx, double dz, int bg, double u0, Bubbles bub, T* state) {
  __shared__ double s_hr[3], s_ht[3], s_z[3];
  const int NX = nx + 2 * kHs, NZ = nz + 2 * kHs;
  const long long plane = (long long)NX * NZ;
  const int k = blockIdx.x;
  const double zm = linspace_at(-kHs * dz, (nz + kHs) * dz, NZ, k);
  if (threadIdx.x < 3) {
    const double z = add_(zm, mul_(c_qp[threadIdx.x], dz));
    s_z[threadIdx.x] = z;
    hydro(bg, z, &s_hr[threadIdx.x], &s_ht[threadIdx.x]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NX; i += blockDim.x) {
    const double xm = linspace_at(-kHs * dx, (nx + kHs) * dx, NX, i);
    double acc[4][3];
#pragma unroll
    for (int qa = 0; qa < 3; ++qa) {
      const double z = s_z[qa], hr = s_hr[qa], ht = s_ht[qa];
#pragma unroll
      for (int qb = 0; qb < 3; ++qb) {
        const double x = add_(xm, mul_(c_qp[qb], dx));
        double t = 0.0;
        for (int n = 0; n < bub.n; ++n) t = add_(t, ellipse_cos2(x, z, bub.b[n]));
        const double W = mul_(c_qw[qa], c_qw[qb]);
        const double r = 0.0;
        const double v0 = mul_(r, W);
        const double v1 = mul_(mul_(add_(r, hr), u0), W);
        const double v2 = mul_(mul_(add_(r, hr), 0.0), W);
        const double v3 = mul_(sub_(mul_(add_(r, hr), add_(t, ht)), mul_(hr, ht)), W);
        if (qb == 0) {
          acc[0][qa] = v0; acc[1][qa] = v1; acc[2][qa] = v2; acc[3][qa] = v3;
        } else {
          acc[0][qa] = add_(acc[0][qa], v0); acc[1][qa] = add_(acc[1][qa], v1);
          acc[2][qa] = add_(acc[2][qa], v2); acc[3][qa] = add_(acc[3][qa], v3);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      MW_AT(state, q * plane + (long long)k * NX + i, 4 * plane) = (T)add_(add_(acc[q][0], acc[q][1]), acc[q][2]);
  }
}

// Backgrounds, ics/initial.py:84-105.
__global__ void k_init_background(int nz, double dz, int bg, double* hyc, double* hytc, double* hyi, double* hyti,
                                  double* hypi) {
  const int NZ = nz + 2 * kHs;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < NZ; k += gridDim.x * blockDim.x) {
    const double z = linspace_at((-kHs + 0.5) * dz, (nz + kHs + 0.5) * dz, NZ, k);
    double hr, ht;
    hydro(bg, z, &hr, &ht);
    const double sumw = add_(add_(c_qw[0], c_qw[1]), c_qw[2]);
    MW_AT(hyc, k, NZ) = mul_(hr, sumw);
    const double a = mul_(ht, hr);
    MW_AT(hytc, k, NZ) = add_(add_(mul_(a, c_qw[0]), mul_(a, c_qw[1])), mul_(a, c_qw[2]));
    if (k <= nz) {
      const double ze = linspace_at(0.0, (nz + 1) * dz, nz + 1, k);
      hydro(bg, ze, &hr, &ht);
      MW_AT(hyi, k, nz + 1) = hr;
      MW_AT(hyti, k, nz + 1) = mul_(hr, ht);
      MW_AT(hypi, k, nz + 1) = mul_(kC0, pow(mul_(hr, ht), kGamma));
    }
  }
}

// GravityBCSourceTerm, solve/source.py:20-50
__global__ void k_gravity_source(int nx, int nz, double xlen, double zlen, const double* hyc, double* src) {
  const double dx = xlen / nx, dz = zlen / nz;
  double B[5] = {0.01, xlen / 8, 1000.0, 500.0, 500.0};
  const long long n = (long long)nx * nz;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nx), i = (int)(idx % nx);
    const double z = linspace_at(dz / 2.0, zlen + dz / 2.0, nz, k);
    const double x = linspace_at(dx / 2.0, xlen + dx / 2.0, nx, i);
    MW_AT(src, idx, n) = mul_(ellipse_cos2(x, z, B), MW_AT(hyc, k + kHs, nz + 2 * kHs));
  }
}

// ---------------------------------------------------------------------------
// compute_stats, post/stats.py:8-35.  Level 1: block b reduces rows
// [b*rpb, (b+1)*rpb) into workspace[2b .. 2b+1]; level 2 reduces the block
// partials.  Both levels use fixed trees, so the result does not depend on
// scheduling.
constexpr int kStatThreads = 256;
constexpr int kStatMaxBlocks = 1024;

// Sum of a and b over the NT threads of the block, in a fixed order (so the
// result is bit-reproducible): a shuffle tree inside each warp, then the warp
// sums by the same tree in warp 0.  Thread 0 ends with the sums; wa / wb hold
// NT / 32 doubles of shared memory.
template <int NT>
__device__ __forceinline__ void block_sum2(double& a, double& b, double* wa, double* wb) {
  static_assert(NT % 32 == 0 && NT / 32 <= 32, "block size");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = add_(a, __shfl_down_sync(0xffffffffu, a, o));
    b = add_(b, __shfl_down_sync(0xffffffffu, b, o));
  }
  if (lane == 0) {
    wa[w] = a;
    wb[w] = b;
  }
  __syncthreads();
  if (w == 0) {
    a = lane < NT / 32 ? wa[lane] : 0.0;
    b = lane < NT / 32 ? wb[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = add_(a, __shfl_down_sync(0xffffffffu, a, o));
      b = add_(b, __shfl_down_sync(0xffffffffu, b, o));
    }
  }
}

__device__ __forceinline__ double load_state(const double* p) { return *p; }
__device__ __forceinline__ double load_state(const float* p) { return split::f2d(*p); }

// Per cell the reference forms p = C0 (rho th)^gamma and t = th / (p0 / p)^(Rd/Cp),
// two powers; since gamma Rd / Cp = Rd / Cv = gamma - 1, the internal energy
// rho Cv t is Cv K (rho theta)^gamma with K = (C0 / p0)^(Rd/Cp), and with
// rho theta = (rho theta)_bg (1 + d) it is Pr (1 + ((1 + d)^gamma - 1)),
// Pr = Cv K (rho theta)_bg^gamma formed once per row (ck = Cv K from the
// host), the bracket by the binomial series of the stage kernels (degree per
// warp, expm1 / log1p for |d| >= 1/8).  ke = ((rho u)^2 + (rho w)^2) / rho
// with one reciprocal.  The same quantities as the reference's up to a few
// roundings per cell (the sums agree to ~1e-16 relative).
__constant__ ieee::Series c_stats_pow_g = ieee::make_series(kGamma);

template <typename T>
__global__ void __launch_bounds__(kStatThreads) k_stats_partial(int nx, int nz, int rpb, double ck, const double* hyc,
                                                                const double* hytc, const T* state, double* part) {
  __shared__ double sm[kStatThreads / 32], se[kStatThreads / 32];
  const int NX = nx + 2 * kHs;
  const long long plane = (long long)NX * (nz + 2 * kHs);
  const int lane = threadIdx.x & 31;
  double m = 0.0, e = 0.0;
  const int k0 = blockIdx.x * rpb, k1 = min(k0 + rpb, nz);
  for (int k = k0; k < k1; ++k) {
    const int kk = k + kHs;
    const double hr = MW_AT(hyc, kk, nz + 2 * kHs), hrt = MW_AT(hytc, kk, nz + 2 * kHs);
    double pr = 0.0;
    if (lane == 0) pr = ck * pow(hrt, kGamma);  // one power per warp and row
    pr = __shfl_sync(0xffffffffu, pr, 0);
    const double irt = 1.0 / hrt;
    for (int base = 0; base < nx; base += kStatThreads) {
      const int i = base + threadIdx.x;
      const bool act = i < nx;
      const unsigned mask = __ballot_sync(0xffffffffu, act);  // the lanes of this row step
      if (act) {
        const long long o = (long long)kk * NX + i + kHs;
        const double rho = load_state(&MW_AT(state, o, 4 * plane)) + hr;
        const double ri = ieee::rcp(rho, mask);
        const double ru = load_state(&MW_AT(state, plane + o, 4 * plane));
        const double rw = load_state(&MW_AT(state, 2 * plane + o, 4 * plane));
        const double ke = fma(ru, ru, rw * rw) * ri;
        const double d = load_state(&MW_AT(state, 3 * plane + o, 4 * plane)) * irt;
        bool big;
        const int n = ieee::series_degree(d, mask, c_stats_pow_g, big);
        double f = d * ieee::series_g(d, n, c_stats_pow_g);  // (1 + d)^gamma - 1
        if (__any_sync(mask, big)) {
          if (big) f = expm1(kGamma * log1p(d));
        }
        m += rho;
        e += ke + fma(pr, f, pr);
      }
    }
  }
  block_sum2<kStatThreads>(m, e, sm, se);
  if (threadIdx.x == 0) {
    MW_AT(part, 2 * blockIdx.x, 2 * gridDim.x) = m;
    MW_AT(part, 2 * blockIdx.x + 1, 2 * gridDim.x) = e;
  }
}

__global__ void __launch_bounds__(kStatMaxBlocks) k_stats_final(int nblocks, double dx, double dz, const double* part,
                                                                double* out2) {
  __shared__ double sm[kStatMaxBlocks / 32], se[kStatMaxBlocks / 32];
  const int t = threadIdx.x;
  double m = t < nblocks ? MW_AT(part, 2 * t, 2 * nblocks) : 0.0;
  double e = t < nblocks ? MW_AT(part, 2 * t + 1, 2 * nblocks) : 0.0;
  block_sum2<kStatMaxBlocks>(m, e, sm, se);
  if (t == 0) {
    MW_AT(out2, 0, 2) = mul_(mul_(m, dx), dz);
    MW_AT(out2, 1, 2) = mul_(mul_(e, dx), dz);
  }
}

int stats_blocks(int nz, int* rpb) {
  const int nb = nz < kStatMaxBlocks ? nz : kStatMaxBlocks;
  *rpb = (nz + nb - 1) / nb;
  return (nz + *rpb - 1) / *rpb;
}

template <typename T>
int run_stats(int nx, int nz, double dx, double dz, const double* hyc, const double* hytc, const T* state,
              void* workspace, size_t workspace_bytes, double* out2, cudaStream_t stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(hyc && hytc && state && workspace && out2, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(finite_pos(dx) && finite_pos(dz), MW_ERR_INVALID_ARG, "dx, dz must be finite and positive");
  MW_REQUIRE(aligned(state) && aligned(hyc) && aligned(hytc) && aligned(out2) && ((uintptr_t)workspace % 8) == 0,
             MW_ERR_ALIGN, "misaligned pointer");
  const size_t need = mw_stats_workspace_bytes(nx, nz);
  MW_REQUIRE(workspace_bytes >= need, MW_ERR_WORKSPACE, "stats workspace needs %zu bytes, got %zu", need,
             workspace_bytes);
  int rpb;
  const int nb = stats_blocks(nz, &rpb);
  const double ck = kCv * std::pow(kC0 / kP0, kRd / kCp);  // Cv (C0 / p0)^(Rd/Cp)
  k_stats_partial<T><<<nb, kStatThreads, 0, stream>>>(nx, nz, rpb, ck, hyc, hytc, state, (double*)workspace);
  st = check_launch("stats partial launch");
  if (st) return st;
  k_stats_final<<<1, kStatMaxBlocks, 0, stream>>>(nb, dx, dz, (const double*)workspace, out2);
  return check_launch("stats final launch");
}

// compute_solution_variables, post/stats.py:38-69
__global__ void k_solution_vars(int nx, int nz, const double* hyc, const double* hytc, const double* state,
                                double* out) {
  const int NX = nx + 2 * kHs;
  const long long plane = (long long)NX * (nz + 2 * kHs);
  const long long n = (long long)nx * nz;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nx), i = (int)(idx % nx);
    const long long o = (long long)(k + kHs) * NX + i + kHs;
    const double hr = MW_AT(hyc, k + kHs, nz + 2 * kHs), hrt = MW_AT(hytc, k + kHs, nz + 2 * kHs);
    const double d = MW_AT(state, o, 4 * plane);
    MW_AT(out, idx, 4 * n) = d;
    MW_AT(out, n + idx, 4 * n) = div_(MW_AT(state, plane + o, 4 * plane), add_(hr, d));
    MW_AT(out, 2 * n + idx, 4 * n) = div_(MW_AT(state, 2 * plane + o, 4 * plane), add_(hr, d));
    MW_AT(out, 3 * n + idx, 4 * n) = sub_(div_(add_(MW_AT(state, 3 * plane + o, 4 * plane), hrt), add_(hr, d)),
                                          div_(hrt, hr));
  }
}

// ---------------------------------------------------------------------------
// Unfused pieces.
__global__ void k_set_bc(int nx, int nz, const double* hyc, double* f, int dir) {
  const int NX = nx + 2 * kHs;
  const long long plane = (long long)NX * (nz + 2 * kHs);
  if (dir == MW_DIR_X) {  // ics/bcs.py:35-39, interior rows
    const long long n = 4LL * nz;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
      const int q = (int)(idx / nz), k = (int)(idx % nz);
      const long long row = q * plane + (long long)(k + kHs) * NX;
      auto at = [&](int c) -> double& { return MW_AT(f, row + c, 4 * plane); };
      at(0) = at(nx);
      at(1) = at(nx + 1);
      at(nx + kHs) = at(kHs);
      at(nx + kHs + 1) = at(kHs + 1);
    }
  } else {  // ics/bcs.py:92-148, all nx+4 columns
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < NX; c += gridDim.x * blockDim.x) {
      auto at = [&](int q, int r) -> double& { return MW_AT(f, q * plane + (long long)r * NX + c, 4 * plane); };
      auto hc = [&](int r) { return MW_AT(hyc, r, nz + 2 * kHs); };
      at(WMOM, 0) = 0.0;
      at(WMOM, 1) = 0.0;
      at(WMOM, nz + kHs) = 0.0;
      at(WMOM, nz + kHs + 1) = 0.0;
      at(UMOM, 0) = mul_(div_(at(UMOM, kHs), hc(kHs)), hc(0));
      at(UMOM, 1) = mul_(div_(at(UMOM, kHs), hc(kHs)), hc(1));
      at(UMOM, nz + kHs) = mul_(div_(at(UMOM, nz + kHs - 1), hc(nz + kHs - 1)), hc(nz + kHs));
      at(UMOM, nz + kHs + 1) = mul_(div_(at(UMOM, nz + kHs - 1), hc(nz + kHs - 1)), hc(nz + kHs + 1));
      for (int q = 0; q < 4; q += 3) {  // DENS and RHOT
        at(q, 0) = at(q, kHs);
        at(q, 1) = at(q, kHs);
        at(q, nz + kHs) = at(q, nz + kHs - 1);
        at(q, nz + kHs + 1) = at(q, nz + kHs - 1);
      }
    }
  }
}

// scipy.signal.convolve(mode="same")[..., 2:-1] accumulation order
__device__ __forceinline__ double interp4_rn(double s0, double s1, double s2, double s3) {
  const double k0 = -1.0 / 12, k1 = 7.0 / 12;
  return add_(add_(add_(mul_(s0, k0), mul_(s1, k1)), mul_(s2, k1)), mul_(s3, k0));
}
__device__ __forceinline__ double diff3_rn(double s0, double s1, double s2, double s3) {
  return add_(add_(add_(mul_(s0, -1.0), mul_(s1, 3.0)), mul_(s2, -3.0)), mul_(s3, 1.0));
}

__global__ void k_interpolate(int nx, int nz, const double* s, double* vals, double* d3, int dir) {
  const int NX = nx + 2 * kHs;
  const long long plane = (long long)NX * (nz + 2 * kHs);
  const int ni = dir == MW_DIR_X ? nx + 1 : nx;  // columns of the output
  const int nk = dir == MW_DIR_X ? nz : nz + 1;  // rows of the output
  const long long n = 4LL * nk * ni;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(idx / ((long long)nk * ni));
    const int r = (int)((idx / ni) % nk), i = (int)(idx % ni);
    double t[4];
    const long long base = dir == MW_DIR_X ? q * plane + (long long)(r + kHs) * NX + i
                                           : q * plane + (long long)r * NX + i + kHs;
    const long long step = dir == MW_DIR_X ? 1 : NX;
#pragma unroll
    for (int j = 0; j < 4; ++j) t[j] = MW_AT(s, base + j * step, 4 * plane);
    MW_AT(vals, idx, n) = interp4_rn(t[0], t[1], t[2], t[3]);
    MW_AT(d3, idx, n) = diff3_rn(t[0], t[1], t[2], t[3]);
  }
}

struct FluxArgs {
  int nx, nz;
  double hv;
  const double *hyc, *hytc, *hyi, *hyti, *hypi;
  const double* vals;
  double* d3;
  double* flux;
  int dir;
};

__global__ void k_flux(FluxArgs a) {
  const int ni = a.dir == MW_DIR_X ? a.nx + 1 : a.nx;
  const int nk = a.dir == MW_DIR_X ? a.nz : a.nz + 1;
  const long long vplane = (long long)nk * ni;               // vals/d3 plane
  const long long fplane = (long long)(a.nz + 1) * (a.nx + 1);  // flux plane
  const long long n = vplane;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / ni), i = (int)(idx % ni);
    double v[4], d[4];
    for (int q = 0; q < 4; ++q) {
      v[q] = MW_AT(a.vals, q * vplane + idx, 4 * vplane);
      d[q] = MW_AT(a.d3, q * vplane + idx, 4 * vplane);
    }
    const long long fo = (long long)r * (a.nx + 1) + i;
    auto F = [&](int q) -> double& { return MW_AT(a.flux, q * fplane + fo, 4 * fplane); };
    if (a.dir == MW_DIR_X) {  // interpolate.py:105-129
      const double rho = add_(v[DENS], MW_AT(a.hyc, r + kHs, a.nz + 2 * kHs));
      const double u = div_(v[UMOM], rho);
      const double w = div_(v[WMOM], rho);
      const double t = div_(add_(v[RHOT], MW_AT(a.hytc, r + kHs, a.nz + 2 * kHs)), rho);
      const double p = mul_(kC0, pow(mul_(rho, t), kGamma));
      F(0) = sub_(mul_(rho, u), mul_(a.hv, d[DENS]));
      F(1) = sub_(add_(mul_(rho, mul_(u, u)), p), mul_(a.hv, d[UMOM]));
      F(2) = sub_(mul_(mul_(rho, u), w), mul_(a.hv, d[WMOM]));
      F(3) = sub_(mul_(mul_(rho, u), t), mul_(a.hv, d[RHOT]));
    } else {  // interpolate.py:153-186
      const double rho = add_(v[DENS], MW_AT(a.hyi, r, a.nz + 1));
      const double u = div_(v[UMOM], rho);
      double w = div_(v[WMOM], rho);
      const double t = div_(add_(v[RHOT], MW_AT(a.hyti, r, a.nz + 1)), rho);
      const double p = sub_(mul_(kC0, pow(mul_(rho, t), kGamma)), MW_AT(a.hypi, r, a.nz + 1));
      if (r == 0 || r == a.nz) {
        w = 0.0;
        d[DENS] = 0.0;
        MW_AT(a.d3, DENS * vplane + idx, 4 * vplane) = 0.0;
      }
      F(0) = sub_(mul_(rho, w), mul_(a.hv, d[DENS]));
      F(1) = sub_(mul_(mul_(rho, w), u), mul_(a.hv, d[UMOM]));
      F(2) = sub_(add_(mul_(rho, mul_(w, w)), p), mul_(a.hv, d[WMOM]));
      F(3) = sub_(mul_(mul_(rho, w), t), mul_(a.hv, d[RHOT]));
    }
  }
}

__global__ void k_tend(int nx, int nz, double d, const double* flux, const double* forcing, const double* srcw,
                       double* tend, int dir) {
  const int NX = nx + 2 * kHs;
  const long long splane = (long long)NX * (nz + 2 * kHs);
  const long long fplane = (long long)(nz + 1) * (nx + 1);
  const long long tplane = (long long)nz * nx;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < tplane;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nx), i = (int)(idx % nx);
    const long long f0 = (long long)k * (nx + 1) + i;
    const long long f1 = dir == MW_DIR_X ? f0 + 1 : f0 + (nx + 1);
    for (int q = 0; q < 4; ++q) {
      double t = div_(-sub_(MW_AT(flux, q * fplane + f1, 4 * fplane), MW_AT(flux, q * fplane + f0, 4 * fplane)), d);
      if (q == WMOM && dir == MW_DIR_Z)
        t = sub_(t, mul_(MW_AT(forcing, DENS * splane + (long long)(k + kHs) * NX + i + kHs, 4 * splane), kGrav));
      if (q == WMOM && srcw) t = add_(t, MW_AT(srcw, idx, tplane));
      MW_AT(tend, q * tplane + idx, 4 * tplane) = t;
    }
  }
}

__global__ void k_update(int nx, int nz, const double* init, const double* tend, double* out, double dt) {
  const int NX = nx + 2 * kHs;
  const long long splane = (long long)NX * (nz + 2 * kHs);
  const long long tplane = (long long)nz * nx;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < 4 * tplane;
       idx += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(idx / tplane);
    const long long r = idx % tplane;
    const int k = (int)(r / nx), i = (int)(r % nx);
    const long long o = q * splane + (long long)(k + kHs) * NX + i + kHs;
    MW_AT(out, o, 4 * splane) = add_(MW_AT(init, o, 4 * splane), mul_(dt, MW_AT(tend, idx, 4 * tplane)));
  }
}

__global__ void k_add_source(int nx, int nz, const double* srcw, double* tend) {
  const long long tplane = (long long)nz * nx;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < tplane;
       idx += (long long)gridDim.x * blockDim.x)
    MW_AT(tend, WMOM * tplane + idx, 4 * tplane) =
        add_(MW_AT(tend, WMOM * tplane + idx, 4 * tplane), MW_AT(srcw, idx, tplane));
}

inline unsigned grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 65535LL * 16) b = 65535LL * 16;
  return (unsigned)b;
}

int check_bubbles(int nbubble, const double* bubbles, Bubbles* out) {
  MW_REQUIRE(nbubble >= 0 && nbubble <= MW_MAX_BUBBLES, MW_ERR_INVALID_ARG, "nbubble must be in [0, %d]",
             MW_MAX_BUBBLES);
  MW_REQUIRE(nbubble == 0 || bubbles, MW_ERR_INVALID_ARG, "bubbles must not be NULL when nbubble > 0");
  out->n = nbubble;
  for (int n = 0; n < MW_MAX_BUBBLES; ++n)
    for (int j = 0; j < 5; ++j) out->b[n][j] = n < nbubble ? bubbles[5 * n + j] : 0.0;
  for (int n = 0; n < nbubble; ++n) {
    MW_REQUIRE(std::isfinite(out->b[n][0]) && std::isfinite(out->b[n][1]) && std::isfinite(out->b[n][2]),
               MW_ERR_INVALID_ARG, "bubble %d: non-finite amplitude or centre", n);
    MW_REQUIRE(finite_pos(out->b[n][3]) && finite_pos(out->b[n][4]), MW_ERR_INVALID_ARG,
               "bubble %d: radii must be finite and positive", n);
  }
  return MW_OK;
}

template <typename T>
int run_init(int nx, int nz, double xlen, double zlen, int background, double u0, int nbubble, const double* bubbles,
             T* state, double* hyc, double* hytc, double* hyi, double* hyti, double* hypi, cudaStream_t stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(finite_pos(xlen) && finite_pos(zlen), MW_ERR_INVALID_ARG, "xlen, zlen must be finite and positive");
  MW_REQUIRE(std::isfinite(u0), MW_ERR_INVALID_ARG, "u0 must be finite");
  MW_REQUIRE(background == MW_BG_CONST_THETA || background == MW_BG_BVFREQ, MW_ERR_INVALID_ARG,
             "unknown background %d", background);
  MW_REQUIRE(state && hyc && hytc && hyi && hyti && hypi, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(aligned(state) && aligned(hyc) && aligned(hytc) && aligned(hyi) && aligned(hyti) && aligned(hypi),
             MW_ERR_ALIGN, "misaligned pointer");
  Bubbles b;
  st = check_bubbles(nbubble, bubbles, &b);
  if (st) return st;
  const double dx = xlen / nx, dz = zlen / nz;
  k_init_state<T><<<nz + 2 * kHs, 256, 0, stream>>>(nx, nz, dx, dz, background, u0, b, state);
  st = check_launch("initial condition launch");
  if (st) return st;
  k_init_background<<<grid_for(nz + 2 * kHs, 128), 128, 0, stream>>>(nz, dz, background, hyc, hytc, hyi, hyti, hypi);
  return check_launch("background launch");
}

}  // namespace
}  // namespace mw

using namespace mw;

extern "C" int mw_init_f64(int nx, int nz, double xlen, double zlen, int background, double u0, int nbubble,
                           const double* bubbles, double* state, double* hyc, double* hytc, double* hyi, double* hyti,
                           double* hypi, void* stream) {
  return run_init<double>(nx, nz, xlen, zlen, background, u0, nbubble, bubbles, state, hyc, hytc, hyi, hyti, hypi,
                          (cudaStream_t)stream);
}

extern "C" int mw_init_f32(int nx, int nz, double xlen, double zlen, int background, double u0, int nbubble,
                           const double* bubbles, float* state, double* hyc, double* hytc, double* hyi, double* hyti,
                           double* hypi, void* stream) {
  return run_init<float>(nx, nz, xlen, zlen, background, u0, nbubble, bubbles, state, hyc, hytc, hyi, hyti, hypi,
                         (cudaStream_t)stream);
}

extern "C" int mw_gravity_source_f64(int nx, int nz, double xlen, double zlen, const double* hyc, double* src_w,
                                     void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(finite_pos(xlen) && finite_pos(zlen), MW_ERR_INVALID_ARG, "xlen, zlen must be finite and positive");
  MW_REQUIRE(hyc && src_w, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(aligned(hyc) && aligned(src_w), MW_ERR_ALIGN, "misaligned pointer");
  k_gravity_source<<<grid_for((long long)nx * nz, 256), 256, 0, (cudaStream_t)stream>>>(nx, nz, xlen, zlen, hyc, src_w);
  return check_launch("gravity source launch");
}

extern "C" size_t mw_stats_workspace_bytes(int nx, int nz) {
  (void)nx;
  if (nz < 1) return 0;
  int rpb;
  return sizeof(double) * 2 * (size_t)stats_blocks(nz, &rpb);
}

extern "C" int mw_stats_f64(int nx, int nz, double dx, double dz, const double* hyc, const double* hytc,
                            const double* state, void* workspace, size_t workspace_bytes, double* out2, void* stream) {
  return run_stats<double>(nx, nz, dx, dz, hyc, hytc, state, workspace, workspace_bytes, out2, (cudaStream_t)stream);
}

extern "C" int mw_stats_f32(int nx, int nz, double dx, double dz, const double* hyc, const double* hytc,
                            const float* state, void* workspace, size_t workspace_bytes, double* out2, void* stream) {
  return run_stats<float>(nx, nz, dx, dz, hyc, hytc, state, workspace, workspace_bytes, out2, (cudaStream_t)stream);
}

extern "C" int mw_solution_variables_f64(int nx, int nz, const double* hyc, const double* hytc, const double* state,
                                         double* out, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(hyc && hytc && state && out, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(aligned(hyc) && aligned(hytc) && aligned(state) && aligned(out), MW_ERR_ALIGN, "misaligned pointer");
  k_solution_vars<<<grid_for((long long)nx * nz, 256), 256, 0, (cudaStream_t)stream>>>(nx, nz, hyc, hytc, state, out);
  return check_launch("solution variables launch");
}

extern "C" int mw_set_bc_f64(int nx, int nz, const double* hyc, double* state, int direction, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(hyc && state, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(aligned(hyc) && aligned(state), MW_ERR_ALIGN, "misaligned pointer");
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 or 1");
  const long long n = direction == MW_DIR_X ? 4LL * nz : nx + 2 * kHs;
  k_set_bc<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(nx, nz, hyc, state, direction);
  return check_launch("set_bc launch");
}

extern "C" int mw_interpolate_f64(int nx, int nz, const double* state, double* vals, double* d3, int direction,
                                  void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(state && vals && d3, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(aligned(state) && aligned(vals) && aligned(d3), MW_ERR_ALIGN, "misaligned pointer");
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 or 1");
  const long long n = direction == MW_DIR_X ? 4LL * nz * (nx + 1) : 4LL * (nz + 1) * nx;
  k_interpolate<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(nx, nz, state, vals, d3, direction);
  return check_launch("interpolate launch");
}

extern "C" int mw_flux_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                           const double* hyi, const double* hyti, const double* hypi, const double* vals, double* d3,
                           double* flux, int direction, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(finite_pos(dx) && finite_pos(dz) && finite_pos(dt_full), MW_ERR_INVALID_ARG,
             "dx, dz, dt_full must be finite and positive");
  MW_REQUIRE(hyc && hytc && hyi && hyti && hypi && vals && d3 && flux, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 or 1");
  FluxArgs a;
  a.nx = nx;
  a.nz = nz;
  a.hv = -kHvBeta * (direction == MW_DIR_X ? dx : dz) / (16 * dt_full);
  a.hyc = hyc;
  a.hytc = hytc;
  a.hyi = hyi;
  a.hyti = hyti;
  a.hypi = hypi;
  a.vals = vals;
  a.d3 = d3;
  a.flux = flux;
  a.dir = direction;
  const long long n = direction == MW_DIR_X ? (long long)nz * (nx + 1) : (long long)(nz + 1) * nx;
  k_flux<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(a);
  return check_launch("flux launch");
}

extern "C" int mw_tend_f64(int nx, int nz, double dx, double dz, const double* flux, const double* state_forcing,
                           const double* src_w, double* tend, int direction, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(finite_pos(dx) && finite_pos(dz), MW_ERR_INVALID_ARG, "dx, dz must be finite and positive");
  MW_REQUIRE(flux && state_forcing && tend, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 or 1");
  k_tend<<<grid_for((long long)nx * nz, 256), 256, 0, (cudaStream_t)stream>>>(
      nx, nz, direction == MW_DIR_X ? dx : dz, flux, state_forcing, src_w, tend, direction);
  return check_launch("tend launch");
}

extern "C" int mw_update_f64(int nx, int nz, const double* init, const double* tend, double* out, double dt_stage,
                             void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(init && tend && out, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(std::isfinite(dt_stage), MW_ERR_INVALID_ARG, "dt_stage must be finite");
  k_update<<<grid_for(4LL * nx * nz, 256), 256, 0, (cudaStream_t)stream>>>(nx, nz, init, tend, out, dt_stage);
  return check_launch("update launch");
}

extern "C" int mw_add_source_f64(int nx, int nz, const double* src_w, double* tend, void* stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(src_w && tend, MW_ERR_INVALID_ARG, "NULL pointer argument");
  k_add_source<<<grid_for((long long)nx * nz, 256), 256, 0, (cudaStream_t)stream>>>(nx, nz, src_w, tend);
  return check_launch("add_source launch");
}

// ---------------------------------------------------------------------------
// Non-finite values of the interior (failure detection after a step).
namespace mw {
namespace {
// Adds the number of non-finite interior values to *count (when non-NULL);
// the step entry points' check instead sets flag[0] = 1 and adds the count to
// flag[1] (two 32-bit words: the decision does not depend on the count, which
// may wrap for more than 2^32 values).
template <typename T>
__global__ void k_count_nonfinite(int nx, int nz, const T* s, unsigned long long* count, unsigned* flag) {
  const int pitch = nx + 2 * kHs;
  const long long plane = (long long)(nz + 2 * kHs) * pitch;
  const long long n = 4LL * nz * nx;
  unsigned c = 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long q = e / ((long long)nz * nx), r = e - q * nz * nx;
    const int k = (int)(r / nx), i = (int)(r - (long long)k * nx);
    const T v = MW_AT(s, q * plane + (long long)(k + kHs) * pitch + i + kHs, 4 * plane);
    c += !isfinite(v);
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) {
    if (count) atomicAdd(count, (unsigned long long)c);
    if (flag) {
      atomicOr(flag, 1u);
      atomicAdd(flag + 1, c);
    }
  }
}

template <typename T>
int count_nonfinite(int nx, int nz, const T* state, unsigned long long* count, unsigned* flag, cudaStream_t stream) {
  int st = check_grid(nx, nz);
  if (st) return st;
  MW_REQUIRE(state && (count || flag), MW_ERR_INVALID_ARG, "NULL pointer argument");
  const long long n = 4LL * nz * nx;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 8);
  k_count_nonfinite<T><<<(unsigned)blocks, 256, 0, stream>>>(nx, nz, state, count, flag);
  return check_launch("non-finite count launch");
}
}  // namespace

// The MW_FLAG_CHECK_FINITE tail of the step entry points (blocking).  It
// allocates nothing: the two 32-bit words it counts into are lent by the
// caller -- the first 8 bytes of the step's scratch array, whose contents
// after a step are unspecified (4-byte alignment suffices).
template <typename T>
int check_finite_blocking(int nx, int nz, const T* state, void* counter8, cudaStream_t stream) {
  MW_REQUIRE(counter8 && ((uintptr_t)counter8 % 4) == 0, MW_ERR_INVALID_ARG, "non-finite check: bad counter word");
  unsigned* d = static_cast<unsigned*>(counter8);
  unsigned h[2] = {0u, 0u};
  cudaError_t e = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned), stream);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "non-finite check: %s", cudaGetErrorString(e));
  int st = count_nonfinite<T>(nx, nz, state, nullptr, d, stream);
  if (st) return st;
  e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "non-finite check: %s", cudaGetErrorString(e));
  if (h[0]) return fail(MW_ERR_NONFINITE, "%u non-finite interior values (modulo 2^32) in the state after the step", h[1]);
  return MW_OK;
}
template int check_finite_blocking<double>(int, int, const double*, void*, cudaStream_t);
template int check_finite_blocking<float>(int, int, const float*, void*, cudaStream_t);

#if MW_CHECK
MW_OOB_COUNTER(oob_count_aux)
#endif
}  // namespace mw

extern "C" int mw_count_nonfinite_f64(int nx, int nz, const double* state, unsigned long long* count, void* stream) {
  return mw::count_nonfinite(nx, nz, state, count, nullptr, (cudaStream_t)stream);
}
extern "C" int mw_count_nonfinite_f32(int nx, int nz, const float* state, unsigned long long* count, void* stream) {
  return mw::count_nonfinite(nx, nz, state, count, nullptr, (cudaStream_t)stream);
}

