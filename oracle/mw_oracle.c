/*
 * mw_oracle.c -- CPU restatement of the PyMiniWeather finite-volume time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the CUDA path is checked
 * against it, and bench.py times it as the CPU baseline.  Nothing on the
 * product path (pyminiweather_gb300) may link or call it.
 *
 * It restates, operation for operation, the NumPy/SciPy FP64 code of the
 * reference package (shriram-jagan/pyminiweather) so that rounding follows the
 * same order of operations:
 *   - interface interpolation as scipy.signal.convolve(mode="same")[..., 2:-1]
 *     accumulates it: ((s0*k3 + s1*k2) + s2*k1) + s3*k0
 *     (pyminiweather/solve/interpolate.py:33-43, 69-79);
 *   - Euler fluxes + hyperviscosity (interpolate.py:82-186);
 *   - tendencies and the gravity term (interpolate.py:189-250);
 *   - halo fill, periodic in x on interior rows and solid wall in z on all
 *     columns, written in place into the forcing array (ics/bcs.py:8-39, 67-148);
 *   - the stage update out = init + dt*tend (solve/step.py:80-82);
 *   - RK3 with alternating direction order (solve/step.py:85-143);
 *   - the 3x3 Gauss-Legendre initial condition and hydrostatic background
 *     (ics/initial.py:11-105, ics/initial_conditions.py:26-81, 96-268,
 *     utils/utils.py:5-51, data/quadrature.py:15-39, mesh.py:25-112);
 *   - the gravity-wave forcing (solve/source.py:20-50);
 *   - mass / total energy (post/stats.py:8-35).
 * Compile with -ffp-contract=off: NumPy evaluates each binary operation
 * separately, so no multiply-add may be fused here.
 *
 * Parity pin: validated against outputs of the reference itself, run in the
 * build container, committed as the .npz files under tests/golden, made by
 * tests/golden/gen_golden.py.
 * NumPy's float64 pow on that machine is an AVX-512 SVML variant that differs
 * from libm pow by about 1 ulp, so the oracle matches the reference to
 * rounding level (checked in tests/test_oracle_golden.py), not bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mw_oracle.h"

/* pyminiweather/data/constants.py:13-27 */
static const double HV_BETA = 0.05;
static const double P0 = 1.0e5;
static const double C0 = 27.5629410929725921310572974482;
static const double GAMMA = 1.40027894002789400278940027894;
static const double GRAV = 9.8;
static const double CP = 1004.0;
static const double CV = 717.0;
static const double RD = 287.0;
static const double PI = 3.14159265358979323846264338327;
static const double THETA0 = 300.0;
static const double EXNER0 = 1.0;

/* pyminiweather/data/quadrature.py:15-30 */
static const double QP[3] = {0.112701665379258311482073460022, 0.500000000000000000000000000000,
                             0.887298334620741688517926539980};
static const double QW[3] = {0.277777777777777777777777777779, 0.444444444444444444444444444444,
                             0.277777777777777777777777777779};

#define HS 2
enum { DENS = 0, UMOM = 1, WMOM = 2, RHOT = 3 };

int mwo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void mwo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* numpy.linspace(start, stop, num, endpoint=False)[k]: step = (stop-start)/num,
 * y = k*step + start, two separate roundings. */
static inline double linspace_at(double start, double stop, int num, int k) {
  double step = (stop - start) / (double)num;
  return (double)k * step + start;
}

/* hydro_const_theta, ics/initial_conditions.py:26-52 */
static void hydro_const_theta(double z, double* hr, double* ht) {
  double exner = EXNER0 - GRAV * z / (CP * THETA0);
  double p = P0 * pow(exner, CP / RD);
  *ht = THETA0;
  *hr = pow(p / C0, 1.0 / GAMMA) / THETA0;
}

/* hydro_const_bvfreq, ics/initial_conditions.py:54-81 */
static void hydro_const_bvfreq(double z, double bv0, double* hr, double* ht) {
  double t = THETA0 * exp(bv0 * bv0 / GRAV * z);
  double exner = EXNER0 - GRAV * GRAV / (CP * bv0 * bv0) * (t - THETA0) / (t * THETA0);
  double p = P0 * pow(exner, CP / RD);
  *ht = t;
  *hr = pow(p / C0, 1.0 / GAMMA) / t;
}

static void hydro(int bg, double z, double* hr, double* ht) {
  if (bg == MWO_BG_BVFREQ)
    hydro_const_bvfreq(z, 0.02, hr, ht);
  else
    hydro_const_theta(z, hr, ht);
}

/* sample_ellipse_cosine, utils/utils.py:5-51 */
static double ellipse_cos2(double x, double z, double amp, double x0, double z0, double xr, double zr) {
  double a = (x - x0) / xr;
  double b = (z - z0) / zr;
  double dist = sqrt(a * a + b * b) * PI / 2.0;
  if (dist <= PI / 2.0) {
    double c = cos(dist);
    return amp * (c * c);
  }
  return 0.0;
}

/* init(), ics/initial.py:11-105.  state is (4, nz+4, nx+4); backgrounds are
 * hy_dens_cell/hy_dens_theta_cell (nz+4) and the three interface arrays (nz+1). */
void mwo_init(int nx, int nz, double xlen, double zlen, int bg, double u0, int nbubble,
              const double* bubbles, double* state, double* hy_dens_cell, double* hy_dens_theta_cell,
              double* hy_dens_int, double* hy_dens_theta_int, double* hy_pressure_int) {
  const double dx = xlen / nx, dz = zlen / nz;
  const int NX = nx + 2 * HS, NZ = nz + 2 * HS;
  const size_t plane = (size_t)NX * NZ;
  /* MeshData.get_mesh_int_ext, mesh.py:37-51 */
  const double xs = -HS * dx, xe = (nx + HS) * dx;
  const double zs = -HS * dz, ze = (nz + HS) * dz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NZ; ++k) {
    double zm = linspace_at(zs, ze, NZ, k);
    for (int i = 0; i < NX; ++i) {
      double xm = linspace_at(xs, xe, NX, i);
      double acc[4][3];
      for (int a = 0; a < 3; ++a) {
        double z = zm + QP[a] * dz;
        double hr, ht;
        hydro(bg, z, &hr, &ht);
        for (int b = 0; b < 3; ++b) {
          double x = xm + QP[b] * dx;
          double t = 0.0;
          for (int q = 0; q < nbubble; ++q) {
            const double* B = bubbles + 5 * q;
            t = t + ellipse_cos2(x, z, B[0], B[1], B[2], B[3], B[4]);
          }
          const double r = 0.0, u = u0, w = 0.0;
          double W = QW[a] * QW[b];
          double v0 = r * W;
          double v1 = ((r + hr) * u) * W;
          double v2 = ((r + hr) * w) * W;
          double v3 = ((r + hr) * (t + ht) - hr * ht) * W;
          if (b == 0) {
            acc[0][a] = v0; acc[1][a] = v1; acc[2][a] = v2; acc[3][a] = v3;
          } else {
            acc[0][a] += v0; acc[1][a] += v1; acc[2][a] += v2; acc[3][a] += v3;
          }
        }
      }
      for (int v = 0; v < 4; ++v)
        state[v * plane + (size_t)k * NX + i] = (acc[v][0] + acc[v][1]) + acc[v][2];
    }
  }
  /* cell-centre background, initial.py:84-95 */
  const double sumw = (QW[0] + QW[1]) + QW[2];
  for (int k = 0; k < NZ; ++k) {
    double z = linspace_at((-HS + 0.5) * dz, (nz + HS + 0.5) * dz, NZ, k);
    double hr, ht;
    hydro(bg, z, &hr, &ht);
    hy_dens_cell[k] = hr * sumw;
    double a = ht * hr;
    hy_dens_theta_cell[k] = (a * QW[0] + a * QW[1]) + a * QW[2];
  }
  /* interface background, initial.py:100-105 */
  for (int k = 0; k <= nz; ++k) {
    double z = linspace_at(0.0, (nz + 1) * dz, nz + 1, k);
    double hr, ht;
    hydro(bg, z, &hr, &ht);
    hy_dens_int[k] = hr;
    hy_dens_theta_int[k] = hr * ht;
    hy_pressure_int[k] = C0 * pow(hr * ht, GAMMA);
  }
}

/* GravityBCSourceTerm, solve/source.py:20-50: wpert*hy_dens_cell at interior
 * cell centres, (nz, nx). */
void mwo_gravity_source(int nx, int nz, double xlen, double zlen, const double* hy_dens_cell, double* src) {
  const double dx = xlen / nx, dz = zlen / nz;
  for (int k = 0; k < nz; ++k) {
    double z = linspace_at(dz / 2.0, zlen + dz / 2.0, nz, k);
    for (int i = 0; i < nx; ++i) {
      double x = linspace_at(dx / 2.0, xlen + dx / 2.0, nx, i);
      double w = ellipse_cos2(x, z, 0.01, xlen / 8, 1000.0, 500.0, 500.0);
      src[(size_t)k * nx + i] = w * hy_dens_cell[k + HS];
    }
  }
}

/* set_bc_x, ics/bcs.py:35-39 (the injection branch is not restated). */
static void bc_x_row(int nx, double* row) {
  row[0] = row[nx];
  row[1] = row[nx + 1];
  row[nx + HS] = row[HS];
  row[nx + HS + 1] = row[HS + 1];
}

/* set_bc_z, ics/bcs.py:92-148, all nx+4 columns. */
static void bc_z(int nx, int nz, const double* hyc, double* f) {
  const int NX = nx + 2 * HS, NZ = nz + 2 * HS;
  const size_t plane = (size_t)NX * NZ;
  double* D = f + DENS * plane;
  double* U = f + UMOM * plane;
  double* Wm = f + WMOM * plane;
  double* T = f + RHOT * plane;
#define R(A, k) ((A) + (size_t)(k) * NX)
  for (int c = 0; c < NX; ++c) {
    R(Wm, 0)[c] = 0.0;
    R(Wm, 1)[c] = 0.0;
    R(Wm, nz + HS)[c] = 0.0;
    R(Wm, nz + HS + 1)[c] = 0.0;
    R(U, 0)[c] = R(U, HS)[c] / hyc[HS] * hyc[0];
    R(U, 1)[c] = R(U, HS)[c] / hyc[HS] * hyc[1];
    R(U, nz + HS)[c] = R(U, nz + HS - 1)[c] / hyc[nz + HS - 1] * hyc[nz + HS];
    R(U, nz + HS + 1)[c] = R(U, nz + HS - 1)[c] / hyc[nz + HS - 1] * hyc[nz + HS + 1];
    R(D, 0)[c] = R(D, HS)[c];
    R(D, 1)[c] = R(D, HS)[c];
    R(D, nz + HS)[c] = R(D, nz + HS - 1)[c];
    R(D, nz + HS + 1)[c] = R(D, nz + HS - 1)[c];
    R(T, 0)[c] = R(T, HS)[c];
    R(T, 1)[c] = R(T, HS)[c];
    R(T, nz + HS)[c] = R(T, nz + HS - 1)[c];
    R(T, nz + HS + 1)[c] = R(T, nz + HS - 1)[c];
  }
#undef R
}

/* scipy.signal.convolve(mode="same") accumulation order for the 4-tap kernels
 * [k0,k1,k2,k3]: fourth-order [-1/12, 7/12, 7/12, -1/12] (data/fields.py:94-97)
 * and the third-difference kernel [1, -3, 3, -1]. */
static inline double interp4(double s0, double s1, double s2, double s3) {
  const double k0 = -1.0 / 12, k1 = 7.0 / 12, k2 = 7.0 / 12, k3 = -1.0 / 12;
  return ((s0 * k3 + s1 * k2) + s2 * k1) + s3 * k0;
}
static inline double diff3(double s0, double s1, double s2, double s3) {
  const double k0 = 1.0, k1 = -3.0, k2 = 3.0, k3 = -1.0;
  return ((s0 * k3 + s1 * k2) + s2 * k1) + s3 * k0;
}

/* One discrete_step (solve/step.py:21-82) in direction dir (0 = x, 1 = z).
 * The halo of `forcing` is written as the reference writes it.  `out` may
 * alias `forcing` or `init`.  src_w (nz, nx) is the optional gravity-wave
 * forcing added to the w tendency (NULL for none). */
void mwo_dirstage(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                  const double* hyi, const double* hyti, const double* hypi, const double* src_w,
                  const double* init, double* forcing, double* out, double dt_stage, int dir) {
  const int NX = nx + 2 * HS, NZ = nz + 2 * HS;
  const size_t plane = (size_t)NX * NZ;
  if (dir == MWO_DIR_X) {
    const double hv = -HV_BETA * dx / (16 * dt_full);
#pragma omp parallel
    {
      double* buf = (double*)malloc(sizeof(double) * (size_t)(4 * (nx + 1) + 4 * nx));
      double* F = buf;                       /* 4 x (nx+1) */
      double* tend = buf + 4 * (nx + 1);     /* 4 x nx */
#pragma omp for schedule(static)
      for (int k = 0; k < nz; ++k) {
        const int kk = k + HS;
        const double* s[4];
        for (int v = 0; v < 4; ++v) {
          double* row = forcing + v * plane + (size_t)kk * NX;
          bc_x_row(nx, row);
          s[v] = row;
        }
        for (int i = 0; i <= nx; ++i) {
          double val[4], d3[4];
          for (int v = 0; v < 4; ++v) {
            val[v] = interp4(s[v][i], s[v][i + 1], s[v][i + 2], s[v][i + 3]);
            d3[v] = diff3(s[v][i], s[v][i + 1], s[v][i + 2], s[v][i + 3]);
          }
          double rho = val[DENS] + hyc[kk];
          double u = val[UMOM] / rho;
          double w = val[WMOM] / rho;
          double t = (val[RHOT] + hytc[kk]) / rho;
          double p = C0 * pow(rho * t, GAMMA);
          F[0 * (nx + 1) + i] = rho * u - hv * d3[DENS];
          F[1 * (nx + 1) + i] = rho * (u * u) + p - hv * d3[UMOM];
          F[2 * (nx + 1) + i] = rho * u * w - hv * d3[WMOM];
          F[3 * (nx + 1) + i] = rho * u * t - hv * d3[RHOT];
        }
        for (int v = 0; v < 4; ++v)
          for (int i = 0; i < nx; ++i)
            tend[v * nx + i] = -(F[v * (nx + 1) + i + 1] - F[v * (nx + 1) + i]) / dx;
        if (src_w)
          for (int i = 0; i < nx; ++i) tend[WMOM * nx + i] = tend[WMOM * nx + i] + src_w[(size_t)k * nx + i];
        for (int v = 0; v < 4; ++v) {
          const double* in = init + v * plane + (size_t)kk * NX + HS;
          double* o = out + v * plane + (size_t)kk * NX + HS;
          for (int i = 0; i < nx; ++i) o[i] = in[i] + dt_stage * tend[v * nx + i];
        }
      }
      free(buf);
    }
  } else {
    const double hv = -HV_BETA * dz / (16 * dt_full);
    bc_z(nx, nz, hyc, forcing);
    const int CB = 32; /* column block: the z pass couples rows only */
    const int nblk = (nx + CB - 1) / CB;
#pragma omp parallel
    {
      double* G = (double*)malloc(sizeof(double) * (size_t)4 * (nz + 1) * CB);
#pragma omp for schedule(static)
      for (int b = 0; b < nblk; ++b) {
        const int c0 = b * CB;
        const int cn = (nx - c0) < CB ? (nx - c0) : CB;
        for (int k = 0; k <= nz; ++k) {
          for (int j = 0; j < cn; ++j) {
            const int c = c0 + j + HS;
            double val[4], d3[4];
            for (int v = 0; v < 4; ++v) {
              const double* col = forcing + v * plane + c;
              double s0 = col[(size_t)k * NX], s1 = col[(size_t)(k + 1) * NX];
              double s2 = col[(size_t)(k + 2) * NX], s3 = col[(size_t)(k + 3) * NX];
              val[v] = interp4(s0, s1, s2, s3);
              d3[v] = diff3(s0, s1, s2, s3);
            }
            double rho = val[DENS] + hyi[k];
            double u = val[UMOM] / rho;
            double w = val[WMOM] / rho;
            double t = (val[RHOT] + hyti[k]) / rho;
            double p = C0 * pow(rho * t, GAMMA) - hypi[k];
            if (k == 0 || k == nz) {
              w = 0.0;
              d3[DENS] = 0.0;
            }
            G[(0 * (size_t)(nz + 1) + k) * CB + j] = rho * w - hv * d3[DENS];
            G[(1 * (size_t)(nz + 1) + k) * CB + j] = rho * w * u - hv * d3[UMOM];
            G[(2 * (size_t)(nz + 1) + k) * CB + j] = rho * (w * w) + p - hv * d3[WMOM];
            G[(3 * (size_t)(nz + 1) + k) * CB + j] = rho * w * t - hv * d3[RHOT];
          }
        }
        for (int k = 0; k < nz; ++k) {
          const int kk = k + HS;
          for (int j = 0; j < cn; ++j) {
            const int c = c0 + j + HS;
            double tend[4];
            for (int v = 0; v < 4; ++v)
              tend[v] = -(G[(v * (size_t)(nz + 1) + k + 1) * CB + j] - G[(v * (size_t)(nz + 1) + k) * CB + j]) / dz;
            tend[WMOM] = tend[WMOM] - forcing[DENS * plane + (size_t)kk * NX + c] * GRAV;
            if (src_w) tend[WMOM] = tend[WMOM] + src_w[(size_t)k * nx + c - HS];
            for (int v = 0; v < 4; ++v) {
              size_t o = v * plane + (size_t)kk * NX + c;
              out[o] = init[o] + dt_stage * tend[v];
            }
          }
        }
      }
      free(G);
    }
  }
}

/* evolve, solve/step.py:85-143.  *reverse is the module-global direction flag:
 * 0 runs z then x, 1 runs x then z; it is toggled after every step. */
void mwo_evolve(int nx, int nz, double dx, double dz, double dt, const double* hyc, const double* hytc,
                const double* hyi, const double* hyti, const double* hypi, const double* src_w, double* state,
                double* state_tmp, int nsteps, int* reverse) {
  for (int s = 0; s < nsteps; ++s) {
    int dirs[2];
    if (*reverse) {
      dirs[0] = MWO_DIR_X; dirs[1] = MWO_DIR_Z;
    } else {
      dirs[0] = MWO_DIR_Z; dirs[1] = MWO_DIR_X;
    }
    for (int d = 0; d < 2; ++d) {
      mwo_dirstage(nx, nz, dx, dz, dt, hyc, hytc, hyi, hyti, hypi, src_w, state, state, state_tmp, dt / 3, dirs[d]);
      mwo_dirstage(nx, nz, dx, dz, dt, hyc, hytc, hyi, hyti, hypi, src_w, state, state_tmp, state_tmp, dt / 2, dirs[d]);
      mwo_dirstage(nx, nz, dx, dz, dt, hyc, hytc, hyi, hyti, hypi, src_w, state, state_tmp, state, dt / 1, dirs[d]);
    }
    *reverse = *reverse ? 0 : 1;
  }
}

/* compute_stats, post/stats.py:8-35.  Sums are pairwise over each row and the
 * row sums pairwise again; NumPy's blocking differs, so totals agree with the
 * reference to rounding level only. */
static double pairwise(const double* a, size_t n) {
  if (n <= 8) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += a[i];
    return s;
  }
  size_t h = n / 2;
  return pairwise(a, h) + pairwise(a + h, n - h);
}

void mwo_stats(int nx, int nz, double dx, double dz, const double* hyc, const double* hytc, const double* state,
               double* mass_energy) {
  const int NX = nx + 2 * HS, NZ = nz + 2 * HS;
  const size_t plane = (size_t)NX * NZ;
  double* rows = (double*)malloc(sizeof(double) * 2 * (size_t)nz);
#pragma omp parallel
  {
    double* m = (double*)malloc(sizeof(double) * (size_t)nx);
    double* e = (double*)malloc(sizeof(double) * (size_t)nx);
#pragma omp for schedule(static)
    for (int k = 0; k < nz; ++k) {
      const int kk = k + HS;
      for (int i = 0; i < nx; ++i) {
        size_t o = (size_t)kk * NX + i + HS;
        double rho = state[DENS * plane + o] + hyc[kk];
        double u = state[UMOM * plane + o] / rho;
        double w = state[WMOM * plane + o] / rho;
        double th = (state[RHOT * plane + o] + hytc[kk]) / rho;
        double p = C0 * pow(rho * th, GAMMA);
        double t = th / pow(P0 / p, RD / CP);
        double ke = rho * (u * u + w * w);
        double ie = rho * CV * t;
        m[i] = rho;
        e[i] = ke + ie;
      }
      rows[k] = pairwise(m, nx);
      rows[nz + k] = pairwise(e, nx);
    }
    free(m);
    free(e);
  }
  mass_energy[0] = pairwise(rows, nz) * dx * dz;
  mass_energy[1] = pairwise(rows + nz, nz) * dx * dz;
  free(rows);
}
