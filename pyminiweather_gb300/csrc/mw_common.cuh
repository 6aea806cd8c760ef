// mw_common.cuh -- constants, host-side argument checks and error plumbing
// shared by the translation units of libminiweather_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "../../include/miniweather_gb300.h"

namespace mw {

// Physical constants, pyminiweather/data/constants.py:13-27.
constexpr double kHvBeta = 0.05;
constexpr double kP0 = 1.0e5;
constexpr double kC0 = 27.5629410929725921310572974482;
constexpr double kGamma = 1.40027894002789400278940027894;
constexpr double kGrav = 9.8;
constexpr double kCp = 1004.0;
constexpr double kCv = 717.0;
constexpr double kRd = 287.0;
constexpr double kPi = 3.14159265358979323846264338327;
constexpr double kTheta0 = 300.0;
constexpr double kExner0 = 1.0;

constexpr int kHs = 2;  // halo width (params["hs"], fixed at 2 by the reference CLI)
enum { DENS = 0, UMOM = 1, WMOM = 2, RHOT = 3 };

// Geometry of one (4, nz+4, nx+4) state array.
struct Geom {
  int nx, nz;
  int pitch;          // nx + 4
  long long plane;    // (nz + 4) * (nx + 4)
};

inline Geom make_geom(int nx, int nz) {
  Geom g;
  g.nx = nx;
  g.nz = nz;
  g.pitch = nx + 2 * kHs;
  g.plane = (long long)(nz + 2 * kHs) * (nx + 2 * kHs);
  return g;
}

// ---------------------------------------------------------------------------
// Host-side error state (one message per calling thread).
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int check_launch(const char* what);

inline bool finite_pos(double v) { return std::isfinite(v) && v > 0.0; }

template <typename T>
inline bool aligned(const T* p) {
  return ((uintptr_t)p % alignof(T)) == 0;
}

inline bool ranges_overlap(const void* a, size_t abytes, const void* b, size_t bbytes) {
  uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
  return a0 < b0 + bbytes && b0 < a0 + abytes;
}

int check_grid(int nx, int nz);

// Rows per z CTA for a single-grid launch: the largest tile up to max_rows
// that still gives about two CTAs per SM (152 SMs), at least 8 rows.
inline int z_tile_rows(int nx, int nz, int cols_per_cta, int max_rows) {
  const long long ncb = (nx + cols_per_cta - 1) / cols_per_cta;
  long long t = (long long)nz * ncb / 304;
  if (t > max_rows) t = max_rows;
  if (t < 8) t = 8;
  return (int)t;
}

}  // namespace mw

#define MW_REQUIRE(cond, code, ...)            \
  do {                                         \
    if (!(cond)) return mw::fail((code), __VA_ARGS__); \
  } while (0)
