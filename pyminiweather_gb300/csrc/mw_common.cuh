// mw_common.cuh -- constants, host-side argument checks and error plumbing
// shared by the translation units of libminiweather_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "../../include/miniweather_gb300.h"

// MW_CHECK=1 builds the bounds-checked library (a debug build): the kernels
// that access memory through MW_AT count every index outside its array
// instead of touching memory there, and mw_debug_oob_count reads the count.
#ifndef MW_CHECK
#define MW_CHECK 0
#endif

namespace mw {

#if MW_CHECK
static __device__ unsigned long long g_oob_count;           // per translation unit
static __device__ __align__(16) unsigned char g_oob_sink[128];  // stands in for out-of-range elements

template <typename T, typename I>
__device__ __forceinline__ T& checked_at(T* p, I i, long long n) {
  static_assert(sizeof(T) <= sizeof(g_oob_sink), "element larger than the sink");
  if ((long long)i < 0 || (long long)i >= n) {
    atomicAdd(&g_oob_count, 1ULL);
    return *reinterpret_cast<T*>(g_oob_sink);
  }
  return p[i];
}
#define MW_AT(p, i, n) (::mw::checked_at((p), (i), (long long)(n)))
// Adds this translation unit's count to *out (and resets it).
#define MW_OOB_COUNTER(fn)                                                          \
  int fn(unsigned long long* out, bool reset) {                                     \
    unsigned long long v = 0;                                                       \
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_oob_count, sizeof(v));               \
    if (e == cudaSuccess && reset) {                                                \
      const unsigned long long z = 0;                                               \
      e = cudaMemcpyToSymbol(g_oob_count, &z, sizeof(z));                           \
    }                                                                               \
    if (e != cudaSuccess) return fail(MW_ERR_CUDA, "oob counter: %s", cudaGetErrorString(e)); \
    *out += v;                                                                      \
    return MW_OK;                                                                   \
  }
#else
#define MW_AT(p, i, n) ((p)[(i)])
#endif

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

inline bool valid_f64_mode(int m) { return m == MW_F64_NATIVE || m == MW_F64_SPLIT || m == MW_F64_IEEE; }

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
