// mw_split_stage.cu -- FP64-storage direction-stage kernels with the interior
// arithmetic in double-FP32 (see mw_split.cuh): the GB300 form of
// discrete_step (pyminiweather/solve/step.py:21-82).
//
// Loads and stores are FP64; each loaded value is split once into (h, l);
// interpolation, fluxes, pressure and flux divergence run on the FP32 pipe;
// the stage update out = init + increment is one FP64 add per value.
//
// Quantities are carried scaled by 12 (mw_split_flux.cuh): A = 12 vals, and
// the background terms, pressure and hyperviscosity coefficient are scaled to
// match; the flux divergence is multiplied by dt / (12 d).  Pressure is
// P_row ((1 + delta)^gamma - 1) with P_row = C0 (rho theta)_bg^gamma: in z the
// reference's p - hy_pressure_int (interpolate.py:163-165); in x the row
// constant cancels in the flux difference.
#include <algorithm>
#include <atomic>

#include "mw_common.cuh"
#include "mw_ensemble.cuh"
#include "mw_split.cuh"
#include "mw_split2.cuh"
#include "mw_split_flux.cuh"

namespace mw {
using namespace split;

namespace s32 {
typedef int sidx;
#include "mw_split_stage_impl.cuh"
}  // namespace s32

namespace s64 {
typedef long long sidx;
#include "mw_split_stage_impl.cuh"
}  // namespace s64

// Arrays whose four planes span fewer than 2^31 elements take the 32-bit-index
// kernels.  Output rows [r0, r1) (the whole grid: 0, nz); fmt 0 FP64 throughout, 1 forcing
// (== init) FP64 and out as double-FP32 pairs, 2 forcing as pairs.
int launch_stage_split(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                       const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                       const double* init, double* forcing, double* out, double dt_stage, int direction,
                       unsigned flags, int r0, int r1, int fmt, cudaStream_t stream) {
  const bool small = 4 * make_geom(nx, nz).plane < (1LL << 31) && !(flags & MW_FLAG_INDEX64);
  return (small ? s32::launch_stage_split : s64::launch_stage_split)(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti,
                                                                     hypi, srcw, init, forcing, out, dt_stage,
                                                                     direction, flags, r0, r1, fmt, stream);
}

static_assert(sizeof(RowS) <= kEnsRowBytes, "row-constant table entry size");

__global__ void k_ens_row_table(const double* hyc, const double* hytc, long long n, RowS* table) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
    const double hrt = MW_AT(hytc, j, n);
    MW_AT(table, j, n) = row_consts(MW_AT(hyc, j, n), hrt, kC0 * pow(hrt, kGamma));
  }
}

int launch_ens_split_rowtable(const double* hyc, const double* hytc, long long n, void* table, cudaStream_t stream) {
  if (n <= 0) return MW_OK;
  MW_REQUIRE(((uintptr_t)table % 16) == 0, MW_ERR_ALIGN, "row table misaligned");
  const long long blocks = std::min<long long>((n + 127) / 128, 4096);
  k_ens_row_table<<<(unsigned)blocks, 128, 0, stream>>>(hyc, hytc, n, (RowS*)table);
  return check_launch("ensemble row-table launch");
}

#if MW_CHECK
MW_OOB_COUNTER(oob_count_split_stage)
#endif

// Ensemble members are planned with fewer than 2^31 elements per state array.
int launch_ens_split(const EnsStage& es, int grid) { return s32::launch_ens_split(es, grid); }
int ens_split_occupancy(int direction, int* blocks_per_sm) { return s32::ens_split_occupancy(direction, blocks_per_sm); }

}  // namespace mw
