// mw_ensemble.cuh -- shared types of the ensemble path: one persistent launch
// per direction-stage advances every member of an ensemble of uneven grids.
#pragma once

#include <cuda_runtime.h>

#include "../../include/miniweather_gb300.h"

namespace mw {

// Stage constants of one member for one direction-stage, formed on the host
// when the plan is built, exactly as the single-grid launches form them.
// Split form: (h, l) float pairs of 12 hv, 12 d, 12 dz g and dt_stage / (12 d),
// and dt_stage / (12 d) * 2^896 in FP64.  FP32 form: hv, dt_stage / d and
// dt_stage rounded to float.  IEEE-FP64 form: -12 hv, dt_stage / (12 d),
// dt_stage and -dt_stage g.  Entry (member * 2 + (direction == z)) * 3 + stage
// (stage 0, 1, 2: dt/3, dt/2, dt).
struct EnsMemberConsts {
  float hv12[2], d12[2], gz12[2], c12[2];
  double c12s;
  float hv_f, c_f, dt_f, pad;
  double HV, c, dt, gdt;
};
static_assert(sizeof(EnsMemberConsts) == 88, "EnsMemberConsts layout");

// Work cursor of the persistent launches, in the plan.  The work lists are
// sorted by decreasing cost, and a warp (x) or CTA (z) that is free takes the
// next item, so a launch ends on its cheapest items.  `next` hands out list
// positions; `done` counts the CTAs that found the list empty, and the last of
// them resets both for the next launch on the plan (the launches of a step
// call are ordered by its stream).
struct EnsCursor {
  unsigned next, done, pad[2];
};

// Arguments of one ensemble direction-stage launch (T = state storage type).
template <typename T>
struct EnsStageT {
  const mw_ens_member* members;  // device
  const int2* items;             // device work list of this direction
  EnsCursor* cursor;             // device, in the plan
  int n_items;
  int z_tile;      // rows per z item
  int direction;   // MW_DIR_X / MW_DIR_Z
  int stage_div;   // the stage uses dt / stage_div (3, 2, 1)
  int fmt;         // split form: storage format of forcing / out (kF64, kToPair, kFromPair)
  unsigned flags;
  const double* hyc;
  const double* hytc;
  const double* hyi;
  const double* hyti;
  const double* hypi;
  const T* init;
  T* forcing;
  T* out;
  const void* xrows;  // split form: row constants indexed like the cell-centre backgrounds
  long long n_xrows;  // entries of xrows
  const void* mconsts;  // EnsMemberConsts per (member, direction, stage), written with the plan
  int n_members;
  cudaStream_t stream;
};
using EnsStage = EnsStageT<double>;

// Index of member e's entry for this launch's direction and stage in mconsts.
template <typename T>
__host__ __device__ inline int mconsts_index(const EnsStageT<T>& es, int e) {
  return (e * 2 + (es.direction == MW_DIR_X ? 0 : 1)) * 3 + (3 - es.stage_div);
}

// Launchers (defined next to the kernels they launch).
int launch_ens_split(const EnsStage& es, int grid);
int ens_split_occupancy(int direction, int* blocks_per_sm);
int launch_ens_f32(const EnsStageT<float>& es, int grid);
int ens_f32_occupancy(int direction, int* blocks_per_sm);
int launch_ens_ieee(const EnsStage& es, int grid);
int ens_ieee_occupancy(int direction, int* blocks_per_sm);

constexpr int kEnsZTileMax = 64;
constexpr int kEnsZCols = 64;  // columns per z work item (one CTA of kEnsZCols threads)
constexpr size_t kEnsRowBytes = 40;  // one row's background constants: four double-FP32 pairs (split form,
                                     // 32 B used) or five FP64 values (IEEE-FP64 form)

constexpr int kEnsConstsPerMember = 6;
inline size_t ens_consts_off(const mw_ens_plan_info& info) {
  return (info.xrows_off + kEnsRowBytes * (size_t)info.n_xrows + 15) & ~(size_t)15;
}

inline size_t ens_cursor_off(const mw_ens_plan_info& info) {
  return (ens_consts_off(info) + sizeof(EnsMemberConsts) * kEnsConstsPerMember * (size_t)info.n_members + 15) &
         ~(size_t)15;
}

#ifdef __CUDACC__
// The next list position for the calling warp (all 32 lanes call it).
__device__ __forceinline__ unsigned ens_take_warp(EnsCursor* c) {
  unsigned v = 0;
  if ((threadIdx.x & 31) == 0) v = atomicAdd(&c->next, 1u);
  return __shfl_sync(0xffffffffu, v, 0);
}
// The next list position for the calling CTA (every thread calls it): thread
// 0 takes it into one of two shared slots, alternated so that a slot is not
// rewritten before every thread has read it.
__device__ __forceinline__ unsigned ens_take_cta(EnsCursor* c, unsigned* slot, int& parity) {
  if (threadIdx.x == 0) slot[parity] = atomicAdd(&c->next, 1u);
  __syncthreads();
  const unsigned v = slot[parity];
  parity ^= 1;
  return v;
}
// Every thread of the CTA, once it has stopped taking items.
__device__ __forceinline__ void ens_finish(EnsCursor* c) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&c->done, 1u) == gridDim.x - 1) {  // every other CTA has stopped taking
      atomicExch(&c->next, 0u);
      atomicExch(&c->done, 0u);
    }
  }
}
#endif

// Row-constant tables of the split / IEEE-FP64 ensemble x kernels: entry j from hyc[j], hytc[j].
int launch_ens_split_rowtable(const double* hyc, const double* hytc, long long n, void* table, cudaStream_t stream);
int launch_ens_ieee_rowtable(const double* hyc, const double* hytc, long long n, void* table, cudaStream_t stream);

}  // namespace mw
