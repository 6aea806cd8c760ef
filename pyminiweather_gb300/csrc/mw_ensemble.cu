// mw_ensemble.cu -- host side of the ensemble path: work plans and the time
// step that advances every member with one persistent launch per
// direction-stage (6 per step).
//
// The plan lives in caller-provided device memory:
//   [members: n x mw_ens_member][x items: int2 (member, row)]
//   [z items: int2 (member, column block + ncb * z tile)]
//   [row constants: n_xrows x 40 B, written by each FP64 step call]
//   [stage constants: n x 6 x EnsMemberConsts, written with the plan]
//   [work cursor: EnsCursor, zero between launches]
// x work items are member rows (one warp walks the segments of the row); z items
// are kEnsZCols-column x z_tile-row tiles.  Each list is sorted by decreasing
// cost (x: row length; z: tile rows, then used columns), members in order
// within a cost, and the persistent warps (x) / CTAs (z) take items from the
// cursor as they become free.
#include <algorithm>
#include <type_traits>
#include <cstring>
#include <numeric>
#include <vector>

#include <cmath>

#include "mw_common.cuh"
#include "mw_ensemble.cuh"
#include "mw_split.cuh"

namespace mw {
namespace {


size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

int check_members(int n, const mw_ens_member* m, int z_tile) {
  MW_REQUIRE(n >= 1, MW_ERR_INVALID_ARG, "n_members must be >= 1");
  MW_REQUIRE(m != nullptr, MW_ERR_INVALID_ARG, "members must not be NULL");
  MW_REQUIRE(z_tile >= 1 && z_tile <= kEnsZTileMax, MW_ERR_INVALID_ARG, "z_tile must be in [1, %d]", kEnsZTileMax);
  for (int e = 0; e < n; ++e) {
    const int st = check_grid(m[e].nx, m[e].nz);
    if (st) return fail(st, "member %d: %s", e, mw_last_error());
    MW_REQUIRE(finite_pos(m[e].dx) && finite_pos(m[e].dz) && finite_pos(m[e].dt), MW_ERR_INVALID_ARG,
               "member %d: dx, dz, dt must be finite and positive", e);
    MW_REQUIRE(m[e].state_off >= 0 && m[e].cell_off >= 0 && m[e].int_off >= 0, MW_ERR_INVALID_ARG,
               "member %d: negative offset", e);
    MW_REQUIRE(4 * make_geom(m[e].nx, m[e].nz).plane < (1LL << 31), MW_ERR_SHAPE,
               "member %d: a member's state array must hold fewer than 2^31 values", e);
  }
  // members' state blocks must not overlap (each is written by its own items)
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int a, int b) { return m[a].state_off < m[b].state_off; });
  for (int j = 0; j + 1 < n; ++j) {
    const mw_ens_member& a = m[order[j]];
    const long long size = 4LL * (a.nx + 2 * kHs) * (a.nz + 2 * kHs);
    MW_REQUIRE(a.state_off + size <= m[order[j + 1]].state_off, MW_ERR_ALIAS,
               "members %d and %d overlap in the state buffers", order[j], order[j + 1]);
  }
  return MW_OK;
}

int layout(int n, const mw_ens_member* m, int z_tile, mw_ens_plan_info* info) {
  long long nxi = 0, nzi = 0, nrows = 0;
  for (int e = 0; e < n; ++e) {
    nrows = std::max(nrows, m[e].cell_off + m[e].nz + 2LL * kHs);
    nxi += m[e].nz;
    nzi += (long long)((m[e].nx + kEnsZCols - 1) / kEnsZCols) * ((m[e].nz + z_tile - 1) / z_tile);
  }
  MW_REQUIRE(nxi < (1LL << 31) && nzi < (1LL << 31), MW_ERR_SHAPE, "ensemble too large for one work list");
  info->n_members = n;
  info->n_x_items = (int)nxi;
  info->n_z_items = (int)nzi;
  info->z_tile = z_tile;
  info->members_off = 0;
  info->x_items_off = align16(sizeof(mw_ens_member) * (size_t)n);
  info->z_items_off = align16(info->x_items_off + sizeof(int2) * (size_t)nxi);
  info->xrows_off = align16(info->z_items_off + sizeof(int2) * (size_t)nzi);
  info->n_xrows = nrows;
  info->bytes = ens_cursor_off(*info) + sizeof(EnsCursor);
  return MW_OK;
}

int num_sms(int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "device query: %s", cudaGetErrorString(e));
  return MW_OK;
}

// fmts: storage format of the three RK stages' forcing / output (the split
// form keeps s1 as pairs; the other forms store every stage as T).
// row_table(table): writes the x row-constant table once per call (or nothing).
template <typename T, typename Launch, typename Occ, typename RowTable>
int ens_step(void* plan, const mw_ens_plan_info* info, const double* hyc, const double* hytc, const double* hyi,
             const double* hyti, const double* hypi, T* S, T* Tmp, T* A, int nsteps, int* reverse, unsigned flags,
             int grid_x, int grid_z, cudaStream_t stream, Launch launch, Occ occupancy, const int fmts[3],
             RowTable row_table) {
  MW_REQUIRE(plan && info, MW_ERR_INVALID_ARG, "plan and info must not be NULL");
  MW_REQUIRE(((uintptr_t)plan % 16) == 0, MW_ERR_ALIGN, "plan must be 16-byte aligned");
  MW_REQUIRE(hyc && hytc && hyi && hyti && hypi, MW_ERR_INVALID_ARG, "background buffers must not be NULL");
  MW_REQUIRE(S && Tmp && A, MW_ERR_INVALID_ARG, "state buffers must not be NULL");
  MW_REQUIRE(S != Tmp && S != A && Tmp != A, MW_ERR_ALIAS, "state, state_tmp and scratch must be separate buffers");
  MW_REQUIRE(aligned(S) && aligned(Tmp) && aligned(A), MW_ERR_ALIGN, "state buffers misaligned");
  MW_REQUIRE(reverse != nullptr && nsteps >= 0, MW_ERR_INVALID_ARG, "bad nsteps / reverse");
  MW_REQUIRE(info->z_tile >= 1 && info->z_tile <= kEnsZTileMax, MW_ERR_INVALID_ARG, "plan info: bad z_tile");
  int sms = 0, st;
  if (grid_x <= 0 || grid_z <= 0) {
    if ((st = num_sms(&sms))) return st;
  }
  if (grid_x <= 0) {
    int b = 0;
    if ((st = occupancy(MW_DIR_X, &b))) return st;
    grid_x = std::max(1, b) * sms;
  }
  if (grid_z <= 0) {
    int b = 0;
    if ((st = occupancy(MW_DIR_Z, &b))) return st;
    grid_z = std::max(1, b) * sms;
  }
  EnsStageT<T> es;
  es.members = (const mw_ens_member*)((const char*)plan + info->members_off);
  es.cursor = (EnsCursor*)((char*)plan + ens_cursor_off(*info));
  es.z_tile = info->z_tile;
  es.flags = flags;
  es.hyc = hyc;
  es.hytc = hytc;
  es.hyi = hyi;
  es.hyti = hyti;
  es.hypi = hypi;
  es.stream = stream;
  const int2* xi = (const int2*)((const char*)plan + info->x_items_off);
  const int2* zi = (const int2*)((const char*)plan + info->z_items_off);
  es.xrows = (const char*)plan + info->xrows_off;
  es.mconsts = (const char*)plan + ens_consts_off(*info);
  es.n_xrows = info->n_xrows;
  es.n_members = info->n_members;
  if (nsteps > 0 && (st = row_table((char*)plan + info->xrows_off))) return st;
  for (int n = 0; n < nsteps; ++n) {
    const int dirs[2] = {*reverse ? MW_DIR_X : MW_DIR_Z, *reverse ? MW_DIR_Z : MW_DIR_X};
    for (int d = 0; d < 2; ++d) {
      es.direction = dirs[d];
      es.items = dirs[d] == MW_DIR_X ? xi : zi;
      es.n_items = dirs[d] == MW_DIR_X ? info->n_x_items : info->n_z_items;
      const int grid = dirs[d] == MW_DIR_X ? grid_x : grid_z;
      T* ins[3] = {S, S, S};
      T* frc[3] = {S, A, Tmp};
      T* outs[3] = {A, Tmp, S};
      const int div[3] = {3, 2, 1};
      for (int s = 0; s < 3; ++s) {
        es.init = ins[s];
        es.forcing = frc[s];
        es.out = outs[s];
        es.stage_div = div[s];
        es.fmt = fmts[s];
        if ((st = launch(es, grid))) return st;
      }
    }
    *reverse = *reverse ? 0 : 1;
  }
  return MW_OK;
}

}  // namespace
}  // namespace mw

using namespace mw;

extern "C" int mw_ensemble_plan_info(int n_members, const mw_ens_member* members, int z_tile,
                                     mw_ens_plan_info* info) {
  int st = check_members(n_members, members, z_tile);
  if (st) return st;
  MW_REQUIRE(info != nullptr, MW_ERR_INVALID_ARG, "info must not be NULL");
  return layout(n_members, members, z_tile, info);
}

extern "C" int mw_ensemble_plan(int n_members, const mw_ens_member* members, int z_tile, void* plan_device,
                                size_t plan_bytes, mw_ens_plan_info* info, void* stream) {
  int st = mw_ensemble_plan_info(n_members, members, z_tile, info);
  if (st) return st;
  MW_REQUIRE(plan_device != nullptr, MW_ERR_INVALID_ARG, "plan_device must not be NULL");
  MW_REQUIRE(((uintptr_t)plan_device % 16) == 0, MW_ERR_ALIGN, "plan_device must be 16-byte aligned");
  MW_REQUIRE(plan_bytes >= info->bytes, MW_ERR_WORKSPACE, "plan needs %zu bytes, got %zu", info->bytes, plan_bytes);
  std::vector<unsigned char> host(info->bytes, 0);
  std::memcpy(host.data() + info->members_off, members, sizeof(mw_ens_member) * (size_t)n_members);
  int2* xi = (int2*)(host.data() + info->x_items_off);
  int2* zi = (int2*)(host.data() + info->z_items_off);
  EnsMemberConsts* mc = (EnsMemberConsts*)(host.data() + ens_consts_off(*info));
  for (int e = 0; e < n_members; ++e) {
    const mw_ens_member& m = members[e];
    for (int dir = 0; dir < 2; ++dir) {
      const double d = dir == 0 ? m.dx : m.dz;
      const double hv = -kHvBeta * d / (16 * m.dt);
      for (int k = 0; k < 3; ++k) {
        const double dts = m.dt / (double)(3 - k);  // dt/3, dt/2, dt/1 as evolve forms them
        EnsMemberConsts& c = mc[(e * 2 + dir) * 3 + k];
        const split::dwc hv12 = split::split_host(12.0 * hv), d12 = split::split_host(12.0 * d),
                         gz12 = split::split_host(12.0 * m.dz * kGrav), c12 = split::split_host(dts / (12.0 * d));
        c.hv12[0] = hv12.h, c.hv12[1] = hv12.l;
        c.d12[0] = d12.h, c.d12[1] = d12.l;
        c.gz12[0] = gz12.h, c.gz12[1] = gz12.l;
        c.c12[0] = c12.h, c.c12[1] = c12.l;
        c.c12s = dts / (12.0 * d) * split::kTwoPow896;  // exact: a power-of-two scale
        c.hv_f = (float)hv;
        c.c_f = (float)(dts / d);
        c.dt_f = (float)dts;
        c.pad = 0.0f;
        c.HV = 12.0 * kHvBeta * d / (16 * m.dt);  // as launch_stage_ieee forms them
        c.c = dts / (12.0 * d);
        c.dt = dts;
        c.gdt = -dts * kGrav;
        MW_REQUIRE(std::isfinite(c.c12s), MW_ERR_INVALID_ARG,
                   "member %d: dt / (12 d) = %g is above the split form's range", e, dts / (12.0 * d));
      }
    }
  }
  long long a = 0, b = 0;
  for (int e = 0; e < n_members; ++e) {
    for (int k = 0; k < members[e].nz; ++k) xi[a++] = make_int2(e, k);
    const int ncb = (members[e].nx + kEnsZCols - 1) / kEnsZCols;
    const int ntile = (members[e].nz + z_tile - 1) / z_tile;
    for (int t = 0; t < ntile; ++t)
      for (int cb = 0; cb < ncb; ++cb) zi[b++] = make_int2(e, cb + ncb * t);
  }
  // decreasing cost, stable: an x row costs its length; a z tile its rows (a
  // CTA marches them whatever its used columns), then its used columns
  std::stable_sort(xi, xi + a, [&](int2 p, int2 q) { return members[p.x].nx > members[q.x].nx; });
  auto tile_cost = [&](int2 it) {
    const mw_ens_member& m = members[it.x];
    const int ncb = (m.nx + kEnsZCols - 1) / kEnsZCols;
    const int cb = it.y % ncb, z0 = (it.y / ncb) * z_tile;
    return std::make_pair(std::min(z_tile, m.nz - z0), std::min(kEnsZCols, m.nx - cb * kEnsZCols));
  };
  std::stable_sort(zi, zi + b, [&](int2 p, int2 q) { return tile_cost(p) > tile_cost(q); });
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(plan_device, host.data(), info->bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "plan upload: %s", cudaGetErrorString(e));
  return MW_OK;
}

extern "C" int mw_ensemble_step_f64(void* plan_device, const mw_ens_plan_info* info, const double* hyc,
                                    const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                                    double* state, double* state_tmp, double* scratch, int nsteps, int* reverse,
                                    int f64_mode, unsigned flags, int grid_x, int grid_z, void* stream) {
  MW_REQUIRE(f64_mode == MW_F64_SPLIT || f64_mode == MW_F64_IEEE, MW_ERR_INVALID_ARG,
             "ensembles with FP64 storage run f64_mode MW_F64_IEEE or MW_F64_SPLIT");
  cudaStream_t s = (cudaStream_t)stream;
  if (f64_mode == MW_F64_IEEE) {
    const int fmts[3] = {0, 0, 0};
    return ens_step<double>(plan_device, info, hyc, hytc, hyi, hyti, hypi, state, state_tmp, scratch, nsteps, reverse,
                            flags, grid_x, grid_z, s,
                            [](const EnsStageT<double>& es, int g) { return launch_ens_ieee(es, g); },
                            [](int d, int* b) { return ens_ieee_occupancy(d, b); }, fmts,
                            [&](void* t) { return launch_ens_ieee_rowtable(hyc, hytc, info->n_xrows, t, s); });
  }
  const int fmts[3] = {1, 2, 0};  // s1 kept in scratch as pairs (kToPair, kFromPair, kF64)
  return ens_step<double>(plan_device, info, hyc, hytc, hyi, hyti, hypi, state, state_tmp, scratch, nsteps, reverse,
                          flags, grid_x, grid_z, s,
                          [](const EnsStageT<double>& es, int g) { return launch_ens_split(es, g); },
                          [](int d, int* b) { return ens_split_occupancy(d, b); }, fmts,
                          [&](void* t) { return launch_ens_split_rowtable(hyc, hytc, info->n_xrows, t, s); });
}

extern "C" int mw_ensemble_step_f32(void* plan_device, const mw_ens_plan_info* info, const double* hyc,
                                    const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                                    float* state, float* state_tmp, float* scratch, int nsteps, int* reverse,
                                    unsigned flags, int grid_x, int grid_z, void* stream) {
  const int fmts[3] = {0, 0, 0};
  return ens_step<float>(plan_device, info, hyc, hytc, hyi, hyti, hypi, state, state_tmp, scratch, nsteps, reverse,
                         flags, grid_x, grid_z, (cudaStream_t)stream,
                         [](const EnsStageT<float>& es, int g) { return launch_ens_f32(es, g); },
                         [](int d, int* b) { return ens_f32_occupancy(d, b); }, fmts, [](void*) { return MW_OK; });
}

extern "C" int mw_ensemble_occupancy(int form, int direction, int* blocks_per_sm) {
  MW_REQUIRE(blocks_per_sm != nullptr, MW_ERR_INVALID_ARG, "blocks_per_sm must not be NULL");
  MW_REQUIRE(direction == MW_DIR_X || direction == MW_DIR_Z, MW_ERR_INVALID_ARG, "direction must be 0 or 1");
  MW_REQUIRE(form >= 0 && form <= 2, MW_ERR_INVALID_ARG, "form must be 0 (FP64 split), 1 (FP32) or 2 (IEEE FP64)");
  if (form == 1) return ens_f32_occupancy(direction, blocks_per_sm);
  return form == 2 ? ens_ieee_occupancy(direction, blocks_per_sm) : ens_split_occupancy(direction, blocks_per_sm);
}
