// mw_split_stage_impl.cuh -- body of mw_split_stage.cu, compiled twice: with
// 32-bit element indices (sidx = int, arrays whose four planes span fewer
// than 2^31 elements: no 64-bit address arithmetic) and with 64-bit ones.
// The including file opens the namespace and defines sidx.  No include guard.

namespace {

constexpr int kXThreads = 256;
#ifndef MW_ZSPLIT_MIN_BLOCKS
#define MW_ZSPLIT_MIN_BLOCKS 5  // z CTAs per SM the register allocation must allow (one fewer
                                // for the pair-reading stage, whose march needs more registers)
#endif
constexpr int kZThreads = 128;  // single grid: columns per z CTA (ensemble: mw::kEnsZCols)
constexpr int kZTileMax = 64;  // rows per shared-memory row-constant table
constexpr int kZMinRows = 8;   // single grid: fewest rows per z CTA
// Single-grid x: warps walk 31-cell segments independently (32 interfaces each).
constexpr int kWCells = 31;
constexpr int kWVals = kWCells + 4;  // staged cells x0-2 .. x0+32
constexpr int kXWarps = kXThreads / 32;
constexpr int kXRowsMax = 64;        // rows of one x CTA's range (row-constant table)

struct SplitArgs {
  int nx, nz, pitch;
  sidx plane;  // 32-bit in the instance for arrays of fewer than 2^31 values
  const double* hyc;
  const double* hytc;
  const double* hyi;
  const double* hyti;
  const double* hypi;
  const double* srcw;
  const double* init;
  double* forcing;
  double* out;
  unsigned flags;
  dwc hv12;              // 12 * hv
  double c12s;           // 2^896 dt_stage / (12 d): out = init + c12s * 2^-896 (F(i) - F(i+1))
  dwc d12;               // 12 d (source term: dt * src = c12 * 12 d * src)
  dwc gz12;              // 12 dz grav (z gravity term: dt g rho' = c12 * 12 dz g rho')
  dwc c12;               // dt_stage / (12 d) as a pair (the pair-format update of stage 1)
};

// Storage format of a stage's forcing and output (the RK3 intermediate s1 is
// internal to a step and may be kept as double-FP32 pairs, 8 bytes a value):
//   kF64      forcing, init and out FP64 (the C-ABI stage, stage 3)
//   kToPair   forcing FP64 and equal to init, out as (h, l) pairs (stage 1)
//   kFromPair forcing as (h, l) pairs, init and out FP64 (stage 2)
enum { kF64 = 0, kToPair = 1, kFromPair = 2 };

// A loaded 8-byte value as a pair: FP64 split, or the (h, l) floats themselves.
template <int FMT>
__device__ __forceinline__ dw as_pair(double v) {
  if (FMT == kFromPair) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return {__uint_as_float((unsigned)b), __uint_as_float((unsigned)(b >> 32))};
  }
  return from_f64(v);
}
__device__ __forceinline__ double pair_bits(dw d) {
  return __longlong_as_double((long long)(((unsigned long long)__float_as_uint(d.l) << 32) | __float_as_uint(d.h)));
}

// Forcing value at row k (the wall rule in the halo rows), as loaded: FP64,
// or the bits of an (h, l) pair for kFromPair.
template <int FMT>
__device__ __forceinline__ double zval64(const SplitArgs& a, int q, int k, int col) {
  if (k >= 0 && k < a.nz) return MW_AT(a.forcing, q * (sidx)a.plane + (sidx)(k + kHs) * a.pitch + col, 4 * (long long)a.plane);
  if (q == WMOM) return 0.0;
  const int src = k < 0 ? kHs : a.nz + kHs - 1;
  const double s = MW_AT(a.forcing, q * (sidx)a.plane + (sidx)src * a.pitch + col, 4 * (long long)a.plane);
  if (q == UMOM) {
    if (FMT == kFromPair)
      return pair_bits(mul(as_pair<FMT>(s), from_f64(MW_AT(a.hyc, k + kHs, a.nz + 2 * kHs) / MW_AT(a.hyc, src, a.nz + 2 * kHs))));
    return s / MW_AT(a.hyc, src, a.nz + 2 * kHs) * MW_AT(a.hyc, k + kHs, a.nz + 2 * kHs);
  }
  return s;
}

// Wall halo rows of one column of the forcing array: -2, -1 (bottom) from
// row 0 and nz, nz+1 (top) from row nz-1.
__device__ __forceinline__ void write_z_halo_column(const SplitArgs& a, int col, bool bottom, bool top) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    if (!(h == 0 ? bottom : top)) continue;
    const int r0 = h == 0 ? -2 : a.nz;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double v0 = zval64<kF64>(a, q, r0, col), v1 = zval64<kF64>(a, q, r0 + 1, col);
      MW_AT(a.forcing, q * (sidx)a.plane + (sidx)(r0 + kHs) * a.pitch + col, 4 * (long long)a.plane) = v0;
      MW_AT(a.forcing, q * (sidx)a.plane + (sidx)(r0 + 1 + kHs) * a.pitch + col, 4 * (long long)a.plane) = v1;
    }
  }
}

// out = init + c12 (F(i) - F(i+1)): one FP64 add (merging the pair, scaled by
// 2^-896) and one FP64 FMA per value; c12s = c12 * 2^896 undoes the scale.
__device__ __forceinline__ double update(double init, dw dF, double c12s) { return fma(c12s, to_f64_scaled(dF), init); }

// ---------------------------------------------------------------------------
// Tiles.  Both the single-grid kernels and the persistent ensemble kernels
// call these; every thread of the CTA must call them (they contain barriers).

struct SmemZ {
  RowS row[kZTileMax + 1];
};

// out = init + c12 (F(i) - F(i+1)) for the four variables (paired differences,
// then per value one FP64 add merging the pair and one FP64 FMA).
// One test per cell for non-finite increments: h - h is 0 for finite h and
// NaN otherwise; only then are the four values merged with the per-value check.
// kToPair: out = init + c12 (F(i) - F(i+1)) in pair arithmetic from the
// init pairs ip (the forcing's own pairs), stored as (h, l) floats.
template <int FMT>
__device__ __forceinline__ void store_update(const SplitArgs& a, sidx o, const double iv[4], const dw2 ip[2],
                                             dw2 dF[2]) {
  if (FMT == kToPair) {
    const dw c = ld(a.c12);
    const dw2 cv = splat(c);
    const float2 cn = f2splat(-c.h);
    float2* out = reinterpret_cast<float2*>(a.out);
#pragma unroll
    for (int pr = 0; pr < 2; ++pr) {
      const dw2 r = add2(ip[pr], mul2n(dF[pr], cv, cn));
      MW_AT(out, (2 * pr) * a.plane + o, 4 * (long long)a.plane) = make_float2(r.h.x, r.l.x);
      MW_AT(out, (2 * pr + 1) * a.plane + o, 4 * (long long)a.plane) = make_float2(r.h.y, r.l.y);
    }
    return;
  }
  const dw d[4] = {lo_of(dF[0]), hi_of(dF[0]), lo_of(dF[1]), hi_of(dF[1])};
  const float2 z = f2add(f2sub(dF[0].h, dF[0].h), f2sub(dF[1].h, dF[1].h));
  double v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = fma(a.c12s, to_f64_scaled_finite(d[q]), iv[q]);
  if (!(z.x + z.y == 0.0f)) {
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = update(iv[q], d[q], a.c12s);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) MW_AT(a.out, q * a.plane + o, 4 * (long long)a.plane) = v[q];
}

// x, single grid: the CTA owns the contiguous range [g0, g1) of the row-major
// list of 31-cell segments (nseg per row) and splits it evenly over its eight
// warps.  Each warp walks its segments with no CTA barrier: lane l stages cell
// x0-2+l (lanes 0..2 also x0+30+l) in its own shared-memory slice, evaluates
// the flux at interface x0+l, and lanes 0..30 update cells x0..x0+30 from the
// fluxes of their own and the next lane's interface.  The next segment's
// values are loaded one segment ahead.  The row constants (an FP64 pow per
// row) are formed once per CTA for all rows of its range.
struct SmemXW {
  dw2 sS[kXWarps][2][kWVals + 1];  // [warp][pair][staged cell]
  dw2 sF[kXWarps][2][32];          // [warp][pair][interface]
  RowS row[kXRowsMax];
};

__device__ __forceinline__ RowS x_row_consts(const SplitArgs& a, int k) {
  const double hrt = MW_AT(a.hytc, k + kHs, a.nz + 2 * kHs);
  return row_consts(MW_AT(a.hyc, k + kHs, a.nz + 2 * kHs), hrt, kC0 * pow(hrt, kGamma));
}

// row_at(k): the row constants of row k.  prologue() runs once, after the
// first segment's loads are issued (so that their latency overlaps it), also
// when the range is empty (it may contain a CTA barrier).
template <int FMT, typename RowAt, typename Prologue>
__device__ __forceinline__ void x_warp_segments(const SplitArgs& a, int nseg, long long g0, long long g1,
                                                RowAt row_at, bool halo, SmemXW& sm, Prologue prologue) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (g0 >= g1) {
    prologue();
    return;
  }
  const Hv2 hv = make_hv2(ld(a.hv12));
  const dw d12 = ld(a.d12);
  int k = (int)(g0 / nseg), sg = (int)(g0 - (long long)k * nseg);
  // The three cells beyond the 32 lanes' (x0+30 .. x0+32) are spread over
  // lanes 0..11, one value each (variable lane & 3 of cell x0+30+(lane>>2)),
  // so their conversion costs the warp one value's instructions, not four.
  const int xq = lane & 3, xj = lane >> 2;
  auto load = [&](int kk, int x0, double v0[4], double& v1) {
    const sidx row = (sidx)(kk + kHs) * a.pitch;
    const int c0 = x0 - 2 + lane, c1 = x0 + 30 + xj;
    if (c0 <= a.nx + 1) {
      const sidx col = wrap_x(c0, a.nx) + kHs;
#pragma unroll
      for (int q = 0; q < 4; ++q) v0[q] = __ldg(&MW_AT(a.forcing, q * a.plane + row + col, 4 * (long long)a.plane));
    }
    if (lane < 12 && c1 <= a.nx + 1) v1 = __ldg(&MW_AT(a.forcing, xq * a.plane + row + wrap_x(c1, a.nx) + kHs, 4 * (long long)a.plane));
  };
  double v0[4] = {0, 0, 0, 0}, v1 = 0.0;
  load(k, sg * kWCells, v0, v1);
  prologue();
  for (long long g = g0; g < g1; ++g) {
    const int x0 = sg * kWCells;
    const sidx row = (sidx)(k + kHs) * a.pitch;
    {
      const dw2 p0 = pack(as_pair<FMT>(v0[DENS]), as_pair<FMT>(v0[UMOM]));
      const dw2 p1 = pack(as_pair<FMT>(v0[WMOM]), as_pair<FMT>(v0[RHOT]));
      sm.sS[w][0][lane] = p0;
      sm.sS[w][1][lane] = p1;
      if (lane < 12) {
        const dw d = as_pair<FMT>(v1);
        float* e = reinterpret_cast<float*>(&sm.sS[w][xq >> 1][32 + xj]);  // h.x, h.y, l.x, l.y
        e[xq & 1] = d.h;
        e[2 + (xq & 1)] = d.l;
      }
    }
    if (FMT != kFromPair && halo && sg == 0 && lane < 4) {  // columns 0, 1 <- nx, nx+1; nx+2, nx+3 <- 2, 3
      const int dst = lane < 2 ? lane : a.nx + lane, src = lane < 2 ? a.nx + lane : lane;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        MW_AT(a.forcing, q * a.plane + row + dst, 4 * (long long)a.plane) = MW_AT(a.forcing, q * a.plane + row + src, 4 * (long long)a.plane);
    }
    const int kc = k;
    const int i = x0 + lane;
    const bool upd = lane < kWCells && i < a.nx;
    const sidx o = row + i + kHs;
    if (++sg == nseg) {
      sg = 0;
      ++k;
    }
    const bool more = g + 1 < g1;
    if (more) load(k, sg * kWCells, v0, v1);
    double iv[4];
    if (FMT != kToPair && upd) {
#pragma unroll
      for (int q = 0; q < 4; ++q) iv[q] = MW_AT(a.init, q * a.plane + o, 4 * (long long)a.plane);
    }
    __syncwarp();
    if (i <= a.nx) {
      dw2 s[2][4];
#pragma unroll
      for (int pr = 0; pr < 2; ++pr)
#pragma unroll
        for (int j = 0; j < 4; ++j) s[pr][j] = sm.sS[w][pr][lane + j];
      dw2 F[2];
      flux_x2(s, row_at(kc), hv, F);
      sm.sF[w][0][lane] = F[0];
      sm.sF[w][1][lane] = F[1];
    }
    __syncwarp();
    if (upd) {
      dw2 dF[2] = {sub2(sm.sF[w][0][lane], sm.sF[w][0][lane + 1]), sub2(sm.sF[w][1][lane], sm.sF[w][1][lane + 1])};
      if (a.srcw) {
        const dw ws = add(lo_of(dF[1]), mul(from_f64(MW_AT(a.srcw, (sidx)kc * a.nx + i, (long long)a.nx * a.nz)), d12));
        dF[1].h.x = ws.h;
        dF[1].l.x = ws.l;
      }
      dw2 ip[2];
      if (FMT == kToPair) {  // init is the forcing: its staged pairs at cell x0+lane
        ip[0] = sm.sS[w][0][lane + 2];
        ip[1] = sm.sS[w][1][lane + 2];
      }
      store_update<FMT>(a, o, iv, ip, dF);
    }
    __syncwarp();
  }
}

// z: columns [cb*NT, cb*NT+NT) (the NT threads of the CTA), rows [kbeg, kend), kend - kbeg <=
// kZTileMax: one thread per column marching the rows with a rolling window of
// variable pairs; the next row and the init values are loaded one step ahead;
// the interface row constants are tabled in shared memory.  hbot / htop:
// write the bottom / top wall halo rows of these columns of the forcing array
// (cb == 0 also does the four x-halo columns).
template <int FMT, int NT = kZThreads>
__device__ __forceinline__ void z_march(const SplitArgs& a, int cb, int kbeg, int kend, bool hbot, bool htop,
                                        SmemZ& sm) {
  if (FMT == kFromPair) hbot = htop = false;  // the pair-format forcing (internal scratch) keeps no halo
  __syncthreads();  // the previous table is no longer read
  for (int r = threadIdx.x; r <= kend - kbeg; r += NT) {
    const int k = kbeg + r;
    sm.row[r] = row_consts(MW_AT(a.hyi, k, a.nz + 1), MW_AT(a.hyti, k, a.nz + 1), MW_AT(a.hypi, k, a.nz + 1));
  }
  __syncthreads();
  const int c = cb * NT + threadIdx.x;
  if ((hbot || htop) && cb == 0 && threadIdx.x < 4)
    write_z_halo_column(a, threadIdx.x < 2 ? threadIdx.x : a.nx + threadIdx.x, hbot, htop);
  if (c >= a.nx) return;
  const int col = c + kHs;
  if (hbot || htop) write_z_halo_column(a, col, hbot, htop);
  const Hv2 hv = make_hv2(ld(a.hv12));
  const dw d12 = ld(a.d12), gz12 = ld(a.gz12);
  dw2 w[2][4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = zval64<FMT>(a, q, kbeg - 2 + j, col);
    w[0][j] = pack(as_pair<FMT>(v[DENS]), as_pair<FMT>(v[UMOM]));
    w[1][j] = pack(as_pair<FMT>(v[WMOM]), as_pair<FMT>(v[RHOT]));
  }
  double nxt[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) nxt[q] = zval64<FMT>(a, q, kbeg + 2, col);
  dw2 Fp[2];
  flux_z2(w, sm.row[0], hv, kbeg == 0, Fp);
  for (int k = kbeg; k < kend; ++k) {
    const sidx o = (sidx)(k + kHs) * a.pitch + col;
    double iv[4];
    if (FMT != kToPair) {
#pragma unroll
      for (int q = 0; q < 4; ++q) iv[q] = MW_AT(a.init, q * a.plane + o, 4 * (long long)a.plane);
    }
    double cur[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) cur[q] = nxt[q];
    if (k + 1 < kend) {
#pragma unroll
      for (int q = 0; q < 4; ++q) nxt[q] = zval64<FMT>(a, q, k + 3, col);
    }
    const dw rho_k = lo_of(w[0][2]);
    const dw2 ip[2] = {w[0][2], w[1][2]};  // kToPair: init is the forcing at row k
#pragma unroll
    for (int pr = 0; pr < 2; ++pr) {
      w[pr][0] = w[pr][1];
      w[pr][1] = w[pr][2];
      w[pr][2] = w[pr][3];
    }
    w[0][3] = pack(as_pair<FMT>(cur[DENS]), as_pair<FMT>(cur[UMOM]));
    w[1][3] = pack(as_pair<FMT>(cur[WMOM]), as_pair<FMT>(cur[RHOT]));
    dw2 Fn[2];
    flux_z2(w, sm.row[k + 1 - kbeg], hv, k + 1 == a.nz, Fn);
    dw2 dF[2] = {sub2(Fp[0], Fn[0]), sub2(Fp[1], Fn[1])};
    dw dw_w = sub(lo_of(dF[1]), mul(rho_k, gz12));
    if (a.srcw) dw_w = add(dw_w, mul(from_f64(MW_AT(a.srcw, (sidx)k * a.nx + c, (long long)a.nx * a.nz)), d12));
    dF[1].h.x = dw_w.h;
    dF[1].l.x = dw_w.l;
    store_update<FMT>(a, o, iv, ip, dF);
    Fp[0] = Fn[0];
    Fp[1] = Fn[1];
  }
}

// ---------------------------------------------------------------------------
// Single grid: x CTA (blockIdx.x, row) walks a run of chunks; z CTA is one tile.
#ifndef MW_XSPLIT_SEGS_PER_WARP
#define MW_XSPLIT_SEGS_PER_WARP 48  // segments per warp (0: one resident wave of CTAs)
#endif
#ifndef MW_XSPLIT_MIN_BLOCKS
#define MW_XSPLIT_MIN_BLOCKS 3
#endif
#ifndef MW_XSPLIT_WHOLE_WAVES
#define MW_XSPLIT_WHOLE_WAVES 1  // round the grid up to a whole number of resident waves
#endif
// Segments [gbase, gbase + total) (rows gbase / nseg onwards).
template <int FMT>
__global__ void __launch_bounds__(kXThreads, MW_XSPLIT_MIN_BLOCKS) k_stage_x_split(SplitArgs a, int nseg, long long total,
                                                                                   long long gbase) {
  __shared__ SmemXW sm;
  const long long g0 = gbase + total * blockIdx.x / gridDim.x, g1 = gbase + total * (blockIdx.x + 1) / gridDim.x;
  if (g0 >= g1) return;
  const int row0 = (int)(g0 / nseg), nrows = (int)((g1 - 1) / nseg) - row0 + 1;  // nrows <= kXRowsMax (host)
  const int w = threadIdx.x >> 5;
  const long long n = g1 - g0;
  // the row-constant table (an FP64 pow per row) is formed while the warps'
  // first loads are in flight
  x_warp_segments<FMT>(a, nseg, g0 + n * w / kXWarps, g0 + n * (w + 1) / kXWarps,
                       [&](int k) { return sm.row[k - row0]; }, a.flags & MW_FLAG_WRITE_HALO, sm, [&]() {
                         for (int r = threadIdx.x; r < nrows; r += kXThreads) sm.row[r] = x_row_consts(a, row0 + r);
                         __syncthreads();
                       });
}

// z, single grid: the CTA owns the contiguous range [u0, u1) of the
// column-block-major list of (column block, row) units, at most kZTileMax
// units, so it marches one or two column-block pieces.  The launch sizes the
// grid to a whole number of resident waves of equal ranges.
// Rows [r0, r1) of every column block.
template <int FMT>
__global__ void __launch_bounds__(kZThreads, FMT == kFromPair ? MW_ZSPLIT_MIN_BLOCKS - 1 : MW_ZSPLIT_MIN_BLOCKS)
    k_stage_z_split(SplitArgs a, int ncb, int r0, int r1) {
  __shared__ SmemZ sm;
  const int rows = r1 - r0;
  const long long U = (long long)ncb * rows;
  long long u = U * blockIdx.x / gridDim.x;
  const long long u1 = U * (blockIdx.x + 1) / gridDim.x;
  const bool halo = a.flags & MW_FLAG_WRITE_HALO;
  while (u < u1) {
    const int cb = (int)(u / rows), k0 = r0 + (int)(u - (long long)cb * rows);
    const int kend = (int)std::min<long long>(r1, k0 + (u1 - u));
    z_march<FMT>(a, cb, k0, kend, halo && k0 == 0, halo && kend == a.nz, sm);
    u += kend - k0;
  }
}

// ---------------------------------------------------------------------------
// Ensemble: one persistent launch per stage walks a work list over all
// members (x: one item per member row; z: one item per member column-tile).
__device__ SplitArgs member_args(const EnsStage& es, int e) {
  const mw_ens_member m = MW_AT(es.members, e, es.n_members);
  SplitArgs a;
  a.nx = m.nx;
  a.nz = m.nz;
  a.pitch = m.nx + 2 * kHs;
  a.plane = (sidx)(m.nz + 2 * kHs) * a.pitch;
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
  // stage constants from the plan (formed on the host, no FP64 work per item)
  const EnsMemberConsts& c = MW_AT(reinterpret_cast<const EnsMemberConsts*>(es.mconsts), mconsts_index(es, e),
                                   (long long)kEnsConstsPerMember * es.n_members);
  a.hv12 = {c.hv12[0], c.hv12[1]};
  a.c12s = c.c12s;
  a.d12 = {c.d12[0], c.d12[1]};
  a.gz12 = {c.gz12[0], c.gz12[1]};
  a.c12 = {c.c12[0], c.c12[1]};
  return a;
}

// x items are rows (member, row), one per warp: the warp walks the row's
// 31-cell segments as the single-grid kernel does, with the row constants read
// from the plan's table (written once per step call, no FP64 pow per row).
template <int FMT>
__global__ void __launch_bounds__(kXThreads, MW_XSPLIT_MIN_BLOCKS) k_ens_x_split(EnsStage es) {
  __shared__ SmemXW sm;
  for (unsigned it = ens_take_warp(es.cursor); it < (unsigned)es.n_items; it = ens_take_warp(es.cursor)) {
    const int2 item = MW_AT(es.items, it, es.n_items);  // (member, row)
    const SplitArgs a = member_args(es, item.x);
    const int nseg = (a.nx + kWCells - 1) / kWCells;
    const RowS r = MW_AT(reinterpret_cast<const RowS*>(es.xrows), MW_AT(es.members, item.x, es.n_members).cell_off + item.y + kHs,
                         es.n_xrows);
    x_warp_segments<FMT>(a, nseg, (long long)item.y * nseg, (long long)(item.y + 1) * nseg,
                    [&](int) { return r; }, a.flags & MW_FLAG_WRITE_HALO, sm, []() {});
  }
  ens_finish(es.cursor);
}

template <int FMT>
__global__ void __launch_bounds__(kEnsZCols,
                                  (kZThreads / kEnsZCols) * (FMT == kFromPair ? MW_ZSPLIT_MIN_BLOCKS - 1 : MW_ZSPLIT_MIN_BLOCKS))
    k_ens_z_split(EnsStage es) {
  __shared__ SmemZ sm;
  __shared__ unsigned slot[2];
  int parity = 0;
  for (unsigned it = ens_take_cta(es.cursor, slot, parity); it < (unsigned)es.n_items;
       it = ens_take_cta(es.cursor, slot, parity)) {
    const int2 item = MW_AT(es.items, it, es.n_items);  // (member, column block + ncb * tile)
    const SplitArgs a = member_args(es, item.x);
    const int ncb = (a.nx + kEnsZCols - 1) / kEnsZCols;
    const int cb = item.y % ncb, tile = item.y / ncb;
    const int k0 = tile * es.z_tile, kend = min(k0 + es.z_tile, a.nz);
    const bool halo = a.flags & MW_FLAG_WRITE_HALO;
    z_march<FMT, kEnsZCols>(a, cb, k0, kend, halo && k0 == 0, halo && kend == a.nz, sm);
  }
  ens_finish(es.cursor);
}

}  // namespace

// Resident CTAs per SM of the ensemble z kernel of format FMT, cached per device.
template <int FMT>
int ens_z_per_sm() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_ens_z_split<FMT>, kEnsZCols, 0) != cudaSuccess || v < 1) v = 1;
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

int launch_ens_split(const EnsStage& es, int grid) {
  if (es.n_items == 0) return MW_OK;
  MW_REQUIRE(es.fmt == kF64 || es.fmt == kToPair || es.fmt == kFromPair, MW_ERR_INVALID_ARG, "bad stage format");
  // The grid is sized for the FP64-storage z kernel; the pair-reading one fits
  // fewer CTAs per SM, so its persistent grid shrinks in proportion (one wave of
  // resident CTAs: a CTA beyond it would start only as the list runs out).
  if (es.direction == MW_DIR_Z && es.fmt == kFromPair) {
    const int b0 = ens_z_per_sm<kF64>(), b1 = ens_z_per_sm<kFromPair>();
    if (b1 < b0) grid = std::max(1, (int)((long long)grid * b1 / b0));
  }
  if (es.direction == MW_DIR_X) {
    if (es.fmt == kToPair)
      k_ens_x_split<kToPair><<<grid, kXThreads, 0, es.stream>>>(es);
    else if (es.fmt == kFromPair)
      k_ens_x_split<kFromPair><<<grid, kXThreads, 0, es.stream>>>(es);
    else
      k_ens_x_split<kF64><<<grid, kXThreads, 0, es.stream>>>(es);
  } else {
    if (es.fmt == kToPair)
      k_ens_z_split<kToPair><<<grid, kEnsZCols, 0, es.stream>>>(es);
    else if (es.fmt == kFromPair)
      k_ens_z_split<kFromPair><<<grid, kEnsZCols, 0, es.stream>>>(es);
    else
      k_ens_z_split<kF64><<<grid, kEnsZCols, 0, es.stream>>>(es);
  }
  return check_launch("ensemble split stage launch");
}

int ens_split_occupancy(int direction, int* blocks_per_sm) {
  cudaError_t e = direction == MW_DIR_X
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_ens_x_split<kF64>, kXThreads, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_ens_z_split<kF64>, kEnsZCols, 0);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  return MW_OK;
}

// CTAs of k_stage_x_split (which 0) / k_stage_z_split (which 1) of format fmt
// resident on the current device, cached per device.
template <int FMT>
int resident_ctas(int which, int* out) {
  static std::atomic<int> cache[2][64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(MW_ERR_CUDA, "cudaGetDevice failed");
  const bool cached = dev >= 0 && dev < 64;
  if (cached && (*out = cache[which][dev].load(std::memory_order_relaxed)) > 0) return MW_OK;
  int per_sm = 0, sms = 0;
  cudaError_t e = which == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_x_split<FMT>, kXThreads, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_z_split<FMT>, kZThreads, 0);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  *out = std::max(1, per_sm) * sms;
  if (cached) cache[which][dev].store(*out, std::memory_order_relaxed);
  return MW_OK;
}

template <int FMT>
int launch_stage_split_fmt(int nx, int nz, double dx, double dz, double dt_full, const double* hyc,
                           const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                           const double* srcw, const double* init, double* forcing, double* out, double dt_stage,
                           int direction, unsigned flags, int r0, int r1, cudaStream_t stream) {
  const Geom g = make_geom(nx, nz);
  MW_REQUIRE(0 <= r0 && r0 < r1 && r1 <= nz, MW_ERR_INVALID_ARG, "row range [%d, %d) outside [0, %d)", r0, r1, nz);
  const int rows = r1 - r0;
  SplitArgs a;
  a.nx = nx;
  a.nz = nz;
  a.pitch = g.pitch;
  a.plane = (sidx)g.plane;
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
  const double d = direction == MW_DIR_X ? dx : dz;
  const double hv = -kHvBeta * d / (16 * dt_full);
  a.hv12 = split_host(12.0 * hv);
  a.c12s = dt_stage / (12.0 * d) * kTwoPow896;  // exact: a power-of-two scale
  MW_REQUIRE(std::isfinite(a.c12s), MW_ERR_INVALID_ARG,
             "dt_stage / (12 d) = %g is above the split form's range (use the native FP64 mode)", dt_stage / (12.0 * d));
  a.d12 = split_host(12.0 * d);
  a.gz12 = split_host(12.0 * dz * kGrav);
  a.c12 = split_host(dt_stage / (12.0 * d));
  if (direction == MW_DIR_X) {
    const int nseg = (nx + kWCells - 1) / kWCells;
    const long long total = (long long)nseg * rows;
    int resident = 0, st = resident_ctas<FMT>(0, &resident);
    if (st) return st;
    // One resident wave (at least one segment per warp) for small grids;
    // about MW_XSPLIT_SEGS_PER_WARP segments per warp for large ones, in a
    // whole number of resident waves of equal ranges, so that the block
    // scheduler evens out the warps' speeds; at most kXRowsMax rows per CTA
    // range.
    long long grid = std::min<long long>(resident, (total + kXWarps - 1) / kXWarps);
    if (MW_XSPLIT_SEGS_PER_WARP > 0) grid = std::max<long long>(grid, total / (kXWarps * MW_XSPLIT_SEGS_PER_WARP));
#if MW_XSPLIT_WHOLE_WAVES
    if (grid > resident) grid = (grid + resident - 1) / resident * resident;  // a whole number of waves
#endif
    grid = std::max<long long>(grid, (rows + kXRowsMax - 3) / (kXRowsMax - 2));
    MW_REQUIRE(grid <= 0x7fffffffLL, MW_ERR_SHAPE, "grid too large for the x direction-stage launch");
    k_stage_x_split<FMT><<<(unsigned)grid, kXThreads, 0, stream>>>(a, nseg, total, (long long)r0 * nseg);
  } else {
    const int ncb = (nx + kZThreads - 1) / kZThreads;
    const long long units = (long long)ncb * rows;
    int resident = 0, st = resident_ctas<FMT>(1, &resident);
    if (st) return st;
    long long grid = resident * ((units + (long long)kZTileMax * resident - 1) / ((long long)kZTileMax * resident));
    grid = std::max<long long>(1, std::min<long long>(grid, units / kZMinRows));
    MW_REQUIRE(grid <= 0x7fffffffLL, MW_ERR_SHAPE, "grid too large for the z direction-stage launch");
    k_stage_z_split<FMT><<<(unsigned)grid, kZThreads, 0, stream>>>(a, ncb, r0, r1);
  }
  return check_launch(direction == MW_DIR_X ? "x split direction-stage launch" : "z split direction-stage launch");
}

// fmt: kF64, kToPair (forcing == init, out as pairs) or kFromPair (forcing as pairs).
int launch_stage_split(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                       const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                       const double* init, double* forcing, double* out, double dt_stage, int direction,
                       unsigned flags, int r0, int r1, int fmt, cudaStream_t stream) {
  MW_REQUIRE(fmt == kF64 || fmt == kToPair || fmt == kFromPair, MW_ERR_INVALID_ARG, "bad stage format %d", fmt);
  MW_REQUIRE(fmt != kToPair || init == forcing, MW_ERR_INVALID_ARG, "the pair-output stage needs init == forcing");
  auto fn = fmt == kToPair ? launch_stage_split_fmt<kToPair>
                           : (fmt == kFromPair ? launch_stage_split_fmt<kFromPair> : launch_stage_split_fmt<kF64>);
  return fn(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, srcw, init, forcing, out, dt_stage, direction, flags,
            r0, r1, stream);
}

