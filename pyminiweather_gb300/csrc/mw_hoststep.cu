// mw_hoststep.cu -- one time step of a state held in host memory: copy in,
// step, copy out, with the copies overlapped with the computation by row
// bands (the end-to-end use of the step by a caller whose arrays live on the
// host).
//
// The step runs band by band as a wavefront three bands deep behind the
// copies in, and each band streams out as soon as its last stage is done, so
// the copies in, the computation and the copies out all overlap.  The x
// direction only couples cells of the same row; a z stage over a band reads
// two rows of each neighbouring band, so it follows the previous stage of the
// band above it.  The z stages run in order on the caller's stream and the x
// stages of each band on a second compute stream, so that the short banded
// launches of the two directions overlap (each fills the other's tail); per-band
// events order the two so that every read sees the same data as in
// mw_step_f64 (the results are identical bit for bit).  The copies run on two
// more side streams, ordered against the computation by events.
#include <algorithm>
#include <mutex>

#include "mw_common.cuh"

namespace mw {

int launch_stage_split(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                       const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                       const double* init, double* forcing, double* out, double dt_stage, int direction,
                       unsigned flags, int r0, int r1, int fmt, cudaStream_t stream);
int launch_stage_ieee(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                      const double* hyi, const double* hyti, const double* hypi, const double* srcw,
                      const double* init, double* forcing, double* out, double dt_stage, int direction,
                      unsigned flags, int r0, int r1, cudaStream_t stream);

namespace {

constexpr int kMaxBands = 64;

struct CopyRes {
  bool ready = false;
  cudaStream_t h2d = nullptr, d2h = nullptr, xs = nullptr;  // copies in, copies out, x stages
  cudaEvent_t start = nullptr, done = nullptr, in[kMaxBands] = {};  // in[b]: band b copied in
  cudaEvent_t xdone[kMaxBands] = {}, zdone[kMaxBands] = {};  // band b's x stages / last z stage issued before
};
CopyRes g_res[64];
std::mutex g_mu;  // held while a call enqueues its work: calls share the streams and events of a device

int resources(CopyRes** r) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(MW_ERR_CUDA, "no usable device");
  CopyRes& c = g_res[dev];
  if (!c.ready) {
    cudaError_t e = cudaStreamCreateWithFlags(&c.h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.d2h, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.xs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.start, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming);
    for (int b = 0; b < kMaxBands && e == cudaSuccess; ++b) {
      e = cudaEventCreateWithFlags(&c.in[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.xdone[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.zdone[b], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return fail(MW_ERR_CUDA, "side streams / events: %s", cudaGetErrorString(e));
    c.ready = true;
  }
  *r = &c;
  return MW_OK;
}

// First interior row of band b.  With ten or more bands the first three and
// the last three are half as tall as the others, so that the copies out start
// sooner and the last copy out ends sooner after the last copy in.
long long band_weight_before(int nb, int b) {
  if (nb < 10) return b;
  const int lo = std::min(b, 3), hi = std::max(0, b - (nb - 3));
  return 2LL * b - lo - hi;
}
int band_start(int nz, int nb, int b) {
  return (int)((long long)nz * band_weight_before(nb, b) / band_weight_before(nb, nb));
}

// The array rows a band moves between host and device: its interior rows, plus
// the wall halo rows for the first and last band.
void band_rows(int nz, int nb, int b, int* r0, int* r1, int* a0, int* a1) {
  *r0 = band_start(nz, nb, b);
  *r1 = band_start(nz, nb, b + 1);
  *a0 = b == 0 ? 0 : *r0 + kHs;
  *a1 = b == nb - 1 ? nz + 2 * kHs : *r1 + kHs;
}

cudaError_t copy_band(double* dst, const double* src, const Geom& g, int a0, int a1, cudaMemcpyKind kind,
                      cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 4 && e == cudaSuccess; ++q) {
    const long long off = q * g.plane + (long long)a0 * g.pitch;
    e = cudaMemcpyAsync(dst + off, src + off, sizeof(double) * (size_t)(a1 - a0) * g.pitch, kind, s);
  }
  return e;
}

}  // namespace
}  // namespace mw

using namespace mw;

namespace mw {
template <typename T>
int check_finite_blocking(int nx, int nz, const T* state, void* counter8, cudaStream_t stream);  // mw_aux.cu
}

extern "C" int mw_step_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                           const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                           const double* src_w, double* state, double* state_tmp, double* scratch, int nsteps,
                           int* reverse, int f64_mode, unsigned flags, void* stream);

extern "C" int mw_step_f64_host(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hyc,
                                const double* hytc, const double* hyi, const double* hyti, const double* hypi,
                                const double* src_w, const double* h_in, double* h_out, double* state,
                                double* state_tmp, double* scratch, int* reverse, int f64_mode, unsigned flags,
                                int nbands, void* stream) {
  // argument checks of the step itself (nothing runs for nsteps = 0)
  int st = mw_step_f64(nx, nz, dx, dz, dt_full, dt, hyc, hytc, hyi, hyti, hypi, src_w, state, state_tmp, scratch, 0,
                       reverse, f64_mode, flags, stream);
  if (st) return st;
  MW_REQUIRE(h_in && h_out, MW_ERR_INVALID_ARG, "host state arrays must not be NULL");
  const Geom g = make_geom(nx, nz);
  const size_t bytes = sizeof(double) * 4 * (size_t)g.plane;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = std::max(1, std::min({nbands, kMaxBands, nz / 16}));
  if ((f64_mode != MW_F64_SPLIT && f64_mode != MW_F64_IEEE) || nb == 1) {  // no bands: copy in, step, copy out
    cudaError_t e = cudaMemcpyAsync(state, h_in, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail(MW_ERR_CUDA, "copy in: %s", cudaGetErrorString(e));
    if ((st = mw_step_f64(nx, nz, dx, dz, dt_full, dt, hyc, hytc, hyi, hyti, hypi, src_w, state, state_tmp, scratch, 1,
                          reverse, f64_mode, flags, stream)))
      return st;
    e = cudaMemcpyAsync(h_out, state, bytes, cudaMemcpyDeviceToHost, s);
    return e == cudaSuccess ? MW_OK : fail(MW_ERR_CUDA, "copy out: %s", cudaGetErrorString(e));
  }
  std::lock_guard<std::mutex> lock(g_mu);
  CopyRes* c = nullptr;
  if ((st = resources(&c))) return st;
  double *S = state, *Tmp = state_tmp, *A = scratch;
  // In the split form the first stage of a direction leaves s1 in the scratch
  // array as double-FP32 pairs (format 1) for the second (format 2), as
  // mw_step_f64 does; the IEEE-FP64 form stores FP64 throughout.
  auto stage = [&](const double* init, double* forcing, double* out, double dts, int dir, int r0, int r1,
                   cudaStream_t on) {
    if (f64_mode == MW_F64_IEEE)
      return launch_stage_ieee(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, init, forcing, out, dts,
                               dir, flags, r0, r1, on);
    const int fmt = out == A ? 1 : (forcing == A ? 2 : 0);
    return launch_stage_split(nx, nz, dx, dz, dt_full, hyc, hytc, hyi, hyti, hypi, src_w, init, forcing, out, dts,
                              dir, flags, r0, r1, fmt, on);
  };
  auto rows_of = [&](int b, int* r0, int* r1) {
    int a0, a1;
    band_rows(nz, nb, b, r0, r1, &a0, &a1);
  };
  auto cuda_ok = [&](cudaError_t ee, const char* what) {
    return ee == cudaSuccess ? MW_OK : fail(MW_ERR_CUDA, "%s: %s", what, cudaGetErrorString(ee));
  };
  // the three x stages of band b on the x stream, after `after` (an event of
  // the stream that last touched the band), then xdone[b]
  auto x_band = [&](int b, cudaEvent_t after) {
    int r0, r1, e;
    rows_of(b, &r0, &r1);
    if ((e = cuda_ok(cudaStreamWaitEvent(c->xs, after, 0), "wait"))) return e;
    if ((e = stage(S, S, A, dt / 3, MW_DIR_X, r0, r1, c->xs))) return e;
    if ((e = stage(S, A, Tmp, dt / 2, MW_DIR_X, r0, r1, c->xs))) return e;
    if ((e = stage(S, Tmp, S, dt, MW_DIR_X, r0, r1, c->xs))) return e;
    return cuda_ok(cudaEventRecord(c->xdone[b], c->xs), "record");
  };
  auto z_band = [&](int k, int b) {  // z stage k (0, 1, 2) over the rows of band b, on the caller's stream
    int r0, r1;
    rows_of(b, &r0, &r1);
    if (k == 0) return stage(S, S, A, dt / 3, MW_DIR_Z, r0, r1, s);
    if (k == 1) return stage(S, A, Tmp, dt / 2, MW_DIR_Z, r0, r1, s);
    const int e = stage(S, Tmp, S, dt, MW_DIR_Z, r0, r1, s);
    return e ? e : cuda_ok(cudaEventRecord(c->zdone[b], s), "record");
  };
  cudaError_t e = cudaEventRecord(c->start, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->h2d, c->start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->xs, c->start, 0);
  for (int b = 0; b < nb && e == cudaSuccess; ++b) {
    int r0, r1, a0, a1;
    band_rows(nz, nb, b, &r0, &r1, &a0, &a1);
    e = copy_band(S, h_in, g, a0, a1, cudaMemcpyHostToDevice, c->h2d);
    if (e == cudaSuccess) e = cudaEventRecord(c->in[b], c->h2d);
  }
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "copy in: %s", cudaGetErrorString(e));
  auto wait_on_main = [&](cudaEvent_t ev) { return cuda_ok(cudaStreamWaitEvent(s, ev, 0), "wait"); };
  // the copy out of band b, behind the event `last` recorded after its last stage
  auto band_out = [&](int b, cudaEvent_t last) {
    int r0, r1, a0, a1;
    band_rows(nz, nb, b, &r0, &r1, &a0, &a1);
    cudaError_t ee = cudaStreamWaitEvent(c->d2h, last, 0);
    if (ee == cudaSuccess) ee = copy_band(h_out, S, g, a0, a1, cudaMemcpyDeviceToHost, c->d2h);
    return ee == cudaSuccess ? MW_OK : fail(MW_ERR_CUDA, "copy out: %s", cudaGetErrorString(ee));
  };
  // A wavefront over the bands, three bands deep.  A z stage over band b reads
  // its forcing two rows into bands b - 1 and b + 1, so it follows the previous
  // z stage (or the copy in, or the x stages) of band b + 1; the x stages of a
  // band touch only that band's rows.  Per band the dependences are:
  //   z then x: z1(b) after the copies in of bands b - 1 .. b + 1; z2(b) after
  //     z1(b - 1 .. b + 1); z3(b) after z2(b - 1 .. b + 1); x(b) after z3(b)
  //     and z3(b + 1), which read the state_tmp / scratch / state rows of band
  //     b that x(b) rewrites; the copy out of b after x(b).
  //   x then z: x(b) after the copy in of b; z1(b) after x(b - 1 .. b + 1);
  //     z2, z3 as above; the copy out of b after z3(b).
  // The z stages are issued in wavefront order on the caller's stream, whose
  // order covers every z-to-z dependence (and the z reads that must precede an
  // x write: z then x, iteration i: z1(i), z2(i-1), z3(i-2), then x(i-3) after
  // zdone[i-2]); the x stages go to the x stream after the event their band
  // needs, and the z stream waits for xdone where a z stage reads x results.
  // An x stage of band b and a z stage running beside it never touch the same
  // rows: the z stages issued after x(b) reach down to band b + 1 at most
  // (z then x), or the x stream runs ahead on bands the z stages reach only
  // after waiting for their xdone (x then z).
  auto wavefront = [&]() -> int {
    for (int i = 0; i < nb + 3; ++i) {
      if (*reverse) {  // x then z: iteration i issues x(i), z1(i-1), z2(i-2), z3(i-3), out(i-3)
        if (i < nb && (st = x_band(i, c->in[i]))) return st;
        if (i >= 1 && i <= nb && (st = wait_on_main(c->xdone[std::min(i, nb - 1)]))) return st;
        for (int k = 0; k < 3; ++k) {
          const int b = i - 1 - k;
          if (b >= 0 && b < nb && (st = z_band(k, b))) return st;
        }
        if (i - 3 >= 0 && i - 3 < nb && (st = band_out(i - 3, c->zdone[i - 3]))) return st;
      } else {  // z then x: iteration i issues z1(i), z2(i-1), z3(i-2), x(i-3), out(i-3)
        for (int k = 0; k < 3; ++k) {
          const int b = i - k;
          if (k == 0 && b < nb && (st = wait_on_main(c->in[std::min(b + 1, nb - 1)]))) return st;
          if (b >= 0 && b < nb && (st = z_band(k, b))) return st;
        }
        const int b = i - 3;
        if (b >= 0 && b < nb) {
          if ((st = x_band(b, c->zdone[std::min(b + 1, nb - 1)]))) return st;
          if ((st = band_out(b, c->xdone[b]))) return st;
        }
      }
    }
    return MW_OK;
  };
  st = wavefront();
  // The caller's stream waits for the x stream and both copy streams, also
  // after an error.
  e = cudaEventRecord(c->done, c->xs);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->done, 0);
  if (e == cudaSuccess) e = cudaEventRecord(c->done, c->d2h);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->done, 0);
  if (e == cudaSuccess) e = cudaEventRecord(c->done, c->h2d);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->done, 0);
  if (st) return st;
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "join: %s", cudaGetErrorString(e));
  *reverse = *reverse ? 0 : 1;
  if (flags & MW_FLAG_CHECK_FINITE) return check_finite_blocking(nx, nz, (const double*)state, scratch, s);
  return MW_OK;
}
