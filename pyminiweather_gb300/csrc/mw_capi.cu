// mw_capi.cu -- error reporting of the C ABI.
#include "mw_common.cuh"

namespace mw {

static thread_local char g_last_error[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return MW_OK;
}

int check_grid(int nx, int nz) {
  if (nx < 2 || nz < 1)
    return fail(MW_ERR_SHAPE, "grid %d x %d: need nx >= 2 (periodic halo of width 2) and nz >= 1", nx, nz);
  long long cells = (long long)(nx + 2 * kHs) * (nz + 2 * kHs);
  if (cells * 4 >= (1LL << 40)) return fail(MW_ERR_SHAPE, "grid %d x %d too large", nx, nz);
  return MW_OK;
}

}  // namespace mw

extern "C" const char* mw_last_error(void) { return mw::g_last_error; }

extern "C" const char* mw_status_string(int status) {
  switch (status) {
    case MW_OK: return "ok";
    case MW_ERR_INVALID_ARG: return "invalid argument";
    case MW_ERR_SHAPE: return "unsupported grid shape";
    case MW_ERR_ALIGN: return "misaligned pointer";
    case MW_ERR_ALIAS: return "output overlaps an input";
    case MW_ERR_CUDA: return "CUDA error";
    case MW_ERR_WORKSPACE: return "workspace too small";
    case MW_ERR_NONFINITE: return "non-finite value";
    default: return "unknown status";
  }
}

extern "C" int mw_abi_version(void) { return MW_ABI_VERSION; }

// ---------------------------------------------------------------------------
// Bounds-checked build: out-of-range index count of the checked kernels.
#if MW_CHECK
namespace mw {
int oob_count_split_stage(unsigned long long* out, bool reset);
int oob_count_adjoint_split(unsigned long long* out, bool reset);
int oob_count_ieee_stage(unsigned long long* out, bool reset);
int oob_count_dirstage(unsigned long long* out, bool reset);
int oob_count_aux(unsigned long long* out, bool reset);
int oob_count_adjoint(unsigned long long* out, bool reset);
namespace {
__global__ void k_oob_selftest(double* p, int n) { MW_AT(p, n, n) = 1.0; }  // one index past the end
}  // namespace
MW_OOB_COUNTER(oob_count_capi)
}  // namespace mw
#endif

extern "C" int mw_debug_oob_count(unsigned long long* count, int reset) {
  MW_REQUIRE(count != nullptr, MW_ERR_INVALID_ARG, "count must not be NULL");
  *count = 0;
#if MW_CHECK
  int st;
  if ((st = mw::oob_count_split_stage(count, reset != 0)) || (st = mw::oob_count_adjoint_split(count, reset != 0)) ||
      (st = mw::oob_count_ieee_stage(count, reset != 0)) || (st = mw::oob_count_dirstage(count, reset != 0)) ||
      (st = mw::oob_count_aux(count, reset != 0)) || (st = mw::oob_count_adjoint(count, reset != 0)) ||
      (st = mw::oob_count_capi(count, reset != 0)))
    return st;
  return MW_OK;
#else
  (void)reset;
  return mw::fail(MW_ERR_INVALID_ARG, "not a bounds-checked build (build with MW_CHECK=1)");
#endif
}

extern "C" int mw_debug_oob_selftest(void* stream) {
#if MW_CHECK
  mw::k_oob_selftest<<<1, 1, 0, (cudaStream_t)stream>>>(nullptr, 4);  // the access goes to the sink
  return mw::check_launch("oob self-test launch");
#else
  (void)stream;
  return mw::fail(MW_ERR_INVALID_ARG, "not a bounds-checked build (build with MW_CHECK=1)");
#endif
}


// ---------------------------------------------------------------------------
// FP64 pipe throughput: the denominator of the FP64-pipe roofline, measured on
// the device at hand.  Every thread runs 8 independent chains of FP64 FMAs
// (a <- a m + p), so each warp always has an FP64 instruction ready.
namespace mw {
namespace {
constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 8;
constexpr int kProbeUnroll = 16;
__device__ double g_probe_sink;
__global__ void __launch_bounds__(kProbeThreads) k_fp64_throughput(int iters) {
  double a[kProbeChains];
#pragma unroll
  for (int c = 0; c < kProbeChains; ++c) a[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  const double m = 0.999999, p = 1e-9;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int r = 0; r < kProbeUnroll; ++r)
#pragma unroll
      for (int c = 0; c < kProbeChains; ++c) a[c] = fma(a[c], m, p);
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kProbeChains; ++c) s += a[c];
  if (s == -1.0) g_probe_sink = s;  // never true (s > 0): keeps the chains live without a store per thread
}
}  // namespace
}  // namespace mw

extern "C" int mw_fp64_throughput(int blocks_per_sm, int iters, double* ops_per_second, void* stream) {
  using namespace mw;
  MW_REQUIRE(ops_per_second != nullptr, MW_ERR_INVALID_ARG, "ops_per_second must not be NULL");
  MW_REQUIRE(blocks_per_sm >= 1 && blocks_per_sm <= 8, MW_ERR_INVALID_ARG, "blocks_per_sm must be in [1, 8]");
  MW_REQUIRE(iters >= 1 && iters <= (1 << 16), MW_ERR_INVALID_ARG, "iters must be in [1, 65536]");
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "device query: %s", cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = blocks_per_sm * sms;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    k_fp64_throughput<<<blocks, kProbeThreads, 0, s>>>(iters / 8 + 1);  // warm-up
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e0, s);
  if (e == cudaSuccess) {
    k_fp64_throughput<<<blocks, kProbeThreads, 0, s>>>(iters);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail(MW_ERR_CUDA, "FP64 throughput probe: %s", cudaGetErrorString(e));
  const double ops = (double)blocks * kProbeThreads * (double)iters * kProbeUnroll * kProbeChains;
  *ops_per_second = ms > 0.0f ? ops / (ms * 1e-3) : 0.0;
  return MW_OK;
}
