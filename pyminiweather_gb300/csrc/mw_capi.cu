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

