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
