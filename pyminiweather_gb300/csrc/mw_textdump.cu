// mw_textdump.cu -- the text dump of the reference's driver
// (pyminiweather/__main__.py:220-233: np.savetxt(outfile, array.reshape(-1, last_dim),
// delimiter=",")), written by host threads.
//
// np.savetxt with its default fmt writes every value as "%.18e", values joined
// by "," and rows ended by "\n".  Python formats a float with correctly rounded
// decimal conversion and so does the C library's printf, so the bytes agree;
// the exceptions are the special values, which Python spells "nan", "inf" and
// "-inf" whatever the NaN's sign bit.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mw_common.cuh"

namespace mw {
namespace {

// One value as np.savetxt's "%.18e" writes it; returns the characters written.
int format_value(double v, char* out) {
  if (std::isnan(v)) {
    std::memcpy(out, "nan", 3);
    return 3;
  }
  if (std::isinf(v)) {
    if (v < 0) {
      std::memcpy(out, "-inf", 4);
      return 4;
    }
    std::memcpy(out, "inf", 3);
    return 3;
  }
  return std::snprintf(out, 40, "%.18e", v);
}

void format_rows(const double* a, long long r0, long long r1, long long cols, std::string* out) {
  char buf[48];
  out->clear();
  out->reserve((size_t)((r1 - r0) * cols * 26));
  for (long long r = r0; r < r1; ++r) {
    const double* row = a + r * cols;
    for (long long c = 0; c < cols; ++c) {
      const int n = format_value(row[c], buf);
      out->append(buf, n);
      out->push_back(c + 1 < cols ? ',' : '\n');
    }
  }
}

}  // namespace
}  // namespace mw

using namespace mw;

extern "C" int mw_savetxt_f64(const double* values, long long rows, long long cols, const char* path, int append,
                              int threads) {
  MW_REQUIRE(values != nullptr && path != nullptr, MW_ERR_INVALID_ARG, "NULL pointer argument");
  MW_REQUIRE(rows >= 0 && cols >= 1, MW_ERR_SHAPE, "rows must be >= 0 and cols >= 1");
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, values) == cudaSuccess && attr.type == cudaMemoryTypeDevice)
    return fail(MW_ERR_INVALID_ARG, "values must be host memory (copy the array to the host first)");
  cudaGetLastError();  // an unregistered host pointer leaves no error behind
  FILE* fh = std::fopen(path, append ? "ab" : "wb");
  if (!fh) return fail(MW_ERR_INVALID_ARG, "cannot open %s for writing", path);
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  // blocks of rows: nt threads format one block each, the blocks are written in order
  const long long block = std::max<long long>(1, std::min<long long>(4096, (rows + nt - 1) / nt));
  std::vector<std::string> bufs(nt);
  int st = MW_OK;
  for (long long r = 0; r < rows && st == MW_OK; r += block * nt) {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) {
      const long long r0 = std::min(rows, r + t * block), r1 = std::min(rows, r0 + block);
      if (t == 0)
        continue;
      pool.emplace_back(format_rows, values, r0, r1, cols, &bufs[t]);
    }
    format_rows(values, std::min(rows, r), std::min(rows, r + block), cols, &bufs[0]);
    for (auto& th : pool) th.join();
    for (int t = 0; t < nt && st == MW_OK; ++t)
      if (!bufs[t].empty() && std::fwrite(bufs[t].data(), 1, bufs[t].size(), fh) != bufs[t].size())
        st = fail(MW_ERR_INVALID_ARG, "write to %s failed", path);
    for (auto& b : bufs) b.clear();
  }
  if (std::fclose(fh) != 0 && st == MW_OK) st = fail(MW_ERR_INVALID_ARG, "closing %s failed", path);
  return st;
}
