// The reference's text matrix format (src/common/common.cpp:84-178): SaveMatrix writes each
// row as its values each followed by one space, then a newline; LoadMatrix reads every run
// of decimal digits as one value, in order, whatever separates them.
#include <cmath>
#include <cstdio>
#include <string>

#include "rt_internal.h"

using namespace rt;

extern "C" {

RT_API rt_status rt_save_matrix(const int32_t* a, int64_t rows, int64_t cols, const char* path) {
  clear_error();
  if (!a || !path || rows < 0 || cols < 0) return fail(RT_ERR_INVALID_ARGUMENT, "save_matrix: bad arguments");
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(RT_ERR_INVALID_ARGUMENT, std::string("save_matrix: cannot open ") + path);
  for (int64_t i = 0; i < rows; ++i) {
    for (int64_t j = 0; j < cols; ++j) std::fprintf(f, "%d ", (int)a[i * cols + j]);
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  return ok ? RT_OK : fail(RT_ERR_INVALID_ARGUMENT, std::string("save_matrix: write failed: ") + path);
}

// SaveMatrix(const std::vector<int>&, filename) (:84-86): the square overload, which writes
// floor(sqrt(size)) rows of floor(sqrt(size)) values.
RT_API rt_status rt_save_matrix_square(const int32_t* a, int64_t size, const char* path) {
  const int64_t s = (int64_t)std::floor(std::sqrt((double)size));
  return rt_save_matrix(a, s, s, path);
}

// LoadMatrix(filename) (:155-178): digits only (a '-' is skipped like any separator, as in
// the reference).  Writes at most cap values; *count receives the number found.
RT_API rt_status rt_load_matrix(const char* path, int32_t* out, int64_t cap, int64_t* count) {
  clear_error();
  if (!path || !count) return fail(RT_ERR_INVALID_ARGUMENT, "load_matrix: bad arguments");
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(RT_ERR_INVALID_ARGUMENT, std::string("load_matrix: cannot open ") + path);
  int64_t n = 0;
  int c = std::fgetc(f);
  while (c != EOF) {
    if (c >= '0' && c <= '9') {
      int64_t v = c - '0';
      while ((c = std::fgetc(f)) != EOF && c >= '0' && c <= '9') v = 10 * v + (c - '0');
      if (out && n < cap) out[n] = (int32_t)v;
      ++n;
    } else {
      c = std::fgetc(f);
    }
  }
  std::fclose(f);
  *count = n;
  if (out && n > cap) return fail(RT_ERR_BUFFER_TOO_SMALL, "load_matrix: more values than cap");
  return RT_OK;
}

}  // extern "C"
