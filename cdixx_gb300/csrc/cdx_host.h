// Host helpers shared by the C ABI (parser, .bin I/O, error string).
#pragma once
#include <stddef.h>
#include <string>
#include <vector>

namespace cdx {

// Mirrors of the public codes (include/cdx.h) for code that does not include it.
enum {
  CDX_ERR_ARG_H = 1, CDX_ERR_SIZE_H = 2, CDX_ERR_CUDA_H = 3, CDX_ERR_ALGO_H = 4, CDX_ERR_STATE_H = 5,
  CDX_ERR_IO_H = 6, CDX_ERR_NOMEM_H = 7, CDX_ERR_CONFIG_H = 8, CDX_ERR_NOLIB_H = 9
};
enum {
  ALGO_RAAR_H = 0, ALGO_ER_H = 1, ALGO_POSER_H = 2, ALGO_HIO_H = 3, ALGO_POSHIO_H = 4, ALGO_FHIO_H = 5,
  ALGO_SHRINKWRAP_H = 6, ALGO_XCORRELATION_H = 7, ALGO_KKT_H = 8, ALGO_TV_H = 9
};

int set_error(int code, const std::string& msg);
int set_error_cstr(int code, const char* msg);
const char* last_error();
int algo_expand(const char* f, std::vector<int>& out, size_t limit);
int read_bin(const char* path, int* rows, int* cols, int* is_complex, float* data, size_t cap);
int write_bin(const char* path, const float* data, int rows, int cols, int is_complex);

}  // namespace cdx
