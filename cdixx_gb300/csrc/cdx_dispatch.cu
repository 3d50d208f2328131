// Length -> kernel dispatch for the row/column passes.
#include "cdx_fft.cuh"
#include "cdx_types.h"

namespace cdx {

template <int N> cudaError_t prepare_len();
template <int N> cudaError_t launch_row(const RowArgs&, int, cudaStream_t);
template <int N> cudaError_t launch_col(const ColArgs&, int, cudaStream_t);

#define CDX_FOR_EACH_SIZE(X) \
  X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) \
  X(1536) X(2048) X(3072) X(4096)

#define CASE_PREP(N) case N: return &prepare_len<N>;
#define CASE_ROW(N) case N: return &launch_row<N>;
#define CASE_COL(N) case N: return &launch_col<N>;
#define CASE_L(N) case N: return Geom<N>::L;

PrepLaunch prep_launcher(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_PREP) default: return nullptr; }
}
RowLaunch row_launcher(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_ROW) default: return nullptr; }
}
ColLaunch col_launcher(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_COL) default: return nullptr; }
}
int lines_per_cta(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_L) default: return 0; }
}

}  // namespace cdx
