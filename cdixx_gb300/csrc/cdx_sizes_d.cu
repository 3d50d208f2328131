#include "cdx_sizes.cuh"
namespace cdx {
CDX_INSTANTIATE(3072) CDX_INSTANTIATE(4096)
}
