#include "cdx_sizes.cuh"
namespace cdx {
CDX_INSTANTIATE(1024) CDX_INSTANTIATE(1536) CDX_INSTANTIATE(2048)
}
