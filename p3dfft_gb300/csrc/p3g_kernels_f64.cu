// F64 path kernels (binary64 data, double-float butterflies).
#include "p3g_kernels_impl.cuh"

namespace p3g {
P3G_INSTANTIATE(PathF64)
}  // namespace p3g
