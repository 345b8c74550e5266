// F32 path kernels (binary32 data, compensated twiddles).
#include "p3g_kernels_impl.cuh"

namespace p3g {
P3G_INSTANTIATE(PathF32)
}  // namespace p3g
