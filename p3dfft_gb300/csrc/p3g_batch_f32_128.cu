// Batch kernel for the F32 path with 128-thread CTAs.
#include "p3g_batch_kernels.cuh"

namespace p3g {
P3G_BATCH_INSTANTIATE(PathF32, 128)
}  // namespace p3g
