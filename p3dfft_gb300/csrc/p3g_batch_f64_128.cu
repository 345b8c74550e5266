// Batch kernel for the F64 path with 128-thread CTAs.
#include "p3g_batch_kernels.cuh"

namespace p3g {
P3G_BATCH_INSTANTIATE(PathF64, 128)
}  // namespace p3g
