// Batch kernel for the F64 path with 256-thread CTAs.
#include "p3g_batch_kernels.cuh"

namespace p3g {
P3G_BATCH_INSTANTIATE(PathF64, 256)
}  // namespace p3g
