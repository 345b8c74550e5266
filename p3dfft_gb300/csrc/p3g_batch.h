// Work-item table of the batch kernel, shared by the host code that builds
// it (p3g_batch.cu) and the kernel instantiations (p3g_batch_<path>_<threads>.cu).
#pragma once

#include <cuda_runtime.h>

#include "p3g_kernels.cuh"
#include "p3g_spectrum.cuh"

namespace p3g {
enum BatchKind { kBXr2c = 0, kBFwd = 1, kBBwd = 2, kBXc2r = 3, kBSpec = 4, kBZero = 5 };

struct BatchPass {
  int kind;
  int tiles;   // work items of the pass
  int first;   // queue index of its first item
  int dep;     // pass that must be complete first, -1 = none
  int rows_per_item;  // spectrum passes
  int pipe;    // 1: tiles go through the double-buffered path (cp.async prefetch)
  int chunk;   // X r2c: bytes per cp.async copy of the real lines
  int pad_;
  const StagePlan* sp;
  const float4* tw;
  XParams x;
  SParams s;
  SpecParams spec;
};

constexpr int kBatchSpinLimit = 1 << 22;  // polls of ~1 us: about 4 s

// 128 threads and four CTAs per SM on both paths (128 registers per thread):
// while one CTA waits on its loads or at a barrier the others compute (12 %
// faster than two 256-thread CTAs on uneven grids of sides 48..256).  Tiles
// then hold at most kElemsPerThread x 128 = 2048 points; a batch with a
// longer line runs 256-thread CTAs (two per SM, 4096-point tiles).
constexpr int kBatchThreadsSmall = 128;
constexpr int kBatchThreadsLarge = 256;
template <int T>
__host__ __device__ constexpr int batch_min_blocks() { return 65536 / 128 / T; }

// Points per thread of the double-buffered path (as the pipelined pass
// kernels): 8 on F64, 16 on F32.
template <bool F64>
__host__ __device__ constexpr int batch_pipe_elems() { return F64 ? 8 : 16; }

// Kernel configuration and launch for one path and CTA size, explicitly
// instantiated in the p3g_batch_<path>_<threads>.cu units.  batch_config_t
// opts the kernel in to the largest dynamic shared memory the current device
// allows next to its static shared variables and reads the occupancy for a
// tile of smem bytes.
template <class P, int T>
cudaError_t batch_config_t(size_t smem, int& per_sm, size_t& max_dyn);
template <class P, int T>
cudaError_t batch_launch_t(const BatchPass* d_pass, int npass, int nitems, int* ctl, int buf_elems, int grid,
                           size_t smem, cudaStream_t st);

}  // namespace p3g
