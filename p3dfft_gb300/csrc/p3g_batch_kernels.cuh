// Device code of the batch kernel (see p3g_batch.cu for the design),
// included by the explicit-instantiation units p3g_batch_<path>_<threads>.cu
// so that the four kernels compile in parallel.
#pragma once

#include "p3g_batch.h"
#include "p3g_kernels_impl.cuh"

namespace p3g {

P3G_D int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
P3G_D int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Waits until *cnt >= need.  false when the launch recorded an error or the
// wait ran out (then it records error 2).
P3G_D bool wait_count(const int* cnt, int need, int* err) {
  for (int polls = 0;; ++polls) {
    if (ld_acquire(cnt) >= need) {
      __threadfence();
      return true;
    }
    if (ld_relaxed(err) != 0) return false;
    if (polls >= kBatchSpinLimit) {
      atomicExch(err, 2);
      return false;
    }
    __nanosleep(polls < 32 ? 64 : 1000);
  }
}

// Pass lookup: the first-item index of up to kFirstCache passes is copied to
// shared memory at kernel start, so finding an item's pass is a binary
// search in shared memory instead of a chain of dependent global loads.
constexpr int kFirstCache = 1024;

P3G_D int find_pass(const BatchPass* __restrict__ passes, const int* s_first, int npass, int it) {
  int lo = 0, hi = npass - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const int f = mid < kFirstCache ? s_first[mid] : passes[mid].first;
    if (f <= it) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// cp.async copies of a double-buffered item's input tile into buf.
template <class P>
P3G_D void batch_issue(const BatchPass& bp, int tile, typename P::W* buf) {
  switch (bp.kind) {
    case kBXr2c: xr2c_copy<P>(bp.x, bp.chunk, buf, tile * bp.x.M, 0); break;
    case kBXc2r: xc2r_copy<P>(bp.x, buf, tile * bp.x.M, 0); break;
    default: {
      const int o1 = tile / bp.s.xtiles;
      strided_copy<P, true>(bp.s, buf, tile - o1 * bp.s.xtiles, o1, 0);
      break;
    }
  }
}

// Transform and store a double-buffered item whose tile is in buf.
template <class P>
P3G_D void batch_process_pipe(const BatchPass& bp, int tile, typename P::W* buf) {
  constexpr int E = batch_pipe_elems<P::kF64>();
  switch (bp.kind) {
    case kBXr2c: {  // the first FFT stage reads the raw line pairs
      const int k = range_k(bp.x.range);
      uint32_t amax = 0;
      Tile<P> t{buf, nullptr, bp.x.M, bp.x.log2m, bp.x.LS, 1, bp.x.ps, k, &amax};
      cta_fft<P, -1, E, kLineMajor, kRawR2C>(t, bp.sp, bp.tw);
      xr2c_store<P>(bp.x, buf, tile * bp.x.M, 0, k);
      range_flush(bp.x.range, amax);
      break;
    }
    case kBXc2r: {  // the first FFT stage reads the raw half spectra
      Tile<P> t{buf, nullptr, bp.x.M, bp.x.log2m, bp.x.LS, 1, bp.x.ps};
      cta_fft<P, 1, E, kLineMajor, kRawC2R>(t, bp.sp, bp.tw);
      xc2r_store<P>(bp.x, buf, tile * bp.x.M, 0, range_k(bp.x.range));
      break;
    }
    default: {
      const int o1 = tile / bp.s.xtiles;
      const int k = range_k(bp.s.range);
      uint32_t amax = 0;
      strided_fix<P>(bp.s, false, buf, k, amax);
      Tile<P> t{buf, nullptr, bp.s.M, bp.s.log2m, 1, bp.s.M};
      if (bp.kind == kBFwd) cta_fft<P, -1, E, kPointMajor>(t, bp.sp, bp.tw);
      else cta_fft<P, 1, E, kPointMajor>(t, bp.sp, bp.tw);
      strided_store<P>(bp.s, buf, tile - o1 * bp.s.xtiles, o1, 0, k);
      range_flush(bp.s.range, amax);
      break;
    }
  }
}

// Single-tile items (plans with generic prime stages, which need a scratch
// tile), spectrum chunks and histogram clears; sm spans both buffers.  Kept
// out of line so that its registers do not weigh on the double-buffered path.
template <class P>
__device__ __noinline__ void batch_process_single(const BatchPass& bp, int tile, typename P::W* sm) {
  switch (bp.kind) {
    case kBXr2c: {
      uint32_t amax = 0;
      x_r2c_tile<P, true>(bp.x, bp.sp, bp.tw, sm, tile, 0, amax);
      range_flush(bp.x.range, amax);
      break;
    }
    case kBFwd:
    case kBBwd: {
      uint32_t amax = 0;
      if (bp.kind == kBFwd) strided_tile<P, -1, true>(bp.s, bp.sp, bp.tw, sm, tile, amax);
      else strided_tile<P, 1, true>(bp.s, bp.sp, bp.tw, sm, tile, amax);
      range_flush(bp.s.range, amax);
      break;
    }
    case kBXc2r: x_c2r_tile<P, true>(bp.x, bp.sp, bp.tw, sm, tile, 0); break;
    case kBSpec: {
      double* hist = reinterpret_cast<double*>(sm);
      const int nwarps = blockDim.x >> 5;
      for (int i = threadIdx.x; i < nwarps * (bp.spec.kmax + 1); i += blockDim.x) hist[i] = 0.0;
      __syncthreads();
      const int r0 = tile * bp.rows_per_item;
      const int r1 = min(r0 + bp.rows_per_item, bp.spec.rows);
      spectrum_rows<P, true>(bp.spec, hist, r0 + (int)(threadIdx.x >> 5), r1, nwarps, 0);
      __syncthreads();
      spectrum_flush(bp.spec, hist, nwarps, 0);
      break;
    }
    case kBZero:
      for (int i = threadIdx.x; i <= bp.spec.kmax; i += blockDim.x) bp.spec.E[i] = 0.0;
      break;
    default: break;
  }
}

// ctl[0] = next queue item, ctl[1] = error, ctl[2 + d] = finished tiles of pass d.
//
// Each CTA holds a current item, the next item (its ticket, pass and whether
// its dependency was already complete when looked up) and one more ticket
// taken ahead.  When the next item is double-buffered and its dependency was
// complete, its tile is copied into the other buffer (cp.async) while the
// current tile is transformed; otherwise the CTA waits for the dependency
// after finishing the current item and loads then.  Between the end of one
// item and the start of the next, warp 1 publishes the finished item (fence +
// counter) while thread 0 looks up the item after next, whose ticket was
// fetched an item earlier: neither latency waits for the other.
template <class P, int T>
__global__ void __launch_bounds__(T, batch_min_blocks<T>())
    k_batch(const BatchPass* __restrict__ passes, int npass, int nitems, int* __restrict__ ctl, int buf_elems) {
  using W = typename P::W;
  __shared__ int s_first[kFirstCache];
  __shared__ int s_item, s_pass, s_ready, s_ok, s_cur, s_cpass;
  W* const buf0 = reinterpret_cast<W*>(p3g_smem);
  int* const err = &ctl[1];
  for (int i = threadIdx.x; i < npass && i < kFirstCache; i += blockDim.x) s_first[i] = passes[i].first;
  __syncthreads();
  // looks up item `it` (thread 0): its pass (-1 past the end or after an
  // error) and whether its dependency is already complete
  auto lookup = [&](int it, int& d, int& ready) {
    d = -1;
    ready = 0;
    if (it < nitems && ld_relaxed(err) == 0) {
      d = find_pass(passes, s_first, npass, it);
      const int dep = passes[d].dep;
      ready = dep < 0 || ld_acquire(&ctl[2 + dep]) >= passes[dep].tiles;
      if (ready) __threadfence();
    }
  };
  int ahead = 0;  // thread 0: the ticket after the next item
  if (threadIdx.x == 0) {
    // first item: wait for its dependency before loading it
    const int it = atomicAdd(&ctl[0], 1);
    int d, r;
    lookup(it, d, r);
    if (d >= 0 && !r && !wait_count(&ctl[2 + passes[d].dep], passes[passes[d].dep].tiles, err)) d = -1;
    s_cur = it;
    s_cpass = d;
    s_item = 0;
    s_pass = -1;
    s_ready = 0;
    if (d >= 0) {
      const int it1 = atomicAdd(&ctl[0], 1);
      ahead = atomicAdd(&ctl[0], 1);
      int d1, r1;
      lookup(it1, d1, r1);
      s_item = it1;
      s_pass = d1;
      s_ready = r1;
    }
  }
  __syncthreads();
  int cur = s_cur, dc = s_cpass, nxt = s_item, dn = s_pass, b = 0;
  bool ready = s_ready != 0;
  if (dc >= 0 && passes[dc].pipe) batch_issue<P>(passes[dc], cur - passes[dc].first, buf0);
  cp_async_commit();
  __syncthreads();  // every thread has read the shared item slots
#pragma unroll 1
  while (dc >= 0) {
    const BatchPass& bc = passes[dc];
    const bool pipe = bc.pipe != 0;
    bool prefetched = false;
    if (pipe && dn >= 0 && ready && passes[dn].pipe) {
      batch_issue<P>(passes[dn], nxt - passes[dn].first, buf0 + (b ^ 1) * buf_elems);
      prefetched = true;
    }
    cp_async_commit();
    if (pipe) {
      cp_async_wait<1>();
      __syncthreads();
      batch_process_pipe<P>(bc, cur - bc.first, buf0 + b * buf_elems);
    } else {
      batch_process_single<P>(bc, cur - bc.first, buf0);
    }
    // the barrier orders every thread's stores before warp 1's gpu-scope
    // fence and counter increment (the grid-barrier pattern)
    __syncthreads();
    if (threadIdx.x == 32) {
      __threadfence();
      atomicAdd(&ctl[2 + dc], 1);
    }
    if (threadIdx.x == 0) {
      int d2 = -1, r2 = 0;
      const int it2 = ahead;
      if (dn >= 0) {
        ahead = atomicAdd(&ctl[0], 1);
        lookup(it2, d2, r2);
      }
      s_item = it2;
      s_pass = d2;
      s_ready = r2;
    }
    __syncthreads();
    const bool cur_ready = ready;
    cur = nxt;
    dc = dn;
    b ^= 1;
    nxt = s_item;
    dn = s_pass;
    ready = s_ready != 0;
    if (dc >= 0 && !prefetched) {
      if (!cur_ready) {
        if (threadIdx.x == 0) {
          const int dep = passes[dc].dep;
          s_ok = wait_count(&ctl[2 + dep], passes[dep].tiles, err) ? 1 : 0;
        }
        __syncthreads();
        if (!s_ok) dc = -1;
      }
      if (dc >= 0 && passes[dc].pipe) batch_issue<P>(passes[dc], cur - passes[dc].first, buf0 + b * buf_elems);
      cp_async_commit();
    }
  }
  cp_async_wait<0>();
}

template <class P, int T>
cudaError_t batch_config_t(size_t smem, int& per_sm, size_t& max_dyn) {
  cudaFuncAttributes fa{};
  int dev = 0, optin = 0;
  cudaError_t e = cudaFuncGetAttributes(&fa, k_batch<P, T>);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const size_t dyn = (size_t)optin - fa.sharedSizeBytes;
  e = opt_in_smem((const void*)k_batch<P, T>, (int)dyn);
  if (e != cudaSuccess) return e;
  max_dyn = dyn;
  if (smem > max_dyn) return cudaErrorInvalidValue;
  per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<P, T>, T, smem);
  if (e == cudaSuccess && per_sm < 1) per_sm = 1;
  return e;
}

template <class P, int T>
cudaError_t batch_launch_t(const BatchPass* d_pass, int npass, int nitems, int* ctl, int buf_elems, int grid,
                           size_t smem, cudaStream_t st) {
  k_batch<P, T><<<grid, T, smem, st>>>(d_pass, npass, nitems, ctl, buf_elems);
  return cudaGetLastError();
}

#define P3G_BATCH_INSTANTIATE(P, T)                                                                      \
  template cudaError_t batch_config_t<P, T>(size_t, int&, size_t&);                                        \
  template cudaError_t batch_launch_t<P, T>(const BatchPass*, int, int, int*, int, int, size_t, cudaStream_t);

}  // namespace p3g
