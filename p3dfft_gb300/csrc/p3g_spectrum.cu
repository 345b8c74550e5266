// Shell spectrum of a forward transform's output: p3g_spectrum.
//
// Restates compute_spectrum of the reference's spectrum sample
// (sample/FORTRAN/driver_spec.F90:263-341) for a single rank: every kept mode
// (kx, ky, kz) of the complex output is binned by ik = int(sqrt(k^2) + 0.5)
// with ky, kz folded to |frequency| the way the sample folds them
// (index > n/2 -> n - index + 1, 1-based), and E(ik) accumulates k^2 |B|^2.
// The serving form's power spectrum uses the same binning with unit weight
// and counts the conjugate partner of every mode with 0 < kx and 2 kx != nx.
//
// Arithmetic: each warp takes one row of the fast axis (x, or z in the
// STRIDE1 layout) 32 modes at a time.  The mode weight w = k^2 |B|^2 is formed
// in double-float (binary32 pairs with FMA-exact products; GB300 runs binary64
// FMA at about 1/70 of the binary32 rate), equal bins among the 32 lanes are
// contiguous (|k| is monotone along x, and monotone on each side of the fold
// along z), so a segmented shuffle reduction gives one partial sum per run of
// equal bins; the run head converts its sum to binary64 and adds it to the
// warp's private binary64 histogram in shared memory.  At the end the CTA sums
// its warps' histograms and adds them to E with binary64 atomics.  Summation
// order differs from the sample's sequential loop, so results agree to
// rounding, not bitwise.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "p3g_plan_internal.h"
#include "p3g_spectrum.cuh"

namespace p3g {
namespace {

template <class P>
__global__ void __launch_bounds__(256) k_spectrum(const SpecParams prm) {
  extern __shared__ double p3g_spec_hist[];
  const int nwarps = blockDim.x >> 5;
  for (int i = threadIdx.x; i < nwarps * (prm.kmax + 1); i += blockDim.x) p3g_spec_hist[i] = 0.0;
  __syncthreads();
  spectrum_rows<P, false>(prm, p3g_spec_hist, blockIdx.x * nwarps + (threadIdx.x >> 5), prm.rows, gridDim.x * nwarps,
                          blockIdx.y);
  __syncthreads();
  spectrum_flush(prm, p3g_spec_hist, nwarps, blockIdx.y);
}

constexpr int kSpecThreads = 256;

template <class P>
cudaError_t launch_spectrum(const SpecParams& prm, int nv, int sm_count, cudaStream_t st) {
  const int nbins = prm.kmax + 1;
  int warps = kSpecThreads / 32;
  while (warps > 1 && (size_t)warps * nbins * sizeof(double) > kSpecMaxSmem) warps >>= 1;
  const size_t smem = (size_t)warps * nbins * sizeof(double);
  cudaError_t e = opt_in_smem((const void*)k_spectrum<P>, 227 * 1024);
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spectrum<P>, warps * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long long want = ((long long)prm.rows + warps - 1) / warps;
  long long slots = (long long)sm_count * per_sm / nv;
  if (slots < 1) slots = 1;
  const int gx = (int)(want < slots ? want : slots);
  k_spectrum<P><<<dim3(gx > 0 ? gx : 1, nv), warps * 32, smem, st>>>(prm);
  return cudaGetLastError();
}

}  // namespace
}  // namespace p3g

namespace p3g {

int make_spectrum_params(p3g_plan p, const void* in, double* E, int kmax, double scale, int flags,
                         long long dim_in, SpecParams& prm) {
  if (flags & ~(P3G_SPEC_K2 | P3G_SPEC_HERMITIAN)) return fail(P3G_E_ARG, "unknown spectrum flags");
  if (kmax <= 0)  // driver_spec.F90:198
    kmax = (int)(std::sqrt((double)p->nx * p->nx + (double)p->ny * p->ny + (double)p->nz * p->nz) * 0.5 + 0.5);
  // driver_spec.F90:271-274, with en = the ip=2 extents
  const long long e1 = p->layout == P3G_LAYOUT_STRIDE1 ? p->nzc : p->nxhpc;
  const long long e3 = p->layout == P3G_LAYOUT_STRIDE1 ? p->nxhpc : p->nzc;
  if (4.0 * (double)kmax * kmax < (double)((e1 - 1) * (e1 - 1) + (long long)(p->nyc - 1) * (p->nyc - 1) +
                                            (e3 - 1) * (e3 - 1)))
    return fail(P3G_E_ARG, "Error: kmax is less than it should be (" + std::to_string(kmax) + ")");
  const size_t nbins = (size_t)kmax + 1;
  if (nbins * sizeof(double) > kSpecMaxSmem) return fail(P3G_E_UNSUPPORTED, "kmax too large for the spectrum kernel");
  if (p->nx >= 32768 || p->ny >= 32768 || p->nz >= 32768)
    return fail(P3G_E_UNSUPPORTED, "spectrum supports sides below 32768");
  const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
  if (dim_in <= 0) dim_in = csize;
  if (dim_in < csize) return fail(P3G_E_ARG, "spectrum error: input array dimensions are too low");
  prm = SpecParams{};
  prm.in = in;
  prm.E = E;
  prm.field = dim_in;
  prm.nyc = p->nyc;
  prm.nx = p->nx;
  prm.ny = p->ny;
  prm.nz = p->nz;
  prm.stride1 = p->layout == P3G_LAYOUT_STRIDE1;
  prm.rows = prm.stride1 ? p->nxhpc * p->nyc : p->nzc * p->nyc;
  prm.len = prm.stride1 ? p->nzc : p->nxhpc;
  prm.kmax = kmax;
  prm.flags = flags;
  prm.s2 = scale * scale;
  return P3G_OK;
}

}  // namespace p3g

extern "C" int p3g_spectrum(p3g_plan p, const void* in, double* E, int kmax, double scale, int flags, int nv,
                            long long dim_in, void* stream) {
  using namespace p3g;
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!in || !E) return fail(P3G_E_ARG, "NULL array");
  if (nv <= 0 || nv > 65535) return fail(P3G_E_ARG, "nv out of range");
  SpecParams prm;
  int rc = make_spectrum_params(p, in, E, kmax, scale, flags, dim_in, prm);
  if (rc) return rc;
  const size_t nbins = (size_t)prm.kmax + 1;
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(E, 0, nbins * nv * sizeof(double), st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("spectrum clear: ") + cudaGetErrorString(e));
  e = p->prec == P3G_F64 ? launch_spectrum<PathF64>(prm, nv, p->sm_count, st)
                         : launch_spectrum<PathF32>(prm, nv, p->sm_count, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("spectrum launch: ") + cudaGetErrorString(e));
  p->launches++;
  return P3G_OK;
}
