// Shell-spectrum row processing shared by k_spectrum (p3g_spectrum.cu) and
// the batch kernel (p3g_batch.cu).  See p3g_spectrum.cu for the method.
#pragma once

#include "p3g_kernels.cuh"
#include "../../include/p3dfft_gb300.h"

struct p3g_plan_s;

namespace p3g {

struct SpecParams {
  const void* in;
  double* E;           // nv * (kmax + 1) bins
  long long field;     // element spacing between fields
  int rows, len;       // rows of the fast axis and their length
  int nyc;             // rows decode as (outer, y) with y fastest
  int nx, ny, nz;
  int stride1;         // fast axis is z (1) or x (0)
  int kmax;
  int flags;
  double s2;           // scale^2
};

// ik = floor(sqrt(k2) + 0.5) exactly: the largest m with k2 > m (m - 1).
P3G_D int shell_index(uint32_t k2) {
  int m = (int)(sqrtf((float)k2) + 0.5f);
  while (m > 0 && (unsigned long long)m * (unsigned long long)(m - 1) >= k2) --m;
  while ((unsigned long long)(m + 1) * (unsigned long long)m < k2) ++m;
  return m;
}

// |frequency| of 0-based index i of an axis of n points (driver_spec.F90:294-298)
P3G_D int fold(int i, int n) { return i + 1 > n / 2 ? n - i : i; }

P3G_D df sq(df a) {
  df r;
  r.hi = fmul_rn(a.hi, a.hi);
  float e = ffma(a.hi, a.hi, -r.hi);
  r.lo = ffma(2.0f * a.hi, a.lo, e);
  return r;
}

template <bool CG>
P3G_D void load_mode(const double2* p, df& re, df& im) {
  const double2 v = gload<CG>(p);
  re = d2df(v.x);
  im = d2df(v.y);
}
template <bool CG>
P3G_D void load_mode(const float2* p, df& re, df& im) {
  const float2 v = gload<CG>(p);
  re = df{v.x, 0.0f};
  im = df{v.y, 0.0f};
}

// Rows r_first, r_first + r_step, ... below r_end of field `field`, one warp
// per row; hist_all holds one histogram of kmax + 1 bins per warp (zeroed by
// the caller).
template <class P, bool CG>
P3G_D void spectrum_rows(const SpecParams& prm, double* hist_all, int r_first, int r_end, int r_step, int field) {
  using UC = typename P::UC;
  const int nbins = prm.kmax + 1;
  const int lane = threadIdx.x & 31;
  double* hist = hist_all + (size_t)(threadIdx.x >> 5) * nbins;
  const UC* in = static_cast<const UC*>(prm.in) + (long long)field * prm.field;
  const bool k2w = (prm.flags & P3G_SPEC_K2) != 0;
  const bool herm = (prm.flags & P3G_SPEC_HERMITIAN) != 0;
  const uint32_t le_mask = 0xFFFFFFFFu >> (31 - lane);
  for (int r = r_first; r < r_end; r += r_step) {
    const int y = r % prm.nyc;
    const int outer = r / prm.nyc;
    const int ky = fold(y, prm.ny);
    const UC* row = in + (long long)r * prm.len;
    for (int base = 0; base < prm.len; base += 32) {
      const int i = base + lane;
      int bin = -1 - lane;  // lanes past the row end: a segment of their own
      df w{0.0f, 0.0f};
      if (i < prm.len) {
        const int kx = prm.stride1 ? outer : i;
        const int kz = fold(prm.stride1 ? i : outer, prm.nz);
        const uint32_t k2 = (uint32_t)kx * kx + (uint32_t)ky * ky + (uint32_t)kz * kz;
        bin = shell_index(k2);
        df re, im;
        load_mode<CG>(row + i, re, im);
        w = dadd(sq(re), sq(im));
        if (k2w) {
          const float khi = __uint2float_rn(k2);
          const float klo = (float)((long long)k2 - (long long)khi);
          w = dmulc(w, khi, klo);
        }
        if (herm && kx > 0 && 2 * kx != prm.nx) w = dscale2(w, 2.0f);
      }
      const int prev = __shfl_up_sync(0xFFFFFFFFu, bin, 1);
      const bool head = lane == 0 || prev != bin;
      const uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
      const int seg = __popc(heads & le_mask);
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const float oh = __shfl_down_sync(0xFFFFFFFFu, w.hi, d);
        const float ol = __shfl_down_sync(0xFFFFFFFFu, w.lo, d);
        const int os = __shfl_down_sync(0xFFFFFFFFu, seg, d);
        if (lane + d < 32 && os == seg) w = dadd(w, df{oh, ol});
      }
      // modes beyond kmax are dropped (the sample would write past E)
      if (head && bin >= 0 && bin <= prm.kmax) atomicAdd(hist + bin, (double)w.hi + (double)w.lo);
    }
  }
}

// Sums the CTA's per-warp histograms into E (binary64 atomics, scaled by
// scale^2).  Call after a barrier; nwarps = histograms in hist_all.
P3G_D void spectrum_flush(const SpecParams& prm, const double* hist_all, int nwarps, int field) {
  const int nbins = prm.kmax + 1;
  double* E = prm.E + (long long)field * nbins;
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nwarps; ++k) s += hist_all[(size_t)k * nbins + b];
    if (s != 0.0) atomicAdd(E + b, s * prm.s2);
  }
}

constexpr size_t kSpecMaxSmem = 200 * 1024;

// Validates a spectrum request against the plan and fills prm (kmax <= 0
// selects the sample's default).  Defined in p3g_spectrum.cu.
int make_spectrum_params(p3g_plan_s* p, const void* in, double* E, int kmax, double scale, int flags,
                         long long dim_in, SpecParams& prm);

}  // namespace p3g
