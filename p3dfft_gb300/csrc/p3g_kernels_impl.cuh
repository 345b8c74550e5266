// Pass kernels, instantiated once per path by p3g_kernels_f64.cu / _f32.cu.
#pragma once

#include <algorithm>

#include "p3g_pipe.cuh"

namespace p3g {

extern __shared__ __align__(16) unsigned char p3g_smem[];

template <class P>
struct PathLimits;
template <>
struct PathLimits<PathF64> {  // 2 CTAs of 256 threads per SM, 128 registers
  static constexpr int kMaxThreads = 256;
  static constexpr int kMinBlocks = 2;
};
template <>
struct PathLimits<PathF32> {
  static constexpr int kMaxThreads = 512;
  static constexpr int kMinBlocks = 1;
};

// ---------------------------------------------------------------- X r2c
// Real lines 2p and 2p+1 form z = x1 + i x2; Z = FFT(z);
// X1[k] = (Z[k] + conj Z[N-k]) / 2, X2[k] = -i (Z[k] - conj Z[N-k]) / 2.
// One tile (M line pairs) of field `field`; sm = the tile's shared memory.
template <class P, bool CG>
P3G_D void x_r2c_tile(const XParams& prm, const StagePlan* __restrict__ sp, const float4* __restrict__ tw,
                      typename P::W* sm, int tile, int field, uint32_t& amax) {
  const int kb = range_k(prm.range);
  using W = typename P::W;
  using C = typename P::C;
  const int N = prm.nx;
  const int M = prm.M;
  const int p0 = tile * M;  // first pair of the tile
  const auto* in = static_cast<const typename P::UR*>(prm.in) + field * prm.in_field;

  float* smf = reinterpret_cast<float*>(sm);
  constexpr int kW = sizeof(W) / sizeof(float);  // floats per element: 4 (F64) or 2 (F32)
  const int LS = prm.LS, ps = prm.ps;
  for (int e = threadIdx.x; e < 2 * M * N; e += blockDim.x) {
    const int lt = e / N;
    const int x = e - lt * N;
    const int line = 2 * p0 + lt;
    const int c = lt & 1;
    float* f = smf + ((lt >> 1) * LS + pad_index(x, ps)) * kW;
    if constexpr (P::kF64) {
      df v{0.f, 0.f};
      if (line < prm.nlines) {
        const double u = gload<CG>(in + (long long)line * prm.in_line + x);
        P::track(amax, u);
        v = P::from_ur(u, kb);
      }
      f[c] = v.hi;
      f[2 + c] = v.lo;
    } else {
      f[c] = line < prm.nlines ? gload<CG>(in + (long long)line * prm.in_line + x) : 0.0f;
    }
  }
  __syncthreads();
  Tile<P> t{sm, sm + M * LS, M, prm.log2m, LS, 1, ps};
  cta_fft<P, -1, kElemsPerThread, kLineMajor>(t, sp, tw);
  xr2c_store<P>(prm, sm, p0, field, kb);
}

template <class P>
__global__ void __launch_bounds__(PathLimits<P>::kMaxThreads, PathLimits<P>::kMinBlocks)
    k_x_r2c(const XParams prm, const StagePlan* __restrict__ sp, const float4* __restrict__ tw) {
  uint32_t amax = 0;
  x_r2c_tile<P, false>(prm, sp, tw, reinterpret_cast<typename P::W*>(p3g_smem), blockIdx.x, blockIdx.y, amax);
  range_flush(prm.range, amax);
}

// ---------------------------------------------------------------- X c2r
// Z[k] = X1[k] + i X2[k] (k <= N/2, imaginary parts of DC and Nyquist
// dropped as FFTW's c2r does), Z[N-k] = conj X1[k] + i conj X2[k];
// z = IFFT(Z) (unnormalised) gives x1 = Re z, x2 = Im z.
template <class P, bool CG>
P3G_D void x_c2r_tile(const XParams& prm, const StagePlan* __restrict__ sp, const float4* __restrict__ tw,
                      typename P::W* sm, int tile, int field) {
  const int kb = range_k(prm.range);
  using W = typename P::W;
  using C = typename P::C;
  const int N = prm.nx;
  const int M = prm.M;
  const int p0 = tile * M;
  const W* in = static_cast<const W*>(prm.in) + field * prm.in_field;
  auto* out = static_cast<typename P::UR*>(prm.out) + field * prm.out_field;
  const int nh = N / 2 + 1;
  const int LS = prm.LS, ps = prm.ps;
  for (int e = threadIdx.x; e < M * nh; e += blockDim.x) {
    const int pr = e / nh;
    const int k = e - pr * nh;
    const int line = 2 * (p0 + pr);
    C x1 = P::zero(), x2 = P::zero();
    if (k < prm.nkeep) {
      if (line < prm.nlines) x1 = P::from_w(gload<CG>(in + (long long)line * prm.in_line + k));
      if (line + 1 < prm.nlines) x2 = P::from_w(gload<CG>(in + (long long)(line + 1) * prm.in_line + k));
    }
    if (k == 0 || 2 * k == N) {
      x1 = P::make(P::re(x1), P::re(P::zero()));
      x2 = P::make(P::re(x2), P::re(P::zero()));
    }
    sm[pr * LS + pad_index(k, ps)] = P::to_w(x1 + rot<1>(x2));
    if (k > 0 && 2 * k < N) sm[pr * LS + pad_index(N - k, ps)] = P::to_w(cconj(x1) + rot<1>(cconj(x2)));
  }
  __syncthreads();
  Tile<P> t{sm, sm + M * LS, M, prm.log2m, LS, 1, ps};
  cta_fft<P, 1, kElemsPerThread, kLineMajor>(t, sp, tw);
  const float* smf = reinterpret_cast<const float*>(sm);
  constexpr int kW = sizeof(W) / sizeof(float);
  for (int e = threadIdx.x; e < 2 * M * N; e += blockDim.x) {
    const int lt = e / N;
    const int n = e - lt * N;
    const int line = 2 * p0 + lt;
    if (line >= prm.nlines) continue;
    const int c = lt & 1;
    const float* f = smf + ((lt >> 1) * LS + pad_index(n, ps)) * kW;
    if constexpr (P::kF64) {
      out[(long long)line * prm.out_line + n] = P::to_ur(df{f[c], f[2 + c]}, kb);
    } else {
      out[(long long)line * prm.out_line + n] = f[c];
    }
  }
}

template <class P>
__global__ void __launch_bounds__(PathLimits<P>::kMaxThreads, PathLimits<P>::kMinBlocks)
    k_x_c2r(const XParams prm, const StagePlan* __restrict__ sp, const float4* __restrict__ tw) {
  x_c2r_tile<P, false>(prm, sp, tw, reinterpret_cast<typename P::W*>(p3g_smem), blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------- strided Y/Z

// One tile (M columns x L rows); `bid` enumerates (x tile, o1, o2 = field).
template <class P, int DIR, bool CG>
P3G_D void strided_tile(const SParams& prm, const StagePlan* __restrict__ sp, const float4* __restrict__ tw,
                        typename P::W* sm, long long bid, uint32_t& amax) {
  const int kb = range_k(prm.range);
  using W = typename P::W;
  using C = typename P::C;
  const int M = prm.M;
  const int N = prm.N;
  const int L = prm.L;
  const int xt = (int)(bid % prm.xtiles);
  bid /= prm.xtiles;
  const int o1 = (int)(bid % prm.O1);
  const int o2 = (int)(bid / prm.O1);
  const int x0 = xt * M;
  // per-element strides are 32-bit; their products with row and column
  // indices span the whole field and are formed in 64 bits
  const long long ibase = (long long)o1 * prm.in_o1 + (long long)o2 * prm.in_o2 + (long long)x0 * prm.in_xs;
  const long long obase = (long long)o1 * prm.out_o1 + (long long)o2 * prm.out_o2 + (long long)x0 * prm.out_xs;

  if (prm.pre == 2 && threadIdx.x < M) {  // DST-I odd extension: zero rows 0 and L+1
    sm[threadIdx.x] = P::to_w(P::zero());
    sm[(L + 1) * M + threadIdx.x] = P::to_w(P::zero());
  }
  // element e -> (column m, row j): columns fastest when columns are adjacent
  // in memory, rows fastest when rows are (STRIDE1 user layout)
  const bool in_rows_fast = prm.in_xs != 1;
  const FastDiv div_l(L);
  for (int e = threadIdx.x; e < M * L; e += blockDim.x) {
    int m, j;
    if (in_rows_fast) {
      m = div_l.div(e);
      j = e - m * L;
    } else {
      m = e & (M - 1);
      j = e >> prm.log2m;
    }
    const int src = j >= prm.lmap_a1 ? j - prm.lmap_d : (j < prm.lmap_a0 ? j : -1);
    C v = P::zero();
    if (x0 + m < prm.X && src >= 0)
      v = load_elem<P, CG>(prm.in, prm.in_user, ibase + (long long)m * prm.in_xs + (long long)src * prm.in_axis, kb,
                           amax);
    if (prm.pre == 0) {
      sm[j * M + m] = P::to_w(v);
    } else if (prm.pre == 1) {
      sm[j * M + m] = P::to_w(v);
      if (j >= 1 && j <= L - 2) sm[(2 * (L - 1) - j) * M + m] = P::to_w(v);
    } else {
      sm[(j + 1) * M + m] = P::to_w(v);
      sm[(2 * (L + 1) - (j + 1)) * M + m] = P::to_w(cneg(v));
    }
  }
  __syncthreads();
  Tile<P> t{sm, sm + M * N, M, prm.log2m, 1, M};
  cta_fft<P, DIR, kElemsPerThread, kPointMajor>(t, sp, tw);
  const bool out_rows_fast = prm.out_xs != 1;
  const FastDiv div_lo(prm.Lout);
  for (int e = threadIdx.x; e < M * prm.Lout; e += blockDim.x) {
    int m, jo;
    if (out_rows_fast) {
      m = div_lo.div(e);
      jo = e - m * prm.Lout;
    } else {
      m = e & (M - 1);
      jo = e >> prm.log2m;
    }
    if (x0 + m >= prm.X) continue;
    const int k = jo < prm.smap_s0 ? jo : jo + prm.smap_d;
    C v;
    if (prm.post == 1) v = rot<1>(P::from_w(sm[(k + 1) * M + m]));
    else v = P::from_w(sm[k * M + m]);
    if (prm.tw4) {  // four-step twiddle w_N^(o1 jo)
      const cdf w = load_tw(prm.tw4, (int)(((unsigned long long)o1 * (unsigned long long)jo) %
                                           (unsigned long long)prm.tw4_n));
      v = prm.tw4_conj ? cmul<true>(v, w) : cmul<false>(v, w);
    }
    store_elem<P>(prm.out, prm.out_user, obase + (long long)m * prm.out_xs + (long long)jo * prm.out_axis, v, kb);
  }
}

template <class P, int DIR>
__global__ void __launch_bounds__(PathLimits<P>::kMaxThreads, PathLimits<P>::kMinBlocks)
    k_strided(const SParams prm, const StagePlan* __restrict__ sp, const float4* __restrict__ tw) {
  uint32_t amax = 0;
  strided_tile<P, DIR, false>(prm, sp, tw, reinterpret_cast<typename P::W*>(p3g_smem), blockIdx.x, amax);
  range_flush(prm.range, amax);
}

// ------------------------------------------------------------- Chebyshev
// out(k) = L k old + out(k+2), ftran.F90:412-451, one thread per (x, y)
// pencil.  The F64 path runs this recurrence in binary64 itself (a few
// multiply-adds per mode on a pass bound by its 2 x 16 bytes per mode), so
// it has binary64's range and rounding like the reference; the F32 path in
// binary32.
template <class P>
__global__ void k_cheby(const ChebyParams prm) {
  using UC = typename P::UC;
  using R = typename std::conditional<P::kF64, double, float>::type;
  const int pcl = blockIdx.x * blockDim.x + threadIdx.x;
  if (pcl >= prm.npencil) return;
  UC* d = static_cast<UC*>(prm.data) + blockIdx.y * prm.field + pcl * prm.pstride;
  const int n = prm.nzc;
  const long long zs = prm.zstride;
  const R sc = (R)prm.sc, lf = (R)prm.lfac;
  auto scaled = [&](int k) {
    const UC v = d[k * zs];
    return UC{(R)v.x * sc, (R)v.y * sc};
  };
  UC old = scaled(n - 2);
  const UC top = scaled(n - 1);
  const R f1 = lf * (R)(n - 1) * (R)0.5;
  UC o1{f1 * top.x, f1 * top.y};  // out(nzc-1)
  UC o2{(R)0, (R)0};               // out(nzc)
  d[(n - 2) * zs] = o1;
  d[(n - 1) * zs] = o2;
  for (int k = n - 3; k >= 0; --k) {
    const UC nw = scaled(k);
    const R f = lf * (R)(k + 1);
    const UC val{f * old.x + o2.x, f * old.y + o2.y};
    d[k * zs] = val;
    o2 = o1;
    o1 = val;
    old = nw;
  }
  const UC v0 = d[0];
  d[0] = UC{v0.x * (R)0.5, v0.y * (R)0.5};
}

// ------------------------------------------------- long X lines (four-step)
// X lines longer than one tile go through a complex buffer T of one line per
// pair of real lines (z = x1 + i x2, N = nx points per line, pair p at p N):
// pack before the complex four-step transform and split after it (r2c), merge
// before it and unpack after it (c2r).  A pair whose second line is past the
// field's last line holds zeros there.

P3G_D long long grid_stride_start() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }
P3G_D long long grid_stride() { return (long long)gridDim.x * blockDim.x; }

template <class P>
__global__ void __launch_bounds__(256) k_x_pack(const XLongParams q) {
  using UR = typename P::UR;
  const UR* in = static_cast<const UR*>(q.in);
  typename P::W* T = static_cast<typename P::W*>(q.out);
  const int kb = range_k(q.range);
  const long long total = (long long)((q.nlines + 1) / 2) * q.nx;
  uint32_t amax = 0;
  for (long long e = grid_stride_start(); e < total; e += grid_stride()) {
    const long long pr = e / q.nx, x = e - pr * q.nx;
    const UR a = in[2 * pr * q.in_line + x];
    const UR b = 2 * pr + 1 < q.nlines ? in[(2 * pr + 1) * q.in_line + x] : UR(0);
    P::track(amax, a);
    P::track(amax, b);
    T[e] = P::to_w(P::make(P::from_ur(a, kb), P::from_ur(b, kb)));
  }
  range_flush(q.range, amax);
}

// X1[k] = (Z[k] + conj Z[N-k]) / 2, X2[k] = -i (Z[k] - conj Z[N-k]) / 2
template <class P>
__global__ void __launch_bounds__(256) k_x_split(const XLongParams q) {
  using C = typename P::C;
  const typename P::W* T = static_cast<const typename P::W*>(q.in);
  const int kb = range_k(q.range);
  const long long total = (long long)((q.nlines + 1) / 2) * q.nkeep;
  for (long long e = grid_stride_start(); e < total; e += grid_stride()) {
    const long long pr = e / q.nkeep;
    const int k = (int)(e - pr * q.nkeep);
    const C a = P::from_w(T[pr * q.nx + k]);
    const C b = cconj(P::from_w(T[pr * q.nx + (k == 0 ? 0 : q.nx - k)]));
    const C x1 = cscale2(a + b, 0.5f), x2 = cscale2(rot<-1>(a - b), 0.5f);
    const long long o1 = 2 * pr * q.out_line + k, o2 = o1 + q.out_line;
    if (q.out_user) {
      auto* out = static_cast<typename P::UC*>(q.out);
      out[o1] = P::to_uc(x1, kb);
      if (2 * pr + 1 < q.nlines) out[o2] = P::to_uc(x2, kb);
    } else {
      auto* out = static_cast<typename P::W*>(q.out);
      out[o1] = P::to_w(x1);
      if (2 * pr + 1 < q.nlines) out[o2] = P::to_w(x2);
    }
  }
}

// Z[k] = X1[k] + i X2[k] over every k < N, X[k] = conj X[N-k] above N/2, the
// imaginary parts of the k = 0 and k = N/2 modes dropped (as c2r does),
// modes at or beyond nkeep zero
template <class P>
__global__ void __launch_bounds__(256) k_x_merge(const XLongParams q) {
  using C = typename P::C;
  const typename P::W* in = static_cast<const typename P::W*>(q.in);
  typename P::W* T = static_cast<typename P::W*>(q.out);
  const long long total = (long long)((q.nlines + 1) / 2) * q.nx;
  for (long long e = grid_stride_start(); e < total; e += grid_stride()) {
    const long long pr = e / q.nx;
    const int k = (int)(e - pr * q.nx);
    const bool mir = 2 * k > q.nx;
    const int kk = mir ? q.nx - k : k;
    C x1 = P::zero(), x2 = P::zero();
    if (kk < q.nkeep) {
      x1 = P::from_w(in[2 * pr * q.in_line + kk]);
      if (2 * pr + 1 < q.nlines) x2 = P::from_w(in[(2 * pr + 1) * q.in_line + kk]);
    }
    if (kk == 0 || 2 * kk == q.nx) {
      x1 = P::make(P::re(x1), P::re(P::zero()));
      x2 = P::make(P::re(x2), P::re(P::zero()));
    }
    if (mir) {
      x1 = cconj(x1);
      x2 = cconj(x2);
    }
    T[e] = P::to_w(x1 + rot<1>(x2));
  }
}

template <class P>
__global__ void __launch_bounds__(256) k_x_unpack(const XLongParams q) {
  using UR = typename P::UR;
  const typename P::W* T = static_cast<const typename P::W*>(q.in);
  UR* out = static_cast<UR*>(q.out);
  const int kb = range_k(q.range);
  const long long total = (long long)((q.nlines + 1) / 2) * q.nx;
  for (long long e = grid_stride_start(); e < total; e += grid_stride()) {
    const long long pr = e / q.nx, x = e - pr * q.nx;
    const typename P::C z = P::from_w(T[e]);
    out[2 * pr * q.out_line + x] = P::to_ur(P::re(z), kb);
    if (2 * pr + 1 < q.nlines) out[(2 * pr + 1) * q.out_line + x] = P::to_ur(P::im(z), kb);
  }
}

// kind: 0 pack, 1 split, 2 merge, 3 unpack
template <class P>
cudaError_t launch_x_long(int kind, const XLongParams& q, int sm_count, cudaStream_t st) {
  const long long per = kind == 1 ? q.nkeep : q.nx;
  const long long total = (long long)((q.nlines + 1) / 2) * per;
  const int blocks = (int)std::max(1LL, std::min((total + 255) / 256, (long long)sm_count * 8));
  switch (kind) {
    case 0: k_x_pack<P><<<blocks, 256, 0, st>>>(q); break;
    case 1: k_x_split<P><<<blocks, 256, 0, st>>>(q); break;
    case 2: k_x_merge<P><<<blocks, 256, 0, st>>>(q); break;
    default: k_x_unpack<P><<<blocks, 256, 0, st>>>(q); break;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- launchers
template <class P>
cudaError_t launch_x_r2c(const XParams& p, const StagePlan* sp, const float4* tw, int threads, size_t smem,
                         int nfields, cudaStream_t st) {
  cudaError_t ea = opt_in_smem((const void*)k_x_r2c<P>, 227 * 1024);
  if (ea != cudaSuccess) return ea;
  k_x_r2c<P><<<dim3(p.tiles, nfields), threads, smem, st>>>(p, sp, tw);
  return cudaGetLastError();
}
template <class P>
cudaError_t launch_x_c2r(const XParams& p, const StagePlan* sp, const float4* tw, int threads, size_t smem,
                         int nfields, cudaStream_t st) {
  cudaError_t ea = opt_in_smem((const void*)k_x_c2r<P>, 227 * 1024);
  if (ea != cudaSuccess) return ea;
  k_x_c2r<P><<<dim3(p.tiles, nfields), threads, smem, st>>>(p, sp, tw);
  return cudaGetLastError();
}
template <class P>
cudaError_t launch_strided(const SParams& p, const StagePlan* sp, const float4* tw, bool forward_sign, int threads,
                           size_t smem, int nfields, cudaStream_t st) {
  cudaError_t ea = opt_in_smem((const void*)k_strided<P, -1>, 227 * 1024);
  if (ea == cudaSuccess) ea = opt_in_smem((const void*)k_strided<P, 1>, 227 * 1024);
  if (ea != cudaSuccess) return ea;
  const long long blocks = (long long)p.xtiles * p.O1 * nfields;
  if (blocks <= 0 || blocks > 0x7FFFFFFFLL) return cudaErrorInvalidConfiguration;
  if (forward_sign) k_strided<P, -1><<<(unsigned)blocks, threads, smem, st>>>(p, sp, tw);
  else k_strided<P, 1><<<(unsigned)blocks, threads, smem, st>>>(p, sp, tw);
  return cudaGetLastError();
}
template <class P>
cudaError_t launch_cheby(const ChebyParams& p, int nfields, cudaStream_t st) {
  const int threads = 128;
  k_cheby<P><<<dim3((p.npencil + threads - 1) / threads, nfields), threads, 0, st>>>(p);
  return cudaGetLastError();
}

// Pipelined launchers: E (elements per thread) selects the instantiation.
template <class P, int E>
cudaError_t launch_strided_pipe_e(const CUtensorMap* map, const CUtensorMap* omap, const SPipeParams& p,
                                  const StagePlan* sp, const float4* tw, bool forward_sign, int threads, size_t smem,
                                  int grid, cudaStream_t st) {
  cudaError_t ea = opt_in_smem((const void*)k_strided_pipe<P, -1, E>, 227 * 1024);
  if (ea == cudaSuccess) ea = opt_in_smem((const void*)k_strided_pipe<P, 1, E>, 227 * 1024);
  if (ea != cudaSuccess) return ea;
  if (forward_sign) k_strided_pipe<P, -1, E><<<grid, threads, smem, st>>>(*map, *omap, p, sp, tw);
  else k_strided_pipe<P, 1, E><<<grid, threads, smem, st>>>(*map, *omap, p, sp, tw);
  return cudaGetLastError();
}
template <class P>
cudaError_t launch_strided_pipe(const CUtensorMap* map, const CUtensorMap* omap, const SPipeParams& p,
                                const StagePlan* sp, const float4* tw, bool forward_sign, int E, int threads,
                                size_t smem, int grid, cudaStream_t st) {
  if constexpr (P::kF64) {
    if (E == 8) return launch_strided_pipe_e<P, 8>(map, omap, p, sp, tw, forward_sign, threads, smem, grid, st);
    if (E == 16) return launch_strided_pipe_e<P, 16>(map, omap, p, sp, tw, forward_sign, threads, smem, grid, st);
  } else {
    if (E == 16) return launch_strided_pipe_e<P, 16>(map, omap, p, sp, tw, forward_sign, threads, smem, grid, st);
    if (E == 32) return launch_strided_pipe_e<P, 32>(map, omap, p, sp, tw, forward_sign, threads, smem, grid, st);
  }
  return cudaErrorInvalidValue;
}
template <class P, int E>
cudaError_t launch_xr2c_pipe_e(const XPipeParams& p, const StagePlan* sp, const float4* tw, int threads, size_t smem,
                               int grid, cudaStream_t st) {
  cudaError_t ea = opt_in_smem((const void*)k_xr2c_pipe<P, E>, 227 * 1024);
  if (ea != cudaSuccess) return ea;
  k_xr2c_pipe<P, E><<<grid, threads, smem, st>>>(p, sp, tw);
  return cudaGetLastError();
}
template <class P>
cudaError_t launch_xr2c_pipe(const XPipeParams& p, const StagePlan* sp, const float4* tw, int E, int threads,
                             size_t smem, int grid, cudaStream_t st) {
  if constexpr (P::kF64) {
    if (E == 8) return launch_xr2c_pipe_e<P, 8>(p, sp, tw, threads, smem, grid, st);
    if (E == 16) return launch_xr2c_pipe_e<P, 16>(p, sp, tw, threads, smem, grid, st);
  } else {
    if (E == 16) return launch_xr2c_pipe_e<P, 16>(p, sp, tw, threads, smem, grid, st);
    if (E == 32) return launch_xr2c_pipe_e<P, 32>(p, sp, tw, threads, smem, grid, st);
  }
  return cudaErrorInvalidValue;
}
template <class P, int E>
cudaError_t launch_xc2r_pipe_e(const XPipeParams& p, const StagePlan* sp, const float4* tw, int threads, size_t smem,
                               int grid, cudaStream_t st) {
  cudaError_t ea = opt_in_smem((const void*)k_xc2r_pipe<P, E>, 227 * 1024);
  if (ea != cudaSuccess) return ea;
  k_xc2r_pipe<P, E><<<grid, threads, smem, st>>>(p, sp, tw);
  return cudaGetLastError();
}
template <class P>
cudaError_t launch_xc2r_pipe(const XPipeParams& p, const StagePlan* sp, const float4* tw, int E, int threads,
                             size_t smem, int grid, cudaStream_t st) {
  if constexpr (P::kF64) {
    if (E == 8) return launch_xc2r_pipe_e<P, 8>(p, sp, tw, threads, smem, grid, st);
    if (E == 16) return launch_xc2r_pipe_e<P, 16>(p, sp, tw, threads, smem, grid, st);
  } else {
    if (E == 16) return launch_xc2r_pipe_e<P, 16>(p, sp, tw, threads, smem, grid, st);
    if (E == 32) return launch_xc2r_pipe_e<P, 32>(p, sp, tw, threads, smem, grid, st);
  }
  return cudaErrorInvalidValue;
}

// Resident CTAs per SM of a pipelined kernel (kind 0 strided, 1 r2c, 2 c2r)
// with E elements per thread for the given block size and dynamic shared
// memory; 1 if the query fails.
template <class P, int E>
int pipe_blocks_per_sm_e(int kind, int threads, size_t smem) {
  const void* f = kind == 0 ? (const void*)k_strided_pipe<P, -1, E>
                            : (kind == 1 ? (const void*)k_xr2c_pipe<P, E> : (const void*)k_xc2r_pipe<P, E>);
  int n = 0;
  if (opt_in_smem(f, 227 * 1024) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem) != cudaSuccess || n < 1) {
    cudaGetLastError();
    return 1;
  }
  return n;
}
template <class P>
int pipe_blocks_per_sm(int kind, int E, int threads, size_t smem) {
  if constexpr (P::kF64) {
    return E == 16 ? pipe_blocks_per_sm_e<P, 16>(kind, threads, smem) : pipe_blocks_per_sm_e<P, 8>(kind, threads, smem);
  } else {
    return E == 32 ? pipe_blocks_per_sm_e<P, 32>(kind, threads, smem)
                   : pipe_blocks_per_sm_e<P, 16>(kind, threads, smem);
  }
}

#define P3G_INSTANTIATE(P)                                                                                          \
  template cudaError_t launch_x_r2c<P>(const XParams&, const StagePlan*, const float4*, int, size_t, int,          \
                                       cudaStream_t);                                                              \
  template cudaError_t launch_x_c2r<P>(const XParams&, const StagePlan*, const float4*, int, size_t, int,          \
                                       cudaStream_t);                                                              \
  template cudaError_t launch_strided<P>(const SParams&, const StagePlan*, const float4*, bool, int, size_t, int,  \
                                         cudaStream_t);                                                            \
  template cudaError_t launch_cheby<P>(const ChebyParams&, int, cudaStream_t);                                     \
  template cudaError_t launch_x_long<P>(int, const XLongParams&, int, cudaStream_t);                               \
  template int pipe_blocks_per_sm<P>(int, int, int, size_t);                                                            \
  template cudaError_t launch_strided_pipe<P>(const CUtensorMap*, const CUtensorMap*, const SPipeParams&,         \
                                              const StagePlan*, const float4*, bool, int, int, size_t, int,       \
                                              cudaStream_t);                                                      \
  template cudaError_t launch_xr2c_pipe<P>(const XPipeParams&, const StagePlan*, const float4*, int, int, size_t,  \
                                           int, cudaStream_t);                                                     \
  template cudaError_t launch_xc2r_pipe<P>(const XPipeParams&, const StagePlan*, const float4*, int, int, size_t,  \
                                           int, cudaStream_t);

}  // namespace p3g
