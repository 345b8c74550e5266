// Kernel parameter blocks and launch entry points shared by the host plan.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "p3g_engine.cuh"

namespace p3g {

// Exponent window of the F64 path (range_bias in p3g_arith.cuh).  A pass
// that converts binary64 user data in records the largest |high word| it saw
// (track, atomicMax, null = off) and scales by 2^-k; a pass that converts to
// binary64 user data scales by 2^k.  k is `bias`, or, with auto_max set, the
// range_bias of the largest |high word| a reduction kernel measured on the
// call's input just before.
struct RangeParams {
  unsigned* track;
  const unsigned* auto_max;
  int bias;
  int log2n;
};
P3G_D int range_k(const RangeParams& r) {
  return r.auto_max ? range_bias(__ldcg(r.auto_max), r.log2n) : r.bias;
}
// Adds a thread's largest |high word| to the pass's record: one atomic per
// warp (every lane of the warp must call it).
P3G_D void range_flush(const RangeParams& r, uint32_t amax) {
  if (!r.track) return;
  const uint32_t w = __reduce_max_sync(0xFFFFFFFFu, amax);
  if ((threadIdx.x & 31) == 0 && w != 0u) atomicMax(r.track, w);
}

// X passes: lines along x (contiguous).  Two real lines travel as the real and
// imaginary parts of one complex line of length nx.
struct XParams {
  const void* in;
  void* out;
  long long in_field, out_field;  // element stride between fields (nv)
  int in_line, out_line;          // element stride between lines (below 2^31, checked at plan creation)
  int nlines;                     // lines per field (ny * nz)
  int nx;                         // real line length = complex FFT length
  int nkeep;                      // complex modes per line stored (r2c) / read (c2r)
  int M, log2m;                   // line pairs per tile
  int tiles;                      // tiles per field
  int LS;                         // shared-memory stride between line pairs (>= padded N)
  int ps;                         // line padding shift (see pad_index), 0 = none
  int out_user;                   // r2c: 1 stores the user complex format (X-only transform)
  RangeParams range;              // r2c: binary64 input; c2r (and X-only r2c): binary64 output
};

// Strided Y/Z passes: a tile is M consecutive x columns of one (o1, o2) row
// set, transformed along the axis.  Element (x, j) of the input sits at
// in + x + j*in_axis + o1*in_o1 + o2*in_o2 (elements of 16 B on the F64 path,
// 8 B on the F32 path, for both the workspace and the user format).
struct SParams {
  const void* in;
  void* out;
  int in_user, out_user;  // 1: user complex format, 0: workspace format
  // single per-element strides (along the axis, between x columns: 1, or
  // nyc*nzc for the STRIDE1 user layout) are 32-bit and below 2^31 (plan
  // creation checks the strides themselves); the kernels form their products
  // with row and column indices, which span the whole field, in 64 bits.
  // Row (o1) and field (o2) strides are 64-bit
  int in_axis, out_axis;
  int in_xs, out_xs;
  long long in_o1, in_o2;
  long long out_o1, out_o2;
  int X;            // valid x columns
  int M, log2m;     // tile width (power of two)
  int xtiles, O1;   // tiles per row, number of o1 rows (o2 = fields from the grid)
  int L;            // logical transform length along the axis
  int N;            // FFT length (L, 2(L-1) or 2(L+1))
  int Lout;         // rows stored
  int pre;          // 0: rows as is, 1: DCT-I even extension (N = 2(L-1)), 2: DST-I odd extension (N = 2(L+1))
  int post;         // 0: result row k = buffer[k], 1: DST-I, result k = i*buffer[k+1]
  int lmap_a0, lmap_a1, lmap_d;  // load: row j <- input row j - d if j >= a1, j if j < a0, else 0
  int smap_s0, smap_d;           // store: output row jo <- result row jo (jo < s0) or jo + d
  // 1: 8-byte elements whose rows may start at an odd element (an odd row
  // stride, e.g. the nx/2+1 modes of a binary32 complex row).  Such a row's
  // tiles start one column later and wrap around (the last tile also takes
  // column 0), so that full tiles start on a 16-byte boundary and load two
  // columns per copy.
  int xphase;
  // > 0: the pass's columns are the positions of a plane of rows holding
  // xrow columns each, contiguous in the input (one row set, O1 = 1); the
  // output of position c goes to row c / xrow, column c % xrow
  int xrow;
  RangeParams range;  // user-format input (Z backward) or output (Z forward) of the F64 path
  // first launch of a four-step line (longer than one tile): the stored
  // element of row jo, o1 is multiplied by w_N^(o1 jo) (conjugated with
  // tw4_conj), N = tw4_n, from a table of the N roots (null: no twiddle)
  const float4* tw4;
  int tw4_n;
  int tw4_conj;
};

// First column of tile xt of row (o1, o2) and the row's phase: 0, or 1 when
// xphase is set and the row starts at an odd 8-byte element.  Column x0 + m
// of the tile is valid below X + phase and is column x0 + m - X past X.
P3G_HD int strided_phase(const SParams& s, int o1, int o2) {
  if (!s.xphase) return 0;
  return (int)(((unsigned long long)reinterpret_cast<uintptr_t>(s.in) / 8u + (unsigned long long)o1 * s.in_o1 +
                (unsigned long long)o2 * s.in_o2) & 1u);
}

// Output offset of tile column c: c * out_xs, or with xrow > 0 the offset of
// its row (out_o1 apart) and column.
P3G_HD long long strided_col_out(const SParams& s, int c) {
  if (s.xrow <= 0) return (long long)c * s.out_xs;
  const int r = c / s.xrow;
  return (long long)r * s.out_o1 + (long long)(c - r * s.xrow) * s.out_xs;
}

// Long X lines (four-step, p3g_kernels_impl.cuh): pack, split, merge, unpack.
struct XLongParams {
  const void* in;
  void* out;
  long long in_line, out_line;  // element strides between lines of the real or half-spectrum arrays
  int nlines;                   // lines per field
  int nx;                       // line length N
  int nkeep;                    // half-spectrum modes kept
  int out_user;                 // split: 1 stores the user complex format (X-only transform)
  RangeParams range;            // pack: binary64 input; unpack and user-format split: output
};


struct ChebyParams {
  void* data;          // user complex output of the 'ffc' transform
  long long field;     // element stride between fields
  long long pstride;   // element stride between pencils
  long long zstride;   // element stride along z
  int npencil;         // nxhpc * nyc
  int nzc;
  double sc;           // 1/(nx*ny*(nzc-1))
  double lfac;         // 4/Lz
};

// Global loads.  CG = true reads through L2 only (ld.global.cg): the batch
// kernel reads, within one launch, data that other CTAs wrote after this SM
// may already have cached the same lines in L1.
template <bool CG, class T>
P3G_D T gload(const T* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}
// User-format elements are converted with the exponent bias k (inputs
// times 2^-k, outputs times 2^k) and inputs are tracked into amax.
template <class P, bool CG = false>
P3G_D typename P::C load_elem(const void* base, int user, long long idx, int k, uint32_t& amax) {
  if (user) {
    const typename P::UC v = gload<CG>(static_cast<const typename P::UC*>(base) + idx);
    P::track(amax, v);
    return P::from_uc(v, k);
  }
  return P::from_w(gload<CG>(static_cast<const typename P::W*>(base) + idx));
}
template <class P>
P3G_D void store_elem(void* base, int user, long long idx, typename P::C v, int k) {
  if (user) static_cast<typename P::UC*>(base)[idx] = P::to_uc(v, k);
  else static_cast<typename P::W*>(base)[idx] = P::to_w(v);
}

// Stride of the raw line pairs of the pipelined X c2r tile: nh = N/2+1
// complexes per line, rounded up to even for 8-byte elements so that two
// complexes move with one 16-byte copy.
P3G_HD int xc2r_raw_stride(int nh, int esize) { return esize == 8 ? (nh + 1) & ~1 : nh; }

// Raises a kernel's dynamic shared-memory limit to `bytes` once per device:
// the attribute belongs to the device that is current when it is set, so a
// process that launches on several GPUs sets it on each (thread-safe).
cudaError_t opt_in_smem(const void* func, int bytes);

// Launchers (one per path).  Return the cudaError_t of the launch.
template <class P>
cudaError_t launch_x_r2c(const XParams& p, const StagePlan* sp, const float4* tw, int threads, size_t smem,
                         int nfields, cudaStream_t st);
template <class P>
cudaError_t launch_x_c2r(const XParams& p, const StagePlan* sp, const float4* tw, int threads, size_t smem,
                         int nfields, cudaStream_t st);
template <class P>
cudaError_t launch_strided(const SParams& p, const StagePlan* sp, const float4* tw, bool forward_sign, int threads,
                           size_t smem, int nfields, cudaStream_t st);
template <class P>
cudaError_t launch_cheby(const ChebyParams& p, int nfields, cudaStream_t st);
// long X lines: kind 0 pack, 1 split, 2 merge, 3 unpack (p3g_kernels_impl.cuh)
template <class P>
cudaError_t launch_x_long(int kind, const XLongParams& q, int sm_count, cudaStream_t st);

// pipelined kernels (p3g_pipe.cuh)
struct SPipeParams;
struct XPipeParams;
template <class P>
cudaError_t launch_strided_pipe(const CUtensorMap* map, const CUtensorMap* omap, const SPipeParams& p,
                                const StagePlan* sp, const float4* tw, bool forward_sign, int E, int threads,
                                size_t smem, int grid, cudaStream_t st);
template <class P>
cudaError_t launch_xr2c_pipe(const XPipeParams& p, const StagePlan* sp, const float4* tw, int E, int threads,
                             size_t smem, int grid, cudaStream_t st);
template <class P>
int pipe_blocks_per_sm(int kind, int E, int threads, size_t smem);
template <class P>
cudaError_t launch_xc2r_pipe(const XPipeParams& p, const StagePlan* sp, const float4* tw, int E, int threads,
                             size_t smem, int grid, cudaStream_t st);

}  // namespace p3g
