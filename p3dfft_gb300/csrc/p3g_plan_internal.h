// Internal definition of the plan object shared by the C-ABI translation
// units of libp3dfft_gb300.so (not part of the public headers).
#pragma once

#include <mutex>
#include <string>
#include <vector>

#include "../../include/p3dfft_gb300.h"
#include "p3g_kernels.cuh"

namespace p3g {

// Records msg as the calling thread's p3g_last_error() and returns code.
int fail(int code, const std::string& msg);

struct AxisPlan {
  StagePlan sp{};
  int n = 0;
  int M = 1, log2m = 0, threads = 32;
  size_t smem = 0;
  int sp_index = 0;  // index into the device StagePlan array
  int tw_lo = 0, tw_cnt = 0;  // this axis's contiguous slice of the twiddle table
  int ls = 0, ps = 0;         // X axis: shared-memory line-pair stride and padding shift
  // pipelined kernels (p3g_pipe.cuh): same tile, double buffered
  bool pipe_ok = false;
  int pipe_m = 1, pipe_log2m = 0;  // lines (columns) per pipelined tile
  int pipe_threads = 0;
  int buf_elems = 0;
  size_t pipe_smem = 0;
  int pipe_bps = 1;  // resident CTAs per SM of the pipelined kernel
  int pipe_e = 8;    // elements per thread of the pipelined kernel (PipeLimits)
  int pipe_nbuf = 2; // tile buffers of the pipelined kernel
  // strided passes that store tiles by TMA: three buffers (0: they do not
  // fit without fewer resident CTAs)
  size_t pipe_smem3 = 0;
  // F64 wide pipelined kernels (16 points per thread): a second stage plan
  // with radix-16 stages and its twiddle slice; every other kernel runs sp
  StagePlan spw{};
  int spw_index = -1;  // -1: none, the pipelined kernel runs sp
  int tw_lo_w = 0, tw_cnt_w = 0;
  int ls_w = 0, ps_w = 0;  // X axis: line-pair stride and padding of the wide tiles
  // the pipelined kernel's stage plan index, twiddle slice and X tile layout
  int pipe_sp() const { return spw_index >= 0 ? spw_index : sp_index; }
  int pipe_tw_lo() const { return spw_index >= 0 ? tw_lo_w : tw_lo; }
  int pipe_tw_cnt() const { return spw_index >= 0 ? tw_cnt_w : tw_cnt; }
  int pipe_ls() const { return spw_index >= 0 ? ls_w : ls; }
  int pipe_ps() const { return spw_index >= 0 ? ps_w : ps; }
};

struct TimerRec {
  int slot;
  cudaEvent_t a, b;
};

}  // namespace p3g

struct p3g_plan_s;

namespace p3g {
// Pass parameters of one field's forward (X, Y, Z) and backward (Z, Y, X)
// transform with workspaces wa/wb; zi = Z op index (0 fft, 1 dct, 2 dst,
// 3 none).  Defined in p3g_plan.cu.
// y_zyx keeps the array between the Y and Z passes in [z][y][x] order (the
// forward Y output in place in wa when y is not pruned) as the batch kernel's
// small grids prefer; by default it is wb as [y][z][x], so that the Z pass
// (forward reads, backward writes) walks its lines one pitch apart and each
// pass has at most one side whose lines are a plane apart.
void make_forward_params(p3g_plan_s* p, const void* in, void* out, void* wa, void* wb, int zi, long long dim_in,
                         long long dim_out, XParams& x, SParams& y, SParams& z, bool y_zyx = false);
void make_backward_params(p3g_plan_s* p, const void* in, void* out, void* wa, void* wb, int zi, long long dim_in,
                          long long dim_out, SParams& z, SParams& y, XParams& x, bool y_zyx = false);
// The range check of p3g_plan_check_range on a copy of the plan's device
// words w (d_err[0..2]), for callers that copied them asynchronously.
int plan_range_result(p3g_plan_s* p, const int w[3], int* bias, int* emax);
// Exponent-window parameters of a pass converting the plan's binary64 user
// data in (input = true: tracked) or out; allow_auto = false ignores the
// auto mode (callers that run no reduction first).  Zero on the F32 path.
RangeParams range_params(p3g_plan_s* p, bool input, bool allow_auto);
// Auto mode: clears the measured word and launches the reduction over nv
// binary64 fields of n doubles spaced `field` doubles apart.
int launch_range_scan(p3g_plan_s* p, const void* in, long long n, long long field, int nv, cudaStream_t st);
}  // namespace p3g

struct p3g_plan_s {
  using AxisPlan = p3g::AxisPlan;
  using TimerRec = p3g::TimerRec;
  using StagePlan = p3g::StagePlan;
  int nx, ny, nz, nxc, nyc, nzc, prec, layout, flags;
  int nxh, nxhp, nxhc, nxhpc, nycph, nzcph;
  long long pitch;
  AxisPlan ax_x, ax_y, ax_z[4];  // z: 0 fft, 1 dct (2(nz-1)), 2 dst (2(nz+1)), 3 none
  AxisPlan ax_xc;                 // the X c2r pass's pipelined kernel (ax_x for the rest)
  bool z_ok[4];
  float4* d_tw = nullptr;
  StagePlan* d_sp = nullptr;
  size_t tw_bytes = 0;
  void* wa = nullptr;  // nz*ny*pitch*nv elements
  void* wb = nullptr;  // nz*nyc*pitch*nv elements: the forward Y output ([y][z][x]), pruned-y backward
  size_t w_fields = 0;
  double timers[12];
  std::vector<TimerRec> pending;
  std::vector<cudaEvent_t> free_events;
  long long launches = 0;
  cudaStream_t aux = nullptr;  // second compute stream of the host-array transforms
  std::mutex mu;
  int sm_count = 0;
  // device words: [0] set by a kernel whose bounded wait timed out, [1] the
  // largest |high word| of the binary64 inputs converted since the last range
  // check, [2] the same measured by the auto-bias reduction of the current call
  int* d_err = nullptr;
  bool use_pipe = true, use_tma = true;
  int tx_extra = 0;  // test hook (p3g_plan_block_tiles)
  // four-step passes for Y or Z (FFT) lines longer than one shared-memory
  // tile: n = n1 n2, the first launch transforms length n2 (lz[0], ly[0]),
  // the second length n1 (ly[1], lz[1]); tw4_* is the twiddle-table offset of
  // the n roots w_n^t; wc holds one field between the two launches
  AxisPlan ly[2], lz[2], lx[2];
  bool four_y = false, four_z = false, four_x = false;
  int tw4_y = 0, tw4_z = 0, tw4_x = 0;
  void* wc = nullptr;
  void* wd = nullptr;  // long X lines: one complex line per pair of real lines
  size_t wc_bytes() const;
  int range_mode = P3G_RANGE_FIXED;  // F64 path: exponent bias fixed (ebias) or picked per call on the device
  int ebias = 0;
  int log2n = 0;  // ceil(log2(nx ny 2 (nz + 1))): bound of the transform's gain

  size_t esize() const { return prec == P3G_F64 ? 16 : 8; }
  // long X lines: pairs of real lines per field, and the row pitch of the
  // four-step scratch for them (pairs rounded up to 16 elements)
  long long xpairs() const { return ((long long)ny * nz + 1) / 2; }
  long long xpitch() const { return (xpairs() + 15) / 16 * 16; }
};

inline size_t p3g_plan_s::wc_bytes() const {
  size_t n = (four_y || four_z) ? (size_t)nz * (ny > nyc ? ny : nyc) * pitch : 0;
  if (four_x && (size_t)nx * xpitch() > n) n = (size_t)nx * xpitch();
  return n * esize();
}
