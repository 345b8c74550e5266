// Allocation-free forward transform: p3g_ftran_r2c_noalloc.
//
// Who needs it: callers that must not allocate device memory once they are
// running.  A serving worker that sized its device-memory budget at start-up,
// an application whose framework owns every device allocation through its
// own pool (a stray cudaMalloc would bypass the pool's accounting), and
// latency-critical loops where cudaMalloc/cudaFree would synchronise the
// device and stall other streams.  p3g_ftran_r2c allocates its workspace on
// first use (and grows it for larger nv); this entry point never does.
//
// How: the workspace of the three forward passes lives in the file-scope
// device array below, a fixed kNoAllocScratchBytes that every GPU which loads
// this library's module holds until the process exits.  Host code cannot use
// the array's name as a device address (in host code it is only a host-side
// stand-in), so the first call on each device, with that device current,
// resolves the address with cudaGetSymbolAddress and caches it; that first
// call should therefore happen before any stream capture.  Nothing in the
// workspace needs to start at zero: every element a pass reads was written
// by the previous pass of the same call.  All calls share the one array, so
// calls that overlap on the GPU (different streams, or different plans
// concurrently) race on it; serialise them.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "p3g_plan_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_dev[kMaxDevices] = {};  // device address of the array, per device

// Resolves the scratch array's device address for the current device (once).
int scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return p3g::fail(P3G_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return p3g::fail(P3G_E_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_dev[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return p3g::fail(P3G_E_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_dev[dev] = ptr;
  }
  *out = g_scratch_dev[dev];
  return P3G_OK;
}

// The three forward passes on the single-tile kernels (one tile per CTA, no
// persistent loop), with the pass parameters the allocating path builds.
template <class P>
int forward_passes(p3g_plan p, const void* in, void* out, int zi, bool fsign, void* wa, void* wb,
                   cudaStream_t st) {
  using namespace p3g;
  XParams x;
  SParams y, z;
  const long long rsize = (long long)p->nx * p->ny * p->nz;
  // the Y output in place in wa (no second buffer unless y is pruned)
  make_forward_params(p, in, out, wa, wb, zi, rsize, (long long)p->nxhpc * p->nyc * p->nzc, x, y, z, true);
  x.range = range_params(p, true, true);
  z.range = range_params(p, false, true);
  const int rc = launch_range_scan(p, in, rsize, rsize, 1, st);  // P3G_RANGE_AUTO only
  if (rc) return rc;
  cudaError_t e = launch_x_r2c<P>(x, p->d_sp + p->ax_x.sp_index, p->d_tw, p->ax_x.threads, p->ax_x.smem, 1, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("X r2c launch: ") + cudaGetErrorString(e));
  e = launch_strided<P>(y, p->d_sp + p->ax_y.sp_index, p->d_tw, true, p->ax_y.threads, p->ax_y.smem, 1, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("Y pass launch: ") + cudaGetErrorString(e));
  const AxisPlan& az = p->ax_z[zi];
  e = launch_strided<P>(z, p->d_sp + az.sp_index, p->d_tw, fsign, az.threads, az.smem, 1, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("Z pass launch: ") + cudaGetErrorString(e));
  p->launches += 3;
  return P3G_OK;
}

}  // namespace

extern "C" int p3g_ftran_r2c_noalloc(p3g_plan p, const void* in, void* out, const char* op, void* stream) {
  using namespace p3g;
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!op || !op[0] || !op[1] || !op[2]) return fail(P3G_E_ARG, "op must have 3 letters");
  if (!in || !out) return fail(P3G_E_ARG, "NULL array");
  int zi;
  bool fsign = true;
  switch (op[2]) {
    case 't':
    case 'f': zi = 0; break;
    case 'c': zi = 1; break;
    case 's': zi = 2; break;
    case 'n':
    case '0': zi = 3; break;
    default: return fail(P3G_E_ARG, std::string("Unknown transform type: ") + op[2]);
  }
  if (!p->z_ok[zi]) return fail(P3G_E_UNSUPPORTED, std::string("Z transform '") + op[2] + "' unsupported for nz");
  if (p->four_x || p->four_y || (zi == 0 && p->four_z))
    return fail(P3G_E_UNSUPPORTED, "allocation-free transform: lines longer than one tile need a second workspace");
  const size_t esize = p->esize();
  const size_t wa_bytes = ((size_t)p->nz * p->ny * p->pitch * esize + 255) / 256 * 256;
  const size_t wb_bytes = p->nyc < p->ny ? (size_t)p->nz * p->nyc * p->pitch * esize : 0;
  if (wa_bytes + wb_bytes > kNoAllocScratchBytes)
    return fail(P3G_E_UNSUPPORTED, "allocation-free transform: the grid needs " + std::to_string(wa_bytes + wb_bytes) +
                                       " bytes of workspace, more than its fixed " +
                                       std::to_string(kNoAllocScratchBytes) + "-byte device scratch");
  void* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  void* wa = base;
  void* wb = static_cast<unsigned char*>(base) + wa_bytes;
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return p->prec == P3G_F64 ? forward_passes<PathF64>(p, in, out, zi, fsign, wa, wb, st)
                            : forward_passes<PathF32>(p, in, out, zi, fsign, wa, wb, st);
}
