// The reference's drop-in entry points (include/p3dfft.h) on top of the
// explicit device API.  Built twice: libp3dfft.so (binary64 arrays) and, with
// -DSINGLE_PREC, libp3dfft_single.so (binary32 arrays), mirroring the
// reference's --enable-single build.  -DSTRIDE1 makes the (nzc, nyc, nxhpc)
// output layout the default, as the reference's --enable-stride1 build does;
// p3dfft_gb_set_layout picks the layout at run time before p3dfft_setup.
//
// State follows the reference's module-level SAVE variables
// (build/module.F90:101-176): one global plan set up by p3dfft_setup and torn
// down by p3dfft_clean, 12 accumulating timers, overwrite flag.  Arrays may
// be device memory or host memory: the kernels read and write host arrays in
// place when the GPU can address them (page-locked memory, or any memory on a
// host whose page tables the GPU uses), else they are staged through device
// buffers with H2D and D2H copies inside the call.  Every call is synchronous
// like the reference's.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/p3dfft_gb300.h"

#ifdef SINGLE_PREC
typedef float real_t;
static const int kPrec = P3G_F32;
#else
typedef double real_t;
static const int kPrec = P3G_F64;
#endif

namespace {

p3g_plan g_plan = nullptr;
int g_comm = 0;
int g_status = 0;
bool g_abort = true;
#ifdef STRIDE1
int g_layout = P3G_LAYOUT_STRIDE1;
#else
int g_layout = P3G_LAYOUT_XYZ;
#endif
std::string g_msg;
cudaStream_t g_stream = nullptr;
cudaStream_t g_copy = nullptr;  // host copies overlapped with the Z pass
constexpr int kRowBlocks = 8;
void* g_stage[2] = {nullptr, nullptr};
size_t g_stage_bytes[2] = {0, 0};
int g_nx, g_ny, g_nz, g_nxhpc, g_nyc, g_nzc;
// timers survive p3dfft_clean (the sample programs read them after it) and
// are zeroed by p3dfft_setup (setup.F90:143) and set_timers
double g_timers[12];

// Reference errors print and call MPI_Abort (setup.F90:125-135,181-184,
// ftran.F90:640-643); here they print, record the status and abort unless
// p3dfft_gb_set_abort(0) was called.
void error(int code, const std::string& msg, bool fatal = true) {
  g_status = code;
  g_msg = msg;
  std::fprintf(stderr, "%s\n", msg.c_str());
  if (fatal && g_abort) std::abort();
}

bool check(int rc) {
  if (rc == P3G_OK) return true;
  error(rc, std::string("P3DFFT error: ") + p3g_last_error());
  return false;
}

bool on_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Host arrays the kernels may read and write in place, without staging: page-
// locked (registered) host memory, or any host memory when the GPU reaches
// pageable memory through the host's page tables (a Grace host over
// NVLink-C2C).  P3DFFT_GB_HOST_DIRECT=0 forces staging through device buffers.
bool host_direct(const void* p) {
  static int mode = -1;
  static bool pageable = false;
  if (mode < 0) {
    const char* e = std::getenv("P3DFFT_GB_HOST_DIRECT");
    mode = (e && *e == '0') ? 0 : 1;
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) == cudaSuccess)
      pageable = v != 0;
    cudaGetLastError();
  }
  if (!mode) return false;
  if (pageable) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost && a.devicePointer == p;
}

void* stage(int which, size_t bytes) {
  if (bytes > g_stage_bytes[which]) {
    if (g_stage[which]) cudaFree(g_stage[which]);
    g_stage[which] = nullptr;
    g_stage_bytes[which] = 0;
    if (cudaMalloc(&g_stage[which], bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    g_stage_bytes[which] = bytes;
  }
  return g_stage[which];
}

bool ready() {
  if (!g_plan) {
    // module.F90:230-231: print and return
    error(P3G_E_STATE, "P3DFFT error: call setup before other routines", false);
    return false;
  }
  return true;
}

// The F64 path's binary64 exponent window (p3g_plan_set_range): every call
// runs at the exponent bias its direction needed last (fields of a
// simulation keep their magnitudes from call to call).  A call whose input
// turns out to lie outside the window runs again at the bias that brings it
// in, so no call returns infinities or flushed zeros that the reference's
// binary64 arithmetic would not; a call whose output overwrites its input
// (in place) cannot run again and picks its bias on the device instead (one
// extra read of the input).  The binary32 library has binary32's range, as
// the reference's single-precision build, and the checks return at once.
enum { kFwd = 0, kBwd = 1 };
int g_bias[2] = {0, 0};

// Runs `call` (which enqueues the transform on g_stream) under the range
// policy above; finish synchronises every stream the call used.  Returns false
// after recording an error.
template <class F, class S>
bool ranged(int dir, bool in_place, F&& call, S&& finish) {
  p3g_plan_set_range(g_plan, in_place ? P3G_RANGE_AUTO : P3G_RANGE_FIXED, g_bias[dir]);
  int rc = call();
  const bool synced = finish();
  if (!check(rc)) return false;
  if (!synced) {
    error(P3G_E_CUDA, "P3DFFT error: transform failed");
    return false;
  }
  int need = 0;
  rc = p3g_plan_check_range(g_plan, &need, nullptr);
  if (rc == P3G_E_RANGE) {
    g_bias[dir] = need;
    p3g_plan_set_range(g_plan, P3G_RANGE_FIXED, need);
    rc = call();
    const bool ok = finish();
    if (!check(rc)) return false;
    if (!ok) {
      error(P3G_E_CUDA, "P3DFFT error: transform failed");
      return false;
    }
    rc = p3g_plan_check_range(g_plan, nullptr, nullptr);
  }
  if (in_place) p3g_plan_set_range(g_plan, P3G_RANGE_FIXED, g_bias[dir]);
  return check(rc);
}

// Runs one transform call with host or device arrays.  in_bytes/out_bytes
// cover all nv fields.  Host arrays are used in place only on the real-space
// side (in_real / out_real): the X passes read and write whole contiguous
// lines there, while the Z passes reach the wavenumber-space array in short
// strided runs that cross the host link far slower than one bulk copy.
template <class F>
void run(int dir, const void* in, size_t in_bytes, bool in_real, void* out, size_t out_bytes, bool out_real,
         F&& call) {
  const bool din = on_device(in) || (in_real && host_direct(in));
  const bool dout = on_device(out) || (out_real && host_direct(out));
  const void* dev_in = in;
  void* dev_out = out;
  if (!din) {
    void* s = stage(0, in_bytes);
    if (!s) return error(P3G_E_NOMEM, "P3DFFT error: staging allocation failed");
    if (cudaMemcpyAsync(s, in, in_bytes, cudaMemcpyHostToDevice, g_stream) != cudaSuccess)
      return error(P3G_E_CUDA, "P3DFFT error: host to device copy failed");
    dev_in = s;
  }
  if (!dout) {
    dev_out = stage(1, out_bytes);
    if (!dev_out) return error(P3G_E_NOMEM, "P3DFFT error: staging allocation failed");
  }
  const bool in_place = dev_in == dev_out;
  if (!ranged(dir, in_place, [&] { return call(dev_in, dev_out); },
              [&] { return cudaStreamSynchronize(g_stream) == cudaSuccess; }))
    return;
  if (!dout && cudaMemcpyAsync(out, dev_out, out_bytes, cudaMemcpyDeviceToHost, g_stream) != cudaSuccess)
    return error(P3G_E_CUDA, "P3DFFT error: device to host copy failed");
  if (cudaStreamSynchronize(g_stream) != cudaSuccess) return error(P3G_E_CUDA, "P3DFFT error: transform failed");
  g_status = 0;
}

// Runs an overlapped call (both streams) under the range policy.
template <class F>
void run_overlapped(int dir, F&& call) {
  if (ranged(dir, false, call, [] {
        const cudaError_t a = cudaStreamSynchronize(g_stream), b = cudaStreamSynchronize(g_copy);
        return a == cudaSuccess && b == cudaSuccess;
      }))
    g_status = 0;
}

size_t rsize() { return (size_t)g_nx * g_ny * g_nz; }
size_t csize() { return (size_t)g_nxhpc * g_nyc * g_nzc; }

}  // namespace

extern "C" {

int p3dfft_gb_status(void) { return g_status; }
const char* p3dfft_gb_last_error(void) { return g_msg.c_str(); }
void p3dfft_gb_set_abort(int on) { g_abort = on != 0; }

void p3dfft_gb_set_layout(int layout) {
  if (layout != P3G_LAYOUT_XYZ && layout != P3G_LAYOUT_STRIDE1)
    return error(P3G_E_ARG, "P3DFFT error: unknown layout " + std::to_string(layout));
  if (g_plan) return error(P3G_E_STATE, "P3DFFT error: the layout can only change before p3dfft_setup");
  g_layout = layout;
  g_status = 0;
}

// setup.F90:83-104,107-605 for a single rank.  memsize receives the padded
// in-place size (setup.F90:579-603).
void p3dfft_setup(int* dims, int* nx, int* ny, int* nz, int* comm, int* nxc, int* nyc, int* nzc, int* ow,
                  int* memsize) {
  (void)ow;  // the input of btran is never modified here; OW only allowed it
  if (*nx <= 0 || *ny <= 0 || *nz <= 0)
    return error(P3G_E_ARG, "Invalid dimensions : " + std::to_string(*nx) + " " + std::to_string(*ny) + " " +
                                std::to_string(*nz));
  if (g_plan)
    return error(P3G_E_STATE,
                 "P3DFFT Setup error: the problem is already initialized. \n"
                 "Currently multiple setups not supported.\n"
                 "Quit the library using p3dfft_clean before initializing another setup");
  if (dims[0] <= 0 || dims[1] <= 0 || dims[0] * dims[1] != 1)
    return error(P3G_E_ARG, "Invalid processor geometry: " + std::to_string(dims[0]) + " " +
                                std::to_string(dims[1]) + " for 1 tasks");
  const int cx = nxc ? *nxc : *nx, cy = nyc ? *nyc : *ny, cz = nzc ? *nzc : *nz;
  if (!check(p3g_plan_create(&g_plan, *nx, *ny, *nz, cx, cy, cz, kPrec, g_layout, P3G_FLAG_TIMERS))) return;
  if (!g_stream) cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
  if (!g_copy) cudaStreamCreateWithFlags(&g_copy, cudaStreamNonBlocking);
  std::memset(g_timers, 0, sizeof(g_timers));
  g_bias[kFwd] = g_bias[kBwd] = 0;
  g_comm = comm ? *comm : 0;
  g_nx = *nx;
  g_ny = *ny;
  g_nz = *nz;
  g_nxhpc = cx / 2 + 1;
  g_nyc = cy;
  g_nzc = cz;
  if (memsize) {
    int s[3], e[3];
    p3g_get_dims(g_plan, 3, s, e, memsize);
  }
  g_status = 0;
}

void p3dfft_get_dims(int* start, int* end, int* size, int* conf) {
  if (!ready()) return;
  if (check(p3g_get_dims(g_plan, *conf, start, end, size))) g_status = 0;
}

void p3dfft_get_mpi_info(int* taskid, int* ntasks, int* comm) {
  if (!ready()) return;
  *taskid = 0;
  *ntasks = 1;
  *comm = g_comm;
  g_status = 0;
}


void p3dfft_ftran_r2c(real_t* A, real_t* B, unsigned char* op) {
  if (!ready()) return;
  const char* o = reinterpret_cast<const char*>(op);
  // host output (staged) with a GPU-readable input: copy the Z pass's output
  // to the host in row blocks while later blocks compute
  if (g_layout == P3G_LAYOUT_XYZ && !on_device(B) && (on_device(A) || host_direct(A))) {
    void* st = stage(1, csize() * 2 * sizeof(real_t));
    if (!st) return error(P3G_E_NOMEM, "P3DFFT error: staging allocation failed");
    return run_overlapped(kFwd, [&] { return p3g_ftran_r2c_to_host(g_plan, A, B, st, o, kRowBlocks, g_stream, g_copy); });
  }
  run(kFwd, A, rsize() * sizeof(real_t), true, B, csize() * 2 * sizeof(real_t), false,
      [&](const void* i, void* out) { return p3g_ftran_r2c(g_plan, i, out, o, 1, 0, 0, g_stream); });
}

void p3dfft_btran_c2r(real_t* A, real_t* B, unsigned char* op) {
  if (!ready()) return;
  const char* o = reinterpret_cast<const char*>(op);
  // host input (staged) with a GPU-writable output: row-block copies feed the
  // Z pass as they land
  if (g_layout == P3G_LAYOUT_XYZ && !on_device(A) && (on_device(B) || host_direct(B))) {
    void* st = stage(0, csize() * 2 * sizeof(real_t));
    if (!st) return error(P3G_E_NOMEM, "P3DFFT error: staging allocation failed");
    return run_overlapped(kBwd,
                          [&] { return p3g_btran_c2r_from_host(g_plan, A, st, B, o, kRowBlocks, g_stream, g_copy); });
  }
  run(kBwd, A, csize() * 2 * sizeof(real_t), false, B, rsize() * sizeof(real_t), true,
      [&](const void* i, void* out) { return p3g_btran_c2r(g_plan, i, out, o, 1, 0, 0, g_stream); });
}

// ftran.F90:104-317: nv fields spaced dim_in reals / dim_out complexes apart
void p3dfft_ftran_r2c_many(real_t* A, int* dim_in, real_t* B, int* dim_out, int* nv, unsigned char* op) {
  if (!ready()) return;
  if ((size_t)*dim_in < rsize() || (size_t)*dim_out < csize())
    return error(P3G_E_ARG, "ftran error: input or output array dimensions are too low", false);
  const char* o = reinterpret_cast<const char*>(op);
  const long long di = *dim_in, dout = *dim_out;
  const int n = *nv;
  run(kFwd, A, (size_t)di * n * sizeof(real_t), true, B, (size_t)dout * n * 2 * sizeof(real_t), false,
      [&](const void* i, void* out) { return p3g_ftran_r2c(g_plan, i, out, o, n, di, dout, g_stream); });
}

// btran.F90:104-304
void p3dfft_btran_c2r_many(real_t* A, int* dim_in, real_t* B, int* dim_out, int* nv, unsigned char* op) {
  if (!ready()) return;
  if ((size_t)*dim_in < csize() || (size_t)*dim_out < rsize())
    return error(P3G_E_ARG, "btran error: input or output array dimensions are too low", false);
  const char* o = reinterpret_cast<const char*>(op);
  const long long di = *dim_in, dout = *dim_out;
  const int n = *nv;
  run(kBwd, A, (size_t)di * n * 2 * sizeof(real_t), false, B, (size_t)dout * n * sizeof(real_t), true,
      [&](const void* i, void* out) { return p3g_btran_c2r(g_plan, i, out, o, n, di, dout, g_stream); });
}

// ftran.F90:787-814: X r2c alone into (nx/2+1, ny, nz) complexes
void p3dfft_ftran_r2c_1d(real_t* A, real_t* B) {
  if (!ready()) return;
  const size_t cbytes = (size_t)(g_nx / 2 + 1) * g_ny * g_nz * 2 * sizeof(real_t);
  run(kFwd, A, rsize() * sizeof(real_t), true, B, cbytes, false,
      [&](const void* i, void* out) { return p3g_ftran_r2c_1d(g_plan, i, out, g_stream); });
}

void p3dfft_cheby(real_t* A, real_t* B, real_t* Lz) {
  if (!ready()) return;
  const double lz = *Lz;
  run(kFwd, A, rsize() * sizeof(real_t), true, B, csize() * 2 * sizeof(real_t), false,
      [&](const void* i, void* out) { return p3g_cheby(g_plan, i, out, lz, 1, 0, 0, g_stream); });
}

void p3dfft_cheby_many(real_t* A, int* dim_in, real_t* B, int* dim_out, int* nv, real_t* Lz) {
  if (!ready()) return;
  if ((size_t)*dim_in < rsize() || (size_t)*dim_out < csize())
    return error(P3G_E_ARG, "cheby error: input or output array dimensions are too low", false);
  const double lz = *Lz;
  const long long di = *dim_in, dout = *dim_out;
  const int n = *nv;
  run(kFwd, A, (size_t)di * n * sizeof(real_t), true, B, (size_t)dout * n * 2 * sizeof(real_t), false,
      [&](const void* i, void* out) { return p3g_cheby(g_plan, i, out, lz, n, di, dout, g_stream); });
}

// module.F90:301-424
void p3dfft_clean(void) {
  if (g_plan) {
    p3g_get_timers(g_plan, g_timers);
    p3g_plan_destroy(g_plan);
  }
  g_plan = nullptr;
  for (int i = 0; i < 2; ++i) {
    if (g_stage[i]) cudaFree(g_stage[i]);
    g_stage[i] = nullptr;
    g_stage_bytes[i] = 0;
  }
  g_status = 0;
}

void get_timers(double* timers) {
  if (g_plan) p3g_get_timers(g_plan, g_timers);
  std::memcpy(timers, g_timers, sizeof(g_timers));
}

void set_timers(void) {
  if (g_plan) p3g_set_timers(g_plan);
  std::memset(g_timers, 0, sizeof(g_timers));
}

}  // extern "C"
