// Host plan and C-ABI of the explicit device API (include/p3dfft_gb300.h).
//
// A plan replaces the reference's p3dfft_setup + init_plan (build/setup.F90,
// build/init_plan.F90) for one rank on a 1x1 processor grid: it factors each
// axis length into radix stages, generates the twiddle tables once in FP64
// (long double on the host), uploads them with the stage plans, and sizes the
// per-pass tiles.  Transforms run three passes per direction:
//   forward:  X r2c (user real -> workspace), Y c2c (workspace -> workspace,
//             y pruning on store), Z op (workspace -> user complex, z pruning)
//   backward: Z op (user complex -> workspace, z zero-fill on load), Y c2c
//             (y zero-fill on load), X c2r (workspace -> user real)
// replacing ftran.F90:489-780 / btran.F90:396-679, whose 1x1 path runs the
// same FFTs with seg_copy/seg_zero passes (module.F90:502-706) in between.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include <cudaTypedefs.h>

#include <cstdint>
#include <cstdlib>

#include "../../include/p3dfft_gb300.h"
#include "p3g_pipe.cuh"
#include "p3g_plan_internal.h"

namespace p3g {

static thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

cudaError_t opt_in_smem(const void* func, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  std::lock_guard<std::mutex> lk(mu);
  if (done.count({func, dev})) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done.insert({func, dev});
  return e;
}
#define P3G_CUDA_TRY(call)                                                                 \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail(P3G_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------ factorisation
// Stage radices for length n, ordered by family (32, 16, 8, 4, 2, 3, 5,
// other primes) as cta_fft expects.  Powers of two use the largest radix
// allowed (max_pow2: 16, or 32 for the wide plans, on the F32 path; 8, or 16
// for the wide plans, on F64; 4 or 2 when a tuner asks) with a smaller
// remainder; with 32 the 2^a factor is
// split into the fewest stages of at most 32, as evenly as possible
// (1024 = 32 x 32, 512 = 32 x 16, 256 = 16 x 16, 128 = 16 x 8).
static bool factor(int n, int max_pow2, std::vector<int>& radices) {
  radices.clear();
  int a = 0;
  while (n % 2 == 0) {
    n /= 2;
    ++a;
  }
  std::vector<int> pow2;
  if (max_pow2 >= 32 && a > 0) {
    const int st = (a + 4) / 5;
    for (int i = 0; i < st; ++i) {
      const int bits = a / st + (i < a % st ? 1 : 0);
      pow2.push_back(1 << bits);
    }
    a = 0;
  }
  if (max_pow2 <= 4) {
    while (a >= 2 && max_pow2 == 4) {
      pow2.push_back(4);
      a -= 2;
    }
    while (a >= 1) {
      pow2.push_back(2);
      a -= 1;
    }
  }
  if (max_pow2 >= 16) {
    while (a >= 4 && a != 5) {  // 2^5 = 8*4 beats 16*2
      pow2.push_back(16);
      a -= 4;
    }
  }
  while (a >= 3 && a != 4) {
    pow2.push_back(8);
    a -= 3;
  }
  if (a == 4) {
    pow2.push_back(4);
    pow2.push_back(4);
  } else if (a == 2) {
    pow2.push_back(4);
  } else if (a == 1) {
    pow2.push_back(2);
  } else if (a == 3) {
    pow2.push_back(8);
  }
  for (int r : {32, 16, 8, 4, 2})
    for (int x : pow2)
      if (x == r) radices.push_back(r);
  for (int p : {3, 5}) {
    while (n % p == 0) {
      radices.push_back(p);
      n /= p;
    }
  }
  for (int p = 7; n > 1; p += 2) {
    while (n % p == 0) {
      radices.push_back(p);
      n /= p;
    }
    if ((long long)p * p > n && n > 1) {
      radices.push_back(n);
      n = 1;
    }
  }
  return (int)radices.size() <= kMaxStages;
}

struct HostTw {
  std::vector<float4> v;
  int mark = 0;  // start of the axis being built
  int push_root(long long num, long long den) {  // exp(-2 pi i num/den), split into hi/lo
    const long double two_pi = 6.283185307179586476925286766559L;
    long long t = num % den;
    const long double ang = -two_pi * (long double)t / (long double)den;
    const long double c = cosl(ang), s = sinl(ang);
    const float ch = (float)c, sh = (float)s;
    const float cl = (float)(c - (long double)ch), sl = (float)(s - (long double)sh);
    v.push_back(make_float4(ch, sh, cl, sl));
    return (int)v.size() - 1;
  }
};



static bool build_stages(int n, int max_pow2, HostTw& tw, StagePlan& sp) {
  std::memset(&sp, 0, sizeof(sp));
  tw.mark = (int)tw.v.size();
  sp.n = n;
  std::vector<int> rad;
  if (n > 1 && !factor(n, max_pow2, rad)) return false;
  sp.nstages = (int)rad.size();
  int ns = 1;
  for (int s = 0; s < sp.nstages; ++s) {
    const int r = rad[s];
    sp.radix[s] = r;
    sp.ns[s] = ns;
    switch (r) {
      case 32: sp.cnt[0]++; break;
      case 16: sp.cnt[1]++; break;
      case 8: sp.cnt[2]++; break;
      case 4: sp.cnt[3]++; break;
      case 2: sp.cnt[4]++; break;
      case 3: sp.cnt[5]++; break;
      case 5: sp.cnt[6]++; break;
      default: sp.has_generic = 1; break;
    }
    sp.tw_off[s] = (int)tw.v.size();
    if (ns > 1) {
      for (int k = 0; k < ns; ++k)
        for (int q = 1; q < r; ++q) tw.push_root((long long)q * k, (long long)ns * r);
    } else {
      tw.push_root(0, 1);  // keep offsets valid
    }
    sp.root_off[s] = (int)tw.v.size();
    if (r != 2 && r != 3 && r != 4 && r != 5 && r != 8 && r != 16 && r != 32)
      for (int m = 0; m < r; ++m) tw.push_root(m, r);
    ns *= r;
  }
  return true;
}

static int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

// Tile sizing: M lines of n points so that one tile holds about `budget`
// elements (64 KB), M a power of two not larger than needed, threads =
// ceil(M n / E) rounded up to a warp.
// max_m caps the tile width of strided passes so that one TMA box row
// (M elements) stays within the 256-word box limit.
static bool size_tile(AxisPlan& ap, int n, int lines_avail, bool f64, int max_m = 1 << 30) {
  const int budget = f64 ? 4096 : 8192;
  const int max_threads = f64 ? 256 : 512;
  const size_t esize = f64 ? 16 : 8;
  int M = 1;
  while (M * 2 * n <= budget && M * 2 <= (1 << ilog2(lines_avail > 0 ? lines_avail : 1)) && M * 2 <= max_m) M *= 2;
  auto threads_for = [&](int m) {
    int t = (m * n + kElemsPerThread - 1) / kElemsPerThread;
    t = (t + 31) / 32 * 32;
    return t < 32 ? 32 : t;
  };
  while (M > 1 && threads_for(M) > max_threads) M /= 2;
  if (threads_for(M) > max_threads) return false;
  ap.n = n;
  ap.M = M;
  ap.log2m = ilog2(M);
  ap.threads = threads_for(M);
  ap.smem = (size_t)M * n * esize * (ap.sp.has_generic ? 2 : 1);
  return ap.smem <= 227 * 1024;
}

// Launch shape of a pipelined kernel with E elements per thread: the most
// threads per CTA and the registers per thread its launch bounds allow.
template <class P, int E>
static void pipe_shape(bool xk, int& max_threads, int& regs) {
  max_threads = xk ? XPipeLimits<P, E>::kMaxThreads : PipeLimits<P, E>::kMaxThreads;
  const int blocks = xk ? XPipeLimits<P, E>::kMinBlocks : PipeLimits<P, E>::kMinBlocks;
  regs = std::min(255, 65536 / (max_threads * blocks));
}

// Pipelined kernels: two tile buffers (1 KB aligned), the axis's twiddles
// and two mbarriers in shared memory.  kind: 0 strided, 1 r2c, 2 c2r.  The
// elements per thread follow the axis's stage plans: 16 on F64 and 32 on F32
// when the axis has a wide plan, else 8 and 16.
static void size_pipe(AxisPlan& ap, int kind, bool f64, int thread_cap = 0) {
  ap.pipe_ok = false;
  if (ap.sp.nstages < 1 || ap.sp.has_generic || ap.n < 2) return;
  const size_t esize = f64 ? 16 : 8;
  const bool xk = kind != 0;  // X kernels have their own launch shape (XPipeLimits)
  const int E = f64 ? (ap.spw_index >= 0 ? 16 : 8) : (ap.spw_index >= 0 ? 32 : 16);
  ap.pipe_e = E;
  int max_threads = 0, regs_max = 0;
  if (f64) {
    if (E == 16) pipe_shape<PathF64, 16>(xk, max_threads, regs_max);
    else pipe_shape<PathF64, 8>(xk, max_threads, regs_max);
  } else if (E == 32) pipe_shape<PathF32, 32>(xk, max_threads, regs_max);
  else pipe_shape<PathF32, 16>(xk, max_threads, regs_max);
  if (thread_cap > 0 && thread_cap < max_threads) max_threads = thread_cap;
  const bool tw_shared = !xk;  // the X kernels read the global table
  const int n = ap.n;
  const int nh = n / 2 + 1;
  auto threads_for = [&](int M) {
    int t = (M * n + E - 1) / E;
    t = (t + 31) / 32 * 32;
    return t < 32 ? 32 : t;
  };
  auto smem_for = [&](int M, size_t& buf_bytes, int nbuf = 2) {
    // buffer stride rounded to 1 KB so every buffer (TMA destinations) stays aligned
    const int raw = 2 * xc2r_raw_stride(nh, (int)esize);  // c2r raw line pair
    const int ls = ap.pipe_ls();
    const size_t need = (size_t)(kind == 0 ? M * n : M * (ls > raw ? ls : raw)) * esize;
    buf_bytes = (need + 1023) / 1024 * 1024;
    return 1024 + nbuf * buf_bytes + (tw_shared ? (size_t)ap.pipe_tw_cnt() * 16 : 0) + 8 * nbuf + 16;
  };
  // resident warps per SM for tile width M: registers per thread from the
  // kernel's launch bounds, 2048 threads and ~228 KB of shared memory per SM
  auto warps_for = [&](int M, int nbuf = 2) {
    const int t = threads_for(M);
    size_t bb;
    const size_t sm = smem_for(M, bb, nbuf);
    const int regs = regs_max;
    int b = 65536 / (regs * t);
    b = std::min(b, 2048 / t);
    b = std::min(b, (int)((228 * 1024) / sm));
    return b * t / 32;
  };
  // widest tile whose CTA fits the kernel; a narrower one (down to half of
  // that, at least 2 lines) only when it keeps 1.5x more warps resident,
  // e.g. 540-point lines whose 4-line tile needs 288 threads (one CTA of
  // 9 warps per SM) against 160 threads for 2 lines (three CTAs)
  int M = ap.M;
  while (M > 1 && threads_for(M) > max_threads) M /= 2;
  if (threads_for(M) > max_threads) return;
  const int w0 = warps_for(M);
  if (M >= 4 && 2 * warps_for(M / 2) >= 3 * w0) M /= 2;
  ap.pipe_threads = threads_for(M);
  ap.pipe_m = M;
  ap.pipe_log2m = ilog2(M);
  // a third tile buffer (loads two tiles ahead) for the X kernels where it
  // fits without costing resident warps; the strided kernels load one tile
  // ahead (two loads in flight per CTA ran their scattered rows 3-15 %
  // slower) and take a third buffer only to drain TMA stores (pipe_smem3)
  size_t buf_bytes = 0;
  ap.pipe_nbuf = 2;
  if (xk && smem_for(M, buf_bytes, 3) <= 227 * 1024 && warps_for(M, 3) >= warps_for(M, 2)) ap.pipe_nbuf = 3;
  ap.pipe_smem = smem_for(M, buf_bytes, ap.pipe_nbuf);
  ap.buf_elems = (int)(buf_bytes / esize);
  ap.pipe_ok = ap.pipe_smem <= 227 * 1024;
  // the strided kernels' TMA-store form: a third buffer drains the stores
  ap.pipe_smem3 = 0;
  if (!xk && smem_for(M, buf_bytes, 3) <= 227 * 1024 && warps_for(M, 3) >= warps_for(M, 2))
    ap.pipe_smem3 = smem_for(M, buf_bytes, 3);
}



}  // namespace p3g

using namespace p3g;



namespace {

int ensure_workspace(p3g_plan p, int nv) {
  if ((size_t)nv <= p->w_fields) return P3G_OK;
  if (p->wa) cudaFree(p->wa);
  if (p->wb) cudaFree(p->wb);
  p->wa = p->wb = nullptr;
  p->w_fields = 0;
  const size_t na = (size_t)p->nz * p->ny * p->pitch * nv * p->esize();
  if (cudaMalloc(&p->wa, na) != cudaSuccess) {
    cudaGetLastError();
    p->wa = nullptr;
    return fail(P3G_E_NOMEM, "workspace allocation failed (" + std::to_string(na) + " bytes)");
  }
  {  // the forward Y pass writes wb ([y][z][x], a layout it cannot write in place)
    const size_t nb = (size_t)p->nz * p->nyc * p->pitch * nv * p->esize();
    if (cudaMalloc(&p->wb, nb) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(p->wa);
      p->wa = p->wb = nullptr;
      return fail(P3G_E_NOMEM, "workspace allocation failed (" + std::to_string(nb) + " bytes)");
    }
  }
  if ((p->four_y || p->four_z || p->four_x) && !p->wc) {
    const size_t nc = p->wc_bytes();
    if (cudaMalloc(&p->wc, nc) != cudaSuccess) {
      cudaGetLastError();
      p->wc = nullptr;
      return fail(P3G_E_NOMEM, "workspace allocation failed (" + std::to_string(nc) + " bytes)");
    }
  }
  if (p->four_x && !p->wd) {
    const size_t nd = (size_t)p->xpairs() * p->nx * p->esize();
    if (cudaMalloc(&p->wd, nd) != cudaSuccess) {
      cudaGetLastError();
      p->wd = nullptr;
      return fail(P3G_E_NOMEM, "workspace allocation failed (" + std::to_string(nd) + " bytes)");
    }
  }
  p->w_fields = nv;
  return P3G_OK;
}

cudaEvent_t get_event(p3g_plan p) {
  if (!p->free_events.empty()) {
    cudaEvent_t e = p->free_events.back();
    p->free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct PassTimer {
  p3g_plan p;
  int slot;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  PassTimer(p3g_plan p_, int slot_, cudaStream_t st_) : p(p_), slot(slot_), st(st_) {
    if (p->flags & P3G_FLAG_TIMERS) {
      a = get_event(p);
      cudaEventRecord(a, st);
    }
  }
  void done() {
    if (!a) return;
    cudaEvent_t b = get_event(p);
    cudaEventRecord(b, st);
    p->pending.push_back(TimerRec{slot, a, b});
    a = nullptr;
  }
};

int op_index(char c, bool& forward_sign, bool natural_forward) {
  switch (c) {
    case 't':
    case 'f':
      forward_sign = natural_forward;
      return 0;
    case 'c':
      forward_sign = true;
      return 1;
    case 's':
      forward_sign = true;  // RODFT00 is the same transform in both directions
      return 2;
    case 'n':
    case '0':
      forward_sign = true;
      return 3;
    default:
      return -1;
  }
}

using EncodeTiledFn = PFN_cuTensorMapEncodeTiled_v12000;

EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    else
      cudaGetLastError();
  }
  return fn;
}

// Rows per TMA box: at most 256, boxes land back to back in the tile buffer
// (128-byte aligned), and ceil(L / rows) * rows must fit in the buffer's
// buf_rows rows (rows past L read as zeros through the tensor bounds).
int pick_box_rows(int L, int buf_rows, int M, int esize) {
  for (int b = L < 256 ? L : 256; b >= 1; --b) {
    const long long rows = (long long)((L + b - 1) / b) * b;
    if (rows > buf_rows) continue;
    if (((long long)b * M * esize) % 128 != 0) continue;
    return b;
  }
  return 0;
}

// 4-D map over (x words, axis rows, o1, o2) of a strided pass's source.
bool encode_strided_map(CUtensorMap* m, const void* base, int esize, long long X, long long rows, long long o1n,
                        long long o2n, long long s_axis, long long s_o1, long long s_o2, int M, int brows) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn || reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  const int w = esize / 4;
  if ((long long)M * w > 256 || ((long long)M * esize) % 16 != 0) return false;
  if (o2n == 1) s_o2 = ((s_o1 * o1n * esize + 15) / 16 * 16) / esize + (esize == 8 ? 0 : 0);
  const cuuint64_t dims[4] = {(cuuint64_t)(X * w), (cuuint64_t)rows, (cuuint64_t)o1n, (cuuint64_t)o2n};
  const cuuint64_t strides[3] = {(cuuint64_t)(s_axis * esize), (cuuint64_t)(s_o1 * esize),
                                 (cuuint64_t)(s_o2 * esize)};
  for (int i = 0; i < 3; ++i)
    if (strides[i] % 16 != 0 || strides[i] >= (1ull << 40)) return false;
  if (dims[0] >= (1ull << 32)) return false;
  const cuuint32_t box[4] = {(cuuint32_t)(M * w), (cuuint32_t)brows, 1, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool aligned_to(const void* ptr, size_t a) { return reinterpret_cast<uintptr_t>(ptr) % a == 0; }

// Tensor maps (TMA) are only built over device memory; user arrays in host
// memory that the kernels address directly are read with cp.async.
bool device_memory(const void* ptr) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

template <class P>
int run_strided(p3g_plan p, SParams& s, const AxisPlan& ap, bool fwd_sign, int nv, cudaStream_t st,
                int max_sms = 0) {
  s.M = ap.M;
  s.log2m = ap.log2m;
  s.N = ap.n;
  s.xtiles = (s.X + ap.M - 1) / ap.M;
  const int esize = (int)sizeof(typename P::W);
  if (p->use_pipe && ap.pipe_ok && aligned_to(s.in, esize)) {
    s.M = ap.pipe_m;
    s.log2m = ap.pipe_log2m;
    s.xtiles = (s.X + s.M - 1) / s.M;
    SPipeParams pp{};
    pp.s = s;
    // TMA boxes copy rows one to one: the load map must be the identity
    // (no zero band and no shift; the backward passes of an unpruned grid
    // have a0 == a1 and d == 0)
    const bool identity_rows = (s.lmap_a0 >= s.L && s.lmap_a1 >= s.L) || (s.lmap_d == 0 && s.lmap_a0 >= s.lmap_a1);
    // binary32 user rows of an odd length (the Z backward input, nx/2+1
    // modes) start at odd 8-byte elements, which neither TMA nor 16-byte
    // copies address.  When the rows of a plane are contiguous the pass takes
    // the plane's positions as its columns instead: every tile then starts
    // on a 16-byte boundary and loads by TMA boxes, and the store splits each
    // position into its row and column
    if (!P::kF64 && s.xphase && p->use_tma && s.in_xs == 1 && s.in_o1 == s.X && s.O1 > 1 && !s.tw4 &&
        s.pre <= 1 && identity_rows && aligned_to(s.in, 16) && s.in_axis % 2 == 0 &&
        (nv == 1 || s.in_o2 % 2 == 0) && (long long)s.X * s.O1 < (1ll << 30) && device_memory(s.in)) {
      pp.s.xrow = s.X;
      pp.s.X = s.X * s.O1;
      pp.s.O1 = 1;
      pp.s.in_o1 = (long long)s.in_axis * s.L;
      pp.s.xphase = 0;
      pp.s.xtiles = (pp.s.X + s.M - 1) / s.M;
    }
    pp.c.tiles_per_field = pp.s.xtiles * pp.s.O1;
    pp.c.ntiles = pp.c.tiles_per_field * nv;
    pp.c.tw_base = ap.pipe_tw_lo();
    pp.c.tw_count = ap.pipe_tw_cnt();
    pp.c.buf_elems = ap.buf_elems;
    pp.c.nbuf = ap.pipe_nbuf;
    pp.c.err = p->d_err;
    pp.chunk = esize;
    CUtensorMap map, omap;
    std::memset(&map, 0, sizeof(map));
    std::memset(&omap, 0, sizeof(omap));
    const SParams& q = pp.s;
    if (p->use_tma && q.in_xs == 1 && q.pre <= 1 && identity_rows && !q.xphase &&
        (!q.in_user || device_memory(q.in))) {
      const int brows = pick_box_rows(q.L, ap.n, q.M, esize);
      if (brows > 0 && encode_strided_map(&map, q.in, esize, q.X, q.L, q.O1, nv, q.in_axis, q.in_o1, q.in_o2, q.M,
                                          brows)) {
        pp.use_tma = 1;
        pp.brows = brows;
        pp.nbox = (s.L + brows - 1) / brows;
        pp.box_bytes = brows * s.M * esize;
        pp.tx_extra = p->tx_extra;
      }
    }
    // TMA tile stores: output rows stored one to one (no pruning gap, no DST
    // shift, no four-step twiddle) in device memory, when the axis has room
    // for a third buffer.  Binary64 user output is converted in shared memory
    // first; binary32 user rows of an odd length (not 16-byte aligned) fail
    // the tensor map's stride check and keep the thread stores
    size_t smem = ap.pipe_smem;
    const bool identity_store = q.smap_s0 >= q.Lout || q.smap_d == 0;
    if (pp.use_tma && ap.pipe_smem3 && q.out_xs == 1 && q.post == 0 && identity_store && !q.tw4 &&
        q.xrow == 0 && aligned_to(q.out, 16) && device_memory(q.out)) {
      const int obrows = pick_box_rows(q.Lout, ap.n, q.M, esize);
      if (obrows > 0 && encode_strided_map(&omap, q.out, esize, q.X, q.Lout, q.O1, nv, q.out_axis, q.out_o1,
                                           q.out_o2, q.M, obrows)) {
        pp.tma_store = 1;
        pp.obrows = obrows;
        pp.onbox = (q.Lout + obrows - 1) / obrows;
        pp.c.nbuf = 3;
        smem = ap.pipe_smem3;
      }
    }
    const int slots = (max_sms > 0 && max_sms < p->sm_count ? max_sms : p->sm_count) * ap.pipe_bps;
    const int grid = pp.c.ntiles < slots ? pp.c.ntiles : slots;
    cudaError_t e = launch_strided_pipe<P>(&map, &omap, pp, p->d_sp + ap.pipe_sp(), p->d_tw, fwd_sign, ap.pipe_e,
                                           ap.pipe_threads, smem, grid, st);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("strided pass launch: ") + cudaGetErrorString(e));
    p->launches++;
    return P3G_OK;
  }
  cudaError_t e = launch_strided<P>(s, p->d_sp + ap.sp_index, p->d_tw, fwd_sign, ap.threads, ap.smem, nv, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("strided pass launch: ") + cudaGetErrorString(e));
  p->launches++;
  return P3G_OK;
}

template <class P>
int run_x_r2c(p3g_plan p, XParams& x, int nv, cudaStream_t st, int max_sms = 0) {
  const AxisPlan& ap = p->ax_x;
  using UR = typename P::UR;
  if (p->use_pipe && ap.pipe_ok) {
    const long long us = sizeof(UR);
    int chunk = (int)us;
    if ((x.nx * us) % 16 == 0 && (x.in_field * us) % 16 == 0 && aligned_to(x.in, 16)) chunk = 16;
    else if ((x.nx * us) % 8 == 0 && (x.in_field * us) % 8 == 0 && aligned_to(x.in, 8)) chunk = 8;
    x.M = ap.pipe_m;
    x.log2m = ap.pipe_log2m;
    x.LS = ap.pipe_ls();
    x.ps = ap.pipe_ps();
    x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;
    XPipeParams xp{};
    xp.x = x;
    xp.chunk = chunk;
    xp.c.tiles_per_field = x.tiles;
    xp.c.ntiles = x.tiles * nv;
    xp.c.tw_base = ap.pipe_tw_lo();
    xp.c.tw_count = ap.pipe_tw_cnt();
    xp.c.buf_elems = ap.buf_elems;
    xp.c.nbuf = ap.pipe_nbuf;
    xp.c.err = p->d_err;
    // the tile's 2M real lines are one contiguous run of device memory
    xp.bulk = x.in_line == x.nx && (x.nx * us) % 16 == 0 && (x.in_field * us) % 16 == 0 && aligned_to(x.in, 16) &&
              device_memory(x.in);
    const int slots = (max_sms > 0 && max_sms < p->sm_count ? max_sms : p->sm_count) * ap.pipe_bps;
    const int grid = xp.c.ntiles < slots ? xp.c.ntiles : slots;
    cudaError_t e = launch_xr2c_pipe<P>(xp, p->d_sp + ap.pipe_sp(), p->d_tw, ap.pipe_e, ap.pipe_threads,
                                        ap.pipe_smem, grid, st);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("X r2c launch: ") + cudaGetErrorString(e));
    p->launches++;
    return P3G_OK;
  }
  cudaError_t e = launch_x_r2c<P>(x, p->d_sp + ap.sp_index, p->d_tw, ap.threads, ap.smem, nv, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("X r2c launch: ") + cudaGetErrorString(e));
  p->launches++;
  return P3G_OK;
}

template <class P>
int run_x_c2r(p3g_plan p, XParams& x, int nv, cudaStream_t st, int max_sms = 0) {
  const AxisPlan& ap = p->ax_xc;
  if (p->use_pipe && ap.pipe_ok) {
    x.M = ap.pipe_m;
    x.log2m = ap.pipe_log2m;
    x.LS = ap.pipe_ls();
    x.ps = ap.pipe_ps();
    x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;
    XPipeParams xp{};
    xp.x = x;
    xp.chunk = (int)sizeof(typename P::W);
    xp.c.tiles_per_field = x.tiles;
    xp.c.ntiles = x.tiles * nv;
    xp.c.tw_base = ap.pipe_tw_lo();
    xp.c.tw_count = ap.pipe_tw_cnt();
    xp.c.buf_elems = ap.buf_elems;
    xp.c.nbuf = ap.pipe_nbuf;
    xp.c.err = p->d_err;
    {
      // every mode of a line arrives by one bulk copy of its nh complexes
      // rounded up to 16 bytes, which the line pitch and the raw stride hold
      const long long es = (long long)sizeof(typename P::W);
      const int nh = x.nx / 2 + 1;
      xp.bulk = x.nkeep == nh && (x.in_line * es) % 16 == 0 && (x.in_field * es) % 16 == 0 &&
                (long long)x.in_line * es >= ((nh * es + 15) / 16) * 16 && aligned_to(x.in, 16) &&
                device_memory(x.in);
    }
    const int slots = (max_sms > 0 && max_sms < p->sm_count ? max_sms : p->sm_count) * ap.pipe_bps;
    const int grid = xp.c.ntiles < slots ? xp.c.ntiles : slots;
    cudaError_t e = launch_xc2r_pipe<P>(xp, p->d_sp + ap.pipe_sp(), p->d_tw, ap.pipe_e, ap.pipe_threads,
                                        ap.pipe_smem, grid, st);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("X c2r launch: ") + cudaGetErrorString(e));
    p->launches++;
    return P3G_OK;
  }
  cudaError_t e = launch_x_c2r<P>(x, p->d_sp + ap.sp_index, p->d_tw, ap.threads, ap.smem, nv, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("X c2r launch: ") + cudaGetErrorString(e));
  p->launches++;
  return P3G_OK;
}

// A Y or Z pass on lines longer than one tile, as two strided launches
// through the scratch wc (four-step, n = n1 n2, j = j1 + n1 j2, k = k2 + n2 k1):
// the first transforms each j1's subsequence j2 (length n2, rows n1 apart),
// multiplies the result by w_n^(j1 k2) on its store and writes wc as
// [field o1][k2][j1][x]; the second transforms each k2's row of j1 (length
// n1) and stores output index k2 + n2 k1.  s is the one-launch pass (identity
// load and store maps, no DCT/DST extension); its fields run one after another.
template <class P>
int run_four(p3g_plan p, const SParams& s, AxisPlan* sub, int tw4, bool fwd_sign, int nv, cudaStream_t st,
             int max_sms = 0, long long Pw = 0) {
  const int n2 = sub[0].n, n1 = sub[1].n;
  const long long N = (long long)n1 * n2;
  if (Pw <= 0) Pw = p->pitch;  // scratch row pitch (at least s.X)
  const size_t es = p->esize();
  for (int f = 0; f < nv; ++f) {
    const char* in = static_cast<const char*>(s.in) + (size_t)f * s.in_o2 * es;
    char* out = static_cast<char*>(s.out) + (size_t)f * s.out_o2 * es;
    SParams a{};
    a.in = in;
    a.in_user = s.in_user;
    a.in_xs = s.in_xs;
    a.in_axis = (int)(n1 * (long long)s.in_axis);
    a.in_o1 = s.in_axis;
    a.in_o2 = s.in_o1;
    a.out = p->wc;
    a.out_xs = 1;
    a.out_axis = (int)(n1 * Pw);
    a.out_o1 = Pw;
    a.out_o2 = N * Pw;
    a.X = s.X;
    a.O1 = n1;
    a.L = a.N = a.Lout = n2;
    a.lmap_a0 = a.lmap_a1 = n2;
    a.smap_s0 = n2;
    a.xphase = s.xphase;
    a.range = s.range;
    a.tw4 = p->d_tw + tw4;
    a.tw4_n = (int)N;
    a.tw4_conj = fwd_sign ? 0 : 1;
    int rc = run_strided<P>(p, a, sub[0], fwd_sign, s.O1, st, max_sms);
    if (rc) return rc;
    SParams b{};
    b.in = p->wc;
    b.in_xs = 1;
    b.in_axis = (int)Pw;
    b.in_o1 = n1 * Pw;
    b.in_o2 = N * Pw;
    b.out = out;
    b.out_user = s.out_user;
    b.out_xs = s.out_xs;
    b.out_axis = (int)(n2 * (long long)s.out_axis);
    b.out_o1 = s.out_axis;
    b.out_o2 = s.out_o1;
    b.X = s.X;
    b.O1 = n2;
    b.L = b.N = b.Lout = n1;
    b.lmap_a0 = b.lmap_a1 = n1;
    b.smap_s0 = n1;
    b.range = s.range;
    rc = run_strided<P>(p, b, sub[1], fwd_sign, s.O1, st, max_sms);
    if (rc) return rc;
  }
  return P3G_OK;
}

// The Y pass or the Z pass of a direction, one launch or four-step.
template <class P>
int run_y(p3g_plan p, SParams& y, bool fwd_sign, int nv, cudaStream_t st, int max_sms = 0) {
  if (p->four_y) return run_four<P>(p, y, p->ly, p->tw4_y, fwd_sign, nv, st, max_sms);
  return run_strided<P>(p, y, p->ax_y, fwd_sign, nv, st, max_sms);
}
template <class P>
int run_z(p3g_plan p, SParams& z, int zi, bool fwd_sign, int nv, cudaStream_t st) {
  if (zi == 0 && p->four_z) return run_four<P>(p, z, p->lz, p->tw4_z, fwd_sign, nv, st);
  return run_strided<P>(p, z, p->ax_z[zi], fwd_sign, nv, st);
}

// Long X lines: the pair buffer wd as a strided pass over pairs (columns,
// nx apart) along x (rows, adjacent), transformed in place by run_four.
SParams x_long_pass(p3g_plan p, int nlines) {
  SParams s{};
  s.in = s.out = p->wd;
  s.in_xs = s.out_xs = p->nx;
  s.in_axis = s.out_axis = 1;
  s.X = (nlines + 1) / 2;
  s.O1 = 1;
  s.L = s.N = s.Lout = p->nx;
  s.lmap_a0 = s.lmap_a1 = p->nx;
  s.smap_s0 = p->nx;
  return s;
}
int x_long(p3g_plan p, int kind, const XLongParams& q, cudaStream_t st) {
  const cudaError_t e = p->prec == P3G_F64 ? launch_x_long<PathF64>(kind, q, p->sm_count, st)
                                           : launch_x_long<PathF32>(kind, q, p->sm_count, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("long X line launch: ") + cudaGetErrorString(e));
  p->launches++;
  return P3G_OK;
}

// The X passes of a direction, one launch or (lines longer than one tile)
// pack / four-step / split per field.
template <class P>
int run_xr2c(p3g_plan p, XParams& x, int nv, cudaStream_t st, int max_sms = 0) {
  if (!p->four_x) return run_x_r2c<P>(p, x, nv, st, max_sms);
  const size_t ur = sizeof(typename P::UR), es = p->esize();
  for (int f = 0; f < nv; ++f) {
    XLongParams q{};
    q.in = static_cast<const char*>(x.in) + (size_t)f * x.in_field * ur;
    q.out = p->wd;
    q.in_line = x.in_line;
    q.nlines = x.nlines;
    q.nx = x.nx;
    q.nkeep = x.nkeep;
    q.range = x.range;
    int rc = x_long(p, 0, q, st);
    if (rc) return rc;
    SParams s = x_long_pass(p, x.nlines);
    if ((rc = run_four<P>(p, s, p->lx, p->tw4_x, true, 1, st, max_sms, p->xpitch()))) return rc;
    q.in = p->wd;
    q.out = static_cast<char*>(x.out) + (size_t)f * x.out_field * es;
    q.out_line = x.out_line;
    q.out_user = x.out_user;
    if ((rc = x_long(p, 1, q, st))) return rc;
  }
  return P3G_OK;
}
template <class P>
int run_xc2r(p3g_plan p, XParams& x, int nv, cudaStream_t st, int max_sms = 0) {
  if (!p->four_x) return run_x_c2r<P>(p, x, nv, st, max_sms);
  const size_t ur = sizeof(typename P::UR), es = p->esize();
  for (int f = 0; f < nv; ++f) {
    XLongParams q{};
    q.in = static_cast<const char*>(x.in) + (size_t)f * x.in_field * es;
    q.out = p->wd;
    q.in_line = x.in_line;
    q.nlines = x.nlines;
    q.nx = x.nx;
    q.nkeep = x.nkeep;
    int rc = x_long(p, 2, q, st);
    if (rc) return rc;
    SParams s = x_long_pass(p, x.nlines);
    if ((rc = run_four<P>(p, s, p->lx, p->tw4_x, false, 1, st, max_sms, p->xpitch()))) return rc;
    q.in = p->wd;
    q.out = static_cast<char*>(x.out) + (size_t)f * x.out_field * ur;
    q.out_line = x.out_line;
    q.range = x.range;
    if ((rc = x_long(p, 3, q, st))) return rc;
  }
  return P3G_OK;
}

}  // namespace

namespace p3g {

// Largest |high word| (sign cleared) of nv binary64 fields into *out.
__global__ void __launch_bounds__(256) k_range_scan(const double* __restrict__ in, long long n, long long field,
                                                    unsigned* out) {
  const double* f = in + blockIdx.y * field;
  uint32_t m = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if ((reinterpret_cast<uintptr_t>(f) & 15) == 0) {
    const double2* f2 = reinterpret_cast<const double2*>(f);
    for (; i < n / 2; i += stride) {
      const double2 v = __ldcs(f2 + i);
      m = max(m, (uint32_t)__double2hiint(v.x) & 0x7FFFFFFFu);
      m = max(m, (uint32_t)__double2hiint(v.y) & 0x7FFFFFFFu);
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) m = max(m, (uint32_t)__double2hiint(f[n - 1]) & 0x7FFFFFFFu);
  } else {
    for (; i < n; i += stride) m = max(m, (uint32_t)__double2hiint(__ldcs(f + i)) & 0x7FFFFFFFu);
  }
  m = __reduce_max_sync(0xFFFFFFFFu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

RangeParams range_params(p3g_plan p, bool input, bool allow_auto) {
  RangeParams r{};
  if (p->prec != P3G_F64) return r;
  r.track = input ? reinterpret_cast<unsigned*>(p->d_err + 1) : nullptr;
  r.auto_max = allow_auto && p->range_mode == P3G_RANGE_AUTO ? reinterpret_cast<const unsigned*>(p->d_err + 2)
                                                             : nullptr;
  r.bias = p->ebias;
  r.log2n = p->log2n;
  return r;
}

int launch_range_scan(p3g_plan p, const void* in, long long n, long long field, int nv, cudaStream_t st) {
  if (p->prec != P3G_F64 || p->range_mode != P3G_RANGE_AUTO) return P3G_OK;
  cudaError_t e = cudaMemsetAsync(p->d_err + 2, 0, sizeof(int), st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("range scan: ") + cudaGetErrorString(e));
  const long long want = (n / 2 + 255) / 256;
  const int gx = (int)std::max(1LL, std::min(want, (long long)p->sm_count * 8 / std::max(1, nv) + 1));
  k_range_scan<<<dim3(gx, nv), 256, 0, st>>>(static_cast<const double*>(in), n, field,
                                               reinterpret_cast<unsigned*>(p->d_err + 2));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("range scan launch: ") + cudaGetErrorString(e));
  p->launches++;
  return P3G_OK;
}

// Pass parameters of a forward transform: X r2c user real -> wa, Y wa ->
// wb ([y][z][x]) keeping y modes 0..nycph-1 and the top
// nyc-nycph (seg_copy_y, ftran.F90:736-738), Z ybuf -> user complex with the
// Z op and z pruning (seg_copy_z, ftran.F90:705-706).
void make_forward_params(p3g_plan p, const void* in, void* out, void* wa, void* wb, int zi, long long dim_in,
                         long long dim_out, XParams& x, SParams& y, SParams& z, bool y_zyx) {
  const long long P_ = p->pitch;
  const long long wa_field = (long long)p->nz * p->ny * P_;
  const long long wb_field = (long long)p->nz * p->nyc * P_;
  // the Y output: wb as [y][z][x], or (y_zyx) [z][y][x] in wa itself unless
  // y is pruned
  void* ybuf = y_zyx && p->nyc == p->ny ? wa : wb;
  const long long y_field = y_zyx && p->nyc == p->ny ? wa_field : wb_field;
  x = XParams{};
  x.in = in;
  x.out = wa;
  x.in_field = dim_in;
  x.out_field = wa_field;
  x.in_line = p->nx;
  x.out_line = (int)P_;
  x.nlines = p->ny * p->nz;
  x.nx = p->nx;
  x.nkeep = p->nxhpc;
  x.M = p->ax_x.M;
  x.log2m = p->ax_x.log2m;
  x.LS = p->ax_x.ls;
  x.ps = p->ax_x.ps;
  x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;

  y = SParams{};
  y.in_xs = y.out_xs = 1;
  y.in = wa;
  y.out = ybuf;
  y.in_axis = (int)P_;
  y.in_o1 = (long long)p->ny * P_;
  y.in_o2 = wa_field;
  // the Y output (Z input) is stored [y][z][x]: the Z pass then reads its
  // lines at a stride of one row (pitch) instead of a whole plane, and the
  // scattered accesses move to the Y pass's stores
  y.out_axis = (int)(y_zyx ? P_ : p->nz * P_);
  y.out_o1 = y_zyx ? (long long)p->nyc * P_ : P_;
  y.out_o2 = y_field;
  y.X = p->nxhpc;
  y.O1 = p->nz;
  y.L = p->ny;
  y.Lout = p->nyc;
  y.lmap_a0 = p->ny;
  y.lmap_a1 = p->ny;
  y.smap_s0 = p->nycph;
  y.smap_d = p->ny - p->nyc;
  y.M = p->ax_y.M;
  y.log2m = p->ax_y.log2m;
  y.N = p->ax_y.n;
  y.xtiles = (y.X + y.M - 1) / y.M;

  const AxisPlan& az = p->ax_z[zi];
  z = SParams{};
  z.in_xs = z.out_xs = 1;
  z.in = ybuf;
  z.out = out;
  z.out_user = 1;
  z.in_axis = (int)(y_zyx ? p->nyc * P_ : P_);
  z.in_o1 = y_zyx ? P_ : (long long)p->nz * P_;
  z.in_o2 = y_field;
  if (p->layout == P3G_LAYOUT_STRIDE1) {  // (nzc, nyc, nxhpc), z fastest (module.F90:245-254)
    z.out_axis = 1;
    z.out_o1 = p->nzc;
    z.out_xs = p->nyc * p->nzc;
  } else {
    z.out_axis = p->nxhpc * p->nyc;
    z.out_o1 = p->nxhpc;
  }
  z.out_o2 = dim_out;
  z.X = p->nxhpc;
  z.O1 = p->nyc;
  z.L = p->nz;
  z.Lout = p->nzc;
  z.pre = zi == 1 ? 1 : (zi == 2 ? 2 : 0);
  z.post = zi == 2 ? 1 : 0;
  z.lmap_a0 = p->nz;
  z.lmap_a1 = p->nz;
  z.smap_s0 = p->nzcph;
  z.smap_d = p->nz - p->nzc;
  z.M = az.M;
  z.log2m = az.log2m;
  z.N = az.n;
  z.xtiles = (z.X + z.M - 1) / z.M;
}

// Pass parameters of a backward transform: Z user complex -> zbuf ([y][z][x]
// in wb; y_zyx: [z][y][x], in wa unless y is pruned) with the z zero fill
// (seg_copy_z + seg_zero_z, btran.F90:553-555), Y zbuf -> wa with the y zero
// fill (seg_copy_y + seg_zero_y, btran.F90:585-588), X c2r wa -> user real
// with x modes beyond nxhpc read as zero (seg_zero_x, btran.F90:662-663).
void make_backward_params(p3g_plan p, const void* in, void* out, void* wa, void* wb, int zi, long long dim_in,
                          long long dim_out, SParams& z, SParams& y, XParams& x, bool y_zyx) {
  const long long P_ = p->pitch;
  const long long wa_field = (long long)p->nz * p->ny * P_;
  const long long wb_field = (long long)p->nz * p->nyc * P_;
  const bool in_wa = y_zyx && p->nyc == p->ny;
  void* zbuf = in_wa ? wa : wb;
  const long long z_field = in_wa ? wa_field : wb_field;
  const AxisPlan& az = p->ax_z[zi];
  z = SParams{};
  z.in_xs = z.out_xs = 1;
  z.in = in;
  z.out = zbuf;
  z.in_user = 1;
  if (p->layout == P3G_LAYOUT_STRIDE1) {
    z.in_axis = 1;
    z.in_o1 = p->nzc;
    z.in_xs = p->nyc * p->nzc;
  } else {
    z.in_axis = p->nxhpc * p->nyc;
    z.in_o1 = p->nxhpc;
  }
  z.in_o2 = dim_in;
  // binary32 complex rows of nxhpc modes start at odd elements for odd nxhpc
  z.xphase = p->prec == P3G_F32 && z.in_xs == 1;
  // the Z output (Y input) as [y][z][x]: the Z pass stores each line one
  // pitch apart, so only its user-format reads are a plane apart
  z.out_axis = (int)(y_zyx ? p->nyc * P_ : P_);
  z.out_o1 = y_zyx ? P_ : (long long)p->nz * P_;
  z.out_o2 = z_field;
  z.X = p->nxhpc;
  z.O1 = p->nyc;
  z.L = p->nz;
  z.Lout = p->nz;
  z.pre = zi == 1 ? 1 : (zi == 2 ? 2 : 0);
  z.post = zi == 2 ? 1 : 0;
  z.lmap_a0 = p->nzcph;
  z.lmap_a1 = p->nz - p->nzcph;
  z.lmap_d = p->nz - p->nzc;
  z.smap_s0 = p->nz;
  z.M = az.M;
  z.log2m = az.log2m;
  z.N = az.n;
  z.xtiles = (z.X + z.M - 1) / z.M;

  y = SParams{};
  y.in_xs = y.out_xs = 1;
  y.in = zbuf;
  y.out = wa;
  y.in_axis = (int)(y_zyx ? P_ : p->nz * P_);
  y.in_o1 = y_zyx ? (long long)p->nyc * P_ : P_;
  y.in_o2 = z_field;
  y.out_axis = (int)P_;
  y.out_o1 = (long long)p->ny * P_;
  y.out_o2 = wa_field;
  y.X = p->nxhpc;
  y.O1 = p->nz;
  y.L = p->ny;
  y.Lout = p->ny;
  y.lmap_a0 = p->nycph;
  y.lmap_a1 = p->ny - p->nycph;
  y.lmap_d = p->ny - p->nyc;
  y.smap_s0 = p->ny;
  y.M = p->ax_y.M;
  y.log2m = p->ax_y.log2m;
  y.N = p->ax_y.n;
  y.xtiles = (y.X + y.M - 1) / y.M;

  x = XParams{};
  x.in = wa;
  x.out = out;
  x.in_field = wa_field;
  x.out_field = dim_out;
  x.in_line = (int)P_;
  x.out_line = p->nx;
  x.nlines = p->ny * p->nz;
  x.nx = p->nx;
  x.nkeep = p->nxhpc;
  x.M = p->ax_x.M;
  x.log2m = p->ax_x.log2m;
  x.LS = p->ax_x.ls;
  x.ps = p->ax_x.ps;
  x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;
}

}  // namespace p3g

namespace {

template <class P>
int do_ftran(p3g_plan p, const void* in, void* out, const char* op, int nv, long long dim_in, long long dim_out,
             cudaStream_t st) {
  bool fsign = true;
  const int zi = op_index(op[2], fsign, true);
  if (zi < 0) return fail(P3G_E_ARG, std::string("Unknown transform type: ") + op[2]);
  if (!p->z_ok[zi]) return fail(P3G_E_UNSUPPORTED, std::string("Z transform '") + op[2] + "' unsupported for nz");
  int rc = ensure_workspace(p, nv);
  if (rc) return rc;
  XParams x;
  SParams y, z;
  make_forward_params(p, in, out, p->wa, p->wb, zi, dim_in, dim_out, x, y, z);
  x.range = range_params(p, true, true);
  z.range = range_params(p, false, true);
  if ((rc = launch_range_scan(p, in, (long long)p->nx * p->ny * p->nz, dim_in, nv, st))) return rc;
  {
    PassTimer tm(p, 4, st);
    if ((rc = run_xr2c<P>(p, x, nv, st))) return rc;
    tm.done();
  }
  {
    PassTimer tm(p, 6, st);
    if ((rc = run_y<P>(p, y, true, nv, st))) return rc;
    tm.done();
  }
  {
    PassTimer tm(p, 7, st);
    if ((rc = run_z<P>(p, z, zi, fsign, nv, st))) return rc;
    tm.done();
  }
  return P3G_OK;
}

template <class P>
int do_btran(p3g_plan p, const void* in, void* out, const char* op, int nv, long long dim_in, long long dim_out,
             cudaStream_t st) {
  bool fsign = false;
  const int zi = op_index(op[0], fsign, false);
  if (zi < 0) return fail(P3G_E_ARG, std::string("Unknown transform type: ") + op[0]);
  if (!p->z_ok[zi]) return fail(P3G_E_UNSUPPORTED, std::string("Z transform '") + op[0] + "' unsupported for nz");
  int rc = ensure_workspace(p, nv);
  if (rc) return rc;
  SParams z, y;
  XParams x;
  make_backward_params(p, in, out, p->wa, p->wb, zi, dim_in, dim_out, z, y, x);
  z.range = range_params(p, true, true);
  x.range = range_params(p, false, true);
  if ((rc = launch_range_scan(p, in, 2LL * p->nxhpc * p->nyc * p->nzc, 2 * dim_in, nv, st))) return rc;
  {
    PassTimer tm(p, 8, st);
    if ((rc = run_z<P>(p, z, zi, fsign, nv, st))) return rc;
    tm.done();
  }
  {
    PassTimer tm(p, 9, st);
    if ((rc = run_y<P>(p, y, false, nv, st))) return rc;
    tm.done();
  }
  {
    PassTimer tm(p, 11, st);
    if ((rc = run_xc2r<P>(p, x, nv, st))) return rc;
    tm.done();
  }
  return P3G_OK;
}

// Row blocks of the Z pass: block c covers y in [c*nyc/K, (c+1)*nyc/K).
struct RowBlock {
  int y0, y1;
};
std::vector<RowBlock> row_blocks(int nyc, int chunks) {
  std::vector<RowBlock> r;
  if (chunks < 1) chunks = 1;
  if (chunks > nyc) chunks = nyc;
  for (int c = 0; c < chunks; ++c)
    r.push_back({(int)((long long)c * nyc / chunks), (int)((long long)(c + 1) * nyc / chunks)});
  return r;
}

// The Z pass of rows [y0, y1): the same parameters with shifted bases.
SParams z_rows(const SParams& z, int y0, int y1, size_t esize) {
  SParams c = z;
  c.O1 = y1 - y0;
  c.in = static_cast<const unsigned char*>(z.in) + (size_t)y0 * z.in_o1 * esize;
  c.out = static_cast<unsigned char*>(z.out) + (size_t)y0 * z.out_o1 * esize;
  return c;
}

struct EventSet {
  std::vector<cudaEvent_t> ev;
  explicit EventSet(size_t n) : ev(n, nullptr) {
    for (auto& e : ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  }
  ~EventSet() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// z-slabs of the X and Y passes: slab c covers planes [c*nz/K, (c+1)*nz/K).
XParams x_planes(const XParams& x, int ny, int z0, int z1, size_t in_es, size_t out_es) {
  XParams s = x;
  s.in = static_cast<const unsigned char*>(x.in) + (size_t)z0 * ny * x.in_line * in_es;
  s.out = static_cast<unsigned char*>(x.out) + (size_t)z0 * ny * x.out_line * out_es;
  s.nlines = ny * (z1 - z0);
  s.tiles = ((s.nlines + 1) / 2 + s.M - 1) / s.M;
  return s;
}
SParams y_planes(const SParams& y, int z0, int z1, size_t es) {
  SParams s = y;
  s.O1 = z1 - z0;
  s.in = static_cast<const unsigned char*>(y.in) + (size_t)z0 * y.in_o1 * es;
  s.out = static_cast<unsigned char*>(y.out) + (size_t)z0 * y.out_o1 * es;
  return s;
}

int aux_stream(p3g_plan p, cudaStream_t& aux) {
  if (!p->aux && cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    p->aux = nullptr;
    return fail(P3G_E_CUDA, "stream creation failed");
  }
  aux = p->aux;
  return P3G_OK;
}

// When the real array lives in host memory the X pass is bound by the host
// link, not by the SMs: the X and Y passes then run in z-slabs on two
// streams, the X pass of slab k+1 (on a third of the SMs) reading the host
// while the Y pass of slab k computes on the rest.
constexpr int kZSlabs = 8;

// Forward transform into a host array: X and Y passes, then the Z pass in row
// blocks, each block's output copied to the host on cs while the next block
// computes.
template <class P>
int do_ftran_to_host(p3g_plan p, const void* in, void* out_host, void* stage, const char* op, int chunks,
                     cudaStream_t st, cudaStream_t cs) {
  bool fsign = true;
  const int zi = op_index(op[2], fsign, true);
  if (zi < 0) return fail(P3G_E_ARG, std::string("Unknown transform type: ") + op[2]);
  if (!p->z_ok[zi]) return fail(P3G_E_UNSUPPORTED, std::string("Z transform '") + op[2] + "' unsupported for nz");
  int rc = ensure_workspace(p, 1);
  if (rc) return rc;
  const long long rsize = (long long)p->nx * p->ny * p->nz;
  const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
  XParams x;
  SParams y, z;
  make_forward_params(p, in, stage, p->wa, p->wb, zi, rsize, csize, x, y, z);
  x.range = range_params(p, true, true);
  z.range = range_params(p, false, true);
  if ((rc = launch_range_scan(p, in, rsize, rsize, 1, st))) return rc;
  const size_t es = p->esize();
  if (!device_memory(in) && p->nz >= 2) {
    cudaStream_t aux;
    if ((rc = aux_stream(p, aux))) return rc;
    const int x_sms = std::max(1, p->sm_count / 3), y_sms = p->sm_count - x_sms;
    const auto slabs = row_blocks(p->nz, kZSlabs);
    EventSet ev(slabs.size() + 2);
    cudaError_t e = cudaEventRecord(ev.ev[0], st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev.ev[0], 0);
    for (size_t k = 0; k < slabs.size() && e == cudaSuccess; ++k) {
      XParams xs = x_planes(x, p->ny, slabs[k].y0, slabs[k].y1, sizeof(typename P::UR), es);
      {
        PassTimer tm(p, 4, st);
        if ((rc = run_xr2c<P>(p, xs, 1, st, x_sms))) return rc;
        tm.done();
      }
      e = cudaEventRecord(ev.ev[k + 1], st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev.ev[k + 1], 0);
      if (e != cudaSuccess) break;
      SParams ys = y_planes(y, slabs[k].y0, slabs[k].y1, es);
      PassTimer tm(p, 6, aux);
      if ((rc = run_y<P>(p, ys, true, 1, aux, y_sms))) return rc;
      tm.done();
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev.ev[slabs.size() + 1], aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev.ev[slabs.size() + 1], 0);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("stream order: ") + cudaGetErrorString(e));
  } else {
    {
      PassTimer tm(p, 4, st);
      if ((rc = run_xr2c<P>(p, x, 1, st))) return rc;
      tm.done();
    }
    {
      PassTimer tm(p, 6, st);
      if ((rc = run_y<P>(p, y, true, 1, st))) return rc;
      tm.done();
    }
  }
  const auto blocks = row_blocks(p->nyc, chunks);
  EventSet evs(blocks.size());
  const size_t pitch = (size_t)p->nyc * p->nxhpc * es;
  for (size_t c = 0; c < blocks.size(); ++c) {
    const int y0 = blocks[c].y0, y1 = blocks[c].y1;
    SParams zc = z_rows(z, y0, y1, es);
    {
      PassTimer tm(p, 7, st);
      if ((rc = run_z<P>(p, zc, zi, fsign, 1, st))) return rc;
      tm.done();
    }
    cudaError_t e = cudaEventRecord(evs.ev[c], st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, evs.ev[c], 0);
    const size_t off = (size_t)y0 * p->nxhpc * es;
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(static_cast<unsigned char*>(out_host) + off, pitch,
                            static_cast<const unsigned char*>(stage) + off, pitch, (size_t)(y1 - y0) * p->nxhpc * es,
                            p->nzc, cudaMemcpyDeviceToHost, cs);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("device to host copy: ") + cudaGetErrorString(e));
  }
  return P3G_OK;
}

// Backward transform from a host array: the input is copied in row blocks on
// cs and the Z pass of each block starts as soon as its copy has landed; then
// the Y and X passes.
template <class P>
int do_btran_from_host(p3g_plan p, const void* in_host, void* stage, void* out, const char* op, int chunks,
                       cudaStream_t st, cudaStream_t cs) {
  bool fsign = false;
  const int zi = op_index(op[0], fsign, false);
  if (zi < 0) return fail(P3G_E_ARG, std::string("Unknown transform type: ") + op[0]);
  if (!p->z_ok[zi]) return fail(P3G_E_UNSUPPORTED, std::string("Z transform '") + op[0] + "' unsupported for nz");
  int rc = ensure_workspace(p, 1);
  if (rc) return rc;
  const long long rsize = (long long)p->nx * p->ny * p->nz;
  const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
  SParams z, y;
  XParams x;
  make_backward_params(p, stage, out, p->wa, p->wb, zi, csize, rsize, z, y, x);
  z.range = range_params(p, true, true);
  x.range = range_params(p, false, true);
  // the auto bias needs the whole input's largest magnitude before the first
  // block's Z pass: measured on the host array itself
  if ((rc = launch_range_scan(p, in_host, 2 * csize, 2 * csize, 1, st))) return rc;
  const size_t es = p->esize();
  const auto blocks = row_blocks(p->nyc, chunks);
  EventSet evs(blocks.size());
  const size_t pitch = (size_t)p->nyc * p->nxhpc * es;
  // the copies must not overwrite the stage while earlier work on st reads it
  EventSet start(1);
  cudaError_t e = cudaEventRecord(start.ev[0], st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, start.ev[0], 0);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("stream order: ") + cudaGetErrorString(e));
  for (size_t c = 0; c < blocks.size(); ++c) {
    const int y0 = blocks[c].y0, y1 = blocks[c].y1;
    const size_t off = (size_t)y0 * p->nxhpc * es;
    e = cudaMemcpy2DAsync(static_cast<unsigned char*>(stage) + off, pitch,
                          static_cast<const unsigned char*>(in_host) + off, pitch, (size_t)(y1 - y0) * p->nxhpc * es,
                          p->nzc, cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaEventRecord(evs.ev[c], cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, evs.ev[c], 0);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("host to device copy: ") + cudaGetErrorString(e));
    SParams zc = z_rows(z, y0, y1, es);
    PassTimer tm(p, 8, st);
    if ((rc = run_z<P>(p, zc, zi, fsign, 1, st))) return rc;
    tm.done();
  }
  if (!device_memory(out) && p->nz >= 2) {
    // host output: the Y pass of slab k+1 computes while the X pass of slab k
    // writes its lines over the host link
    cudaStream_t aux;
    if ((rc = aux_stream(p, aux))) return rc;
    const int x_sms = std::max(1, p->sm_count / 3), y_sms = p->sm_count - x_sms;
    const auto slabs = row_blocks(p->nz, kZSlabs);
    EventSet ev(slabs.size() + 1);
    for (size_t k = 0; k < slabs.size() && e == cudaSuccess; ++k) {
      SParams ys = y_planes(y, slabs[k].y0, slabs[k].y1, es);
      {
        PassTimer tm(p, 9, st);
        if ((rc = run_y<P>(p, ys, false, 1, st, y_sms))) return rc;
        tm.done();
      }
      e = cudaEventRecord(ev.ev[k], st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev.ev[k], 0);
      if (e != cudaSuccess) break;
      XParams xs = x_planes(x, p->ny, slabs[k].y0, slabs[k].y1, es, sizeof(typename P::UR));
      PassTimer tm(p, 11, aux);
      if ((rc = run_xc2r<P>(p, xs, 1, aux, x_sms))) return rc;
      tm.done();
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev.ev[slabs.size()], aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev.ev[slabs.size()], 0);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("stream order: ") + cudaGetErrorString(e));
    return P3G_OK;
  }
  {
    PassTimer tm(p, 9, st);
    if ((rc = run_y<P>(p, y, false, 1, st))) return rc;
    tm.done();
  }
  {
    PassTimer tm(p, 11, st);
    if ((rc = run_xc2r<P>(p, x, 1, st))) return rc;
    tm.done();
  }
  return P3G_OK;
}

bool valid_op(const char* op) { return op && op[0] && op[1] && op[2]; }

}  // namespace

namespace p3g {
// p3g_plan_check_range on words w copied from the plan's d_err.
int plan_range_result(p3g_plan p, const int w[3], int* bias, int* emax) {
  const uint32_t amax = (uint32_t)w[1];
  const int ebits = (int)(amax >> 20);
  if (emax) *emax = ebits == 0 ? -1075 : ebits - 1023;
  const int need = range_bias(amax, p->log2n);
  if (bias) *bias = need;
  if (p->prec != P3G_F64 || p->range_mode == P3G_RANGE_AUTO || ebits == 0 || ebits == 2047) return P3G_OK;
  // inside the window at the plan's bias?
  const int E = ebits - 1023 - p->ebias;
  if (E >= kRangeLo && E <= kRangeTop - p->log2n) return P3G_OK;
  return fail(P3G_E_RANGE, "F64 transform input of largest magnitude 2^" + std::to_string(ebits - 1023) +
                               " is outside the exponent window at bias " + std::to_string(p->ebias) +
                               " (results invalid): call again after p3g_plan_set_range(plan, P3G_RANGE_FIXED, " +
                               std::to_string(need) + ") or with P3G_RANGE_AUTO");
}
}  // namespace p3g

extern "C" {

int p3g_version(void) { return 100; }

const char* p3g_last_error(void) { return g_last_error.c_str(); }

int p3g_plan_create(p3g_plan* out, int nx, int ny, int nz, int nxc, int nyc, int nzc, int precision, int layout,
                    int flags) {
  return p3g_plan_create_tuned(out, nx, ny, nz, nxc, nyc, nzc, precision, layout, flags, 0, 0);
}

int p3g_plan_create_tuned(p3g_plan* out, int nx, int ny, int nz, int nxc, int nyc, int nzc, int precision,
                          int layout, int flags, int max_radix, int max_lines) {
  if (!out) return fail(P3G_E_ARG, "plan pointer is NULL");
  if (max_radix != 0 && max_radix != 2 && max_radix != 4 && max_radix != 8 && max_radix != 16 &&
      !(max_radix == 32 && precision == P3G_F32))
    return fail(P3G_E_ARG, "max_radix must be 0, 2, 4, 8, 16 (or 32 on the F32 path)");
  if (max_lines < 0 || (max_lines & (max_lines - 1)) != 0)
    return fail(P3G_E_ARG, "max_lines must be 0 or a power of two");
  *out = nullptr;
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return fail(P3G_E_ARG, "Invalid dimensions : " + std::to_string(nx) + " " + std::to_string(ny) + " " +
                               std::to_string(nz));
  if (nxc <= 0) nxc = nx;
  if (nyc <= 0) nyc = ny;
  if (nzc <= 0) nzc = nz;
  if (nxc > nx || nyc > ny || nzc > nz) return fail(P3G_E_ARG, "pruned sizes must not exceed the grid");
  if (precision != P3G_F64 && precision != P3G_F32) return fail(P3G_E_ARG, "unknown precision");
  if (layout != P3G_LAYOUT_XYZ && layout != P3G_LAYOUT_STRIDE1) return fail(P3G_E_ARG, "unknown layout");
  auto* p = new p3g_plan_s();
  p->nx = nx;
  p->ny = ny;
  p->nz = nz;
  p->nxc = nxc;
  p->nyc = nyc;
  p->nzc = nzc;
  p->prec = precision;
  p->layout = layout;
  p->flags = flags;
  p->nxh = nx / 2;
  p->nxhp = p->nxh + 1;
  p->nxhc = nxc / 2;
  p->nxhpc = p->nxhc + 1;
  p->nycph = (nyc + 1) / 2;
  p->nzcph = (nzc + 1) / 2;
  std::memset(p->timers, 0, sizeof(p->timers));
  const bool f64 = precision == P3G_F64;
  const long long align = f64 ? 8 : 16;  // 128-byte workspace rows
  p->pitch = (p->nxhpc + align - 1) / align * align;

  HostTw tw;
  std::vector<StagePlan> sps;
  int strided_max_m = f64 ? 64 : 128;  // 256 words per TMA box row
  const int x_max_m = max_lines > 0 ? max_lines : (1 << 30);
  if (max_lines > 0 && max_lines < strided_max_m) strided_max_m = max_lines;
  // largest power-of-two radix: the tuner's cap, else 8 on the F64 path; on
  // F32, 32 for power-of-two lengths (their radix-32 stages run with 32
  // elements per thread) and 16 for the mixed-radix ones
  auto axis_pow2 = [&](int n) {
    if (max_radix > 0) return max_radix;
    if (f64) return 8;
    return (n & (n - 1)) == 0 ? 32 : 16;
  };
  // Every axis has a stage plan of radices up to 8 (F64) or 16 (F32) for the
  // kernels that run 8 or 16 points per thread (and the single-tile and batch
  // kernels); power-of-two lines add a wide plan for the wide pipelined
  // kernels: radix 32 on F32 (every axis), radix 16 on F64, where it pays off
  // on the Y pass only (1024 points: 8.2 -> 7.8 ms at 1024^3; the X passes'
  // 128-thread CTAs and the Z passes' user-format stores ran slower with it)
  auto wide_ok = [&](const AxisPlan& ap, int n) {
    if ((n & (n - 1)) != 0) return false;
    if (f64) return &ap == &p->ax_y && (max_radix == 0 || max_radix >= 16) && n >= 256;
    return max_radix == 0 || max_radix >= 32;
  };
  auto add_axis = [&](AxisPlan& ap, int n, int lines) -> bool {
    if (!build_stages(n, std::min(axis_pow2(n), f64 ? 8 : 16), tw, ap.sp)) return false;
    ap.tw_lo = tw.mark;
    ap.tw_cnt = (int)tw.v.size() - tw.mark;
    if (!size_tile(ap, n, lines, f64, &ap == &p->ax_x ? x_max_m : strided_max_m)) return false;
    ap.sp_index = (int)sps.size();
    sps.push_back(ap.sp);
    // the wide plan (1024 = 16 x 16 x 4 against 8 x 8 x 4 x 4 on F64, 32 x 32
    // against 16 x 16 x 4 on F32), kept when it has a wide stage
    if (wide_ok(ap, n)) {
      StagePlan w;
      if (build_stages(n, f64 ? 16 : 32, tw, w) && w.cnt[f64 ? 1 : 0] > 0) {
        ap.spw = w;
        ap.tw_lo_w = tw.mark;
        ap.tw_cnt_w = (int)tw.v.size() - tw.mark;
        ap.spw_index = (int)sps.size();
        sps.push_back(w);
      }
    }
    return true;
  };

  auto bad = [&](const std::string& m) {
    delete p;
    return fail(P3G_E_UNSUPPORTED, m);
  };
  // single per-element strides (a plane's row pitch, the Y output's row
  // stride nz*pitch, the STRIDE1 column stride nyc*nzc) are 32-bit kernel parameters;
  // offsets (their products with indices) are formed in 64 bits
  if ((long long)p->pitch * std::max(ny, nz) >= (1LL << 31) || (long long)p->nxhpc * p->nyc >= (1LL << 31) ||
      (long long)p->nyc * p->nzc >= (1LL << 31))
    return bad("a plane of more than 2^31 elements is not supported");
  const bool x_fits = add_axis(p->ax_x, nx, (ny * nz + 1) / 2);
  {
    // line padding for the X tiles (pad_index in p3g_engine.cuh): only for
    // all-power-of-two plans whose every N/R is a multiple of the first radix
    AxisPlan& ax = p->ax_x;
    const int nh2 = 2 * (nx / 2 + 1);
    auto pad_of = [&](const StagePlan& sp, int& ps, int& ls) {
      ps = 0;
      if (sp.nstages > 0 && !sp.has_generic) {
        const int r0 = sp.radix[0];
        bool ok = (r0 & (r0 - 1)) == 0 && r0 >= 4;
        for (int i = 0; ok && i < sp.nstages; ++i) {
          const int r = sp.radix[i];
          ok = (r & (r - 1)) == 0 && (nx / r) % r0 == 0;
        }
        if (ok) ps = ilog2(r0);
      }
      ls = nx + (ps ? nx >> ps : 0);
      if (ls < nh2) ls = nh2;
    };
    pad_of(ax.sp, ax.ps, ax.ls);
    if (ax.spw_index >= 0) pad_of(ax.spw, ax.ps_w, ax.ls_w);
    if (!x_fits) ax.ls = 0;
    ax.smem = (size_t)ax.M * ax.ls * (f64 ? 16 : 8) * (ax.sp.has_generic ? 2 : 1);
    if (ax.smem > 227 * 1024) {
      delete p;
      return fail(P3G_E_UNSUPPORTED, "x length " + std::to_string(nx) + " is too long");
    }
  }
  // lines longer than one tile: four-step passes, n = n1 n2 with n1 the
  // divisor nearest below sqrt(n) for which both lengths fit a tile, and the
  // n roots of unity for the twiddle between the two launches
  auto split_four = [&](AxisPlan* sub, int n, int& tw4, int lines) -> bool {
    for (int n1 = (int)std::sqrt((double)n); n1 >= 2; --n1) {
      if (n % n1) continue;
      if (!add_axis(sub[0], n / n1, lines) || !add_axis(sub[1], n1, lines)) continue;
      tw4 = (int)tw.v.size();
      for (int t = 0; t < n; ++t) tw.push_root(t, n);
      return true;
    }
    return false;
  };
  if (!add_axis(p->ax_y, ny, p->nxhpc)) {
    if (nyc != ny || !split_four(p->ly, ny, p->tw4_y, p->nxhpc))
      return bad("y length " + std::to_string(ny) + " is too long" + (nyc != ny ? " for a pruned transform" : ""));
    p->four_y = true;
  }
  p->z_ok[0] = add_axis(p->ax_z[0], nz, p->nxhpc);
  if (!p->z_ok[0] && nzc == nz && split_four(p->lz, nz, p->tw4_z, p->nxhpc)) p->z_ok[0] = p->four_z = true;
  if (!x_fits) {
    if (!split_four(p->lx, nx, p->tw4_x, (int)std::min<long long>(p->xpairs(), 1 << 30)))
      return bad("x length " + std::to_string(nx) + " is too long");
    p->four_x = true;
  }
  p->z_ok[1] = nz >= 2 && add_axis(p->ax_z[1], 2 * (nz - 1), p->nxhpc);
  p->z_ok[2] = add_axis(p->ax_z[2], 2 * (nz + 1), p->nxhpc);
  p->z_ok[3] = add_axis(p->ax_z[3], 1, p->nxhpc);
  if (p->z_ok[3]) {  // 'none': a copy pass of nz rows, no stages
    p->ax_z[3].n = nz;
    sps[p->ax_z[3].sp_index].n = nz;
    p->ax_z[3].sp.n = nz;
    if (!size_tile(p->ax_z[3], nz, p->nxhpc, f64, strided_max_m)) p->z_ok[3] = false;
  }
  if (!p->z_ok[0] && !p->z_ok[1] && !p->z_ok[3]) return bad("z length " + std::to_string(nz) + " is too long");
  // the wide kernels take fewer points per tile line set (fewer threads per
  // CTA); an axis whose wide tile does not fit runs the narrow kernels
  auto narrow_if_unfit = [&](AxisPlan& ap, int kind) {
    if (!ap.pipe_ok && ap.spw_index >= 0) {
      ap.spw_index = -1;
      size_pipe(ap, kind, f64);
    }
  };
  auto size_x = [&] {  // r2c and c2r share the tile; c2r needs the larger buffer
    size_pipe(p->ax_x, 1, f64);
    AxisPlan c2r = p->ax_x;
    size_pipe(c2r, 2, f64);
    if (!c2r.pipe_ok || c2r.pipe_threads != p->ax_x.pipe_threads || c2r.pipe_m != p->ax_x.pipe_m)
      p->ax_x.pipe_ok = false;
    p->ax_x.buf_elems = c2r.buf_elems;
    p->ax_x.pipe_smem = c2r.pipe_smem;
    p->ax_x.pipe_nbuf = c2r.pipe_nbuf;
  };
  size_x();
  if (!p->ax_x.pipe_ok && p->ax_x.spw_index >= 0) {
    p->ax_x.spw_index = -1;
    size_x();
  }
  // the X c2r pass: the same kernel shape, except on the F32 path, whose
  // c2r pass runs the 16-point kernel (1024^3: 3.01 -> 2.80 ms; the r2c pass
  // is faster with the radix-32 one, 2.56 against 2.72 ms)
  p->ax_xc = p->ax_x;
  if (!f64 && p->ax_xc.spw_index >= 0) {
    // and in CTAs of at most 128 threads, six per SM, for power-of-two lines
    // of 512 points or more (1024: 2.80 -> 2.69 ms; on 768-point lines the
    // smaller CTAs were slower, 1.82 -> 1.88 ms)
    p->ax_xc.spw_index = -1;
    size_pipe(p->ax_xc, 2, f64, nx >= 512 && (nx & (nx - 1)) == 0 ? 128 : 0);
    if (!p->ax_xc.pipe_ok) size_pipe(p->ax_xc, 2, f64);
  }
  size_pipe(p->ax_y, 0, f64);
  narrow_if_unfit(p->ax_y, 0);
  for (int i = 0; i < 2; ++i) {
    if (p->four_y) {
      size_pipe(p->ly[i], 0, f64);
      narrow_if_unfit(p->ly[i], 0);
    }
    if (p->four_z) {
      size_pipe(p->lz[i], 0, f64);
      narrow_if_unfit(p->lz[i], 0);
    }
  }
  for (int i = 0; i < 4; ++i)
    if (p->z_ok[i]) {
      size_pipe(p->ax_z[i], 0, f64);
      narrow_if_unfit(p->ax_z[i], 0);
    }
  {
    auto bps = [&](AxisPlan& ap, int kind) {
      if (!ap.pipe_ok) return;
      auto occ = [&](size_t sm) {
        return f64 ? pipe_blocks_per_sm<PathF64>(kind, ap.pipe_e, ap.pipe_threads, sm)
                   : pipe_blocks_per_sm<PathF32>(kind, ap.pipe_e, ap.pipe_threads, sm);
      };
      ap.pipe_bps = occ(ap.pipe_smem);
      if (ap.pipe_smem3 && occ(ap.pipe_smem3) < ap.pipe_bps) ap.pipe_smem3 = 0;
    };
    bps(p->ax_x, 2);
    bps(p->ax_xc, 2);
    bps(p->ax_y, 0);
    for (int i = 0; i < 2; ++i) {
      if (p->four_y) bps(p->ly[i], 0);
      if (p->four_z) bps(p->lz[i], 0);
    }
    for (int i = 0; i < 4; ++i) bps(p->ax_z[i], 0);
  }
  {
    const char* e = std::getenv("P3G_NO_PIPE");
    p->use_pipe = !(e && *e && *e != '0');
    e = std::getenv("P3G_NO_TMA");
    p->use_tma = !(e && *e && *e != '0');
  }
  if (cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) {
    cudaGetLastError();
    p->sm_count = 132;
  }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, dev);
  }

  {
    const long double gain = (long double)nx * (long double)ny * 2.0L * (long double)(nz + 1);
    int l = 0;
    while ((long double)std::ldexp(1.0, l) < gain) ++l;
    p->log2n = l;
  }
  p->tw_bytes = tw.v.size() * sizeof(float4);
  if (cudaMalloc(&p->d_tw, p->tw_bytes) != cudaSuccess ||
      cudaMalloc(&p->d_sp, sps.size() * sizeof(StagePlan)) != cudaSuccess ||
      cudaMalloc(&p->d_err, 4 * sizeof(int)) != cudaSuccess || cudaMemset(p->d_err, 0, 4 * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (p->d_tw) cudaFree(p->d_tw);
    delete p;
    return fail(P3G_E_NOMEM, "plan table allocation failed");
  }
  if (cudaMemcpy(p->d_tw, tw.v.data(), p->tw_bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->d_sp, sps.data(), sps.size() * sizeof(StagePlan), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(p->d_tw);
    cudaFree(p->d_sp);
    delete p;
    return fail(P3G_E_CUDA, "plan table upload failed");
  }
  *out = p;
  return P3G_OK;
}

int p3g_plan_destroy(p3g_plan p) {
  if (!p) return P3G_OK;
  for (auto& r : p->pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : p->free_events) cudaEventDestroy(e);
  if (p->aux) cudaStreamDestroy(p->aux);
  if (p->wa) cudaFree(p->wa);
  if (p->wb) cudaFree(p->wb);
  if (p->wc) cudaFree(p->wc);
  if (p->wd) cudaFree(p->wd);
  if (p->d_tw) cudaFree(p->d_tw);
  if (p->d_sp) cudaFree(p->d_sp);
  if (p->d_err) cudaFree(p->d_err);
  delete p;
  return P3G_OK;
}

int p3g_get_dims(p3g_plan p, int conf, int start[3], int end[3], int size[3]) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (conf == 1) {
    const int s[3] = {p->nx, p->ny, p->nz};
    for (int i = 0; i < 3; ++i) {
      start[i] = 1;
      end[i] = size[i] = s[i];
    }
  } else if (conf == 2) {
    int s[3] = {p->nxhpc, p->nyc, p->nzc};
    if (p->layout == P3G_LAYOUT_STRIDE1) {
      s[0] = p->nzc;
      s[2] = p->nxhpc;
    }
    for (int i = 0; i < 3; ++i) {
      start[i] = 1;
      end[i] = size[i] = s[i];
    }
  } else if (conf == 3) {
    // setup.F90:580-603 at 1x1: pad1 = 2*max(nz*nyc*nxhpc, ny*nz*nxhpc) - nx*ny*nz
    long long pad1 = 2LL * std::max((long long)p->nz * p->nyc * p->nxhpc, (long long)p->ny * p->nz * p->nxhpc) -
                     (long long)p->nx * p->ny * p->nz;
    if (pad1 < 0) pad1 = 0;
    const long long den = (long long)p->nx * p->ny;
    const long long padi = pad1 / den + (pad1 % den ? 1 : 0);
    const int s[3] = {p->nx, p->ny, (int)(p->nz + padi)};
    for (int i = 0; i < 3; ++i) {
      start[i] = 0;
      end[i] = size[i] = s[i];
    }
  } else {
    return fail(P3G_E_ARG, "conf must be 1, 2 or 3");
  }
  return P3G_OK;
}

int p3g_ftran_r2c_to_host(p3g_plan p, const void* in, void* out_host, void* stage, const char* op, int chunks,
                          void* stream, void* copy_stream) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!valid_op(op)) return fail(P3G_E_ARG, "op must have 3 letters");
  if (!in || !out_host || !stage) return fail(P3G_E_ARG, "NULL array");
  if (p->layout != P3G_LAYOUT_XYZ) return fail(P3G_E_UNSUPPORTED, "row-block copies need the XYZ layout");
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream), cs = static_cast<cudaStream_t>(copy_stream);
  return p->prec == P3G_F64 ? do_ftran_to_host<PathF64>(p, in, out_host, stage, op, chunks, st, cs)
                            : do_ftran_to_host<PathF32>(p, in, out_host, stage, op, chunks, st, cs);
}

int p3g_btran_c2r_from_host(p3g_plan p, const void* in_host, void* stage, void* out, const char* op, int chunks,
                            void* stream, void* copy_stream) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!valid_op(op)) return fail(P3G_E_ARG, "op must have 3 letters");
  if (!in_host || !out || !stage) return fail(P3G_E_ARG, "NULL array");
  if (p->layout != P3G_LAYOUT_XYZ) return fail(P3G_E_UNSUPPORTED, "row-block copies need the XYZ layout");
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream), cs = static_cast<cudaStream_t>(copy_stream);
  return p->prec == P3G_F64 ? do_btran_from_host<PathF64>(p, in_host, stage, out, op, chunks, st, cs)
                            : do_btran_from_host<PathF32>(p, in_host, stage, out, op, chunks, st, cs);
}

int p3g_ftran_r2c(p3g_plan p, const void* in, void* out, const char* op, int nv, long long dim_in, long long dim_out,
                  void* stream) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!valid_op(op)) return fail(P3G_E_ARG, "op must have 3 letters");
  if (nv <= 0 || nv > 65535) return fail(P3G_E_ARG, "nv out of range");
  if (!in || !out) return fail(P3G_E_ARG, "NULL array");
  const long long rsize = (long long)p->nx * p->ny * p->nz;
  const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
  if (dim_in <= 0) dim_in = rsize;
  if (dim_out <= 0) dim_out = csize;
  if (dim_in < rsize) return fail(P3G_E_ARG, "ftran error: input array dimensions are too low");
  if (dim_out < csize) return fail(P3G_E_ARG, "ftran error: output array dimensions are too low");
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return p->prec == P3G_F64 ? do_ftran<PathF64>(p, in, out, op, nv, dim_in, dim_out, st)
                            : do_ftran<PathF32>(p, in, out, op, nv, dim_in, dim_out, st);
}

int p3g_btran_c2r(p3g_plan p, const void* in, void* out, const char* op, int nv, long long dim_in, long long dim_out,
                  void* stream) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!valid_op(op)) return fail(P3G_E_ARG, "op must have 3 letters");
  if (nv <= 0 || nv > 65535) return fail(P3G_E_ARG, "nv out of range");
  if (!in || !out) return fail(P3G_E_ARG, "NULL array");
  const long long rsize = (long long)p->nx * p->ny * p->nz;
  const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
  if (dim_in <= 0) dim_in = csize;
  if (dim_out <= 0) dim_out = rsize;
  if (dim_in < csize) return fail(P3G_E_ARG, "btran error: input array dimensions are too low");
  if (dim_out < rsize) return fail(P3G_E_ARG, "btran error: output array dimensions are too low");
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return p->prec == P3G_F64 ? do_btran<PathF64>(p, in, out, op, nv, dim_in, dim_out, st)
                            : do_btran<PathF32>(p, in, out, op, nv, dim_in, dim_out, st);
}

int p3g_ftran_r2c_1d(p3g_plan p, const void* in, void* out, void* stream) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (!in || !out) return fail(P3G_E_ARG, "NULL array");
  XParams x{};
  x.in = in;
  x.out = out;
  x.in_field = (long long)p->nx * p->ny * p->nz;
  x.out_field = (long long)p->nxhp * p->ny * p->nz;
  x.in_line = p->nx;
  x.out_line = p->nxhp;
  x.nlines = p->ny * p->nz;
  x.nx = p->nx;
  x.nkeep = p->nxhp;  // every mode: the X transform alone is not pruned
  x.M = p->ax_x.M;
  x.log2m = p->ax_x.log2m;
  x.LS = p->ax_x.ls;
  x.ps = p->ax_x.ps;
  x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;
  x.out_user = 1;
  x.range = range_params(p, true, true);
  std::lock_guard<std::mutex> lk(p->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = launch_range_scan(p, in, x.in_field, x.in_field, 1, st);
  if (rc) return rc;
  return p->prec == P3G_F64 ? run_xr2c<PathF64>(p, x, 1, st) : run_xr2c<PathF32>(p, x, 1, st);
}

int p3g_cheby(p3g_plan p, const void* in, void* out, double lz, int nv, long long dim_in, long long dim_out,
              void* stream) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (p->nzc < 2) return fail(P3G_E_ARG, "Chebyshev transform needs nzc >= 2");
  if (!(lz != 0.0)) return fail(P3G_E_ARG, "Lz must be non-zero");
  int rc = p3g_ftran_r2c(p, in, out, "ffc", nv, dim_in, dim_out, stream);
  if (rc) return rc;
  const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
  if (dim_out <= 0) dim_out = csize;
  std::lock_guard<std::mutex> lk(p->mu);
  ChebyParams c{};
  c.data = out;
  c.field = dim_out;
  c.npencil = p->nxhpc * p->nyc;
  c.nzc = p->nzc;
  if (p->layout == P3G_LAYOUT_STRIDE1) {
    c.pstride = p->nzc;
    c.zstride = 1;
  } else {
    c.pstride = 1;
    c.zstride = (long long)p->nxhpc * p->nyc;
  }
  c.sc = 1.0 / ((double)p->nx * (double)p->ny * (double)(p->nzc - 1));
  c.lfac = 4.0 / lz;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  PassTimer tm(p, 7, st);
  cudaError_t e = p->prec == P3G_F64 ? launch_cheby<PathF64>(c, nv, st) : launch_cheby<PathF32>(c, nv, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("cheby launch: ") + cudaGetErrorString(e));
  p->launches++;
  tm.done();
  return P3G_OK;
}

int p3g_get_timers(p3g_plan p, double timers[12]) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  std::lock_guard<std::mutex> lk(p->mu);
  for (auto& r : p->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess)
      p->timers[r.slot] += ms * 1e-3;
    p->free_events.push_back(r.a);
    p->free_events.push_back(r.b);
  }
  p->pending.clear();
  std::memcpy(timers, p->timers, sizeof(p->timers));
  return P3G_OK;
}

int p3g_set_timers(p3g_plan p) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  double tmp[12];
  p3g_get_timers(p, tmp);
  std::lock_guard<std::mutex> lk(p->mu);
  std::memset(p->timers, 0, sizeof(p->timers));
  return P3G_OK;
}

long long p3g_plan_device_bytes(p3g_plan p) {
  if (!p) return 0;
  long long b = (long long)p->tw_bytes + 6LL * sizeof(StagePlan);
  if (p->wa) b += (long long)p->nz * p->ny * p->pitch * p->w_fields * p->esize();
  if (p->wb) b += (long long)p->nz * p->nyc * p->pitch * p->w_fields * p->esize();
  if (p->wc) b += (long long)p->wc_bytes();
  if (p->wd) b += p->xpairs() * p->nx * (long long)p->esize();
  return b;
}

long long p3g_plan_launches(p3g_plan p) { return p ? p->launches : 0; }

int p3g_plan_set_range(p3g_plan p, int mode, int bias) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (mode != P3G_RANGE_FIXED && mode != P3G_RANGE_AUTO) return fail(P3G_E_ARG, "unknown range mode");
  if (bias < -1100 || bias > 1100) return fail(P3G_E_ARG, "exponent bias out of range");
  std::lock_guard<std::mutex> lk(p->mu);
  p->range_mode = mode;
  p->ebias = bias;
  return P3G_OK;
}

int p3g_plan_check_range(p3g_plan p, int* bias, int* emax) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  if (p->prec != P3G_F64) {  // binary32 inputs are not tracked: nothing to read
    if (bias) *bias = 0;
    if (emax) *emax = -1075;
    return P3G_OK;
  }
  int w[3] = {0, 0, 0};
  cudaError_t e = cudaMemcpy(w, p->d_err, sizeof(w), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(p->d_err + 1, 0, sizeof(int));
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("range read: ") + cudaGetErrorString(e));
  return plan_range_result(p, w, bias, emax);
}


int p3g_plan_status(p3g_plan p) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  int flag = 0;
  if (cudaMemcpy(&flag, p->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(P3G_E_CUDA, std::string("status read: ") + cudaGetErrorString(cudaGetLastError()));
  if (flag) {
    // reported once: the record is cleared for the calls that follow
    if (cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) cudaGetLastError();
    return fail(P3G_E_CUDA, "a pipelined pass timed out waiting for its tile copy (results invalid)");
  }
  return p3g_plan_check_range(p, nullptr, nullptr);
}

int p3g_plan_block_tiles(p3g_plan p, int on) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  std::lock_guard<std::mutex> lk(p->mu);
  p->tx_extra = on ? 16 : 0;
  return P3G_OK;
}

int p3g_plan_set_options(p3g_plan p, int use_pipe, int use_tma) {
  if (!p) return fail(P3G_E_STATE, "P3DFFT error: call setup before other routines");
  p->use_pipe = use_pipe != 0;
  p->use_tma = use_tma != 0;
  return P3G_OK;
}

}  // extern "C"
