// Batches of independent transforms in one persistent launch: p3g_batch_*.
//
// A batch holds a list of jobs (forward, backward, round trip, or forward +
// shell spectrum), each on its own plan (any sizes, one precision per batch)
// and its own device workspace.  Every job is a chain of passes (X, Y, Z
// forward; Z, Y, X backward; spectrum), every pass a set of tiles, and every
// tile one work item of a single queue.  One persistent kernel (grid = SMs x
// resident CTAs) takes items in queue order with an atomic ticket; an item
// whose pass depends on the job's previous pass waits (bounded) until all
// tiles of that pass have been counted done.  Items are taken in queue
// order and every dependency points to an earlier item, which a running CTA
// already holds, so the launch makes progress whether or not all CTAs are
// resident.
//
// Queue order (the schedule): jobs in windows of `window` jobs; inside a
// window pass-major (every job's X pass, then every job's Y pass, ...).  A
// small window keeps a job's passes close together in time, so the data of a
// small grid is still in the 129 MB L2 when its next pass reads it; a large
// window gives each pass more parallel tiles.  The autotuner picks it.
//
// Visibility between CTAs: the CTA barrier after a tile's stores, then thread
// 0's gpu-scope fence and one atomic increment of the pass counter; the waiting CTA's
// thread 0 polls the counter with ld.acquire.gpu and fences; the CTA then
// reads the data through L2 only (ld.global.cg), so no stale L1 line from an
// earlier pass is seen.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "p3g_batch.h"
#include "p3g_plan_internal.h"

namespace p3g {
namespace {

// Double-buffered path: halve the tile width until the tile fits E points per
// thread; returns the buffer size in elements (0 when it cannot fit), room
// for the packed tile or the raw line pairs, whichever is larger.
size_t pipe_fit_x(XParams& x, int E, int esize, int threads) {
  const int nh = x.nx / 2 + 1;
  auto fits = [&](int M) { return (long long)M * x.nx <= (long long)E * threads; };
  while (x.M > 1 && !fits(x.M)) {
    x.M >>= 1;
    x.log2m--;
  }
  if (!fits(x.M)) return 0;
  x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;
  const int raw = 2 * xc2r_raw_stride(nh, esize);
  return (size_t)x.M * (x.LS > raw ? x.LS : raw);
}
size_t pipe_fit_s(SParams& s, int E, int threads) {
  while (s.M > 1 && (long long)s.M * s.N > (long long)E * threads) {
    s.M >>= 1;
    s.log2m--;
  }
  if ((long long)s.M * s.N > (long long)E * threads) return 0;
  s.xtiles = (s.X + s.M - 1) / s.M;
  return (size_t)s.M * s.N;
}

// Halve the plan's tile width until one tile fits the batch CTA; returns the
// tile's shared-memory bytes (0 when even one line is too long).
size_t fit_x(XParams& x, const AxisPlan& ap, size_t esize, int threads) {
  const long long tile = (long long)kElemsPerThread * threads;
  while (x.M > 1 && (long long)x.M * x.nx > tile) {
    x.M >>= 1;
    x.log2m--;
  }
  if ((long long)x.M * x.nx > tile) return 0;
  x.tiles = ((x.nlines + 1) / 2 + x.M - 1) / x.M;
  return (size_t)x.M * x.LS * esize * (ap.sp.has_generic ? 2 : 1);
}
size_t fit_s(SParams& s, const AxisPlan& ap, size_t esize, int threads) {
  const long long tile = (long long)kElemsPerThread * threads;
  while (s.M > 1 && (long long)s.M * s.N > tile) {
    s.M >>= 1;
    s.log2m--;
  }
  if ((long long)s.M * s.N > tile) return 0;
  s.xtiles = (s.X + s.M - 1) / s.M;
  return (size_t)s.M * s.N * esize * (ap.sp.has_generic ? 2 : 1);
}

template <class P>
cudaError_t batch_config(size_t smem, int threads, int& per_sm, size_t& max_dyn) {
  return threads == kBatchThreadsSmall ? batch_config_t<P, kBatchThreadsSmall>(smem, per_sm, max_dyn)
                                       : batch_config_t<P, kBatchThreadsLarge>(smem, per_sm, max_dyn);
}

template <class P>
cudaError_t batch_launch(const BatchPass* d_pass, int npass, int nitems, int* ctl, int buf_elems, int grid,
                         int threads, size_t smem, cudaStream_t st) {
  return threads == kBatchThreadsSmall
             ? batch_launch_t<P, kBatchThreadsSmall>(d_pass, npass, nitems, ctl, buf_elems, grid, smem, st)
             : batch_launch_t<P, kBatchThreadsLarge>(d_pass, npass, nitems, ctl, buf_elems, grid, smem, st);
}

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

// Workspace of one job inside its work buffer: wa | wb (Y pruning) | complex
// field (round trip and spectrum jobs).
struct JobLayout {
  size_t wa, wb, cplx, total;
};
JobLayout job_layout(p3g_plan p, int kind) {
  JobLayout l{};
  const size_t es = p->esize();
  l.wa = round256((size_t)p->nz * p->ny * p->pitch * es);
  l.wb = p->nyc < p->ny ? round256((size_t)p->nz * p->nyc * p->pitch * es) : 0;
  l.cplx = (kind == P3G_JOB_ROUNDTRIP || kind == P3G_JOB_SPECTRUM)
               ? round256((size_t)p->nxhpc * p->nyc * p->nzc * es)
               : 0;
  l.total = l.wa + l.wb + l.cplx;
  return l;
}

}  // namespace
}  // namespace p3g

using namespace p3g;

struct p3g_batch_s {
  int prec = P3G_F64;
  int sm_count = 0;
  std::vector<BatchPass> host;
  std::vector<p3g_plan> plans;  // the jobs' plans (their range records)
  BatchPass* d_pass = nullptr;
  size_t pass_cap = 0;
  int* d_ctl = nullptr;
  size_t ctl_cap = 0;
  // page-locked staging of the pass table, copied on the launch stream by
  // the next launch (dirty); `staged` marks the end of that copy, so the
  // next set_jobs overwrites the staging only after it.  No call waits on
  // the copy engines' queues, which other streams' bulk copies may fill.
  BatchPass* h_pass = nullptr;
  size_t h_cap = 0;
  bool dirty = false;
  cudaEvent_t staged = nullptr;
  bool staged_pending = false;
  // the launch's error word, copied to page-locked memory after the kernel
  // on the launch stream; `done` marks the copy
  int* h_err = nullptr;
  cudaEvent_t done = nullptr;
  bool done_pending = false;
  // the F64 jobs' plans' range words (d_err[0..2] each), copied after the
  // kernel on the launch stream (and the range record cleared there)
  int* h_range = nullptr;
  size_t h_range_cap = 0;  // plans
  int npass = 0, nitems = 0;
  size_t smem = 0;
  int buf_elems = 0;
  int threads = 0, grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;
  std::mutex mu;
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

// Every job's chain of passes for CTAs of `threads` threads: tile widths,
// double-buffered or single-tile items, and the shared memory the items need
// (smem bytes for single-tile and spectrum items, buf_elems per buffer of the
// double-buffered ones).  fit = false when a line is longer than the tile.
static int build_chains(p3g_batch b, int njobs, const p3g_job* jobs, int threads,
                        std::vector<std::vector<BatchPass>>& chains, size_t& smem, size_t& buf_elems, bool& fit) {
  const bool f64 = b->prec == P3G_F64;
  const int pipe_e = f64 ? batch_pipe_elems<true>() : batch_pipe_elems<false>();
  const int nwarps = threads / 32;
  chains.assign(njobs, {});
  smem = 0;
  buf_elems = 0;
  fit = true;
  for (int j = 0; j < njobs; ++j) {
    const p3g_job& jb = jobs[j];
    p3g_plan p = jb.plan;
    const std::string who = "job " + std::to_string(j) + ": ";
    if (!p) return fail(P3G_E_ARG, who + "plan is NULL");
    if (p->prec != b->prec) return fail(P3G_E_ARG, who + "plan precision differs from the batch's");
    if (jb.kind < P3G_JOB_ROUNDTRIP || jb.kind > P3G_JOB_SPECTRUM) return fail(P3G_E_ARG, who + "unknown kind");
    if (!jb.in || !jb.out || !jb.work) return fail(P3G_E_ARG, who + "NULL array");
    if (!p->z_ok[0]) return fail(P3G_E_UNSUPPORTED, who + "Z FFT unsupported for nz");
    if (p->four_x || p->four_y || p->four_z) return fail(P3G_E_UNSUPPORTED, who + "lines longer than one tile (four-step)");
    const JobLayout L = job_layout(p, jb.kind);
    unsigned char* w = static_cast<unsigned char*>(jb.work);
    void* wa = w;
    void* wb = L.wb ? w + L.wa : nullptr;
    void* cplx = L.cplx ? w + L.wa + L.wb : nullptr;
    const StagePlan* dsp = p->d_sp;
    bool fits = true;
    const size_t es = p->esize();
    // double-buffered when the axis has no generic prime stage and its tile
    // fits the pipelined CTA; else single-tile (scratch tile, no prefetch)
    auto x_pass = [&](int kind, const XParams& x) {
      BatchPass q{};
      q.kind = kind;
      q.x = x;
      const AxisPlan& ap = p->ax_x;
      size_t pe = 0;
      if (!ap.sp.has_generic && ap.sp.nstages > 0 && x.nx >= 2) {
        XParams t = x;
        pe = pipe_fit_x(t, pipe_e, (int)es, threads);
        if (pe) q.x = t;
      }
      if (pe) {
        q.pipe = 1;
        buf_elems = std::max(buf_elems, pe);
        const size_t ur = f64 ? 8 : 4;
        q.chunk = (int)ur;
        const uintptr_t a = reinterpret_cast<uintptr_t>(x.in);
        if ((x.nx * ur) % 16 == 0 && a % 16 == 0) q.chunk = 16;
        else if ((x.nx * ur) % 8 == 0 && a % 8 == 0) q.chunk = 8;
      } else {
        const size_t need = fit_x(q.x, ap, es, threads);
        fits = fits && need > 0;
        smem = std::max(smem, need);
      }
      q.tiles = q.x.tiles;
      q.sp = dsp + ap.sp_index;
      q.tw = p->d_tw;
      chains[j].push_back(q);
    };
    auto s_pass = [&](int kind, const SParams& s, const AxisPlan& ap) {
      BatchPass q{};
      q.kind = kind;
      q.s = s;
      size_t pe = 0;
      if (!ap.sp.has_generic && ap.sp.nstages > 0 && s.N >= 2) {
        SParams t = s;
        pe = pipe_fit_s(t, pipe_e, threads);
        if (pe) q.s = t;
      }
      if (pe) {
        q.pipe = 1;
        buf_elems = std::max(buf_elems, pe);
      } else {
        const size_t need = fit_s(q.s, ap, es, threads);
        fits = fits && need > 0;
        smem = std::max(smem, need);
      }
      q.tiles = q.s.xtiles * q.s.O1;
      q.sp = dsp + ap.sp_index;
      q.tw = p->d_tw;
      chains[j].push_back(q);
    };
    const long long rsize = (long long)p->nx * p->ny * p->nz;
    const long long csize = (long long)p->nxhpc * p->nyc * p->nzc;
    if (jb.kind == P3G_JOB_SPECTRUM) {
      SpecParams sp;
      int rc = make_spectrum_params(p, cplx, static_cast<double*>(jb.out), jb.kmax, jb.scale, jb.flags, csize, sp);
      if (rc) return rc;
      BatchPass q{};
      q.kind = kBZero;
      q.spec = sp;
      q.tiles = 1;
      chains[j].push_back(q);
    }
    if (jb.kind != P3G_JOB_BACKWARD) {
      XParams x;
      SParams y, z;
      void* fout = jb.kind == P3G_JOB_FORWARD ? jb.out : cplx;
      make_forward_params(p, jb.in, fout, wa, wb, 0, rsize, csize, x, y, z, true);
      x.range = range_params(p, true, false);
      z.range = range_params(p, false, false);
      x_pass(kBXr2c, x);
      s_pass(kBFwd, y, p->ax_y);
      s_pass(kBFwd, z, p->ax_z[0]);
    }
    if (jb.kind == P3G_JOB_ROUNDTRIP || jb.kind == P3G_JOB_BACKWARD) {
      SParams z, y;
      XParams x;
      const void* bin = jb.kind == P3G_JOB_BACKWARD ? jb.in : cplx;
      make_backward_params(p, bin, jb.out, wa, wb, 0, csize, rsize, z, y, x, true);
      if (jb.kind == P3G_JOB_BACKWARD) z.range = range_params(p, true, false);  // user input
      x.range = range_params(p, false, false);
      s_pass(kBBwd, z, p->ax_z[0]);
      s_pass(kBBwd, y, p->ax_y);
      x_pass(kBXc2r, x);
    }
    if (!fits) {
      fit = false;
      return P3G_OK;
    }
    if (jb.kind == P3G_JOB_SPECTRUM) {
      BatchPass q = chains[j][0];
      q.kind = kBSpec;
      q.rows_per_item = nwarps * 4;
      q.tiles = (q.spec.rows + q.rows_per_item - 1) / q.rows_per_item;
      smem = std::max(smem, (size_t)nwarps * (q.spec.kmax + 1) * sizeof(double));
      chains[j].push_back(q);
    }
  }
  return P3G_OK;
}

extern "C" {

long long p3g_job_work_bytes(p3g_plan plan, int kind) {
  if (!plan || kind < P3G_JOB_ROUNDTRIP || kind > P3G_JOB_SPECTRUM) {
    fail(P3G_E_ARG, "invalid plan or job kind");
    return -1;
  }
  return (long long)job_layout(plan, kind).total;
}

int p3g_batch_create(p3g_batch* out, int precision) {
  if (!out) return fail(P3G_E_ARG, "batch pointer is NULL");
  *out = nullptr;
  if (precision != P3G_F64 && precision != P3G_F32) return fail(P3G_E_ARG, "unknown precision");
  auto* b = new p3g_batch_s();
  b->prec = precision;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&b->h_err), sizeof(int), cudaHostAllocDefault);
  if (e == cudaSuccess) *b->h_err = 0;
  if (e != cudaSuccess) {
    if (b->staged) cudaEventDestroy(b->staged);
    if (b->done) cudaEventDestroy(b->done);
    delete b;
    return fail(P3G_E_CUDA, std::string("batch create: ") + cudaGetErrorString(e));
  }
  *out = b;
  return P3G_OK;
}

int p3g_batch_destroy(p3g_batch b) {
  if (!b) return P3G_OK;
  b->drop_graph();
  if (b->d_pass) cudaFree(b->d_pass);
  if (b->d_ctl) cudaFree(b->d_ctl);
  if (b->h_pass) cudaFreeHost(b->h_pass);
  if (b->h_err) cudaFreeHost(b->h_err);
  if (b->h_range) cudaFreeHost(b->h_range);
  if (b->staged) cudaEventDestroy(b->staged);
  if (b->done) cudaEventDestroy(b->done);
  delete b;
  return P3G_OK;
}

int p3g_batch_set_jobs(p3g_batch b, int njobs, const p3g_job* jobs, int window) {
  if (!b) return fail(P3G_E_STATE, "batch is NULL");
  if (njobs <= 0 || !jobs) return fail(P3G_E_ARG, "no jobs");
  if (window <= 0) window = njobs;
  std::lock_guard<std::mutex> lk(b->mu);
  const bool f64 = b->prec == P3G_F64;
  // per job: its chain of passes; 128-thread CTAs unless a line needs the
  // 256-thread tile
  std::vector<std::vector<BatchPass>> chains;
  size_t smem = 0;        // single-tile and spectrum items (bytes)
  size_t buf_elems = 0;   // one buffer of the double-buffered items (elements)
  int threads = kBatchThreadsSmall;
  for (;;) {
    bool fit = false;
    const int rc = build_chains(b, njobs, jobs, threads, chains, smem, buf_elems, fit);
    if (rc != P3G_OK) return rc;
    if (fit) break;
    if (threads == kBatchThreadsLarge)
      return fail(P3G_E_UNSUPPORTED, "a line is longer than a batch tile (4096 points)");
    threads = kBatchThreadsLarge;
  }
  {
    const size_t es = f64 ? 16 : 8;
    buf_elems = (buf_elems + 1) / 2 * 2;  // keeps the second buffer 16-byte aligned
    smem = std::max(smem, 2 * buf_elems * es);
  }
  if (smem > 227 * 1024) return fail(P3G_E_UNSUPPORTED, "a job's tile exceeds shared memory");
  // queue: windows of jobs, pass-major inside a window
  std::vector<BatchPass> table;
  std::vector<int> last(njobs, -1);
  long long items = 0;
  for (int w0 = 0; w0 < njobs; w0 += window) {
    const int w1 = std::min(njobs, w0 + window);
    size_t depth = 0;
    for (int j = w0; j < w1; ++j) depth = std::max(depth, chains[j].size());
    for (size_t s = 0; s < depth; ++s)
      for (int j = w0; j < w1; ++j) {
        if (s >= chains[j].size()) continue;
        BatchPass q = chains[j][s];
        q.dep = last[j];
        q.first = (int)items;
        items += q.tiles;
        last[j] = (int)table.size();
        table.push_back(q);
      }
  }
  if (items > 0x7FFFFFF0LL) return fail(P3G_E_UNSUPPORTED, "too many work items");
  int per_sm = 1;
  size_t max_dyn = 0;
  cudaError_t e = f64 ? batch_config<PathF64>(smem, threads, per_sm, max_dyn)
                      : batch_config<PathF32>(smem, threads, per_sm, max_dyn);
  if (e != cudaSuccess && smem > max_dyn && max_dyn > 0)
    return fail(P3G_E_UNSUPPORTED, "a job's tile needs " + std::to_string(smem) + " bytes of shared memory, above " +
                                       std::to_string(max_dyn));
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch kernel attributes: ") + cudaGetErrorString(e));
  const size_t pass_bytes = table.size() * sizeof(BatchPass);
  const size_t ctl_bytes = (2 + table.size()) * sizeof(int);
  b->drop_graph();
  // the table (device and staging) and the counters grow by at least 2x, so
  // that a server's batches stop reallocating (cudaFree waits for the whole
  // device) after a few launches
  auto grow = [](size_t need, size_t cap) { return std::max(need, std::max<size_t>(2 * cap, 16384)); };
  if (b->staged_pending) {  // the last upload has read the staging
    e = cudaEventSynchronize(b->staged);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch table upload: ") + cudaGetErrorString(e));
    b->staged_pending = false;
  }
  if (pass_bytes > b->pass_cap) {
    const size_t cap = grow(pass_bytes, b->pass_cap);
    if (b->d_pass) cudaFree(b->d_pass);
    b->d_pass = nullptr;
    b->pass_cap = 0;
    if (cudaMalloc(&b->d_pass, cap) != cudaSuccess) {
      cudaGetLastError();
      return fail(P3G_E_NOMEM, "batch table allocation failed");
    }
    b->pass_cap = cap;
  }
  if (pass_bytes > b->h_cap) {
    const size_t cap = grow(pass_bytes, b->h_cap);
    if (b->h_pass) cudaFreeHost(b->h_pass);
    b->h_pass = nullptr;
    b->h_cap = 0;
    if (cudaHostAlloc(reinterpret_cast<void**>(&b->h_pass), cap, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return fail(P3G_E_NOMEM, "batch table staging allocation failed");
    }
    b->h_cap = cap;
  }
  if (ctl_bytes > b->ctl_cap) {
    const size_t cap = grow(ctl_bytes, b->ctl_cap);
    if (b->d_ctl) cudaFree(b->d_ctl);
    b->d_ctl = nullptr;
    b->ctl_cap = 0;
    if (cudaMalloc(&b->d_ctl, cap) != cudaSuccess) {
      cudaGetLastError();
      return fail(P3G_E_NOMEM, "batch counter allocation failed");
    }
    b->ctl_cap = cap;
  }
  std::memcpy(b->h_pass, table.data(), pass_bytes);
  b->dirty = true;
  b->host = std::move(table);
  b->plans.clear();
  for (int j = 0; j < njobs; ++j)
    if (std::find(b->plans.begin(), b->plans.end(), jobs[j].plan) == b->plans.end()) b->plans.push_back(jobs[j].plan);
  if (f64 && b->plans.size() > b->h_range_cap) {
    const size_t cap = std::max<size_t>(b->plans.size(), 2 * b->h_range_cap);
    if (b->h_range) cudaFreeHost(b->h_range);
    b->h_range = nullptr;
    b->h_range_cap = 0;
    if (cudaHostAlloc(reinterpret_cast<void**>(&b->h_range), cap * 3 * sizeof(int), cudaHostAllocDefault) !=
        cudaSuccess) {
      cudaGetLastError();
      return fail(P3G_E_NOMEM, "batch range staging allocation failed");
    }
    b->h_range_cap = cap;
  }
  b->npass = (int)b->host.size();
  b->nitems = (int)items;
  b->smem = smem;
  b->buf_elems = (int)buf_elems;
  b->threads = threads;
  const long long slots = (long long)b->sm_count * per_sm;
  b->grid = (int)std::max(1LL, std::min(slots, items));
  return P3G_OK;
}

// The pass table's copy from its staging (when set_jobs changed it), the
// counter clear, the kernel and the copy of its error word, all on st.
static int batch_upload(p3g_batch b, cudaStream_t st) {
  if (!b->dirty) return P3G_OK;
  // after the previous launch (which reads the table), on whichever stream
  cudaError_t e = b->done_pending ? cudaStreamWaitEvent(st, b->done, 0) : cudaSuccess;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_pass, b->h_pass, (size_t)b->npass * sizeof(BatchPass), cudaMemcpyHostToDevice,
                                  st);
  if (e == cudaSuccess) e = cudaEventRecord(b->staged, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch table upload: ") + cudaGetErrorString(e));
  b->staged_pending = true;
  b->dirty = false;
  return P3G_OK;
}

static int batch_enqueue(p3g_batch b, cudaStream_t st) {
  const size_t ctl_bytes = (2 + (size_t)b->npass) * sizeof(int);
  cudaError_t e = cudaMemsetAsync(b->d_ctl, 0, ctl_bytes, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch clear: ") + cudaGetErrorString(e));
  e = b->prec == P3G_F64
          ? batch_launch<PathF64>(b->d_pass, b->npass, b->nitems, b->d_ctl, b->buf_elems, b->grid, b->threads,
                                  b->smem, st)
          : batch_launch<PathF32>(b->d_pass, b->npass, b->nitems, b->d_ctl, b->buf_elems, b->grid, b->threads,
                                  b->smem, st);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  e = cudaMemcpyAsync(b->h_err, b->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (b->prec == P3G_F64)
    for (size_t i = 0; i < b->plans.size() && e == cudaSuccess; ++i) {
      e = cudaMemcpyAsync(b->h_range + 3 * i, b->plans[i]->d_err, 3 * sizeof(int), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(b->plans[i]->d_err + 1, 0, sizeof(int), st);
    }
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch status copy: ") + cudaGetErrorString(e));
  return P3G_OK;
}

int p3g_batch_launch(p3g_batch b, void* stream) {
  if (!b || b->nitems == 0) return fail(P3G_E_STATE, "batch has no jobs");
  std::lock_guard<std::mutex> lk(b->mu);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = batch_upload(b, st);
  if (rc == P3G_OK) rc = batch_enqueue(b, st);
  if (rc == P3G_OK) {
    if (cudaEventRecord(b->done, st) != cudaSuccess)
      return fail(P3G_E_CUDA, std::string("batch launch: ") + cudaGetErrorString(cudaGetLastError()));
    b->done_pending = true;
    b->launches++;
  }
  return rc;
}

int p3g_batch_capture(p3g_batch b) {
  if (!b || b->nitems == 0) return fail(P3G_E_STATE, "batch has no jobs");
  std::lock_guard<std::mutex> lk(b->mu);
  b->drop_graph();
  cudaStream_t cs = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("capture stream: ") + cudaGetErrorString(e));
  // the table goes to the device before the capture: replays reuse it
  int urc = batch_upload(b, cs);
  if (urc == P3G_OK && cudaStreamSynchronize(cs) != cudaSuccess)
    urc = fail(P3G_E_CUDA, std::string("batch table upload: ") + cudaGetErrorString(cudaGetLastError()));
  if (urc != P3G_OK) {
    cudaStreamDestroy(cs);
    return urc;
  }
  b->staged_pending = false;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  int rc = P3G_OK;
  if (e == cudaSuccess) {
    rc = batch_enqueue(b, cs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    if (e == cudaSuccess && rc == P3G_OK) {
      b->graph = g;
      e = cudaGraphInstantiate(&b->exec, g, 0);
    } else if (g) {
      cudaGraphDestroy(g);
    }
  }
  cudaStreamDestroy(cs);
  if (rc) return rc;
  if (e != cudaSuccess) {
    b->drop_graph();
    return fail(P3G_E_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
  }
  return P3G_OK;
}

int p3g_batch_replay(p3g_batch b, void* stream) {
  if (!b || !b->exec) return fail(P3G_E_STATE, "batch has no captured graph");
  std::lock_guard<std::mutex> lk(b->mu);
  cudaError_t e = cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess) e = cudaEventRecord(b->done, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
  b->done_pending = true;
  b->launches++;
  return P3G_OK;
}

int p3g_batch_status(p3g_batch b, void* stream) {
  if (!b) return fail(P3G_E_STATE, "batch is NULL");
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess && b->done_pending) e = cudaEventSynchronize(b->done);
  if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("batch: ") + cudaGetErrorString(e));
  if (!b->done_pending) return P3G_OK;
  const int err = *static_cast<volatile int*>(b->h_err);
  if (err) return fail(P3G_E_CUDA, "batch kernel: a dependency wait timed out");
  // the F64 jobs' binary64 inputs against the exponent window at their plans'
  // biases, from the words copied after the kernel
  if (b->prec == P3G_F64)
    for (size_t i = 0; i < b->plans.size(); ++i) {
      int w[3];
      for (int k = 0; k < 3; ++k) w[k] = static_cast<volatile int*>(b->h_range)[3 * i + k];
      const int rc = plan_range_result(b->plans[i], w, nullptr, nullptr);
      if (rc) return rc;
    }
  return P3G_OK;
}

int p3g_batch_block_pass(p3g_batch b, int pass) {
  if (!b || b->nitems == 0) return fail(P3G_E_STATE, "batch has no jobs");
  if (pass < 0 || pass >= b->npass) return fail(P3G_E_ARG, "pass index out of range");
  std::lock_guard<std::mutex> lk(b->mu);
  // waiters compare the pass's done-counter with this device copy of its tile
  // count; one more than the pass has makes every dependent wait run out
  // (in the staging, uploaded by the next launch)
  if (b->staged_pending) {
    cudaError_t e = cudaEventSynchronize(b->staged);
    if (e != cudaSuccess) return fail(P3G_E_CUDA, std::string("block pass: ") + cudaGetErrorString(e));
    b->staged_pending = false;
  }
  b->h_pass[pass].tiles = b->host[pass].tiles + 1;
  b->dirty = true;
  b->drop_graph();
  return P3G_OK;
}

int p3g_batch_info(p3g_batch b, long long info[5]) {
  if (!b) return fail(P3G_E_STATE, "batch is NULL");
  info[0] = b->npass;
  info[1] = b->nitems;
  info[2] = b->grid;
  info[3] = b->launches;
  info[4] = b->threads;
  return P3G_OK;
}

}  // extern "C"
