// Pipelined (persistent, multi-buffered) pass kernels.
//
// Each CTA walks a strided list of tiles (grid = SMs x resident CTAs).  While
// it transforms tile i in one shared buffer, the copy of the next tile (two
// tiles ahead in the X kernels with three buffers) is already in flight (TMA
// tensor tiles, bulk copies or cp.async), so HBM traffic overlaps the
// butterflies.  Each strided tile goes through: a fix-up step in shared
// memory (format conversion of user data, DCT-I/DST-I extension), the
// Stockham stages of p3g_engine.cuh with the pass's twiddles held in shared
// memory for the life of the CTA, and a store step with the pruning map and
// output format conversion fused in, or, for rows stored one to one, TMA
// tensor stores issued by one thread (with a third buffer, so a buffer is
// reloaded only after its store has read it).
#pragma once

#include <type_traits>

#include "p3g_async.cuh"
#include "p3g_kernels.cuh"

namespace p3g {

// ------------------------------------------------------------ parameters
struct PipeCommon {
  int ntiles;               // tiles over all fields
  int tiles_per_field;
  int tw_base, tw_count;    // this pass's slice of the twiddle table (float4)
  int buf_elems;            // elements (W) per buffer
  int nbuf;                 // tile buffers (2 or 3): loads run nbuf - 1 tiles ahead (nbuf - 2 with TMA stores)
  int* err;                 // device error flag
};

struct SPipeParams {
  SParams s;
  PipeCommon c;
  int use_tma;              // 1: TMA tensor tiles, 0: cp.async
  int brows, nbox;          // TMA: rows per box, boxes per tile
  int box_bytes;
  int tx_extra;             // test hook: bytes the barrier expects beyond the boxes (0)
  int chunk;                // cp.async bytes per element copy (16 or 8)
  // 1: the transformed tile leaves by TMA stores (one thread, asynchronous)
  // in onbox boxes of obrows rows; the kernel then keeps nbuf = 3 buffers
  // and loads one tile ahead, so a buffer is reloaded two iterations after
  // its store was issued
  int tma_store;
  int obrows, onbox;
};

struct XPipeParams {
  XParams x;
  PipeCommon c;
  int chunk;                // r2c: cp.async bytes per copy (4, 8 or 16)
  // 1: thread 0 loads tiles with 1-D bulk copies on an mbarrier (r2c: the
  // tile's 2M contiguous real lines in one copy, full tiles only; c2r: one
  // copy per line of every mode), else every thread issues cp.async
  int bulk;
};

P3G_D unsigned char* align1k(unsigned char* p) {
  return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Tiles hold at most 4096 (F64) or 8192 (F32) elements; a thread holds E
// of them per stage: on the F64 path 16 for axes with radix-16 stages (one
// 16-point butterfly per thread and stage: 1024 = 16 x 16 x 4) and 8
// otherwise (512 threads, 16 warps per SM to hide the latency of the
// dependent double-float chains); on the F32 path 32 for axes with radix-32
// stages (one 32-point butterfly per thread and stage takes a 1024-point line
// through two stages) and 16 otherwise.
template <class P, int E>
struct PipeLimits {
  // one radix-32 (F32) or radix-16 (F64) butterfly per thread and stage
  static constexpr bool kWide = P::kF64 ? E == 16 : E == 32;
  static constexpr int kMaxThreads = (P::kF64 ? 4096 : 8192) / E;
  // 128 registers per thread (with a larger budget the scheduler hoists
  // shared-memory loads across codelets and spills), except for the wide
  // kernels: one 256-thread CTA per SM (its two 64 KB tiles fill shared
  // memory) with up to 255 registers for the 32- or 16-point butterflies
  static constexpr int kMinBlocks = kWide ? 1 : 65536 / 128 / kMaxThreads;
};

// X passes: 256-thread CTAs, three per SM (85 registers; for the F32
// radix-32 stages 64-thread CTAs, six per SM, with up to 170 registers: 1024
// points X r2c 2.57 -> 2.49 ms at 1024^3 against three 128-thread CTAs; the
// F64 radix-16 kernel keeps 128-thread CTAs), with the twiddles
// read from the global table through L1 instead of a shared-memory copy,
// which leaves room for three double-buffered tiles per SM.  The X passes
// gain from the extra resident CTAs; the strided passes, whose tiles must
// stay wide for their long-stride DRAM rows, keep PipeLimits.
template <class P, int E>
struct XPipeLimits {
  static constexpr int kMaxThreads = PipeLimits<P, E>::kWide ? (P::kF64 ? 128 : 64) : 256;
  static constexpr int kMinBlocks = PipeLimits<P, E>::kWide && !P::kF64 ? 6 : 3;
};

// Largest radix compiled into a pipelined kernel (cta_fft's MAXR).
template <class P, int E>
struct PipeMaxR {
  static constexpr int value = P::kF64 ? (E == 16 ? 16 : 8) : (E == 32 ? 32 : 16);
};



// ------------------------------------------------------------ strided Y/Z
template <class P>
struct StridedSmem {
  typename P::W* buf0;
  float4* tw;
  uint64_t* mbar;
};
template <class P>
P3G_D StridedSmem<P> strided_smem(const PipeCommon& pc) {
  extern __shared__ unsigned char p3g_pipe_smem[];
  StridedSmem<P> r;
  r.buf0 = reinterpret_cast<typename P::W*>(align1k(p3g_pipe_smem));
  r.tw = reinterpret_cast<float4*>(r.buf0 + pc.nbuf * pc.buf_elems);
  r.mbar = reinterpret_cast<uint64_t*>(r.tw + pc.tw_count);
  return r;
}

P3G_D void strided_decode(const SPipeParams& q, int tile, int& xt, int& o1, int& o2) {
  o2 = tile / q.c.tiles_per_field;
  const int r = tile - o2 * q.c.tiles_per_field;
  o1 = r / q.s.xtiles;
  xt = r - o1 * q.s.xtiles;
}

// cp.async copies of one strided tile (columns xt*M.., row block o1, field
// o2) into dst, without a commit; the DCT-I/DST-I extension rows are extra
// copies of the same elements (the DST-I negation happens in the fix-up
// step).
template <class P, bool WALK = false>
P3G_D void strided_copy(const SParams& s, typename P::W* dst, int xt, int o1, int o2) {
  using W = typename P::W;
  const int M = s.M, L = s.L;
  const int ph = strided_phase(s, o1, o2);
  const int x0 = xt * M + ph;
  const long long ib0 = (long long)o1 * s.in_o1 + (long long)o2 * s.in_o2;
  const long long ib = ib0 + (long long)x0 * s.in_xs;
  const char* in = static_cast<const char*>(s.in);
  constexpr int esz = (int)sizeof(W);
  auto one = [&](int m, int j) {
    const int src = j >= s.lmap_a1 ? j - s.lmap_d : (j < s.lmap_a0 ? j : -1);
    const int c = x0 + m;
    const bool ok = src >= 0 && c < s.X + ph;
    const int cw = c < s.X ? c : c - s.X;  // the phase-shifted row's last tile wraps to column 0
    const char* g = ok ? in + (ib0 + (long long)cw * s.in_xs + (long long)src * s.in_axis) * esz : in;
    const uint32_t nb = ok ? (uint32_t)esz : 0u;
    int r0 = j, r1 = -1;
    if (s.pre == 2) {
      r0 = j + 1;
      r1 = 2 * (L + 1) - (j + 1);
    } else if (s.pre == 1 && j >= 1 && j <= L - 2) {
      r1 = 2 * (L - 1) - j;
    }
    if constexpr (esz == 16) {
      cp_async16(dst + r0 * M + m, g, nb);
      if (r1 >= 0) cp_async16(dst + r1 * M + m, g, nb);
      if (s.pre == 2 && j == 0) {  // rows 0 and L+1 of the odd extension are zero
        cp_async16(dst + m, in, 0);
        cp_async16(dst + (L + 1) * M + m, in, 0);
      }
    } else {
      cp_async8(dst + r0 * M + m, g, nb);
      if (r1 >= 0) cp_async8(dst + r1 * M + m, g, nb);
      if (s.pre == 2 && j == 0) {
        cp_async8(dst + m, in, 0);
        cp_async8(dst + (L + 1) * M + m, in, 0);
      }
    }
  };
  const int T = blockDim.x;
  if constexpr (esz == 8) {
    // 8-byte elements with adjacent columns: two columns per 16-byte copy when
    // the tile's first column and the row stride keep the pair 16-byte aligned
    // (a tile whose pair would cross the last valid column copies singly)
    const bool pairs = s.in_xs == 1 && M >= 2 && ((ib | s.in_axis) & 1) == 0 &&
                       (reinterpret_cast<uintptr_t>(in) & 15) == 0 && x0 + M <= s.X;
    if (pairs) {
      const int MP = M >> 1, lmp = s.log2m - 1;
      const bool identity =
          s.pre == 0 && ((s.lmap_a0 >= L && s.lmap_a1 >= L) || (s.lmap_d == 0 && s.lmap_a0 >= s.lmap_a1));
      if (WALK && identity && (T & (MP - 1)) == 0) {
        // rows one to one: each thread keeps one column pair and walks its
        // rows with addresses advanced by constant steps (faster inside the
        // batch kernel; slower for the long lines of the pass kernels, whose
        // loads are measured ~10 % slower with it)
        const int m = 2 * (threadIdx.x & (MP - 1));
        const int j0 = threadIdx.x >> lmp, js = T >> lmp;
        const char* g = in + (ib + m + (long long)j0 * s.in_axis) * esz;
        const long long gstep = (long long)js * s.in_axis * esz;
        W* d = dst + j0 * M + m;
#pragma unroll 4
        for (int j = j0; j < L; j += js, g += gstep, d += js * M) cp_async16(d, g, 16u);
        return;
      }
      for (int e = threadIdx.x; e < MP * L; e += T) {
        const int m = 2 * (e & (MP - 1));
        const int j = e >> lmp;
        const int src = j >= s.lmap_a1 ? j - s.lmap_d : (j < s.lmap_a0 ? j : -1);
        const bool ok = src >= 0;
        const char* g = ok ? in + (ib + m + (long long)src * s.in_axis) * esz : in;
        const uint32_t nb = ok ? 16u : 0u;
        int r0 = j, r1 = -1;
        if (s.pre == 2) {
          r0 = j + 1;
          r1 = 2 * (L + 1) - (j + 1);
        } else if (s.pre == 1 && j >= 1 && j <= L - 2) {
          r1 = 2 * (L - 1) - j;
        }
        cp_async16(dst + r0 * M + m, g, nb);
        if (r1 >= 0) cp_async16(dst + r1 * M + m, g, nb);
        if (s.pre == 2 && j == 0) {
          cp_async16(dst + m, in, 0);
          cp_async16(dst + (L + 1) * M + m, in, 0);
        }
      }
      return;
    }
  }
  if (s.in_xs != 1) {  // rows adjacent in memory (STRIDE1 user layout): rows fastest
    const FastDiv div_l(L);
    for (int e = threadIdx.x; e < M * L; e += T) {
      const int m = (int)div_l.div(e);
      one(m, e - m * L);
    }
  } else if ((T & (M - 1)) == 0) {  // each thread keeps one column m: rows strided by T/M
    const int m = threadIdx.x & (M - 1);
    for (int j = threadIdx.x >> s.log2m; j < L; j += T >> s.log2m) one(m, j);
  } else {
    for (int e = threadIdx.x; e < M * L; e += T) one(e & (M - 1), e >> s.log2m);
  }
}

// Copies of one tile into buffer b.  TMA: thread 0 arms the barrier and
// issues the boxes.  cp.async: every thread, one commit group per call.
template <class P>
P3G_D void strided_issue(const SPipeParams& q, const CUtensorMap* tin, int tile, int b) {
  using W = typename P::W;
  const StridedSmem<P> sm = strided_smem<P>(q.c);
  W* dst = sm.buf0 + b * q.c.buf_elems;
  int xt, o1, o2;
  strided_decode(q, tile, xt, o1, o2);
  if (q.use_tma) {
    if (threadIdx.x == 0) {
      constexpr int kWords = sizeof(W) / 4;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&sm.mbar[b], (uint32_t)(q.nbox * q.box_bytes + q.tx_extra));
      for (int i = 0; i < q.nbox; ++i)
        tma_load_4d(dst + i * q.brows * q.s.M, tin, &sm.mbar[b], xt * q.s.M * kWords, i * q.brows, o1, o2);
    }
    return;
  }
  strided_copy<P>(q.s, dst, xt, o1, o2);
  cp_async_commit();
}

// Fix-up of a loaded strided tile, element-wise in place: user format ->
// working format, DST-I negation, DCT-I mirror after a TMA load (tma).
// Ends with a barrier when it changed anything.
template <class P>
P3G_D void strided_fix(const SParams& s, bool tma, typename P::W* sm, int k, uint32_t& amax) {
  using W = typename P::W;
  using C = typename P::C;
  const bool raw_user = s.in_user != 0 && P::kF64;  // binary32 user data is the working format
  if (raw_user || s.pre == 2 || (tma && s.pre == 1)) {
    const int M = s.M, L = s.L;
    const int rows = tma ? L : s.N;
    for (int e = threadIdx.x; e < M * rows; e += blockDim.x) {
      const int m = e & (M - 1);
      const int j = e >> s.log2m;
      C v;
      if (raw_user) {
        const typename P::UC u = reinterpret_cast<const typename P::UC*>(sm)[j * M + m];
        P::track(amax, u);
        v = P::from_uc(u, k);
      } else {
        v = P::from_w(sm[j * M + m]);
      }
      if (s.pre == 2 && j >= L + 2) v = cneg(v);
      const W w = P::to_w(v);
      sm[j * M + m] = w;
      if (tma && s.pre == 1 && j >= 1 && j <= L - 2) sm[(2 * (L - 1) - j) * M + m] = w;
    }
    __syncthreads();
  }
}

// Store of a transformed strided tile with the pruning map and the output
// format (DST-I output rows k+1 times i).
template <class P>
P3G_D void strided_store(const SParams& s, const typename P::W* sm, int xt, int o1, int o2, int kb) {
  using C = typename P::C;
  const int M = s.M;
  const int ph = strided_phase(s, o1, o2);  // the tile's columns as loaded by strided_copy
  const int x0 = xt * M + ph;
  const int xend = s.X + ph;
  const long long obase = (long long)o1 * s.out_o1 + (long long)o2 * s.out_o2;
  auto one = [&](int m, int jo) {
    const int k = jo < s.smap_s0 ? jo : jo + s.smap_d;
    const int c = x0 + m < s.X ? x0 + m : x0 + m - s.X;
    C v;
    if (s.post == 1) v = rot<1>(P::from_w(sm[(k + 1) * M + m]));
    else v = P::from_w(sm[k * M + m]);
    store_elem<P>(s.out, s.out_user, obase + strided_col_out(s, c) + (long long)jo * s.out_axis, v, kb);
  };
  const int T = blockDim.x;
  if (s.tw4) {
    // four-step twiddle w_N^(o1 jo) on every stored element (rows one to one)
    const unsigned long long n4 = (unsigned long long)s.tw4_n;
    for (int e = threadIdx.x; e < M * s.Lout; e += T) {
      const int m = e & (M - 1), jo = e >> s.log2m;
      if (x0 + m >= xend) continue;
      const int c = x0 + m < s.X ? x0 + m : x0 + m - s.X;
      C v = P::from_w(sm[jo * M + m]);
      const cdf w = load_tw(s.tw4, (int)(((unsigned long long)o1 * (unsigned long long)jo) % n4));
      v = s.tw4_conj ? cmul<true>(v, w) : cmul<false>(v, w);
      store_elem<P>(s.out, s.out_user, obase + strided_col_out(s, c) + (long long)jo * s.out_axis, v, kb);
    }
    return;
  }
  if (s.out_xs == 1 && s.post == 0 && (s.smap_s0 >= s.Lout || s.smap_d == 0) && (T & (M - 1)) == 0) {
    // rows stored one to one (no pruning gap, no DST shift): each thread keeps
    // one column and walks its rows with a shared-memory address and an
    // output pointer advanced by constant steps
    const int m = threadIdx.x & (M - 1);
    if (x0 + m >= xend) return;
    const int c = x0 + m < s.X ? x0 + m : x0 + m - s.X;
    const int j0 = threadIdx.x >> s.log2m, js = T >> s.log2m;
    using W = typename P::W;
    uint32_t a = (uint32_t)__cvta_generic_to_shared(sm) + (uint32_t)((j0 * M + m) * (int)sizeof(W));
    const uint32_t astep = (uint32_t)(T * (int)sizeof(W));
    const long long o = obase + strided_col_out(s, c) + (long long)j0 * s.out_axis;
    const long long ostep = (long long)js * s.out_axis;
    if (s.out_user) {
      typename P::UC* d = static_cast<typename P::UC*>(s.out) + o;
#pragma unroll 4
      for (int jo = j0; jo < s.Lout; jo += js, a += astep, d += ostep) *d = P::to_uc(P::from_w(lds(a, (W*)nullptr)), kb);
    } else {
      W* d = static_cast<W*>(s.out) + o;
#pragma unroll 4
      for (int jo = j0; jo < s.Lout; jo += js, a += astep, d += ostep) *d = lds(a, (W*)nullptr);
    }
    return;
  }
  if (s.out_xs != 1) {  // rows adjacent in memory (STRIDE1 user layout): rows fastest
    const FastDiv div_lo(s.Lout);
    for (int e = threadIdx.x; e < M * s.Lout; e += T) {
      const int m = (int)div_lo.div(e);
      if (x0 + m < xend) one(m, e - m * s.Lout);
    }
  } else if ((T & (M - 1)) == 0) {
    const int m = threadIdx.x & (M - 1);
    if (x0 + m < xend)
      for (int jo = threadIdx.x >> s.log2m; jo < s.Lout; jo += T >> s.log2m) one(m, jo);
  } else {
    for (int e = threadIdx.x; e < M * s.Lout; e += T) {
      const int m = e & (M - 1);
      if (x0 + m < xend) one(m, e >> s.log2m);
    }
  }
}

// Waits for the copies of tile slot it (buffer it % nbuf): cp.async groups
// (nbuf - 1 may stay in flight) or the TMA mbarrier; false after a time-out.
P3G_D void cp_async_wait_ahead(int nbuf) {
  if (nbuf >= 3) cp_async_wait<2>();
  else cp_async_wait<1>();
}

template <class P, int DIR, int E>
__global__ void __launch_bounds__(PipeLimits<P, E>::kMaxThreads, PipeLimits<P, E>::kMinBlocks)
    k_strided_pipe(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout,
                   const __grid_constant__ SPipeParams pp, const StagePlan* __restrict__ sp,
                   const float4* __restrict__ tw_g) {
  const int nb = pp.c.nbuf;
  const int la = nb - 1 - pp.tma_store;  // tiles loaded ahead of the current one
  {
    const StridedSmem<P> sm = strided_smem<P>(pp.c);
    for (int i = threadIdx.x; i < pp.c.tw_count; i += blockDim.x) sm.tw[i] = __ldg(tw_g + pp.c.tw_base + i);
    if (threadIdx.x == 0 && pp.use_tma) {
      for (int i = 0; i < nb; ++i) mbar_init(&sm.mbar[i], 1);
      mbar_fence_init();
    }
  }
  __syncthreads();
  const int k = range_k(pp.s.range);
  uint32_t amax = 0;
  int it = 0;
  int tile = blockIdx.x;
  // tiles of the first la iterations in flight before the loop
  for (int j = 0; j < la; ++j) {
    const int t = tile + j * (int)gridDim.x;
    if (t < pp.c.ntiles) strided_issue<P>(pp, &tin, t, j);
    else if (!pp.use_tma) cp_async_commit();
  }
  int b = 0, ph = 0;  // buffer of iteration it and the parity of its use
#pragma unroll 1
  for (; tile < pp.c.ntiles; tile += gridDim.x, ++it) {
    bool ok = true;
    {
      const SPipeParams& q = pp;
      // into the buffer of iteration it + la - nb (with TMA stores: the
      // store issued two iterations ago, which must have read its tile)
      const int ahead = tile + la * (int)gridDim.x;
      const int bl = b + la >= nb ? b + la - nb : b + la;
      if (ahead < q.c.ntiles) {
        if (q.tma_store && threadIdx.x == 0) bulk_wait_read<1>();
        strided_issue<P>(q, &tin, ahead, bl);
      } else if (!q.use_tma) {
        cp_async_commit();  // one group per iteration
      }
      if (q.use_tma) ok = mbar_wait_bounded(&strided_smem<P>(q.c).mbar[b], ph, q.c.err);
      else cp_async_wait_ahead(nb);
    }
    if (__syncthreads_or(!ok)) break;
    strided_fix<P>(pp.s, pp.use_tma != 0, strided_smem<P>(pp.c).buf0 + b * pp.c.buf_elems, k, amax);
    {
      const SPipeParams& q = pp;
      const StridedSmem<P> sm = strided_smem<P>(q.c);
      Tile<P> t{sm.buf0 + b * q.c.buf_elems, nullptr, q.s.M, q.s.log2m, 1, q.s.M};
      cta_fft<P, DIR, E, kPointMajor, kRawNone, PipeMaxR<P, E>::value>(t, sp, sm.tw, q.c.tw_base);
    }
    {
      int xt, o1, o2;
      strided_decode(pp, tile, xt, o1, o2);
      const typename P::W* tb = strided_smem<P>(pp.c).buf0 + b * pp.c.buf_elems;
      if (pp.tma_store) {
        if constexpr (P::kF64) {
          if (pp.s.out_user) {  // binary64 user format, converted in place (16 bytes each)
            typename P::W* tm = strided_smem<P>(pp.c).buf0 + b * pp.c.buf_elems;
            const int ne = pp.s.Lout * pp.s.M;
            for (int e = threadIdx.x; e < ne; e += blockDim.x)
              reinterpret_cast<typename P::UC*>(tm)[e] = P::to_uc(P::from_w(tm[e]), k);
          }
        }
        fence_proxy_async_smem();  // this thread's tile writes, before the async-proxy reads
        __syncthreads();
        if (threadIdx.x == 0) {
          constexpr int kWords = sizeof(typename P::W) / 4;
          for (int i = 0; i < pp.onbox; ++i)
            tma_store_4d(&tout, tb + i * pp.obrows * pp.s.M, xt * pp.s.M * kWords, i * pp.obrows, o1, o2);
          bulk_commit_group();
        }
      } else {
        strided_store<P>(pp.s, tb, xt, o1, o2, k);
      }
    }
    __syncthreads();
    if (++b == nb) {
      b = 0;
      ph ^= 1;
    }
  }
  // early exit after a timed-out wait: wait (bounded) for the copies of the
  // tiles issued and not yet consumed
  if (pp.use_tma) {
    if (threadIdx.x == 0) {
      const StridedSmem<P> sm = strided_smem<P>(pp.c);
      for (int j = 0; j <= la; ++j)
        if (tile + j * (int)gridDim.x < pp.c.ntiles) {
          const int i = it + j;
          mbar_wait_bounded(&sm.mbar[i % nb], (i / nb) & 1, nullptr);
        }
    }
  } else {
    cp_async_wait<0>();
  }
  // the tile stores must have completed before the CTA's shared memory goes
  if (pp.tma_store && threadIdx.x == 0) bulk_wait_all();
  range_flush(pp.s.range, amax);
}

// ---------------------------------------------------------------- X passes
template <class P>
P3G_D typename P::W* xpipe_buf(const PipeCommon& pc, int b) {
  extern __shared__ unsigned char p3g_pipe_smem[];
  return reinterpret_cast<typename P::W*>(align1k(p3g_pipe_smem)) + b * pc.buf_elems;
}
// the bulk copies' mbarriers, one per buffer, after the buffers
template <class P>
P3G_D uint64_t* xpipe_mbar(const PipeCommon& pc) {
  return reinterpret_cast<uint64_t*>(xpipe_buf<P>(pc, pc.nbuf));
}

// cp.async of CH bytes (16, 8 or 4)
template <int CH>
P3G_D void cp_async_n(void* d, const void* g, uint32_t nb) {
  if constexpr (CH == 16) cp_async16(d, g, nb);
  else if constexpr (CH == 8) cp_async8(d, g, nb);
  else cp_async4(d, g, nb);
}

// Line by line: each thread copies every blockDim.x-th chunk of each line, with
// the line's addresses formed once (lines at least blockDim.x chunks long).
template <class P, int CH>
P3G_D void xr2c_copy_lines(const XParams& x, const char* in, char* dst, int p0) {
  using UR = typename P::UR;
  const int lbytes = x.nx * (int)sizeof(UR);
  const int step = (int)blockDim.x * CH;
  for (int lt = 0; lt < 2 * x.M; ++lt) {
    const int line = 2 * p0 + lt;
    const bool ok = line < x.nlines;
    const char* g = in + (ok ? (long long)line * x.in_line * (long long)sizeof(UR) : 0LL);
    char* d = dst + lt * lbytes;
    const uint32_t nb = ok ? (uint32_t)CH : 0u;
    for (int c = (int)threadIdx.x * CH; c < lbytes; c += step) cp_async_n<CH>(d + c, g + c, nb);
  }
}

// r2c: real lines 2p, 2p+1 of the tile (first pair p0 of field `field`)
// copied raw ([line][x]) into dst, `chunk` bytes per copy, without a commit.
template <class P>
P3G_D void xr2c_copy(const XParams& x, int chunk, typename P::W* dst_w, int p0, int field) {
  using UR = typename P::UR;
  const int M = x.M, N = x.nx;
  const char* in = reinterpret_cast<const char*>(static_cast<const UR*>(x.in) + field * x.in_field);
  char* dst = reinterpret_cast<char*>(dst_w);
  const int cpl = N * (int)sizeof(UR) / chunk;  // copies per line
  if (cpl >= (int)blockDim.x) {
    if (chunk == 16) xr2c_copy_lines<P, 16>(x, in, dst, p0);
    else if (chunk == 8) xr2c_copy_lines<P, 8>(x, in, dst, p0);
    else xr2c_copy_lines<P, 4>(x, in, dst, p0);
    return;
  }
  const FastDiv fcpl((uint32_t)cpl);
  for (int e = threadIdx.x; e < 2 * M * cpl; e += blockDim.x) {
    const int lt = (int)fcpl.div((uint32_t)e);
    const int c = e - lt * cpl;
    const int line = 2 * p0 + lt;
    const bool ok = line < x.nlines;
    const char* g = ok ? in + (long long)line * x.in_line * (long long)sizeof(UR) + (long long)c * chunk : in;
    char* d = dst + ((long long)lt * N * (long long)sizeof(UR) + (long long)c * chunk);
    const uint32_t nb = ok ? (uint32_t)chunk : 0u;
    if (chunk == 16) cp_async16(d, g, nb);
    else if (chunk == 8) cp_async8(d, g, nb);
    else cp_async4(d, g, nb);
  }
}

// r2c tiles that arrive by one bulk copy: bulk loads on and the tile's 2M
// lines all inside the field (a partial tile is zero-filled by cp.async)
P3G_D bool xr2c_tile_bulk(const XPipeParams& q, int tile) {
  if (!q.bulk) return false;
  const int field = tile / q.c.tiles_per_field;
  const int p0 = (tile - field * q.c.tiles_per_field) * q.x.M;
  return 2 * (p0 + q.x.M) <= q.x.nlines;
}

// Copies of one r2c tile into buffer b: one bulk copy by thread 0 (with an
// empty commit group so that every tile counts one group) or cp.async.
template <class P>
P3G_D void xr2c_issue(const XPipeParams& q, int tile, int b) {
  using UR = typename P::UR;
  const int field = tile / q.c.tiles_per_field;
  const int p0 = (tile - field * q.c.tiles_per_field) * q.x.M;
  if (xr2c_tile_bulk(q, tile)) {
    if (threadIdx.x == 0) {
      uint64_t* bar = xpipe_mbar<P>(q.c) + b;
      const uint32_t bytes = (uint32_t)(2 * q.x.M * q.x.nx) * (uint32_t)sizeof(UR);
      const UR* src = static_cast<const UR*>(q.x.in) + field * q.x.in_field + (long long)2 * p0 * q.x.nx;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(bar, bytes);
      bulk_load(xpipe_buf<P>(q.c, b), src, bytes, bar);
    }
  } else {
    xr2c_copy<P>(q.x, q.chunk, xpipe_buf<P>(q.c, b), p0, field);
  }
  cp_async_commit();
}


// X1[k] = (Z[k] + conj Z[N-k]) / 2, X2[k] = -i (Z[k] - conj Z[N-k]) / 2,
// modes k < nkeep stored to the working layout (USER: the user complex
// format, for the X-only transform).
template <class P, bool USER>
P3G_D void xr2c_store_t(const XParams& x, const typename P::W* sm, int p0, int field, int kb) {
  using C = typename P::C;
  using O = typename std::conditional<USER, typename P::UC, typename P::W>::type;
  const int N = x.nx, nk = x.nkeep;
  O* out = static_cast<O*>(x.out) + field * x.out_field;
  const FastDiv fnk((uint32_t)nk);
  for (int e = threadIdx.x; e < x.M * nk; e += blockDim.x) {
    const int pr = (int)fnk.div((uint32_t)e);
    const int k = e - pr * nk;
    const int line = 2 * (p0 + pr);
    if (line >= x.nlines) continue;
    const C a = P::from_w(sm[pr * x.LS + pad_index(k, x.ps)]);
    const C bb = cconj(P::from_w(sm[pr * x.LS + pad_index(k == 0 ? 0 : N - k, x.ps)]));
    const C r1 = cscale2(a + bb, 0.5f), r2 = cscale2(rot<-1>(a - bb), 0.5f);
    if constexpr (USER) {
      out[(long long)line * x.out_line + k] = P::to_uc(r1, kb);
      if (line + 1 < x.nlines) out[(long long)(line + 1) * x.out_line + k] = P::to_uc(r2, kb);
    } else {
      out[(long long)line * x.out_line + k] = P::to_w(r1);
      if (line + 1 < x.nlines) out[(long long)(line + 1) * x.out_line + k] = P::to_w(r2);
    }
  }
}
// kb: the exponent bias of the user-format output (X-only transform)
template <class P>
P3G_D void xr2c_store(const XParams& x, const typename P::W* sm, int p0, int field, int kb) {
  if (x.out_user) xr2c_store_t<P, true>(x, sm, p0, field, kb);
  else xr2c_store_t<P, false>(x, sm, p0, field, kb);
}

template <class P, int E>
__global__ void __launch_bounds__(XPipeLimits<P, E>::kMaxThreads, XPipeLimits<P, E>::kMinBlocks)
    k_xr2c_pipe(const __grid_constant__ XPipeParams pp, const StagePlan* __restrict__ sp,
                const float4* __restrict__ tw_g) {
  const int k = range_k(pp.x.range);
  const int nb = pp.c.nbuf;
  uint32_t amax = 0;
  int it = 0;
  int tile = blockIdx.x;
  if (pp.bulk && threadIdx.x == 0) {
    for (int i = 0; i < nb; ++i) mbar_init(xpipe_mbar<P>(pp.c) + i, 1);
    mbar_fence_init();
  }
  __syncthreads();
  for (int j = 0; j < nb - 1; ++j) {
    const int t = tile + j * (int)gridDim.x;
    if (t < pp.c.ntiles) xr2c_issue<P>(pp, t, j);
    else cp_async_commit();
  }
  int b = 0, ph = 0;  // buffer of iteration it and the parity of its use
#pragma unroll 1
  for (; tile < pp.c.ntiles; tile += gridDim.x, ++it) {
    const int ahead = tile + (nb - 1) * (int)gridDim.x;
    if (ahead < pp.c.ntiles) xr2c_issue<P>(pp, ahead, b == 0 ? nb - 1 : b - 1);
    else cp_async_commit();
    cp_async_wait_ahead(nb);
    const bool ok = !xr2c_tile_bulk(pp, tile) || mbar_wait_bounded(xpipe_mbar<P>(pp.c) + b, ph, pp.c.err);
    if (__syncthreads_or(!ok)) break;
    {
      // the first FFT stage reads the raw line pairs (packing fused into it)
      Tile<P> t{xpipe_buf<P>(pp.c, b), nullptr, pp.x.M, pp.x.log2m, pp.x.LS, 1, pp.x.ps, k, &amax};
      cta_fft<P, -1, E, kLineMajor, kRawR2C, PipeMaxR<P, E>::value>(t, sp, tw_g, 0);
    }
    {
      const int field = tile / pp.c.tiles_per_field;
      const int p0 = (tile - field * pp.c.tiles_per_field) * pp.x.M;
      xr2c_store<P>(pp.x, xpipe_buf<P>(pp.c, b), p0, field, k);
    }
    __syncthreads();
    if (++b == nb) {
      b = 0;
      ph ^= 1;
    }
  }
  cp_async_wait<0>();
  // early exit after a timed-out wait: wait (bounded) for bulk copies in flight
  if (threadIdx.x == 0)
    for (int j = 0; j < nb; ++j) {
      const int t = tile + j * (int)gridDim.x;
      if (t < pp.c.ntiles && xr2c_tile_bulk(pp, t))
        mbar_wait_bounded(xpipe_mbar<P>(pp.c) + (it + j) % nb, ((it + j) / nb) & 1, nullptr);
    }
  range_flush(pp.x.range, amax);
}

// c2r: complex lines 2p, 2p+1 of nh = N/2+1 modes copied raw (pair stride
// 2 nh) into dst, modes beyond nkeep as zeros, without a commit.
template <class P>
P3G_D void xc2r_copy(const XParams& x, typename P::W* dst, int p0, int field) {
  using W = typename P::W;
  const int M = x.M, nh = x.nx / 2 + 1;
  const W* in = static_cast<const W*>(x.in) + field * x.in_field;
  if constexpr (sizeof(W) == 8) {
    // two complexes per 16-byte copy: raw stride rs even, line pitch even
    const int rs = xc2r_raw_stride(nh, 8), hp = rs >> 1;
    if ((x.in_line & 1) == 0 && (reinterpret_cast<uintptr_t>(in) & 15) == 0) {
      if (hp >= (int)blockDim.x) {  // line by line, addresses formed once per line
        for (int lt = 0; lt < 2 * M; ++lt) {
          const int line = 2 * p0 + lt;
          const int keep = line < x.nlines ? x.nkeep : 0;
          const W* g = in + (line < x.nlines ? (long long)line * x.in_line : 0LL);
          W* d = dst + lt * rs;
          for (int k = 2 * (int)threadIdx.x; k < rs; k += 2 * (int)blockDim.x) {
            const int nv = min(max(keep - k, 0), 2);
            cp_async16(d + k, nv ? g + k : in, (uint32_t)(8 * nv));
          }
        }
        return;
      }
      const FastDiv fhp((uint32_t)hp);
      for (int e = threadIdx.x; e < 2 * M * hp; e += blockDim.x) {
        const int lt = (int)fhp.div((uint32_t)e);
        const int k = 2 * (e - lt * hp);
        const int line = 2 * p0 + lt;
        const int nv = line < x.nlines ? min(max(x.nkeep - k, 0), 2) : 0;  // valid elements of the pair
        const W* g = nv ? in + (long long)line * x.in_line + k : in;
        cp_async16(dst + lt * rs + k, g, (uint32_t)(8 * nv));
      }
      return;
    }
    const FastDiv fnh((uint32_t)nh);
    for (int e = threadIdx.x; e < 2 * M * nh; e += blockDim.x) {
      const int lt = (int)fnh.div((uint32_t)e);
      const int k = e - lt * nh;
      const int line = 2 * p0 + lt;
      const bool ok = line < x.nlines && k < x.nkeep;
      const W* g = ok ? in + (long long)line * x.in_line + k : in;
      cp_async8(dst + lt * rs + k, g, ok ? 8u : 0u);
    }
    return;
  }
  if (nh >= (int)blockDim.x) {  // line by line, addresses formed once per line
    for (int lt = 0; lt < 2 * M; ++lt) {
      const int line = 2 * p0 + lt;
      const int keep = line < x.nlines ? x.nkeep : 0;
      const W* g = in + (line < x.nlines ? (long long)line * x.in_line : 0LL);
      W* d = dst + lt * nh;
      for (int k = threadIdx.x; k < nh; k += blockDim.x) {
        const bool ok = k < keep;
        if constexpr (sizeof(W) == 16) cp_async16(d + k, ok ? g + k : in, ok ? 16u : 0u);
        else cp_async8(d + k, ok ? g + k : in, ok ? 8u : 0u);
      }
    }
    return;
  }
  const FastDiv fnh((uint32_t)nh);
  for (int e = threadIdx.x; e < 2 * M * nh; e += blockDim.x) {
    const int lt = (int)fnh.div((uint32_t)e);
    const int k = e - lt * nh;
    const int line = 2 * p0 + lt;
    const bool ok = line < x.nlines && k < x.nkeep;
    const W* g = ok ? in + (long long)line * x.in_line + k : in;
    if constexpr (sizeof(W) == 16) cp_async16(dst + lt * nh + k, g, ok ? 16u : 0u);
    else cp_async8(dst + lt * nh + k, g, ok ? 8u : 0u);
  }
}

// Copies of one c2r tile into buffer b: one bulk copy per line (the nh
// modes rounded up to 16 bytes, into the raw line stride) by thread 0, with an
// empty commit group, or cp.async.
template <class P>
P3G_D void xc2r_issue(const XPipeParams& q, int tile, int b) {
  using W = typename P::W;
  const int field = tile / q.c.tiles_per_field;
  const int p0 = (tile - field * q.c.tiles_per_field) * q.x.M;
  if (q.bulk) {
    if (threadIdx.x == 0) {
      const int nh = q.x.nx / 2 + 1;
      const int rs = xc2r_raw_stride(nh, (int)sizeof(W));
      const uint32_t lbytes = ((uint32_t)nh * (uint32_t)sizeof(W) + 15u) & ~15u;
      const int nl = min(2 * q.x.M, q.x.nlines - 2 * p0);
      uint64_t* bar = xpipe_mbar<P>(q.c) + b;
      const W* in = static_cast<const W*>(q.x.in) + field * q.x.in_field;
      W* dst = xpipe_buf<P>(q.c, b);
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(bar, lbytes * (uint32_t)nl);
      for (int lt = 0; lt < nl; ++lt) bulk_load(dst + lt * rs, in + (long long)(2 * p0 + lt) * q.x.in_line, lbytes, bar);
    }
  } else {
    xc2r_copy<P>(q.x, xpipe_buf<P>(q.c, b), p0, field);
  }
  cp_async_commit();
}

// x1 = Re z, x2 = Im z to the user's real lines (format conversion fused).
// Even N: each thread takes positions n, n+1 of a line pair, reads the two
// complex values once and writes two-element vectors to both lines.
template <class P>
P3G_D void xc2r_store(const XParams& x, const typename P::W* sm, int p0, int field, int k) {
  using W = typename P::W;
  using UR = typename P::UR;
  const int M = x.M, N = x.nx, LS = x.LS, ps = x.ps;
  UR* out = static_cast<UR*>(x.out) + field * x.out_field;
  const bool vec = (N & 1) == 0 && (x.out_line & 1) == 0 &&
                   (reinterpret_cast<uintptr_t>(out) & (2 * sizeof(UR) - 1)) == 0;
  if (vec) {
    const int NH = N >> 1;
    const FastDiv fNH((uint32_t)NH);
    for (int e = threadIdx.x; e < M * NH; e += blockDim.x) {
      const int pr = (int)fNH.div((uint32_t)e);
      const int n = 2 * (e - pr * NH);
      const int line = 2 * (p0 + pr);
      if (line >= x.nlines) continue;
      const W a = sm[pr * LS + pad_index(n, ps)];  // n even: n and n+1 never straddle a pad
      const W b = sm[pr * LS + pad_index(n, ps) + 1];
      UR* o = out + (long long)line * x.out_line + n;
      if constexpr (P::kF64) {
        *reinterpret_cast<double2*>(o) = make_double2(P::to_ur(df{a.x, a.z}, k), P::to_ur(df{b.x, b.z}, k));
        if (line + 1 < x.nlines)
          *reinterpret_cast<double2*>(o + x.out_line) =
              make_double2(P::to_ur(df{a.y, a.w}, k), P::to_ur(df{b.y, b.w}, k));
      } else {
        *reinterpret_cast<float2*>(o) = make_float2(a.x, b.x);
        if (line + 1 < x.nlines) *reinterpret_cast<float2*>(o + x.out_line) = make_float2(a.y, b.y);
      }
    }
    return;
  }
  const float* smf = reinterpret_cast<const float*>(sm);
  constexpr int kW = sizeof(W) / sizeof(float);
  const FastDiv fN((uint32_t)N);
  for (int e = threadIdx.x; e < 2 * M * N; e += blockDim.x) {
    const int lt = (int)fN.div((uint32_t)e);
    const int n = e - lt * N;
    const int line = 2 * p0 + lt;
    if (line >= x.nlines) continue;
    const int c = lt & 1;
    const float* f = smf + ((lt >> 1) * LS + pad_index(n, ps)) * kW;
    if constexpr (P::kF64) out[(long long)line * x.out_line + n] = P::to_ur(df{f[c], f[2 + c]}, k);
    else out[(long long)line * x.out_line + n] = f[c];
  }
}

template <class P, int E>
__global__ void __launch_bounds__(XPipeLimits<P, E>::kMaxThreads, XPipeLimits<P, E>::kMinBlocks)
    k_xc2r_pipe(const __grid_constant__ XPipeParams pp, const StagePlan* __restrict__ sp,
                const float4* __restrict__ tw_g) {
  const int k = range_k(pp.x.range);
  int it = 0;
  const int nb = pp.c.nbuf;
  int tile = blockIdx.x;
  if (pp.bulk && threadIdx.x == 0) {
    for (int i = 0; i < nb; ++i) mbar_init(xpipe_mbar<P>(pp.c) + i, 1);
    mbar_fence_init();
  }
  __syncthreads();
  for (int j = 0; j < nb - 1; ++j) {
    const int t = tile + j * (int)gridDim.x;
    if (t < pp.c.ntiles) xc2r_issue<P>(pp, t, j);
    else cp_async_commit();
  }
  int b = 0, ph = 0;  // buffer of iteration it and the parity of its use
#pragma unroll 1
  for (; tile < pp.c.ntiles; tile += gridDim.x, ++it) {
    const int ahead = tile + (nb - 1) * (int)gridDim.x;
    if (ahead < pp.c.ntiles) xc2r_issue<P>(pp, ahead, b == 0 ? nb - 1 : b - 1);
    else cp_async_commit();
    cp_async_wait_ahead(nb);
    const bool ok = !pp.bulk || mbar_wait_bounded(xpipe_mbar<P>(pp.c) + b, ph, pp.c.err);
    if (__syncthreads_or(!ok)) break;
    {
      // the first FFT stage reads the raw half spectra (Hermitian merge fused into it)
      Tile<P> t{xpipe_buf<P>(pp.c, b), nullptr, pp.x.M, pp.x.log2m, pp.x.LS, 1, pp.x.ps};
      cta_fft<P, 1, E, kLineMajor, kRawC2R, PipeMaxR<P, E>::value>(t, sp, tw_g, 0);
    }
    {
      const int field = tile / pp.c.tiles_per_field;
      const int p0 = (tile - field * pp.c.tiles_per_field) * pp.x.M;
      xc2r_store<P>(pp.x, xpipe_buf<P>(pp.c, b), p0, field, k);
    }
    __syncthreads();
    if (++b == nb) {
      b = 0;
      ph ^= 1;
    }
  }
  cp_async_wait<0>();
  // early exit after a timed-out wait: wait (bounded) for bulk copies in flight
  if (pp.bulk && threadIdx.x == 0)
    for (int j = 0; j < nb; ++j)
      if (tile + j * (int)gridDim.x < pp.c.ntiles)
        mbar_wait_bounded(xpipe_mbar<P>(pp.c) + (it + j) % nb, ((it + j) / nb) & 1, nullptr);
}

}  // namespace p3g
