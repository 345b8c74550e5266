// CTA-level mixed-radix Stockham FFT over a tile of M lines in shared memory.
//
// A tile holds M independent lines of N complex points.  Element (line, j)
// lives at sm[line * LS + j * JS]; the X passes use line-major tiles
// (LS = N, JS = 1), the strided Y/Z passes point-major tiles (LS = 1, JS = M)
// so that consecutive threads touch consecutive x columns.
//
// Each stage of radix R runs the Stockham autosort step (Govindaraju et al.,
// SC'08): butterfly j of a line reads points j + q N/R (q < R), multiplies them
// by w_{Ns R}^{q (j mod Ns)}, runs a register DFT of size R and writes points
// (j / Ns) Ns R + (j mod Ns) + q Ns.  All reads of a stage finish before any
// write (one barrier), so a stage works in place: every thread keeps all of its
// butterflies of the stage in registers (at most ceil(E/R), E = elements per
// thread, which the launch guarantees by using ceil(M N / E) threads).
//
// Radices 2, 3, 4, 5, 8, 16, 32 are register codelets.  Any other prime p runs a
// generic direct-DFT stage through a second shared-memory buffer (O(N p) work).
#pragma once

#include "p3g_codelets.cuh"

namespace p3g {

constexpr int kMaxStages = 20;
constexpr int kElemsPerThread = 16;  // E

struct StagePlan {
  int n;                   // transform length (1 allowed: no stages)
  int nstages;
  int has_generic;         // a stage with a radix outside {2,3,4,5,8,16}
  int cnt[7];              // number of stages of radix 32, 16, 8, 4, 2, 3, 5 (stored in this order, then generic)
  int radix[kMaxStages];
  int ns[kMaxStages];      // sub-transform length before the stage
  int tw_off[kMaxStages];  // float4 offset of this stage's twiddles [k < ns][q-1 < radix-1]
  int root_off[kMaxStages];  // generic stages: float4 offset of the radix-th roots of unity
};

// Twiddles are stored for the forward sign (exp(-2 pi i ...)) as double-float
// complex float4 (re.hi, im.hi, re.lo, im.lo); the backward direction
// multiplies by the conjugate.
P3G_D cdf load_tw(const float4* __restrict__ tw, int idx) {
  const float4 v = tw[idx];  // shared memory (pipelined passes) or global
  return cdf{df{v.x, v.z}, df{v.y, v.w}};
}

// Division by a runtime divisor d <= 2^15 for dividends x < 2^15 with one
// multiply-high: q = floor(2x * ceil(2^31/d) / 2^32).  Exact because the
// magic's excess over 2^31/d is below 1/d and x < 2^15 (the error term stays
// under 1/d).  Tiles hold at most 2^14 elements, so every index fits.
// Powers of two use a shift (m == 0).
struct FastDiv {
  uint32_t d, m, sh;
  P3G_D explicit FastDiv(uint32_t dd) : d(dd), m(0), sh(0) {
    if ((dd & (dd - 1)) == 0) sh = (uint32_t)(__ffs((int)dd) - 1);
    else m = 0x7FFFFFFFu / dd + 1;  // ceil(2^31 / d)
  }
  P3G_D uint32_t div(uint32_t x) const { return m ? __umulhi(x << 1, m) : (x >> sh); }
  P3G_D void divmod(uint32_t x, uint32_t& q, uint32_t& r) const {
    q = div(x);
    r = x - q * d;
  }
};

// Shared-memory element access through 32-bit shared addresses (ld/st.shared)
// rather than generic pointers.
P3G_D float4 lds(uint32_t a, float4*) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
  return v;
}
P3G_D float2 lds(uint32_t a, float2*) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(a));
  return v;
}
P3G_D double lds1(uint32_t a, double*) {
  double v;
  asm volatile("ld.shared.f64 %0, [%1];\n" : "=d"(v) : "r"(a));
  return v;
}
P3G_D float lds1(uint32_t a, float*) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];\n" : "=f"(v) : "r"(a));
  return v;
}
P3G_D void sts(uint32_t a, float4 v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"r"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
}
P3G_D void sts(uint32_t a, float2 v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};\n" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

// Line-major tiles may be padded by one element every 2^ps elements
// (ps = log2 of the plan's first radix, 0 = no padding) so that the first
// stage's stride-R writes hit distinct banks.  For the plans that use it
// (all radices powers of two, every stage's N/R and every later stage's
// sub-length multiples of 2^ps) each stage's R inputs and R outputs stay
// equally spaced in the padded layout.
P3G_D int pad_index(int j, int ps) { return ps ? j + (j >> ps) : j; }

template <class P>
struct Tile {
  typename P::W* sm;       // M lines x N points
  typename P::W* scratch;  // same size, generic stages only
  int M, log2m, LS, JS;    // point-major tiles (LS = 1) always have JS = M
  int ps = 0;              // line-major padding shift (0: none)
  // kRawR2C first stage only: the binary64 exponent bias of the conversion
  // and the thread's running largest |high word| (null: not tracked)
  int ebias = 0;
  uint32_t* amax = nullptr;
  P3G_D int addr(int line, int j) const { return line * LS + (LS == 1 ? j * JS : pad_index(j, ps)); }
  P3G_D uint32_t saddr(int line, int j) const {
    return (uint32_t)__cvta_generic_to_shared(sm) + (uint32_t)((line * LS + j * JS) * (int)sizeof(typename P::W));
  }
  // butterfly b -> (line, j) over M lines x (N / R) butterflies per line
  P3G_D void decode(int b, int per_line, int& line, int& j) const {
    if (LS == 1) {  // point-major: line fastest
      line = b & (M - 1);
      j = b >> log2m;
    } else {
      line = b / per_line;
      j = b - line * per_line;
    }
  }
  P3G_D void decode(int b, const FastDiv& per_line, int& line, int& j) const {
    if (LS == 1) {
      line = b & (M - 1);
      j = b >> log2m;
    } else {
      uint32_t q, r;
      per_line.divmod((uint32_t)b, q, r);
      line = (int)q;
      j = (int)r;
    }
  }
};

// Hardware barrier with a compile-time id.  Each radix uses its own id: with a
// plain __syncthreads() the compiler merges the identical barriers of all
// switch cases in cta_fft, which keeps every case's registers live at once.
template <int ID>
P3G_D void cta_barrier() {
  asm volatile("bar.sync %0;" ::"n"(ID) : "memory");
}

// Tile layouts a kernel can fix at compile time: the strided passes use
// point-major tiles (LS = 1, JS = M), the X passes line-major ones (LS =
// padded N, JS = 1); kAnyLayout reads the layout from the tile.
enum { kAnyLayout = -1, kLineMajor = 0, kPointMajor = 1 };

// One stage of radix R.  FULL: every thread owns exactly MAXB butterflies
// (M N / R == MAXB x blockDim.x, the usual case), so no butterfly needs a
// guard or a placeholder value.  With a known layout the butterfly -> point
// mapping needs no runtime layout test: point-major, butterfly b reads
// element b (line b mod M, position b / M); line-major, b / (N / R) is the
// line.  In the power-of-two families ns is a power of two (they run first),
// so the twiddle index is a mask.
//
// RAW (first stage of a line-major X tile only) reads the tile's raw line
// pairs instead of the packed complex line, so no separate pass precedes the
// FFT:
//   kRawR2C: real lines 2*line, 2*line+1 ([line][x], one user real each);
//            z[p] = x1[p] + i x2[p].
//   kRawC2R: the pair's half spectra (lines 2*line, 2*line+1 at a stride of
//            rs working-format complexes, nh = N/2+1 modes each); the
//            Hermitian extension z[p] = X1[p] + i X2[p] with
//            X[p] = conj X[N-p] above N/2 and the imaginary parts of the
//            p = 0 and p = N/2 modes ignored (as c2r does).
enum { kRawNone = 0, kRawR2C = 1, kRawC2R = 2 };

template <class P, int DIR, int R, int E, int LAY, bool FULL, int RAW = kRawNone>
__device__ __forceinline__ void stage_reg(const Tile<P>& t, int N, int ns, const float4* __restrict__ tw) {
  using C = typename P::C;
  using W = typename P::W;
  constexpr int MAXB = (E + R - 1) / R;
  constexpr bool kPow2 = (R & (R - 1)) == 0;
  constexpr uint32_t kW = (uint32_t)sizeof(W);
  const int per_line = N / R;
  const int T = blockDim.x;
  const bool pm = LAY == kPointMajor || (LAY == kAnyLayout && t.LS == 1);
  const FastDiv fd_line((uint32_t)(pm ? 1 : per_line)), fd_ns((uint32_t)(kPow2 ? 1 : ns));
  const int nb = t.M * per_line;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(t.sm);
  const int ps = pm ? 0 : t.ps;
  // bytes between inputs q, q+1 and between outputs q, q+1
  const uint32_t jstride = pm ? ((uint32_t)per_line << t.log2m) * kW
                              : (uint32_t)(t.JS * (int)kW) * (uint32_t)pad_index(per_line, ps);
  const uint32_t ostride =
      pm ? ((uint32_t)ns << t.log2m) * kW : (uint32_t)(t.JS * (int)kW) * (uint32_t)pad_index(ns, ps);
  // Non-full stages: explicitly initialised, because the arrays are written
  // and read under correlated guards (b < nb) the compiler cannot prove, and
  // inside a persistent tile loop an uninitialised element would otherwise be
  // kept live around the loop, with every codelet's registers.
  C v[MAXB][R];
  uint32_t oaddr[MAXB];
  bool live[MAXB];
  if constexpr (!FULL) {
#pragma unroll
    for (int i = 0; i < MAXB; ++i) {
      oaddr[i] = 0;
#pragma unroll
      for (int q = 0; q < R; ++q) v[i][q] = P::zero();
    }
  }
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    const int b = threadIdx.x + i * T;
    live[i] = FULL || b < nb;
    if (live[i]) {
      int line, j;
      uint32_t ia;
      if (pm) {
        line = b & (t.M - 1);
        j = b >> t.log2m;
        ia = sbase + (uint32_t)b * kW;
      } else {
        uint32_t q, r;
        fd_line.divmod((uint32_t)b, q, r);
        line = (int)q;
        j = (int)r;
        ia = sbase + (uint32_t)(t.addr(line, j) * (int)kW);
      }
      if constexpr (RAW == kRawR2C) {
        using UR = typename P::UR;
        constexpr uint32_t kU = (uint32_t)sizeof(UR);
        const uint32_t ra = sbase + (uint32_t)((2 * line * N + j) * (int)kU);
        const uint32_t rstep = (uint32_t)per_line * kU, lstep = (uint32_t)N * kU;
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const UR x1 = lds1(ra + q * rstep, (UR*)nullptr), x2 = lds1(ra + lstep + q * rstep, (UR*)nullptr);
          if (t.amax) {
            P::track(*t.amax, x1);
            P::track(*t.amax, x2);
          }
          v[i][q] = P::make(P::from_ur(x1, t.ebias), P::from_ur(x2, t.ebias));
        }
      } else if constexpr (RAW == kRawC2R) {
        const int nh = N / 2 + 1;
        const int rs = sizeof(W) == 8 ? (nh + 1) & ~1 : nh;  // raw line stride (xc2r_raw_stride)
        const uint32_t ra = sbase + (uint32_t)(line * 2 * rs * (int)kW);
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const int pt = j + q * per_line;
          const bool mir = 2 * pt > N;
          const int pm = mir ? N - pt : pt;
          C x1 = P::from_w(lds(ra + (uint32_t)(pm * (int)kW), (W*)nullptr));
          C x2 = P::from_w(lds(ra + (uint32_t)((rs + pm) * (int)kW), (W*)nullptr));
          if (pm == 0 || 2 * pm == N) {
            x1 = P::make(P::re(x1), P::re(P::zero()));
            x2 = P::make(P::re(x2), P::re(P::zero()));
          }
          if (mir) {
            x1 = cconj(x1);
            x2 = cconj(x2);
          }
          v[i][q] = x1 + rot<1>(x2);
        }
      } else {
#pragma unroll
        for (int q = 0; q < R; ++q) v[i][q] = P::from_w(lds(ia + q * jstride, (W*)nullptr));
      }
      const int k = kPow2 ? (j & (ns - 1)) : (int)(j - fd_ns.div((uint32_t)j) * (uint32_t)ns);
      if (ns > 1) {
        const float4* twp = tw + k * (R - 1) - 1;
#pragma unroll
        for (int q = 1; q < R; ++q) v[i][q] = cmul<(DIR > 0)>(v[i][q], load_tw(twp, q));
      }
      dft<R, DIR>(v[i]);
      const int jo = (j - k) * R + k;
      oaddr[i] = sbase + (pm ? (uint32_t)(line + (jo << t.log2m)) * kW : (uint32_t)(t.addr(line, jo) * (int)kW));
    }
  }
  cta_barrier<(R == 16 ? 1 : (R == 32 ? 6 : R))>();
#pragma unroll
  for (int i = 0; i < MAXB; ++i) {
    if (live[i]) {
#pragma unroll
      for (int q = 0; q < R; ++q) sts(oaddr[i] + q * ostride, P::to_w(v[i][q]));
    }
  }
  cta_barrier<(R == 16 ? 1 : (R == 32 ? 6 : R))>();
}

// Generic prime radix p: twiddle the inputs into scratch, then each output is
// a direct p-term sum with the p-th roots of unity.
template <class P, int DIR>
__device__ __noinline__ void stage_generic(const Tile<P>& t, int N, int p, int ns, const float4* __restrict__ tw,
                                           const float4* __restrict__ roots) {
  using C = typename P::C;
  const int per_line = N / p;
  const int total = t.M * N;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    int line, idx;
    t.decode(e, N, line, idx);
    const int q = idx / per_line;
    const int j = idx - q * per_line;
    C v = P::from_w(t.sm[t.addr(line, idx)]);
    const int k = j % ns;
    if (q > 0 && ns > 1) v = cmul<(DIR > 0)>(v, load_tw(tw, k * (p - 1) + q - 1));
    t.scratch[t.addr(line, idx)] = P::to_w(v);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    int line, idx;
    t.decode(e, N, line, idx);
    const int kout = idx / per_line;  // output index within the butterfly
    const int j = idx - kout * per_line;
    C acc = P::from_w(t.scratch[t.addr(line, j)]);
    int m = 0;
    for (int q = 1; q < p; ++q) {
      m += kout;
      if (m >= p) m -= p;
      const C x = P::from_w(t.scratch[t.addr(line, j + q * per_line)]);
      acc = acc + (m == 0 ? x : cmul<(DIR > 0)>(x, load_tw(roots, m)));
    }
    const int k = j % ns;
    t.sm[t.addr(line, (j - k) * p + k + kout * ns)] = P::to_w(acc);
  }
  __syncthreads();
}

// Stage s of radix R reads its twiddles at tw_off(s) and has sub-transform
// length ns(s) = product of the radices before it; both follow from the
// family counts, so they are carried in registers instead of being loaded
// per stage (stage 0 owns one placeholder twiddle, see build_stages).
template <class P, int DIR, int R, int E, int LAY, int RAW>
__device__ __forceinline__ void run_family(const Tile<P>& t, const float4* __restrict__ tw, int N, int cnt, int& ns,
                                           int& off, bool& raw) {
  constexpr int MAXB = (E + R - 1) / R;
  const bool full = t.M * (N / R) == MAXB * (int)blockDim.x;
#pragma unroll 1
  for (int c = 0; c < cnt; ++c) {
    if (RAW != kRawNone && raw) {  // the plan's first stage reads the raw line pairs
      if (full) stage_reg<P, DIR, R, E, LAY, true, RAW>(t, N, ns, tw + off);
      else stage_reg<P, DIR, R, E, LAY, false, RAW>(t, N, ns, tw + off);
      raw = false;
    } else if (full) {
      stage_reg<P, DIR, R, E, LAY, true>(t, N, ns, tw + off);
    } else {
      stage_reg<P, DIR, R, E, LAY, false>(t, N, ns, tw + off);
    }
    off += ns > 1 ? ns * (R - 1) : 1;
    ns *= R;
  }
}

// Runs all stages of the plan on the tile (sm must be filled and
// synchronised).  MAXR is the largest power-of-two radix compiled in: 16 on
// the F32 path and 8 on F64, 32 and 16 in the wide pipelined kernels (the
// large codelets need many registers, so only kernels that may use them
// carry them; the plans they run never exceed MAXR).  The plan orders its stages by radix family (16, 8, 4, 2, 3,
// 5, then generic primes) and each family runs in its own loop: a single loop
// with a switch over the radix makes the register allocator keep the live
// ranges of every codelet at once and spill.  Radix 16 is compiled only for
// the F32 path (the F64 codelet needs ~200 registers; radix 8 has the same
// double-float operation count per point for the sizes used here).
// tw points at the twiddle table entry tw_base (the full table with
// tw_base = 0, or a pass's slice copied to shared memory).  E = elements each
// thread holds per stage; the launch uses ceil(M N / E) threads.  LAY: the
// tile layout when the caller knows it (kPointMajor, kLineMajor).  RAW: the
// tile still holds the raw line pairs of an X r2c or c2r tile (kRawR2C,
// kRawC2R; plans without generic stages only), read by the first stage.
template <class P, int DIR, int E = kElemsPerThread, int LAY = kAnyLayout, int RAW = kRawNone,
          int MAXR = P::kF64 ? 8 : 16>
__device__ __forceinline__ void cta_fft(const Tile<P>& t, const StagePlan* __restrict__ sp,
                                        const float4* __restrict__ tw, int tw_base = 0) {
  const int N = __ldg(&sp->n);
  int c[7];
#pragma unroll
  for (int i = 0; i < 7; ++i) c[i] = __ldg(&sp->cnt[i]);
  const int nst = __ldg(&sp->nstages);
  int ns = 1;
  int off = __ldg(&sp->tw_off[0]) - tw_base;
  bool raw = RAW != kRawNone;
  if constexpr (MAXR >= 32) run_family<P, DIR, 32, E, LAY, RAW>(t, tw, N, c[0], ns, off, raw);
  if constexpr (MAXR >= 16) run_family<P, DIR, 16, E, LAY, RAW>(t, tw, N, c[1], ns, off, raw);
  run_family<P, DIR, 8, E, LAY, RAW>(t, tw, N, c[2], ns, off, raw);
  run_family<P, DIR, 4, E, LAY, RAW>(t, tw, N, c[3], ns, off, raw);
  run_family<P, DIR, 2, E, LAY, RAW>(t, tw, N, c[4], ns, off, raw);
  run_family<P, DIR, 3, E, LAY, RAW>(t, tw, N, c[5], ns, off, raw);
  run_family<P, DIR, 5, E, LAY, RAW>(t, tw, N, c[6], ns, off, raw);
  const int sg = c[0] + c[1] + c[2] + c[3] + c[4] + c[5] + c[6];
#pragma unroll 1
  for (int s = sg; s < nst; ++s)
    stage_generic<P, DIR>(t, N, __ldg(&sp->radix[s]), __ldg(&sp->ns[s]), tw + (__ldg(&sp->tw_off[s]) - tw_base),
                          tw + (__ldg(&sp->root_off[s]) - tw_base));
}

}  // namespace p3g
