// Arithmetic building blocks for the GB300 FFT passes.
//
// Two working precisions:
//   * F64 path: data enters and leaves as IEEE binary64, but every butterfly runs
//     in "double-float" arithmetic: a value is an unevaluated sum hi + lo of two
//     binary32 numbers (about 48 significant bits).  GB300 executes FP32 FMA at
//     ~126 lanes/clk/SM against ~1.7 lanes/clk/SM for FP64 FMA, so double-float
//     butterflies are ~10x cheaper than native FP64 ones at the accuracy the
//     P3DFFT double-precision contract needs (normalised L-inf <= 1e-12).
//   * F32 path: plain binary32 data with twiddles kept as hi + lo pairs, so the
//     twiddle product is compensated (x*w_hi + x*w_lo).
//
// Conversions between binary64 and double-float use integer bit manipulation
// only (no FP64 pipe instructions), see d2df / df2d below.  They are
// __host__ __device__ so the CPU tests can check them bit for bit.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define P3G_HD __host__ __device__ __forceinline__
#define P3G_D __device__ __forceinline__
#else
#define P3G_HD inline
#define P3G_D inline
#endif

namespace p3g {

// ---------------------------------------------------------------- bit casts
P3G_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
P3G_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
P3G_HD uint64_t d2u(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
P3G_HD double u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
P3G_HD float u32_to_f32_rn(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return __uint2float_rn(v);
#else
  return (float)v;
#endif
}

// Rounded FP32 ops that the compiler must not fuse into FMAs (error-free
// transformations rely on each operation being rounded separately).
P3G_HD float fadd_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;
  return r;
#endif
}
P3G_HD float fsub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
P3G_HD float fmul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
P3G_HD float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// ---------------------------------------------------------------- types
struct df {
  float hi, lo;
};
struct cdf {  // double-float complex
  df re, im;
};
struct cf {  // binary32 complex
  float re, im;
};

// Knuth TwoSum: s + e == a + b exactly.
P3G_HD void two_sum(float a, float b, float& s, float& e) {
  s = fadd_rn(a, b);
  float bb = fsub_rn(s, a);
  e = fadd_rn(fsub_rn(a, fsub_rn(s, bb)), fsub_rn(b, bb));
}

// ------------------------------------------------- binary64 <-> double-float
// d2df: hi takes the sign, exponent and the top 23 fraction bits of x
// (truncated), lo = the remaining 29 fraction bits, rounded once to 24 bits.
// |hi + lo - x| <= 2^-48 |x| for 2^-74 <= |x| < 2^128.  Below 2^-74 lo is
// dropped (relative error <= 2^-23), below 2^-126 the value flushes to a signed
// zero, at or above 2^128 hi is +-inf: the F64 path has binary32's exponent
// range, and its error bound is relative to the largest magnitude of a field.
//
// d2df_edge handles every exponent; d2df takes a shorter route for binary64
// exponents 949..1150 (2^-74 <= |x| < 2^128, the values FFT data has) and
// gives the same bits: hi is the high word rebiased and funnel-shifted by 3,
// lo = rem * 2^(e-1075) with the sign in the scale and +0 added, so that
// rem == 0 gives +0 as the edge route does.
P3G_HD df d2df_edge(double x) {
  const uint64_t b = d2u(x);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const uint32_t sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7FFu);
  df r;
  if (e < 897) {  // |x| < 2^-126 (also zero and binary64 subnormals)
    r.hi = u2f(sign);
    r.lo = 0.0f;
    return r;
  }
  if (e > 1150) {  // |x| >= 2^128, inf, nan
    const uint32_t nanbit = (e == 2047 && ((hw & 0xFFFFFu) | lw)) ? 0x400000u : 0u;
    r.hi = u2f(sign | 0x7F800000u | nanbit);
    r.lo = 0.0f;
    return r;
  }
  const uint32_t m23 = ((hw & 0xFFFFFu) << 3) | (lw >> 29);
  r.hi = u2f(sign | ((uint32_t)(e - 896) << 23) | m23);
  const uint32_t rem = lw & 0x1FFFFFFFu;
  if (e >= 949 && rem != 0u) {
    // rem * 2^(e-1075): scale by an exact power of two (normal for e >= 949)
    const float lo = u32_to_f32_rn(rem) * u2f((uint32_t)(e - 948) << 23);
    r.lo = u2f(f2u(lo) | sign);
  } else {
    r.lo = 0.0f;
  }
  return r;
}

// (hi:lo) << 3, upper word
P3G_HD uint32_t shl3_funnel(uint32_t lo, uint32_t hi) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, 3);
#else
  return (hi << 3) | (lo >> 29);
#endif
}

P3G_HD df d2df(double x) {
  const uint64_t b = d2u(x);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const uint32_t a = hw & 0x7FFFFFFFu;
  if (a - (949u << 20) >= (202u << 20)) return d2df_edge(x);  // e < 949 or e > 1150
  const uint32_t hb = shl3_funnel(lw, a - (896u << 20)) | (hw & 0x80000000u);
  // 2^(e-1075) = 2^(e_hi - 179) with the sign of x; e_hi >= 53, so the
  // subtraction stays inside the exponent field
  const uint32_t scale = (hb & 0xFF800000u) - (52u << 23);
  df r;
  r.hi = u2f(hb);
  r.lo = ffma(u32_to_f32_rn(lw & 0x1FFFFFFFu), u2f(scale), 0.0f);
  return r;
}

// Nearest integer of a binary32 value below 2^30.
P3G_HD int32_t f32_to_i32_rn(float v) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(v);
#else
  return (int32_t)std::nearbyint(v);
#endif
}

// df2d: hi + lo rounded to binary64 (error <= 1/2 ulp of the result for
// |hi + lo| >= 2^-75, below that the lo part is dropped).  The pair is made
// canonical with TwoSum (s + t == hi + lo, |t| <= ulp32(s)/2), s is widened
// exactly, and t, scaled to binary64 ulps of s (|k| <= 2^29) and rounded to an
// integer with one F2I, is added to the bit pattern.  A step that lowers |s|
// from an exact power of two counts in the half-size ulps of the binade below.
// No step crosses a binade otherwise: the widened s has at least 2^29 ulps of
// mantissa above its binade and at least 2^29 below the next.  Subnormal
// binary32 parts are flushed.
//
// df2d_st converts any canonical pair (s, t); df2d takes a shorter route when
// s's binary32 exponent is 52..254 and s is not a power of two (so no binade
// change can happen): t, its sign taken relative to s, becomes a signed k that
// is added to the 64-bit pattern, with the same result as df2d_st.
P3G_HD double df2d_st(float s, float t) {
  const uint32_t sb = f2u(s);
  const uint32_t sign = sb & 0x80000000u;
  const int es = (int)((sb >> 23) & 0xFFu);
  const uint32_t ms = sb & 0x7FFFFFu;
  if (es == 0) return u2d((uint64_t)sign << 32);
  if (es == 255) return u2d(((uint64_t)(sign | 0x7FF00000u | (ms ? 0x80000u : 0u))) << 32);
  const uint64_t d = ((uint64_t)(sign | ((uint32_t)(es + 896) << 20) | (ms >> 3)) << 32) |
                     ((uint64_t)(ms & 7u) << 29);
  const uint32_t tb = f2u(t);
  const bool down = ((tb ^ sb) & 0x80000000u) != 0u;  // t lowers |s|
  // one binary64 ulp of s is 2^(es-179); 2^(179-es) has biased exponent 306-es
  const int scale_e = 306 - es + ((down && ms == 0u) ? 1 : 0);
  if ((tb & 0x7FFFFFFFu) == 0u || scale_e > 254) return u2d(d);
  const int64_t k = f32_to_i32_rn(u2f(tb & 0x7FFFFFFFu) * u2f((uint32_t)scale_e << 23));
  return u2d(down ? d - (uint64_t)k : d + (uint64_t)k);
}

P3G_HD double df2d(float hi, float lo) {
  float s, t;
  two_sum(hi, lo, s, t);
  const uint32_t sb = f2u(s);
  const uint32_t ex = sb & 0x7F800000u;
  if (ex - (52u << 23) >= (203u << 23) || (sb & 0x7FFFFFu) == 0u) return df2d_st(s, t);
  // widened s: sign | (es + 896) << 20 | ms >> 3 : (ms & 7) << 29
  const uint32_t dh = (((sb >> 3) & 0x0FFFFFFFu) | (sb & 0x80000000u)) + (896u << 20);
  const uint32_t dl = sb << 29;
  // k = t / ulp64(s) rounded, positive when t raises |s|
  const int32_t k = f32_to_i32_rn(u2f(f2u(t) ^ (sb & 0x80000000u)) * u2f((306u << 23) - ex));
  const uint64_t d = ((uint64_t)dh << 32) | dl;
  return u2d(d + (uint64_t)(int64_t)k);
}

// -------------------------------------------- exponent bias (binary64 range)
// The double-float pairs have binary32's exponent range, so the F64 path
// scales a field by an exact power of two 2^-k on its way in (binary64 ->
// double-float) and by 2^k on its way out, with k chosen from the field's
// largest magnitude.  Scaling by a power of two only moves the exponent, so
// the result is the same as the unscaled transform's wherever both exist.

// x * 2^-k as double-float (k = 0: d2df).  Zeros, binary64 subnormals,
// infinities and NaNs keep their class; a result below 2^-1022 flushes to a
// signed zero and one at or above 2^1024 becomes a signed infinity.
P3G_HD df d2df_scaled(double x, int k) {
  if (k == 0) return d2df(x);
  const uint64_t b = d2u(x);
  const uint32_t hw = (uint32_t)(b >> 32);
  const int e = (int)((hw >> 20) & 0x7FFu);
  if (e == 0 || e == 2047) return d2df_edge(x);
  const int e2 = e - k;
  if (e2 < 1) return df{u2f(hw & 0x80000000u), 0.0f};
  if (e2 > 2046) return df{u2f((hw & 0x80000000u) | 0x7F800000u), 0.0f};
  const uint32_t hw2 = (hw & 0x800FFFFFu) | ((uint32_t)e2 << 20);
  return d2df(u2d(((uint64_t)hw2 << 32) | (uint32_t)b));
}

// d * 2^k for a binary64 d (k = 0: d).  Zeros, infinities and NaNs keep their
// class; a result below 2^-1022 flushes to a signed zero, one at or above
// 2^1024 becomes a signed infinity.
P3G_HD double scale_pow2(double d, int k) {
  if (k == 0) return d;
  const uint64_t b = d2u(d);
  const uint32_t hw = (uint32_t)(b >> 32);
  const int e = (int)((hw >> 20) & 0x7FFu);
  if (e == 0 || e == 2047) return d;
  const int e2 = e + k;
  if (e2 < 1) return u2d((uint64_t)(hw & 0x80000000u) << 32);
  if (e2 > 2046) return u2d((uint64_t)((hw & 0x80000000u) | 0x7FF00000u) << 32);
  return u2d(((uint64_t)((hw & 0x800FFFFFu) | ((uint32_t)e2 << 20)) << 32) | (uint32_t)b);
}

// The window of largest magnitudes the F64 path transforms without a bias:
// 2^kRangeLo <= max |x| < 2^(kRangeTop - log2n + 1), where 2^log2n bounds the
// transform's gain (nx ny 2 (nz + 1) covers the DCT-I/DST-I extensions).
// Above it a partial sum could reach binary32's 2^128; below it the low words
// of the pairs (2^-48 of the largest value) would fall out of binary32's
// normal range.
constexpr int kRangeLo = -50;
constexpr int kRangeTop = 124;

// Exponent bias for a field whose largest |high word| (sign cleared) is amax:
// 0 inside the window, else the unbiased exponent E of the largest magnitude
// (which scales it into [1, 2)).  Fields of zeros and binary64 subnormals
// only, and fields holding an infinity or a NaN, are not scaled.
P3G_HD int range_bias(uint32_t amax, int log2n) {
  const int e = (int)(amax >> 20);
  if (e == 0 || e >= 2047) return 0;
  const int E = e - 1023;
  if (E >= kRangeLo && E <= kRangeTop - log2n) return 0;
  return E;
}

// ------------------------------------------------------- double-float ops
// The ops keep (hi, lo) unnormalised: hi is always a rounded partial result and
// lo collects exact error terms and the low-order parts.  The absolute error
// of each op is ~2^-48 of its operands' magnitude, which is what a norm-wise
// FFT error bound needs; no renormalisation happens inside a pass.
P3G_D df dadd(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  df r;
  r.hi = s;
  r.lo = fadd_rn(fadd_rn(a.lo, b.lo), e);
  return r;
}
P3G_D df dsub(df a, df b) {
  float s, e;
  two_sum(a.hi, -b.hi, s, e);
  df r;
  r.hi = s;
  r.lo = fadd_rn(fsub_rn(a.lo, b.lo), e);
  return r;
}
P3G_D df dneg(df a) { return df{-a.hi, -a.lo}; }
// a * c for a double-float constant c (the lo*lo term is below 2^-48)
P3G_D df dmulc(df a, float chi, float clo) {
  df r;
  r.hi = fmul_rn(a.hi, chi);
  float e = ffma(a.hi, chi, -r.hi);
  e = ffma(a.hi, clo, e);
  r.lo = ffma(a.lo, chi, e);
  return r;
}
// exact scaling by a power of two
P3G_D df dscale2(df a, float p2) { return df{a.hi * p2, a.lo * p2}; }

// ------------------------------------------------------------- complex ops
P3G_D cdf operator+(cdf a, cdf b) { return cdf{dadd(a.re, b.re), dadd(a.im, b.im)}; }
P3G_D cdf operator-(cdf a, cdf b) { return cdf{dsub(a.re, b.re), dsub(a.im, b.im)}; }
P3G_D cf operator+(cf a, cf b) { return cf{a.re + b.re, a.im + b.im}; }
P3G_D cf operator-(cf a, cf b) { return cf{a.re - b.re, a.im - b.im}; }

// multiply by s*i with s = +1 or -1
template <int S>
P3G_D cdf rot(cdf a) {
  return S > 0 ? cdf{dneg(a.im), a.re} : cdf{a.im, dneg(a.re)};
}
template <int S>
P3G_D cf rot(cf a) {
  return S > 0 ? cf{-a.im, a.re} : cf{a.im, -a.re};
}
P3G_D cdf cneg(cdf a) { return cdf{dneg(a.re), dneg(a.im)}; }
P3G_D cf cneg(cf a) { return cf{-a.re, -a.im}; }
P3G_D cdf cscale2(cdf a, float p2) { return cdf{dscale2(a.re, p2), dscale2(a.im, p2)}; }
P3G_D cf cscale2(cf a, float p2) { return cf{a.re * p2, a.im * p2}; }
P3G_D cdf cconj(cdf a) { return cdf{a.re, dneg(a.im)}; }
P3G_D cf cconj(cf a) { return cf{a.re, -a.im}; }

// real double-float constant (hi, lo) times complex
P3G_D cdf mulr(cdf a, float chi, float clo) { return cdf{dmulc(a.re, chi, clo), dmulc(a.im, chi, clo)}; }
P3G_D cf mulr(cf a, float chi, float /*clo*/) { return cf{a.re * chi, a.im * chi}; }

// sum of two exact-ish products p1 + s2*p2 where p = x*y, used by the complex
// multiply: returns (x1*y1 + sg*x2*y2) in double-float with lo cross terms.
P3G_D df dot2(df x1, df y1, df x2, df y2, float sg) {
  const float p1 = fmul_rn(x1.hi, y1.hi);
  const float e1 = ffma(x1.hi, y1.hi, -p1);
  const float p2 = fmul_rn(x2.hi, y2.hi) * sg;
  const float e2 = ffma(x2.hi * sg, y2.hi, -p2);
  float s, t;
  two_sum(p1, p2, s, t);
  float lo = fadd_rn(fadd_rn(e1, e2), t);
  lo = ffma(x1.hi, y1.lo, lo);
  lo = ffma(x1.lo, y1.hi, lo);
  lo = ffma(x2.hi * sg, y2.lo, lo);
  lo = ffma(x2.lo * sg, y2.hi, lo);
  return df{s, lo};
}

// a * w (CONJ = false) or a * conj(w) (CONJ = true), w a double-float twiddle
template <bool CONJ>
P3G_D cdf cmul(cdf a, cdf w) {
  if (!CONJ) return cdf{dot2(a.re, w.re, a.im, w.im, -1.0f), dot2(a.re, w.im, a.im, w.re, 1.0f)};
  return cdf{dot2(a.re, w.re, a.im, w.im, 1.0f), dot2(a.im, w.re, a.re, w.im, -1.0f)};
}
// binary32 data times a compensated twiddle (w.hi + w.lo per component)
template <bool CONJ>
P3G_D cf cmul(cf a, cdf w) {
  const float wr = w.re.hi, wrl = w.re.lo;
  const float wi = CONJ ? -w.im.hi : w.im.hi, wil = CONJ ? -w.im.lo : w.im.lo;
  float re = a.re * wrl;
  re = ffma(-a.im, wil, re);
  re = ffma(a.re, wr, re);
  re = ffma(-a.im, wi, re);
  float im = a.re * wil;
  im = ffma(a.im, wrl, im);
  im = ffma(a.re, wi, im);
  im = ffma(a.im, wr, im);
  return cf{re, im};
}
// complex constant c = (cre, cim) (double-float parts)
P3G_D cdf mulcc(cdf a, float crh, float crl, float cih, float cil) {
  const df cr{crh, crl}, ci{cih, cil};
  return cdf{dot2(a.re, cr, a.im, ci, -1.0f), dot2(a.re, ci, a.im, cr, 1.0f)};
}
P3G_D cf mulcc(cf a, float crh, float /*crl*/, float cih, float /*cil*/) {
  return cf{ffma(a.re, crh, -a.im * cih), ffma(a.re, cih, a.im * crh)};
}

#if defined(__CUDACC__)
// ------------------------------------------------ memory formats per path
// F64 path: user data binary64 (double / double2); workspace and shared
// memory hold one complex as float4 (re.hi, im.hi, re.lo, im.lo).
// F32 path: user data and workspace binary32 (float / float2).
struct PathF64 {
  using C = cdf;
  using W = float4;   // workspace / shared-memory element
  using UR = double;  // user real
  using UC = double2; // user complex
  static constexpr bool kF64 = true;
  P3G_D static C from_w(float4 v) { return cdf{df{v.x, v.z}, df{v.y, v.w}}; }
  P3G_D static float4 to_w(C c) { return make_float4(c.re.hi, c.im.hi, c.re.lo, c.im.lo); }
  P3G_D static C from_uc(double2 v) { return cdf{d2df(v.x), d2df(v.y)}; }
  P3G_D static double2 to_uc(C c) { return make_double2(df2d(c.re.hi, c.re.lo), df2d(c.im.hi, c.im.lo)); }
  P3G_D static df from_ur(double v) { return d2df(v); }
  P3G_D static double to_ur(df v) { return df2d(v.hi, v.lo); }
  // with the exponent bias k: inputs times 2^-k, outputs times 2^k
  P3G_D static C from_uc(double2 v, int k) { return cdf{d2df_scaled(v.x, k), d2df_scaled(v.y, k)}; }
  P3G_D static double2 to_uc(C c, int k) {
    return make_double2(scale_pow2(df2d(c.re.hi, c.re.lo), k), scale_pow2(df2d(c.im.hi, c.im.lo), k));
  }
  P3G_D static df from_ur(double v, int k) { return d2df_scaled(v, k); }
  P3G_D static double to_ur(df v, int k) { return scale_pow2(df2d(v.hi, v.lo), k); }
  // largest |high word| seen (the binary64 exponent window's input)
  P3G_D static void track(uint32_t& amax, double v) {
    amax = max(amax, (uint32_t)__double2hiint(v) & 0x7FFFFFFFu);
  }
  P3G_D static void track(uint32_t& amax, double2 v) {
    track(amax, v.x);
    track(amax, v.y);
  }
  P3G_D static C make(df re, df im) { return cdf{re, im}; }
  P3G_D static C zero() { return cdf{df{0.f, 0.f}, df{0.f, 0.f}}; }
  P3G_D static df re(C c) { return c.re; }
  P3G_D static df im(C c) { return c.im; }
};
struct PathF32 {
  using C = cf;
  using W = float2;
  using UR = float;
  using UC = float2;
  static constexpr bool kF64 = false;
  P3G_D static C from_w(float2 v) { return cf{v.x, v.y}; }
  P3G_D static float2 to_w(C c) { return make_float2(c.re, c.im); }
  P3G_D static C from_uc(float2 v) { return cf{v.x, v.y}; }
  P3G_D static float2 to_uc(C c) { return make_float2(c.re, c.im); }
  P3G_D static float from_ur(float v) { return v; }
  P3G_D static float to_ur(float v) { return v; }
  // binary32 data has binary32's range, as the reference's single-precision
  // build: no exponent bias and nothing to track
  P3G_D static C from_uc(float2 v, int) { return cf{v.x, v.y}; }
  P3G_D static float2 to_uc(C c, int) { return make_float2(c.re, c.im); }
  P3G_D static float from_ur(float v, int) { return v; }
  P3G_D static float to_ur(float v, int) { return v; }
  P3G_D static void track(uint32_t&, float) {}
  P3G_D static void track(uint32_t&, float2) {}
  P3G_D static C make(float re, float im) { return cf{re, im}; }
  P3G_D static C zero() { return cf{0.f, 0.f}; }
  P3G_D static float re(C c) { return c.re; }
  P3G_D static float im(C c) { return c.im; }
};
#endif  // __CUDACC__

}  // namespace p3g
