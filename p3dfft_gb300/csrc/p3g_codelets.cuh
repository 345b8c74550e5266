// Register-resident DFT codelets of radix 2, 3, 4, 5, 8, 16 and 32.
//
// DIR = -1 computes X_k = sum_n a_n exp(-2 pi i n k / R) (FFTW_FORWARD),
// DIR = +1 the exp(+...) transform (FFTW_BACKWARD).  Inputs and outputs are in
// natural order in the same array.  Every codelet is written once over the
// complex type C (cdf for the F64 path, cf for the F32 path); constants are
// double-float (hi, lo) pairs of binary32 literals (exact splits of the
// binary64 values, written as hex floats so that no FP64 arithmetic appears
// in device code).
#pragma once

#include "p3g_arith.cuh"

namespace p3g {

// cos/sin constants as (hi, lo) binary32 pairs
#define P3G_SQRT3_2 0x1.bb67aep-1f, 0x1.0b0996p-26f
#define P3G_C5_1 0x1.3c6ef4p-2f, -0x1.1a02d6p-27f
#define P3G_C5_2 -0x1.9e377ap-1f, 0x1.1a02d6p-27f
#define P3G_S5_1 0x1.e6f0e2p-1f, -0x1.97756p-26f
#define P3G_S5_2 0x1.2cf23p-1f, 0x1.1d5698p-27f
#define P3G_SQRT1_2 0x1.6a09e6p-1f, 0x1.9fcef4p-27f
#define P3G_C16_1 0x1.d906bcp-1f, 0x1.e651a8p-26f
#define P3G_S16_1 0x1.87de2ap-2f, 0x1.abaa58p-28f

template <int DIR, class C>
P3G_D void dft2(C* a) {
  const C t = a[0] - a[1];
  a[0] = a[0] + a[1];
  a[1] = t;
}

template <int DIR, class C>
P3G_D void dft3(C* a) {
  const C t1 = a[1] + a[2];
  const C t2 = a[0] + cscale2(t1, -0.5f);
  const C t3 = rot<DIR>(mulr(a[1] - a[2], P3G_SQRT3_2));
  a[0] = a[0] + t1;
  a[1] = t2 + t3;
  a[2] = t2 - t3;
}

template <int DIR, class C>
P3G_D void dft4(C& a0, C& a1, C& a2, C& a3) {
  const C t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = rot<DIR>(a1 - a3);
  a0 = t0 + t2;
  a2 = t0 - t2;
  a1 = t1 + t3;
  a3 = t1 - t3;
}
template <int DIR, class C>
P3G_D void dft4(C* a) {
  dft4<DIR>(a[0], a[1], a[2], a[3]);
}

template <int DIR, class C>
P3G_D void dft5(C* a) {
  const C t1 = a[1] + a[4], t2 = a[2] + a[3], t3 = a[1] - a[4], t4 = a[2] - a[3];
  const C b1 = a[0] + (mulr(t1, P3G_C5_1) + mulr(t2, P3G_C5_2));
  const C b2 = a[0] + (mulr(t1, P3G_C5_2) + mulr(t2, P3G_C5_1));
  const C d1 = rot<DIR>(mulr(t3, P3G_S5_1) + mulr(t4, P3G_S5_2));
  const C d2 = rot<DIR>(mulr(t3, P3G_S5_2) - mulr(t4, P3G_S5_1));
  a[0] = a[0] + (t1 + t2);
  a[1] = b1 + d1;
  a[4] = b1 - d1;
  a[2] = b2 + d2;
  a[3] = b2 - d2;
}

// multiply by w8^1 = (1 + DIR i)/sqrt2 and w8^3 = (-1 + DIR i)/sqrt2
template <int DIR, class C>
P3G_D C mul_w8_1(C a) {
  return mulr(a + rot<DIR>(a), P3G_SQRT1_2);
}
template <int DIR, class C>
P3G_D C mul_w8_3(C a) {
  return mulr(rot<DIR>(a) - a, P3G_SQRT1_2);
}

template <int DIR, class C>
P3G_D void dft8(C* a) {
  dft4<DIR>(a[0], a[2], a[4], a[6]);
  dft4<DIR>(a[1], a[3], a[5], a[7]);
  const C o1 = mul_w8_1<DIR>(a[3]);
  const C o2 = rot<DIR>(a[5]);
  const C o3 = mul_w8_3<DIR>(a[7]);
  const C e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6], o0 = a[1];
  a[0] = e0 + o0;
  a[4] = e0 - o0;
  a[1] = e1 + o1;
  a[5] = e1 - o1;
  a[2] = e2 + o2;
  a[6] = e2 - o2;
  a[3] = e3 + o3;
  a[7] = e3 - o3;
}

// 16 = 4 x 4: inner DFT4 over n2 (stride-4 inputs), twiddle w16^(n1 k2),
// outer DFT4 over n1; output X[k2 + 4 k1].
template <int DIR, class C>
P3G_D void dft16(C* a) {
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) dft4<DIR>(a[n1], a[n1 + 4], a[n1 + 8], a[n1 + 12]);
  // b[n1][k2] lives in a[n1 + 4 k2]
  constexpr float S = DIR > 0 ? 1.0f : -1.0f;
  a[1 + 4] = mulcc(a[1 + 4], P3G_C16_1, S * 0x1.87de2ap-2f, S * 0x1.abaa58p-28f);  // w^1
  a[1 + 8] = mul_w8_1<DIR>(a[1 + 8]);                                                 // w^2
  a[1 + 12] = mulcc(a[1 + 12], P3G_S16_1, S * 0x1.d906bcp-1f, S * 0x1.e651a8p-26f);  // w^3
  a[2 + 4] = mul_w8_1<DIR>(a[2 + 4]);                                                 // w^2
  a[2 + 8] = rot<DIR>(a[2 + 8]);                                                      // w^4
  a[2 + 12] = mul_w8_3<DIR>(a[2 + 12]);                                               // w^6
  a[3 + 4] = mulcc(a[3 + 4], P3G_S16_1, S * 0x1.d906bcp-1f, S * 0x1.e651a8p-26f);    // w^3
  a[3 + 8] = mul_w8_3<DIR>(a[3 + 8]);                                                 // w^6
  a[3 + 12] = cneg(mulcc(a[3 + 12], P3G_C16_1, S * 0x1.87de2ap-2f, S * 0x1.abaa58p-28f));  // w^9 = -w^1
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) dft4<DIR>(a[4 * k2], a[4 * k2 + 1], a[4 * k2 + 2], a[4 * k2 + 3]);
  // now X[k2 + 4 k1] sits in a[4 k2 + k1]: transpose the 4x4 index
  C t[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) t[i] = a[i];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2)
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[k2 + 4 * k1] = t[4 * k2 + k1];
}

// a * w32^E with w32 = exp(DIR 2 pi i / 32): w32^E = w32^(E mod 8) (DIR i)^(E / 8)
// (cos/sin of 2 pi e / 32 for e = 1, 2, 3 as (hi, lo) binary32 pairs; the
// sines are the cosines of 8 - e).
#define P3G_C32_1 0x1.f6297cp-1f, 0x1.feeb96p-26f
#define P3G_C32_2 0x1.d906bcp-1f, 0x1.e651a8p-26f
#define P3G_C32_3 0x1.a9b662p-1f, 0x1.21d434p-26f
#define P3G_C32_5 0x1.1c73b4p-1f, -0x1.9465cep-27f
#define P3G_C32_6 0x1.87de2ap-2f, 0x1.abaa58p-28f
#define P3G_C32_7 0x1.8f8b84p-3f, -0x1.cb2cfcp-30f
template <int DIR, int E, class C>
P3G_D C mul_w32(C a) {
  constexpr int e8 = E % 8, q = (E / 8) % 4;
  constexpr float S = DIR > 0 ? 1.0f : -1.0f;
  C r;
  if constexpr (e8 == 0) r = a;
  else if constexpr (e8 == 4) r = mul_w8_1<DIR>(a);
  else if constexpr (e8 == 1) r = mulcc(a, P3G_C32_1, S * 0x1.8f8b84p-3f, S * -0x1.cb2cfcp-30f);
  else if constexpr (e8 == 2) r = mulcc(a, P3G_C32_2, S * 0x1.87de2ap-2f, S * 0x1.abaa58p-28f);
  else if constexpr (e8 == 3) r = mulcc(a, P3G_C32_3, S * 0x1.1c73b4p-1f, S * -0x1.9465cep-27f);
  else if constexpr (e8 == 5) r = mulcc(a, P3G_C32_5, S * 0x1.a9b662p-1f, S * 0x1.21d434p-26f);
  else if constexpr (e8 == 6) r = mulcc(a, P3G_C32_6, S * 0x1.d906bcp-1f, S * 0x1.e651a8p-26f);
  else r = mulcc(a, P3G_C32_7, S * 0x1.f6297cp-1f, S * 0x1.feeb96p-26f);
  if constexpr (q >= 1) r = rot<DIR>(r);
  if constexpr (q >= 2) r = rot<DIR>(r);
  if constexpr (q >= 3) r = rot<DIR>(r);
  return r;
}

// 32 = 8 x 4: inner DFT4 over n2 (inputs n1 + 8 n2), twiddle w32^(n1 k2),
// outer DFT8 over n1 (contiguous after the inner step); output X[k2 + 4 k1].
template <int DIR, class C>
P3G_D void dft32(C* a) {
#pragma unroll
  for (int n1 = 0; n1 < 8; ++n1) dft4<DIR>(a[n1], a[n1 + 8], a[n1 + 16], a[n1 + 24]);
  // b[n1][k2] lives in a[n1 + 8 k2]
  a[1 + 8] = mul_w32<DIR, 1>(a[1 + 8]);
  a[2 + 8] = mul_w32<DIR, 2>(a[2 + 8]);
  a[3 + 8] = mul_w32<DIR, 3>(a[3 + 8]);
  a[4 + 8] = mul_w32<DIR, 4>(a[4 + 8]);
  a[5 + 8] = mul_w32<DIR, 5>(a[5 + 8]);
  a[6 + 8] = mul_w32<DIR, 6>(a[6 + 8]);
  a[7 + 8] = mul_w32<DIR, 7>(a[7 + 8]);
  a[1 + 16] = mul_w32<DIR, 2>(a[1 + 16]);
  a[2 + 16] = mul_w32<DIR, 4>(a[2 + 16]);
  a[3 + 16] = mul_w32<DIR, 6>(a[3 + 16]);
  a[4 + 16] = mul_w32<DIR, 8>(a[4 + 16]);
  a[5 + 16] = mul_w32<DIR, 10>(a[5 + 16]);
  a[6 + 16] = mul_w32<DIR, 12>(a[6 + 16]);
  a[7 + 16] = mul_w32<DIR, 14>(a[7 + 16]);
  a[1 + 24] = mul_w32<DIR, 3>(a[1 + 24]);
  a[2 + 24] = mul_w32<DIR, 6>(a[2 + 24]);
  a[3 + 24] = mul_w32<DIR, 9>(a[3 + 24]);
  a[4 + 24] = mul_w32<DIR, 12>(a[4 + 24]);
  a[5 + 24] = mul_w32<DIR, 15>(a[5 + 24]);
  a[6 + 24] = mul_w32<DIR, 18>(a[6 + 24]);
  a[7 + 24] = mul_w32<DIR, 21>(a[7 + 24]);
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) dft8<DIR>(a + 8 * k2);
  // now X[k2 + 4 k1] sits in a[8 k2 + k1]: transpose the 4x8 index
  C t[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) t[i] = a[i];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2)
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) a[k2 + 4 * k1] = t[8 * k2 + k1];
}

template <int R, int DIR, class C>
P3G_D void dft(C* a) {
  if constexpr (R == 2) dft2<DIR>(a);
  else if constexpr (R == 3) dft3<DIR>(a);
  else if constexpr (R == 4) dft4<DIR>(a);
  else if constexpr (R == 5) dft5<DIR>(a);
  else if constexpr (R == 8) dft8<DIR>(a);
  else if constexpr (R == 16) dft16<DIR>(a);
  else if constexpr (R == 32) dft32<DIR>(a);
}

}  // namespace p3g
