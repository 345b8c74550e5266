// CPU check of the integer-only binary64 <-> double-float conversions used by
// the F64 path (p3g_arith.cuh).  Built and run by tests/test_conversions.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../p3dfft_gb300/csrc/p3g_arith.cuh"

using p3g::d2df;
using p3g::df2d;

static int failures = 0;
static void fail(const char* what, double x, double got, double ref) {
  if (failures < 20) std::printf("FAIL %s x=%a got=%a ref=%a\n", what, x, got, ref);
  ++failures;
}

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  long n = 0;
  // d2df: |hi + lo - x| <= 2^-48 |x| in [2^-74, 2^127]
  for (int i = 0; i < 2000000; ++i) {
    int ex = -74 + (int)(u01(rng) * 201.0);
    double x = std::ldexp(1.0 + u01(rng), ex);
    if (rng() & 1) x = -x;
    p3g::df r = d2df(x);
    long double s = (long double)r.hi + (long double)r.lo;
    long double err = fabsl(s - (long double)x);
    if (!(err <= ldexpl(fabsl((long double)x), -48))) fail("d2df bound", x, (double)s, x);
    if (std::signbit(r.hi) != std::signbit(x)) fail("d2df sign", x, r.hi, x);
    // round trip through df2d
    double back = df2d(r.hi, r.lo);
    if (!(std::fabs(back - x) <= std::ldexp(std::fabs(x), -47))) fail("roundtrip", x, back, x);
    ++n;
  }
  // exact for values with <= 24+24 significant bits
  for (int i = 0; i < 100000; ++i) {
    float a = (float)(u01(rng) * 2 - 1), b = std::ldexp((float)(u01(rng) * 2 - 1), -30);
    double x = (double)a + (double)b;
    double back = df2d(d2df(x).hi, d2df(x).lo);
    if (!(std::fabs(back - x) <= std::ldexp(std::fabs(x), -47))) fail("exact48", x, back, x);
  }
  // df2d on arbitrary pairs, including cancellation and |lo| > |hi|
  for (int i = 0; i < 2000000; ++i) {
    float hi = (float)std::ldexp(u01(rng) * 2 - 1, (int)(u01(rng) * 60) - 30);
    float lo;
    int mode = (int)(rng() % 4);
    if (mode == 0) lo = hi * (float)std::ldexp(u01(rng) * 2 - 1, -(int)(u01(rng) * 40));
    else if (mode == 1) lo = (float)std::ldexp(u01(rng) * 2 - 1, (int)(u01(rng) * 60) - 30);
    else if (mode == 2) lo = -hi + (float)std::ldexp(u01(rng) * 2 - 1, -40);
    else {  // hi a power of two, lo just below/above
      hi = (float)std::ldexp(1.0, (int)(u01(rng) * 40) - 20);
      if (rng() & 1) hi = -hi;
      lo = (float)std::ldexp(u01(rng) * 2 - 1, std::ilogb(hi) - 24 - (int)(u01(rng) * 4));
    }
    long double exact = (long double)hi + (long double)lo;  // exponents within 64 bits here
    double ref = (double)exact;
    double got = df2d(hi, lo);
    double ulp = ref == 0 ? 0 : std::ldexp(1.0, std::ilogb(ref) - 52);
    if (!(std::fabs(got - ref) <= ulp)) fail("df2d", (double)hi, got, ref);
  }
  // specials
  if (d2df(0.0).hi != 0.0f || !std::signbit(d2df(-0.0).hi)) fail("zero", 0, 0, 0);
  if (!std::isinf(d2df(1e300).hi)) fail("inf", 1e300, 0, 0);
  if (!std::isnan(d2df(std::nan("")).hi)) fail("nan", 0, 0, 0);
  if (d2df(1e-300).hi != 0.0f) fail("tiny", 1e-300, 0, 0);
  if (df2d(0.0f, 0.0f) != 0.0) fail("zero back", 0, 0, 0);
  if (!std::isinf(df2d(INFINITY, 0.0f))) fail("inf back", 0, 0, 0);
  std::printf("checked %ld values, %d failures\n", n, failures);
  return failures ? 1 : 0;
}
