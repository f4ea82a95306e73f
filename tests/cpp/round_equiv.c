/* round_equiv.c -- the FP64-free forms the CUDA kernels use for eflib's
 * fast_roundi / fast_floori / fast_ceili of a float argument and for
 * vector_::length's double square root (eflib/include/eflib/math/math.h:
 * 139-164, vector_generic.h:118-126), checked against the reference's
 * double forms.
 *
 *   round_equiv            every float within 2^20 ulps of each boundary,
 *                          every float with |f| < 2^-20 ... 2^-24 region
 *                          sampled densely, and every 61st float of all 2^32
 *   round_equiv --all      every one of the 2^32 floats (about two minutes)
 *
 * The device forms, restated here with the same IEEE operations:
 *   roundi(f) = floor(f + 0.5 rounded down)
 *   floori(f) = f in [-0x1.01b2b2p-26, 0) ? 0 : floor(f)
 *   ceili(f)  = |f| >= 2^26 ? the double form : f in (0, 0x1.01b2b2p-26] ? 0 : ceil(f)
 *   length    = the float square root
 * Exit status 0 when every checked float agrees. */
#include <fenv.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#pragma STDC FENV_ACCESS ON

static const double EPS = (double)0.5f - 1.5e-8;
static double ref_roundi(double d) { return floor(d + 0.5); }
static double ref_floori(double d) { return ref_roundi(d - EPS); }
static double ref_ceili(double d) { return ref_roundi(d + EPS); }

static float add_rd(float a, float b) {
  fesetround(FE_DOWNWARD);
  volatile float r = a + b;
  fesetround(FE_TONEAREST);
  return r;
}
static double dev_roundi(float f) { return floorf(add_rd(f, 0.5f)); }
static double dev_floori(float f) { return (f < 0.0f && f >= -0x1.01b2b2p-26f) ? 0.0 : floorf(f); }
static double dev_ceili(float f) {
  if (!(fabsf(f) < 0x1p26f)) return ref_ceili((double)f);
  return (f > 0.0f && f <= 0x1.01b2b2p-26f) ? 0.0 : ceilf(f);
}

static long bad = 0, checked = 0;
static int same(double a, double b) { return a == b || (isnan(a) && isnan(b)); }
static void check(uint32_t bits) {
  float f;
  memcpy(&f, &bits, 4);
  double d = f;
  ++checked;
  int ok = same(dev_roundi(f), ref_roundi(d)) && same(dev_floori(f), ref_floori(d)) &&
           same(dev_ceili(f), ref_ceili(d)) && same(dev_roundi(f), ref_floori(0.5 + d));
  if (f >= 0.0f || isnan(f)) {
    float a = (float)sqrt(d), b = sqrtf(f);
    uint32_t ua, ub;
    memcpy(&ua, &a, 4);
    memcpy(&ub, &b, 4);
    ok = ok && (ua == ub || (isnan(a) && isnan(b)));
  }
  if (!ok && bad++ < 10) printf("differs at %08x (%.9g)\n", bits, f);
}

int main(int argc, char** argv) {
  if (argc > 1 && strcmp(argv[1], "--all") == 0) {
    for (uint64_t u = 0; u < (1ull << 32); ++u) check((uint32_t)u);
  } else {
    const float edges[] = {-0x1.01b2b2p-26f, 0x1.01b2b2p-26f, 0.0f, 0.5f, -0.5f, 1.0f, -1.0f, 0x1p23f, 0x1p24f, 0x1p26f, -0x1p26f};
    for (size_t i = 0; i < sizeof(edges) / sizeof(edges[0]); ++i) {
      uint32_t b;
      memcpy(&b, &edges[i], 4);
      for (int64_t k = -(1 << 20); k <= (1 << 20); ++k) check((uint32_t)((int64_t)b + k));
    }
    for (uint32_t b = 0; b < 0x33000000u; b += 7) check(b);              /* 0 .. 2^-25, both signs */
    for (uint32_t b = 0x80000000u; b < 0xB3000000u; b += 7) check(b);
    for (uint64_t u = 0; u < (1ull << 32); u += 61) check((uint32_t)u);
  }
  printf("%ld floats checked, %ld differ\n", checked, bad);
  return bad != 0;
}
