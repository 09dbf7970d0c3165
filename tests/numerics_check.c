/* Device arithmetic restated for a check on the host CPU (test
 * infrastructure):
 *   cube_rn(h)      == h^3 correctly rounded (compared by the caller): the
 *                      FP64 identity the device relies on for h^3 outside
 *                      icube_rn's range, with the CPU's fused multiply-add
 *   slide_est(...)  slide_3's decision of a test on float estimates
 *                      (drop_above_est and approx_f in hc_slide.cu and
 *                      hc_internal.cuh): 0 surely not above, 1 surely
 *                      above, 2 undecided
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

double cube_rn(double h) {
  double p = h * h;
  double e = fma(h, h, -p);
  double q = p * h;
  double f = fma(p, h, -q);
  double c = fma(e, h, f);
  return q + c;
}


/* approx_abs_f: the high word's exponent and 20 mantissa bits as a float */
static float approx_f(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  const int hi = (int)(b >> 32);
  const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
  uint32_t u;
  if (e <= 0) u = 0;
  else if (e >= 255) u = 0x7f800000u;
  else u = ((uint32_t)e << 23) | ((uint32_t)(hi & 0xfffff) << 3);
  if ((int64_t)b < 0) u |= 0x80000000u;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

int slide_est(double e, double e2, double w, int diag) {
  const float fe = approx_f(e), fe2 = approx_f(e2), fw = approx_f(w);
  float est = fe - fe2;
  if (diag) est *= (1.0f / 1.41f);
  const float m = 0x1p-17f * (fabsf(fe) + fabsf(fe2) + fabsf(fw)) + 1e-30f;
  const float t = est - fw;
  if (t < -m) return 0;
  if (t > m) return 1;
  return 2;
}

/* n seeded cases, half of them within a relative 1e-5 (or an absolute
 * 1e-9 * scale) of the threshold; returns the number of decided cases whose
 * decision contradicts the FP64 test, and the decided count in *decided */
long slide_est_check(long n, unsigned seed, long* decided) {
  srand(seed);
  long bad = 0, dec = 0;
  for (long i = 0; i < n; i++) {
    const double r1 = (double)rand() / RAND_MAX, r2 = (double)rand() / RAND_MAX;
    const double r3 = (double)rand() / RAND_MAX, r4 = (double)rand() / RAND_MAX;
    const double scale = pow(10, (int)(r1 * 8) - 3);
    const double e = (r2 * 2 - 1) * scale * 1000;
    double w = (i % 97 == 0) ? 10000.0 : r3 * scale * 50;
    const int diag = (int)(i & 1);
    const double span = diag ? w * 1.41 : w;
    double e2;
    switch ((i >> 1) % 4) {
      case 0: e2 = e - span * (1 + (r4 - 0.5) * 1e-5); break;
      case 1: e2 = e - span + (r4 - 0.5) * 1e-9 * scale; break;
      case 2: e2 = (r4 * 2 - 1) * scale * 1000; break;
      default: e2 = e - (r4 * 2 - 1) * w * 3; break;
    }
    const double drop = diag ? ((e - e2) / 1.41) : (e - e2);
    const int want = drop > w;
    const int got = slide_est(e, e2, w, diag);
    if (got != 2) {
      dec++;
      if (got != want) bad++;
    }
  }
  *decided = dec;
  return bad;
}
