/* The two FP64 identities the device relies on, checked on the host CPU
 * with its fused multiply-add (test infrastructure):
 *   cube_rn(h)      == h^3 correctly rounded (compared by the caller)
 *   div_const(x,y)  == x / y for a fixed divisor y (Markstein)
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

double cube_rn(double h) {
  double p = h * h;
  double e = fma(h, h, -p);
  double q = p * h;
  double f = fma(p, h, -q);
  double c = fma(e, h, f);
  return q + c;
}

double div_const(double x, double y, double r) {
  double q = x * r;
  double e = fma(-q, y, x);
  return fma(e, r, q);
}

/* mismatches of div_const against x / y over n seeded random x */
long div_mismatches(double y, long n, uint64_t seed) {
  double r = 1.0 / y;
  long bad = 0;
  for (long i = 0; i < n; i++) {
    seed = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    uint64_t m = seed >> 12;
    int ex = (int)((seed >> 2) % 1600) - 800;
    double x = ldexp(1.0 + (double)m / 4503599627370496.0, ex);
    if (seed & 1) x = -x;
    if (x / y != div_const(x, y, r)) bad++;
  }
  return bad;
}
