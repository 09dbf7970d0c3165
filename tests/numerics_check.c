/* The FP64 identity the device relies on for h^3 outside icube_rn's
 * range, checked on the host CPU with its fused multiply-add (test
 * infrastructure):
 *   cube_rn(h)      == h^3 correctly rounded (compared by the caller)
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

