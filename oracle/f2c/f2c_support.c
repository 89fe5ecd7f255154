/* The two libf2c helpers the AMOS translation calls, written from their
 * Fortran definitions: SIGN(a, b) = |a| with the sign of b, and a**b. */
#include "f2c.h"
double d_sign(doublereal *a, doublereal *b) {
  double x = (*a >= 0 ? *a : -*a);
  return (*b >= 0 ? x : -x);
}
double pow_dd(doublereal *a, doublereal *b) { return pow(*a, *b); }
