/* Minimal f2c support header, written for this project, sufficient to compile
 * the f2c-translated AMOS Bessel routines that OPTIMET-3D vendors
 * (srcAna/amos.c, srcAna/fortran.c). Used only to build the reference's own
 * Bessel code into oracle/_ref/ for pinning the oracle. */
#ifndef OM_F2C_SHIM_H
#define OM_F2C_SHIM_H
#include <math.h>
typedef long integer;
typedef double doublereal;
typedef float real;
#ifndef abs
#define abs(x) ((x) >= 0 ? (x) : -(x))
#endif
#ifndef min
#define min(a, b) ((a) <= (b) ? (a) : (b))
#endif
#ifndef max
#define max(a, b) ((a) >= (b) ? (a) : (b))
#endif
double d_sign(doublereal *a, doublereal *b);
double pow_dd(doublereal *a, doublereal *b);
#endif
