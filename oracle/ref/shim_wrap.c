/* shim_wrap.c -- routes the reference's libm calls to the oracle's portable
 * functions (linked with -Wl,--wrap=log,--wrap=exp,--wrap=sin,--wrap=cos,
 * --wrap=sincos) so the compiled reference and the GPU replay agree bit for
 * bit.  Test infrastructure (reference build for the CPU oracle). */
#include "../orc_math.h"

double __wrap_log(double x) { return orc_log(x); }
double __wrap_exp(double x) { return orc_exp(x); }
double __wrap_sin(double x) { return orc_sin(x); }
double __wrap_cos(double x) { return orc_cos(x); }
void __wrap_sincos(double x, double *s, double *c) { *s = orc_sin(x); *c = orc_cos(x); }
