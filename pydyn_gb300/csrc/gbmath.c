/* The host build of gbmath.h with the C library's names, for callers that load a libm by path
 * (pydyn's ops.use_libm, the oracle) and for the package's host-side tables (cos of latitudes). */
#include "gbmath.h"

double exp(double x) { return gbm_exp(x); }
double log(double x) { return gbm_log(x); }
double pow(double x, double y) { return gbm_pow(x, y); }
double sin(double x) { return gbm_sin(x); }
double cos(double x) { return gbm_cos(x); }
