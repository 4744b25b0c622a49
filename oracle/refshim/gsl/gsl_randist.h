/* GSL random-distribution stand-in: the Weibull law by inversion of its CDF,
 * x = a * (-ln u)^(1/b) with u uniform on (0,1). */
#ifndef MTH_REFSHIM_GSL_RANDIST_H
#define MTH_REFSHIM_GSL_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_weibull(gsl_rng* r, double a, double b);
#ifdef __cplusplus
}
#endif
#endif
