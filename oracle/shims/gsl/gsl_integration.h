/* GSL integration shim: QAG with the 61-point Gauss-Kronrod rule. */
#ifndef MXS_GSL_INTEGRATION_H
#define MXS_GSL_INTEGRATION_H
#include <math.h> /* GSL headers pull in gsl_math.h / math.h */
#include <stddef.h>
#include "gsl_errno.h"
typedef struct { double (*function)(double x, void* params); void* params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
enum { GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21 = 2, GSL_INTEG_GAUSS31 = 3, GSL_INTEG_GAUSS41 = 4,
       GSL_INTEG_GAUSS51 = 5, GSL_INTEG_GAUSS61 = 6 };
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace* w);
int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs, double epsrel, size_t limit,
                        int key, gsl_integration_workspace* w, double* result, double* abserr);
#endif
