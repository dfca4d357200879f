#ifndef MXS_GSL_INTERP_H
#define MXS_GSL_INTERP_H
#include <math.h> /* GSL headers pull in gsl_math.h / math.h */
#include <stddef.h>
typedef struct { int dummy; } gsl_interp_accel;
typedef struct { const char* name; } gsl_interp_type;
extern const gsl_interp_type* gsl_interp_cspline;
gsl_interp_accel* gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel* a);
#endif
