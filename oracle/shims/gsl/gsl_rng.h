#ifndef MXS_GSL_RNG_H
#define MXS_GSL_RNG_H
typedef struct { unsigned long seed; } gsl_rng;
#endif
