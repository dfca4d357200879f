#ifndef MXS_GSL_RANDIST_H
#define MXS_GSL_RANDIST_H
#include "gsl_rng.h"
#endif
