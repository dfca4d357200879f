#ifndef MXS_GSL_ERRNO_H
#define MXS_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_CONTINUE (-2)
#define GSL_EDOM 1
#define GSL_EMAXITER 11
#define GSL_EROUND 18
typedef void gsl_error_handler_t(const char*, const char*, int, int);
gsl_error_handler_t* gsl_set_error_handler_off(void);
#endif
