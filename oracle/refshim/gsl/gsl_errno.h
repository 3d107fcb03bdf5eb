/* GSL status codes used by the reference (documented values), for
 * oracle/ref.mk (TEST INFRASTRUCTURE). */
#ifndef CMCREF_SHIM_GSL_ERRNO_H
#define CMCREF_SHIM_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_FAILURE (-1)
#define GSL_CONTINUE (-2)
#define GSL_EDOM 1
#define GSL_EINVAL 4
#define GSL_EBADFUNC 9
typedef void gsl_error_handler_t(const char *reason, const char *file, int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler_off(void);
const char *gsl_strerror(int gsl_errno);
#endif
