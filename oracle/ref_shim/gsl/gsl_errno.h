/* REFERENCE BUILD — test infrastructure only.  Stand-in for gsl_errno.h,
 * which the reference includes (include/exshalos/exshalos_h.h:12) without
 * calling anything from it. */
#ifndef EXH_REF_GSL_ERRNO_H
#define EXH_REF_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_EDOM 1
#endif
