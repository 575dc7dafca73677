/* Oracle compat shim: genetIC includes this header but calls nothing from it. */
#ifndef COMPAT_GSL_ERRNO_H
#define COMPAT_GSL_ERRNO_H
#define GSL_SUCCESS 0
#endif
