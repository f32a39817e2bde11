/* Stand-in for the generated parameter header (test-only shim). */
#ifndef LGX_REF_SHIM_PARAMS_H
#define LGX_REF_SHIM_PARAMS_H
#define LIBINT2_MAX_VECLEN 1
#define LIBINT2_CARTGAUSS_MAX_AM 12
#define LIBINT2_CARTGAUSS_MAX_AM_eri 12
#endif
