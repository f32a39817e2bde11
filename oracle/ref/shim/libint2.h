/* Minimal stand-in for the generated <libint2.h> so that the reference's
 * header-only Shell / solid-harmonics / Boys / brute-force ERI code compiles
 * without the generated integral library.  Test-infrastructure only. */
#ifndef LGX_REF_SHIM_LIBINT2_H
#define LGX_REF_SHIM_LIBINT2_H
#include <algorithm>
#include <libint2/config.h>
#include <libint2/util/deprecated.h>
#include <libint2/numeric.h>
#endif
