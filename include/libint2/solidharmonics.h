// libint2::solidharmonics::SolidHarmonicsCoefficients<Real>::coeff (the
// reference's include/libint2/solidharmonics.h:114-174): the coefficient of
// the Cartesian component x^lx y^ly z^lz in the real solid harmonic (l, m),
// m = -l..l, in libint's convention, from liblgx (lgx_solid_coeff) so that
// callers transforming Cartesian sets themselves (the generated-library C
// API returns Cartesian sets) use the coefficients the kernels use.
#ifndef LGX_LIBINT2_SOLIDHARMONICS_H
#define LGX_LIBINT2_SOLIDHARMONICS_H

#include "../lgx.h"

namespace libint2 {
namespace solidharmonics {

template <typename Real>
class SolidHarmonicsCoefficients {
 public:
  static Real coeff(int l, int m, int lx, int ly, int lz) {
    return Real(lgx_solid_coeff(l, m, lx, ly, lz));
  }
};

}  // namespace solidharmonics
}  // namespace libint2

#endif
