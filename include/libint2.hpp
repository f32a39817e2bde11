// Umbrella header of the GB300 libint2 drop-in (the reference's
// include/libint2.hpp): Shell, ShellPair, BasisSet, Atom, Engine,
// initialize/finalize, the derivative-set iterators, plus the batched J/K
// builder of this library.
#ifndef LGX_LIBINT2_HPP
#define LGX_LIBINT2_HPP

#include "lgx.h"
#include "libint2/shell.h"
#include "libint2/basis.h"
#include "libint2/engine.h"
#include "libint2/deriv_iter.h"
#include "libint2/solidharmonics.h"
#include "libint2/jk.h"

#endif
