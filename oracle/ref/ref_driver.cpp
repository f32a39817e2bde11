// Test-infrastructure only: a thin C driver over the REFERENCE's own
// header-only code (libint2::Shell, ShellPair, SolidHarmonicsCoefficients,
// FmEval_Reference2 / FmEval_Taylor, BasisSet, DerivMapGenerator and the
// brute-force ERI of src/bin/test_eri/eri.h), compiled in place from the
// reference tree by oracle/ref/build_ref.sh into oracle/_ref/libref.so.
//
// It exists to pin the CPU restatement in oracle/oracle.cpp (and, through
// committed golden fixtures, the CUDA path) against the reference's own
// arithmetic.  Nothing in the product links it.
#include <libint2/util/cxxstd.h>
#include <libint2/shell.h>
#include <libint2/solidharmonics.h>
#include <libint2/boys.h>
#include <libint2/deriv_map.h>
#include <libint2/deriv_iter.h>
#include <libint2/atom.h>
#include <libint2/basis.h.in>

#include <eri.h>

#include <cstring>
#include <vector>

using libint2::Shell;
using libint2::ShellPair;
using libint2::ScreeningMethod;

namespace {
Shell make_shell(int l, int pure, int nprim, const double* alpha,
                 const double* coeff, const double* O, bool renorm) {
  libint2::svector<double> a(alpha, alpha + nprim);
  libint2::svector<double> c(coeff, coeff + nprim);
  return Shell(a, {{l, pure != 0, c}}, {{O[0], O[1], O[2]}}, renorm);
}
}  // namespace

extern "C" {

// libint2::Shell::Shell(...) + renorm() (shell.h:767-777, 958-999).
int ref_shell_normalize(int l, int pure, int nprim, const double* alpha,
                        const double* coeff_in, double* coeff_out,
                        double* max_ln_coeff_out) {
  const double O[3] = {0, 0, 0};
  Shell s = make_shell(l, pure, nprim, alpha, coeff_in, O, true);
  for (int p = 0; p < nprim; ++p) {
    coeff_out[p] = s.contr[0].coeff[p];
    max_ln_coeff_out[p] = s.max_ln_coeff[p];
  }
  return 0;
}

// SolidHarmonicsCoefficients<double>::coeff (solidharmonics.h:114-174).
double ref_solid_coeff(int l, int m, int lx, int ly, int lz) {
  return libint2::solidharmonics::SolidHarmonicsCoefficients<double>::coeff(
      l, m, lx, ly, lz);
}

// FmEval_Reference2<double>::eval (boys.h:229-246).
void ref_boys_reference2(double T, int mmax, double* F) {
  libint2::FmEval_Reference2<double>::eval(F, T, mmax);
}

// FmEval_Reference<long double>::eval (boys.h:180-188): MacLaurin series in
// extended precision, used to judge both double-precision evaluators.
void ref_boys_reference_ld(double T, int mmax, double* F) {
  std::vector<long double> f(mmax + 1);
  libint2::FmEval_Reference<long double>::eval(f.data(), (long double)T, mmax);
  for (int m = 0; m <= mmax; ++m) F[m] = (double)f[m];
}

// FmEval_Taylor<double,7>::eval (boys.h:679-821).
void ref_boys_taylor(double T, int mmax, double* F) {
  static auto inst = libint2::FmEval_Taylor<double, 7>::instance(20, 1e-15);
  inst->eval(F, T, mmax);
}

// ShellPair::init (shell.h:1138-1256); method 0 = Original, 1 = Conservative.
// Returns the number of surviving primitive pairs; per pair writes
// P[3], K, one_over_gamma, nonsph_screen_fac, ln_scr, p1, p2.
int ref_shellpair_init(const int* l, const int* nprim, const double* alpha1,
                       const double* coeff1, const double* O1,
                       const double* alpha2, const double* coeff2,
                       const double* O2, double ln_prec, int method,
                       double* P, double* K, double* oogamma, double* nonsph,
                       double* ln_scr, int* p1, int* p2, double* AB) {
  Shell s1 = make_shell(l[0], 0, nprim[0], alpha1, coeff1, O1, false);
  Shell s2 = make_shell(l[1], 0, nprim[1], alpha2, coeff2, O2, false);
  ShellPair sp;
  sp.init(s1, s2, ln_prec,
          method == 0 ? ScreeningMethod::Original
                      : ScreeningMethod::Conservative);
  const int n = (int)sp.primpairs.size();
  for (int i = 0; i < n; ++i) {
    const auto& pp = sp.primpairs[i];
    for (int x = 0; x < 3; ++x) P[3 * i + x] = pp.P[x];
    K[i] = pp.K;
    oogamma[i] = pp.one_over_gamma;
    nonsph[i] = pp.nonsph_screen_fac;
    ln_scr[i] = pp.ln_scr;
    p1[i] = pp.p1;
    p2[i] = pp.p2;
  }
  for (int x = 0; x < 3; ++x) AB[x] = sp.AB[x];
  return n;
}

// DerivMapGenerator's xx_xx map for deriv order 1 (deriv_map.h:170-262).
int ref_deriv_map1(int swap_braket, int swap_bra, int swap_ket, int s) {
  static bool init = false;
  if (!init) {
    libint2::DerivMapGenerator::initialize();
    init = true;
  }
  auto& t = libint2::DerivMapGenerator::instance(1, libint2::BraKet::xx_xx);
  return (int)t(swap_braket, swap_bra, swap_ket, s);
}

// Order of the 12 first-derivative shell sets (CartesianDerivIterator<4>(1)).
// Writes, for each set, the index (0..11) of the differentiated coordinate.
int ref_deriv_order1(int* coord_of_set) {
  libint2::CartesianDerivIterator<4> diter(1);
  int di = 0;
  bool last = false;
  do {
    const auto& v = *diter;
    for (int c = 0; c < 12; ++c)
      if (v[c] == 1) coord_of_set[di] = c;
    ++di;
    last = diter.last();
    if (!last) diter.next();
  } while (!last);
  return di;
}

// Order of the 78 second-derivative shell sets (CartesianDerivIterator<4>(2)):
// for each set, the two differentiated coordinates c1 <= c2 (0..11).
int ref_deriv_order2(int* c1, int* c2) {
  libint2::CartesianDerivIterator<4> diter(2);
  int di = 0;
  bool last = false;
  do {
    const auto& v = *diter;
    int a = -1, b = -1;
    for (int c = 0; c < 12; ++c) {
      if (v[c] == 2) a = b = c;
      if (v[c] == 1) (a < 0 ? a : b) = c;
    }
    c1[di] = a;
    c2[di] = b;
    ++di;
    last = diter.last();
    if (!last) diter.next();
  } while (!last);
  return di;
}

// Brute-force contracted shell set from src/bin/test_eri/eri.h:121-468, with
// the contraction loop of tests/unit/test-2body.cc:246-289 and the
// Cartesian->solid-harmonic steps of engine.impl.h:1965-1985 (reference
// solidharmonics transforms).  Shells carry already-normalized coefficients.
// out holds nderiv sets of n1*n2*n3*n4 values in libint's buffer order.
int ref_eri_shellset(const int* l, const int* pure, const int* nprim,
                     const double* alpha_flat, const double* coeff_flat,
                     const double* O, int deriv, double* out) {
  std::vector<Shell> sh;
  int off = 0;
  for (int i = 0; i < 4; ++i) {
    sh.push_back(make_shell(l[i], pure[i], nprim[i], alpha_flat + off,
                            coeff_flat + off, O + 3 * i, false));
    off += nprim[i];
  }
  const int nderiv = deriv == 0 ? 1 : (deriv == 1 ? 12 : 78);
  size_t ncart = 1, npure = 1;
  for (int i = 0; i < 4; ++i) {
    ncart *= sh[i].cartesian_size();
    npure *= sh[i].size();
  }
  std::vector<double> cart(nderiv * ncart, 0.0);

  int ijkl = 0;
  int l0, m0, n0, l1, m1, n1, l2, m2, n2, l3, m3, n3;
  FOR_CART(l0, m0, n0, sh[0].contr[0].l)
  FOR_CART(l1, m1, n1, sh[1].contr[0].l)
  FOR_CART(l2, m2, n2, sh[2].contr[0].l)
  FOR_CART(l3, m3, n3, sh[3].contr[0].l)
  for (size_t p0 = 0; p0 < sh[0].nprim(); ++p0)
    for (size_t p1 = 0; p1 < sh[1].nprim(); ++p1)
      for (size_t p2 = 0; p2 < sh[2].nprim(); ++p2)
        for (size_t p3 = 0; p3 < sh[3].nprim(); ++p3) {
          const double c0123 =
              sh[0].contr[0].coeff[p0] * sh[1].contr[0].coeff[p1] *
              sh[2].contr[0].coeff[p2] * sh[3].contr[0].coeff[p3];
          libint2::CartesianDerivIterator<4> diter(deriv);
          bool last = false;
          int di = 0;
          do {
            cart[di * ncart + ijkl] +=
                c0123 * eri(&(*diter)[0], l0, m0, n0, sh[0].alpha[p0],
                            sh[0].O.data(), l1, m1, n1, sh[1].alpha[p1],
                            sh[1].O.data(), l2, m2, n2, sh[2].alpha[p2],
                            sh[2].O.data(), l3, m3, n3, sh[3].alpha[p3],
                            sh[3].O.data(), 0);
            ++di;
            last = diter.last();
            if (!last) diter.next();
          } while (!last);
        }
  ++ijkl;
  END_FOR_CART
  END_FOR_CART
  END_FOR_CART
  END_FOR_CART

  // Cartesian -> solid harmonics, index by index, as Engine does.
  std::vector<double> a(ncart), b(ncart);
  for (int d = 0; d < nderiv; ++d) {
    std::memcpy(a.data(), cart.data() + d * ncart, ncart * sizeof(double));
    double* src = a.data();
    double* tgt = b.data();
    const size_t nc[4] = {sh[0].cartesian_size(), sh[1].cartesian_size(),
                          sh[2].cartesian_size(), sh[3].cartesian_size()};
    if (sh[0].contr[0].pure) {
      libint2::solidharmonics::transform_first(sh[0].contr[0].l,
                                               nc[1] * nc[2] * nc[3], src, tgt);
      std::swap(src, tgt);
    }
    if (sh[1].contr[0].pure) {
      libint2::solidharmonics::transform_inner(sh[0].size(), sh[1].contr[0].l,
                                               nc[2] * nc[3], src, tgt);
      std::swap(src, tgt);
    }
    if (sh[2].contr[0].pure) {
      libint2::solidharmonics::transform_inner(
          sh[0].size() * sh[1].size(), sh[2].contr[0].l, nc[3], src, tgt);
      std::swap(src, tgt);
    }
    if (sh[3].contr[0].pure) {
      libint2::solidharmonics::transform_last(
          sh[0].size() * sh[1].size() * sh[2].size(), sh[3].contr[0].l, src,
          tgt);
      std::swap(src, tgt);
    }
    std::memcpy(out + d * npure, src, npure * sizeof(double));
  }
  return (int)npure;
}

// BasisSet(name, atoms) (basis.h.in:134-182) for the given atoms (bohr).
// Returns the number of shells; fills per-shell l, pure, nprim, origin and
// the flattened (normalized) exponents/coefficients when buffers are given.
int ref_basis(const char* name, int natoms, const int* Z, const double* xyz,
              int* l, int* pure, int* nprim, double* O, double* alpha,
              double* coeff, int max_flat) {
  std::vector<libint2::Atom> atoms(natoms);
  for (int i = 0; i < natoms; ++i) {
    atoms[i].atomic_number = Z[i];
    atoms[i].x = xyz[3 * i];
    atoms[i].y = xyz[3 * i + 1];
    atoms[i].z = xyz[3 * i + 2];
  }
  libint2::BasisSet bs(name, atoms);
  if (!l) return (int)bs.size();
  int off = 0;
  for (size_t s = 0; s < bs.size(); ++s) {
    l[s] = bs[s].contr[0].l;
    pure[s] = bs[s].contr[0].pure;
    nprim[s] = (int)bs[s].nprim();
    for (int x = 0; x < 3; ++x) O[3 * s + x] = bs[s].O[x];
    for (size_t p = 0; p < bs[s].nprim(); ++p) {
      if (off >= max_flat) return -1;
      alpha[off] = bs[s].alpha[p];
      coeff[off] = bs[s].contr[0].coeff[p];
      ++off;
    }
  }
  return (int)bs.size();
}

}  // extern "C"
