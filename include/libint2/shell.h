// libint2::Shell / ShellPair / ScreeningMethod for the GB300 drop-in.
//
// Same names, members and constructor semantics as the reference
// (include/libint2/shell.h:720-1329 of libint): a Shell holds exponents,
// one contraction {l, pure, coeff} and its origin; construction embeds the
// primitive normalization into the coefficients and renormalizes the
// contraction to unit self-overlap (Shell::renorm, shell.h:958-999), here
// through lgx_shell_normalize.  Generally contracted shells (more than one
// contraction) are not supported, as in Engine::compute2 of the reference
// (engine.impl.h:1168-1171).
#ifndef LGX_LIBINT2_SHELL_H
#define LGX_LIBINT2_SHELL_H

#include <array>
#include <cassert>
#include <cmath>
#include <cstdlib>
#include <limits>
#include <ostream>
#include <stdexcept>
#include <utility>
#include <vector>

#include "../lgx.h"

namespace libint2 {

template <typename T>
using svector = std::vector<T>;

struct Shell {
  typedef double real_t;

  struct Contraction {
    int l;
    bool pure;
    svector<real_t> coeff;
    bool operator==(const Contraction& o) const {
      return l == o.l && pure == o.pure && coeff == o.coeff;
    }
    bool operator!=(const Contraction& o) const { return !(*this == o); }
    size_t cartesian_size() const { return (l + 1) * (l + 2) / 2; }
    size_t size() const { return pure ? (2 * l + 1) : cartesian_size(); }
  };

  svector<real_t> alpha;
  svector<Contraction> contr;
  std::array<real_t, 3> O;
  svector<real_t> max_ln_coeff;

  Shell() = default;
  Shell(svector<real_t> _alpha, svector<Contraction> _contr, std::array<real_t, 3> _O,
        bool embed_normalization_into_coefficients = true)
      : alpha(std::move(_alpha)), contr(std::move(_contr)), O(_O) {
    if (embed_normalization_into_coefficients) renorm();
    update_max_ln_coeff();
  }

  Shell& move(std::array<real_t, 3> new_origin) {
    O = new_origin;
    return *this;
  }
  /// Shell::extract_primitive (shell.h:930-945): primitive p alone, with
  /// coefficient 1 in every contraction; normalized when unit_normalized,
  /// else normalization-free
  Shell extract_primitive(size_t p, bool unit_normalized = true) const {
    svector<Contraction> c;
    c.reserve(contr.size());
    for (const auto& x : contr) c.push_back(Contraction{x.l, x.pure, {real_t(1)}});
    return Shell({alpha.at(p)}, c, O, unit_normalized);
  }
  size_t cartesian_size() const {
    size_t s = 0;
    for (const auto& c : contr) s += c.cartesian_size();
    return s;
  }
  size_t size() const {
    size_t s = 0;
    for (const auto& c : contr) s += c.size();
    return s;
  }
  size_t ncontr() const { return contr.size(); }
  size_t nprim() const { return alpha.size(); }
  bool operator==(const Shell& o) const {
    return O == o.O && alpha == o.alpha && contr == o.contr;
  }
  bool operator!=(const Shell& o) const { return !(*this == o); }

  static char am_symbol(size_t l) {
    static const char s[] = "spdfghikmnoqrtuvwxyz";
    assert(l < sizeof(s) - 1);
    return s[l];
  }

  /// Shell::do_enforce_unit_normalization (shell.h:891-901): with no
  /// argument reports, otherwise sets whether renorm() rescales each
  /// contraction to unit self-overlap (process-wide, default true).
  static bool do_enforce_unit_normalization() { return lgx_enforce_unit_normalization(-1) != 0; }
  static bool do_enforce_unit_normalization(bool flag) {
    return lgx_enforce_unit_normalization(flag ? 1 : 0) != 0;
  }

  /// "unit" shell: exponent 0, coefficient 1, at the origin
  static const Shell& unit() {
    static const Shell u = [] {
      Shell s;
      s.alpha = {0.0};
      s.contr = {{0, false, {1.0}}};
      s.O = {{0, 0, 0}};
      s.max_ln_coeff = {0.0};
      return s;
    }();
    return u;
  }

 private:
  void renorm() {
    for (auto& c : contr) {
      svector<real_t> out(c.coeff.size());
      if (lgx_shell_normalize(c.l, int(alpha.size()), alpha.data(), c.coeff.data(),
                              out.data()) != LGX_OK)
        throw std::invalid_argument("libint2::Shell: invalid shell");
      c.coeff = std::move(out);
    }
  }
  void update_max_ln_coeff() {
    max_ln_coeff.assign(nprim(), -std::numeric_limits<real_t>::max());
    for (size_t p = 0; p < nprim(); ++p)
      for (const auto& c : contr) max_ln_coeff[p] = std::max(max_ln_coeff[p], std::log(std::abs(c.coeff[p])));
  }
};

inline std::ostream& operator<<(std::ostream& os, const Shell& sh) {
  os << "Shell:( O={" << sh.O[0] << "," << sh.O[1] << "," << sh.O[2] << "}\n";
  for (const auto& c : sh.contr)
    os << "  " << Shell::am_symbol(c.l) << (c.pure ? "" : "c") << " nprim=" << sh.nprim()
       << "\n";
  return os << ")";
}

/// Primitive screening methods (shell.h:1041-1059 of the reference).  The
/// GPU path implements Original and Conservative; the Schwarz variants are
/// accepted by the J/K builder, which screens quartets by Schwarz bounds.
enum class ScreeningMethod {
  Original = 0x0001,
  Conservative = 0x0010,
  Schwarz = 0x0100,
  SchwarzInf = 0x1000,
  Invalid = 0x0000
};
inline ScreeningMethod& default_screening_method_ref() {
  static ScreeningMethod m = ScreeningMethod::Original;
  return m;
}
inline ScreeningMethod default_screening_method() { return default_screening_method_ref(); }
inline void default_screening_method(ScreeningMethod m) { default_screening_method_ref() = m; }

/// ShellPair (shell.h:1079-1329): accepted by Engine::compute2 for
/// interface compatibility.  The GPU path builds primitive-pair data on the
/// device, so a ShellPair passed in is not consulted.
struct ShellPair {
  struct PrimPairData {
    double P[3];
    double K;
    double one_over_gamma;
    double nonsph_screen_fac;
    double ln_scr;
    int p1, p2;
  };
  std::vector<PrimPairData> primpairs;
  double AB[3] = {0, 0, 0};
  double ln_prec = std::numeric_limits<double>::lowest();
  ScreeningMethod screening_method_ = ScreeningMethod::Invalid;
  ShellPair() = default;
  template <typename Real>
  ShellPair(const Shell& s1, const Shell& s2, Real ln_prec_,
            ScreeningMethod method = default_screening_method()) {
    init(s1, s2, ln_prec_, method);
  }
  /// Schwarz / SchwarzInf screening of the primitive pairs (shell.h:1258-1328):
  /// pair (p1, p2) is kept when log(nprim1 nprim2 K(p1, p2)) + ln|c1| + ln|c2|
  /// >= ln_prec, K from the caller's evaluator (s1, p1, s2, p2) -> Schwarz
  /// factor of the primitive pair
  template <typename Real, typename SchwarzFactorEvaluator>
  ShellPair(const Shell& s1, const Shell& s2, Real ln_prec_, ScreeningMethod method,
            SchwarzFactorEvaluator&& schwarz_factor) {
    init(s1, s2, ln_prec_, method, std::forward<SchwarzFactorEvaluator>(schwarz_factor));
  }
  template <typename Real, typename SchwarzFactorEvaluator>
  void init(const Shell& s1, const Shell& s2, Real ln_prec_, ScreeningMethod method,
            SchwarzFactorEvaluator&& schwarz_factor) {
    if (method != ScreeningMethod::Schwarz && method != ScreeningMethod::SchwarzInf)
      throw std::invalid_argument("ShellPair: the evaluator form takes Schwarz / SchwarzInf");
    primpairs.clear();
    double AB2 = 0;
    for (int i = 0; i < 3; ++i) {
      AB[i] = s1.O[i] - s2.O[i];
      AB2 += AB[i] * AB[i];
    }
    const double n12 = double(s1.nprim() * s2.nprim());
    for (size_t p1 = 0; p1 < s1.nprim(); ++p1)
      for (size_t p2 = 0; p2 < s2.nprim(); ++p2) {
        const double ln_scr = std::log(n12 * double(schwarz_factor(s1, p1, s2, p2))) +
                              s1.max_ln_coeff[p1] + s2.max_ln_coeff[p2];
        if (ln_scr < ln_prec_) continue;
        const double a1 = s1.alpha[p1], a2 = s2.alpha[p2], oog = 1 / (a1 + a2);
        PrimPairData d;
        for (int i = 0; i < 3; ++i)
          d.P[i] = AB2 == 0 ? s1.O[i] : (a1 * s1.O[i] + a2 * s2.O[i]) * oog;
        d.K = 5.9149671727956128778 * std::exp(-a1 * a2 * oog * AB2) * oog;
        d.one_over_gamma = oog;
        d.nonsph_screen_fac = 0;
        d.ln_scr = ln_scr;
        d.p1 = int(p1);
        d.p2 = int(p2);
        primpairs.push_back(d);
      }
    ln_prec = ln_prec_;
    screening_method_ = method;
  }
  template <typename Real>
  void init(const Shell& s1, const Shell& s2, Real ln_prec_,
            ScreeningMethod method = ScreeningMethod::Original) {
    primpairs.clear();
    double AB2 = 0;
    for (int i = 0; i < 3; ++i) {
      AB[i] = s1.O[i] - s2.O[i];
      AB2 += AB[i] * AB[i];
    }
    for (size_t p1 = 0; p1 < s1.nprim(); ++p1)
      for (size_t p2 = 0; p2 < s2.nprim(); ++p2) {
        const double a1 = s1.alpha[p1], a2 = s2.alpha[p2], g = a1 + a2, oog = 1 / g;
        const double mr = -a1 * a2 * oog * AB2;
        const double ln_scr = mr + s1.max_ln_coeff[p1] + s2.max_ln_coeff[p2];
        if (method == ScreeningMethod::Original && ln_scr < ln_prec_) continue;
        PrimPairData d;
        for (int i = 0; i < 3; ++i)
          d.P[i] = AB2 == 0 ? s1.O[i] : (a1 * s1.O[i] + a2 * s2.O[i]) * oog;
        d.K = 5.9149671727956128778 * std::exp(mr) * oog;
        d.one_over_gamma = oog;
        d.nonsph_screen_fac = 0;
        d.ln_scr = ln_scr;
        d.p1 = int(p1);
        d.p2 = int(p2);
        primpairs.push_back(d);
      }
    ln_prec = ln_prec_;
    screening_method_ = method;
  }
};

}  // namespace libint2

#endif
