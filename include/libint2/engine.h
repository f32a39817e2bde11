// libint2::Engine (Operator::coulomb / erf_coulomb / erfc_coulomb, BraKet
// xx_xx / xs_xx / xs_xs, deriv_order 0, 1 and 2) as a drop-in over liblgx
// (include/lgx.h).
//
// Names and signatures follow the reference's engine.h:444-1064 for this
// path: Engine(Operator, max_nprim, max_l, deriv_order, precision, params,
// braket, screening); compute(s1,s2,s3,s4); compute2<op,braket,deriv>(...);
// results(), nshellsets(), set_precision(), precision(), set(...);
// exceptions lmax_exceeded / using_default_initialized.  compute() returns
// results(): nshellsets() pointers to row-major shell sets in the caller's
// shell order, valid until the next compute on this Engine; results()[0] is
// nullptr when every primitive quartet was screened out
// (engine.impl.h:1781-1784).  The arithmetic runs on the GPU context
// created by libint2::initialize().
#ifndef LGX_LIBINT2_ENGINE_H
#define LGX_LIBINT2_ENGINE_H

#include <array>
#include <limits>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../lgx.h"
#include "shell.h"

namespace libint2 {

/// Operator enum of the reference (engine.h:98-184); coulomb, erf_coulomb
/// and erfc_coulomb are served (the attenuated ones take omega as params).
enum class Operator {
  overlap = 0,
  kinetic,
  nuclear,
  erf_nuclear,
  erfc_nuclear,
  emultipole1,
  emultipole2,
  emultipole3,
  sphemultipole,
  opVop,
  delta,
  coulomb,
  cgtg,
  cgtg_x_coulomb,
  delcgtg2,
  r12,
  erf_coulomb,
  erfc_coulomb,
  stg,
  stg_x_coulomb,
  invalid = -1,
  first_2body_oper = delta,
  last_2body_oper = stg_x_coulomb
};

/// BraKet enum (engine.h:188-206); xx_xx, and the 3- and 2-centre xs_xx /
/// xs_xs through Shell::unit() as the reference does (engine.impl.h:140-175).
enum class BraKet { x_x = 0, xx_xx, xs_xx, xx_xs, xs_xs, invalid = -1 };

enum class CartesianShellNormalization { standard, uniform };

/// libint2::operator_traits<Op> (engine.h:200-371), the part callers use:
/// the parameter type of an operator and its default value (empty for the
/// Coulomb operator, the attenuation omega for erf / erfc_coulomb).
namespace detail {
struct default_operator_traits {
  typedef struct {
  } oper_params_type;
  static oper_params_type default_params() { return oper_params_type{}; }
  static constexpr auto nopers = 1u;
  static constexpr auto intrinsic_deriv_order = 0u;
};
}  // namespace detail
template <Operator Op>
struct operator_traits : public detail::default_operator_traits {};
template <>
struct operator_traits<Operator::erf_coulomb> : public detail::default_operator_traits {
  typedef double oper_params_type;
  static oper_params_type default_params() { return 0.0; }
};
template <>
struct operator_traits<Operator::erfc_coulomb> : public detail::default_operator_traits {
  typedef double oper_params_type;
  static oper_params_type default_params() { return 0.0; }
};

constexpr size_t num_geometrical_derivatives(size_t ncenter, size_t deriv_order) {
  return deriv_order > 0 ? (num_geometrical_derivatives(ncenter, deriv_order - 1) *
                            (3 * ncenter + deriv_order - 1)) /
                               deriv_order
                         : 1;
}

namespace detail {
struct Runtime {
  std::mutex mu;
  lgx_context* ctx = nullptr;
  int device = 0;
};
inline Runtime& runtime() {
  static Runtime r;
  return r;
}
}  // namespace detail

/// libint2::initialize() (initialize.h:76-95): creates the GPU context.
inline void initialize(bool /*verbose*/ = false) {
  auto& r = detail::runtime();
  std::lock_guard<std::mutex> lk(r.mu);
  if (!r.ctx) {
    if (lgx_create(&r.ctx, r.device) != LGX_OK)
      throw std::runtime_error("libint2::initialize: no usable GB300 / sm_100+ CUDA device");
  }
}
inline bool initialized() { return detail::runtime().ctx != nullptr; }
/// libint2::finalize(): releases the GPU context.
inline void finalize() {
  auto& r = detail::runtime();
  std::lock_guard<std::mutex> lk(r.mu);
  if (r.ctx) lgx_destroy(r.ctx);
  r.ctx = nullptr;
}

class Engine {
 public:
  typedef double value_type;
  typedef double scalar_type;
  typedef std::vector<const value_type*> target_ptr_vec;
  static constexpr auto max_ntargets = 12;

  /// thrown when max_l exceeds LGX_MAX_L (engine.h:893-905)
  struct lmax_exceeded : public std::logic_error {
    lmax_exceeded(const char* task_name, size_t lmax_limit, size_t lmax_requested)
        : std::logic_error("Engine::lmax_exceeded"),
          task_name_(task_name),
          lmax_limit_(lmax_limit),
          lmax_requested_(lmax_requested) {}
    const char* task_name() const { return task_name_.c_str(); }
    size_t lmax_limit() const { return lmax_limit_; }
    size_t lmax_requested() const { return lmax_requested_; }
   private:
    std::string task_name_;
    size_t lmax_limit_, lmax_requested_;
  };
  /// thrown when using a default-initialized Engine (engine.h:907-913)
  struct using_default_initialized : public std::logic_error {
    using_default_initialized()
        : std::logic_error("Engine is default-initialized: use the full constructor") {}
  };

  Engine() = default;
  /// erf_coulomb / erfc_coulomb: params = omega, the range-separation
  /// parameter (operator_traits<erf_coulomb>::oper_params_type, engine.h:353-370)
  Engine(Operator oper, size_t max_nprim, int max_l, int deriv_order,
         scalar_type precision, double omega, BraKet braket = BraKet::invalid,
         ScreeningMethod screening = default_screening_method())
      : Engine(oper, max_nprim, max_l, deriv_order, precision, nullptr, braket, screening) {
    set_params(omega);
  }
  /// Coulomb with its (empty) parameters as libint callers pass them:
  /// operator_traits<Operator::coulomb>::default_params()
  Engine(Operator oper, size_t max_nprim, int max_l, int deriv_order, scalar_type precision,
         detail::default_operator_traits::oper_params_type /*params*/,
         BraKet braket = BraKet::invalid, ScreeningMethod screening = default_screening_method())
      : Engine(oper, max_nprim, max_l, deriv_order, precision, nullptr, braket, screening) {}
  Engine(Operator oper, size_t max_nprim, int max_l, int deriv_order = 0,
         scalar_type precision = std::numeric_limits<scalar_type>::epsilon(),
         std::nullptr_t /*params*/ = nullptr, BraKet braket = BraKet::invalid,
         ScreeningMethod screening = default_screening_method())
      : oper_(oper),
        braket_(braket == BraKet::invalid ? BraKet::xx_xx : braket),
        max_nprim_(max_nprim),
        lmax_(max_l),
        deriv_order_(deriv_order),
        screening_(screening) {
    if ((oper_ != Operator::coulomb && oper_ != Operator::erf_coulomb &&
         oper_ != Operator::erfc_coulomb) ||
        (braket_ != BraKet::xx_xx && braket_ != BraKet::xs_xx && braket_ != BraKet::xs_xs))
      throw std::invalid_argument(
          "libint2::Engine (GB300): only Operator::coulomb, erf_coulomb, erfc_coulomb with "
          "BraKet::xx_xx, xs_xx or xs_xs is implemented");
    if (max_l < 0 || max_l > LGX_MAX_L) throw lmax_exceeded("eri", LGX_MAX_L, max_l);
    if (deriv_order < 0 || deriv_order > LGX_MAX_DERIV)
      throw std::invalid_argument("libint2::Engine (GB300): deriv_order must be 0, 1 or 2");
    if (deriv_order == 2 && braket_ != BraKet::xx_xx)
      throw std::invalid_argument("libint2::Engine (GB300): deriv_order 2 needs BraKet::xx_xx");
    set_precision(precision);
    if (!initialized()) initialize();
    targets_.assign(nshellsets(), nullptr);
    initialized_ = true;
  }

  Operator oper() const { return oper_; }
  /// Engine::set_params (engine.h:685-700): omega of erf/erfc_coulomb
  Engine& set_params(double omega) {
    if (!(omega >= 0)) throw std::invalid_argument("Engine::set_params: omega must be >= 0");
    omega_ = omega;
    return *this;
  }
  /// the Coulomb operator's (empty) parameters
  Engine& set_params(detail::default_operator_traits::oper_params_type) { return *this; }
  /// Engine::set(Operator) / set(BraKet) (engine.h:658-684): change the
  /// operator or the braket of a constructed engine (one of those served)
  Engine& set(Operator new_oper) {
    if (new_oper != Operator::coulomb && new_oper != Operator::erf_coulomb &&
        new_oper != Operator::erfc_coulomb)
      throw std::invalid_argument(
          "libint2::Engine (GB300): only Operator::coulomb, erf_coulomb, erfc_coulomb");
    oper_ = new_oper;
    return *this;
  }
  Engine& set(BraKet new_braket) {
    if (new_braket != BraKet::xx_xx && new_braket != BraKet::xs_xx && new_braket != BraKet::xs_xs)
      throw std::invalid_argument("libint2::Engine (GB300): only BraKet::xx_xx, xs_xx, xs_xs");
    if (deriv_order_ == 2 && new_braket != BraKet::xx_xx)
      throw std::invalid_argument("libint2::Engine (GB300): deriv_order 2 needs BraKet::xx_xx");
    braket_ = new_braket;
    targets_.assign(nshellsets(), nullptr);
    return *this;
  }
  double params() const { return omega_; }
  BraKet braket() const { return braket_; }
  int deriv_order() const { return deriv_order_; }
  /// rank of the braket: 4 (xx_xx), 3 (xs_xx), 2 (xs_xs) (engine.h:408-417)
  int braket_rank() const {
    return braket_ == BraKet::xs_xs ? 2 : (braket_ == BraKet::xs_xx ? 3 : 4);
  }
  unsigned int nshellsets() const {
    return unsigned(num_geometrical_derivatives(size_t(braket_rank()), size_t(deriv_order_)));
  }
  const target_ptr_vec& results() const { return targets_; }

  Engine& set_precision(scalar_type prec) {
    if (prec <= 0.) {
      precision_ = 0.;
      ln_precision_ = std::numeric_limits<scalar_type>::lowest();
    } else {
      precision_ = prec;
      ln_precision_ = std::log(prec);
    }
    return *this;
  }
  scalar_type precision() const { return precision_; }
  Engine& set(ScreeningMethod m) {
    screening_ = m;
    return *this;
  }
  Engine& set(CartesianShellNormalization n) {
    if (n != CartesianShellNormalization::standard)
      throw std::invalid_argument("libint2::Engine (GB300): only standard normalization");
    return *this;
  }
  ScreeningMethod screening_method() const { return screening_; }
  Engine& set_max_nprim(size_t n) {
    max_nprim_ = n;
    return *this;
  }
  /// Engine::prescale_by / prescaled_by (engine.h:851-861): every target
  /// integral is multiplied by `sc` (default 1); libint folds it into the
  /// primitive prefactor, here it scales the returned sets.
  Engine& prescale_by(scalar_type sc) {
    scale_ = sc;
    return *this;
  }
  scalar_type prescaled_by() const { return scale_; }
  Engine& set_max_l(int L) {
    if (L > LGX_MAX_L) throw lmax_exceeded("eri", LGX_MAX_L, L);
    lmax_ = L;
    return *this;
  }

  /// Engine::compute (engine.impl.h:140-175): 4 shells for xx_xx, 3 for
  /// xs_xx (bra1 | ket1 ket2), 2 for xs_xs (bra1 | ket1); the missing
  /// positions take Shell::unit() as in the reference.
  const target_ptr_vec& compute(const Shell& s1, const Shell& s2, const Shell& s3,
                                const Shell& s4) {
    if (braket_rank() != 4) throw std::invalid_argument("Engine::compute: braket needs 4 shells");
    return compute_impl(s1, s2, s3, s4);
  }
  const target_ptr_vec& compute(const Shell& s1, const Shell& s2, const Shell& s3) {
    if (braket_rank() != 3) throw std::invalid_argument("Engine::compute: braket needs 3 shells");
    return compute_impl(s1, Shell::unit(), s2, s3);
  }
  const target_ptr_vec& compute(const Shell& s1, const Shell& s2) {
    if (braket_rank() != 2) throw std::invalid_argument("Engine::compute: braket needs 2 shells");
    return compute_impl(s1, Shell::unit(), s2, Shell::unit());
  }
  /// Engine::compute2<op, braket, deriv> (engine.h:787-791).  Precomputed
  /// ShellPair data of the bra / ket (xx_xx, deriv 0 or 1) is used as the
  /// reference uses it (engine.impl.h:1259-1276): when its ln_prec is at
  /// most ln(precision) its primitive pairs are the ones screened (the GPU
  /// rebuilds them at that ln_prec: the data of ShellPair::init with the
  /// engine's Original / Conservative method), else they are recomputed at
  /// the engine precision; a ShellPair of another screening method is
  /// rejected, as the reference asserts.  Deriv 2 recomputes them.
  template <Operator op, BraKet bk, size_t deriv>
  const target_ptr_vec& compute2(const Shell& s1, const Shell& s2, const Shell& s3,
                                 const Shell& s4, const ShellPair* sp12 = nullptr,
                                 const ShellPair* sp34 = nullptr) {
    static_assert((op == Operator::coulomb || op == Operator::erf_coulomb ||
                   op == Operator::erfc_coulomb) &&
                      (bk == BraKet::xx_xx || bk == BraKet::xs_xx || bk == BraKet::xs_xs),
                  "only coulomb / erf_coulomb / erfc_coulomb with xx_xx, xs_xx, xs_xs is "
                  "implemented on the GPU path");
    if (int(deriv) != deriv_order_ || bk != braket_ || op != oper_)
      throw std::invalid_argument("Engine::compute2: deriv_order, operator or braket mismatch");
    for (const ShellPair* sp : {sp12, sp34})
      if (sp && sp->screening_method_ != screening_)
        throw std::invalid_argument(
            "Engine::compute2: received ShellPair initialized for an incompatible screening "
            "method");
    if ((sp12 || sp34) && bk == BraKet::xx_xx && deriv_order_ < 2) {
      const double pl[2] = {
          sp12 && sp12->ln_prec <= ln_precision_ ? double(sp12->ln_prec) : ln_precision_,
          sp34 && sp34->ln_prec <= ln_precision_ ? double(sp34->ln_prec) : ln_precision_};
      return compute_impl(s1, s2, s3, s4, pl);
    }
    return compute_impl(s1, s2, s3, s4);
  }

 private:
  Operator oper_ = Operator::invalid;
  BraKet braket_ = BraKet::invalid;
  size_t max_nprim_ = 0;
  int lmax_ = -1;
  int deriv_order_ = 0;
  scalar_type precision_ = 0, ln_precision_ = 0;
  ScreeningMethod screening_ = ScreeningMethod::Original;
  double omega_ = 0;
  scalar_type scale_ = 1;
  bool initialized_ = false;
  std::vector<value_type> buf_;
  target_ptr_vec targets_;

  // pair_ln: NULL, or the ln_prec of the bra / ket primitive pairs
  const target_ptr_vec& compute_impl(const Shell& s1, const Shell& s2, const Shell& s3,
                                     const Shell& s4, const double* pair_ln = nullptr) {
    if (!initialized_) throw using_default_initialized();
    const Shell* sh[4] = {&s1, &s2, &s3, &s4};
    lgx_shell d[4];
    size_t nv = 1;
    for (int k = 0; k < 4; ++k) {
      if (sh[k]->ncontr() != 1)
        throw std::invalid_argument("generally-contracted shells are not yet supported");
      const int l = sh[k]->contr[0].l;
      if (l > lmax_) throw lmax_exceeded("eri", size_t(lmax_), size_t(l));
      d[k].l = l;
      d[k].pure = sh[k]->contr[0].pure ? 1 : 0;
      d[k].nprim = int(sh[k]->nprim());
      d[k].pad_ = 0;
      for (int x = 0; x < 3; ++x) d[k].origin[x] = sh[k]->O[x];
      d[k].alpha = sh[k]->alpha.data();
      d[k].coeff = sh[k]->contr[0].coeff.data();
      nv *= sh[k]->size();
    }
    const unsigned ns = nshellsets();
    buf_.resize(nv * (deriv_order_ == 2 ? 78 : (deriv_order_ ? 12 : 1)));
    int nsets = 0, nvalues = 0, is_null = 0;
    const int method =
        screening_ == ScreeningMethod::Conservative ? LGX_SCREEN_CONSERVATIVE : LGX_SCREEN_ORIGINAL;
    auto& rt = detail::runtime();
    // the runtime context is shared by every Engine: set this one's operator
    const int opc = oper_ == Operator::erf_coulomb
                        ? LGX_OP_ERF_COULOMB
                        : (oper_ == Operator::erfc_coulomb ? LGX_OP_ERFC_COULOMB : LGX_OP_COULOMB);
    if (lgx_set_operator(rt.ctx, opc, omega_) != LGX_OK)
      throw std::runtime_error(std::string("libint2::Engine::compute: ") + lgx_last_error(rt.ctx));
    const lgx_status st =
        pair_ln ? lgx_compute_shellset_pairs(rt.ctx, d, deriv_order_, precision_, method, pair_ln,
                                             buf_.data(), buf_.size(), &nsets, &nvalues, &is_null)
                : lgx_compute_shellset(rt.ctx, d, deriv_order_, precision_, method, buf_.data(),
                                       buf_.size(), &nsets, &nvalues, &is_null);
    if (st == LGX_ERR_LMAX_EXCEEDED) throw lmax_exceeded("eri", LGX_MAX_L, size_t(lmax_));
    if (st != LGX_OK)
      throw std::runtime_error(std::string("libint2::Engine::compute: ") + lgx_last_error(rt.ctx));
    targets_.assign(ns, nullptr);
    if (is_null) return targets_;
    if (scale_ != scalar_type(1))
      for (size_t i = 0; i < size_t(nsets) * size_t(nvalues); ++i) buf_[i] *= scale_;
    // derivative sets of the real centres only: the unit shells' sets (zero)
    // are left out, which leaves the reference's order (centres A, C, D for
    // xs_xx; A, C for xs_xs; each x, y, z)
    static const int kSet3[9] = {0, 1, 2, 6, 7, 8, 9, 10, 11};
    static const int kSet2[6] = {0, 1, 2, 6, 7, 8};
    for (unsigned s = 0; s < ns; ++s) {
      const int src = (deriv_order_ == 0 || braket_rank() == 4)
                          ? int(s)
                          : (braket_rank() == 3 ? kSet3[s] : kSet2[s]);
      targets_[s] = buf_.data() + size_t(src) * nv;
    }
    return targets_;
  }
};

}  // namespace libint2

#endif
