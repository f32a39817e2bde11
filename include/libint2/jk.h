// Batched, Schwarz-screened J/K build and gradients over a BasisSet: the
// GB300 replacement of the per-quartet Engine loop of compute_2body_fock /
// compute_2body_fock_deriv (tests/hartree-fock/hartree-fock++.cc:1574-2000
// of the reference).  No counterpart class exists in the reference; it
// wraps lgx_set_basis / lgx_jk / lgx_jk_grad.
#ifndef LGX_LIBINT2_JK_H
#define LGX_LIBINT2_JK_H

#include <stdexcept>
#include <string>
#include <vector>

#include "../lgx.h"
#include "basis.h"
#include "engine.h"

namespace libint2 {
namespace gb300 {

class JKBuilder {
 public:
  explicit JKBuilder(const BasisSet& bs, int device = 0) {
    if (lgx_create(&ctx_, device) != LGX_OK)
      throw std::runtime_error("JKBuilder: no usable CUDA device");
    std::vector<int32_t> l, pure, nprim, atom;
    std::vector<double> O, alpha, coeff;
    const auto& s2a = bs.shell2atom_index();
    for (size_t s = 0; s < bs.size(); ++s) {
      l.push_back(bs[s].contr[0].l);
      pure.push_back(bs[s].contr[0].pure ? 1 : 0);
      nprim.push_back(int(bs[s].nprim()));
      atom.push_back(s < s2a.size() ? int(s2a[s]) : 0);
      O.insert(O.end(), bs[s].O.begin(), bs[s].O.end());
      alpha.insert(alpha.end(), bs[s].alpha.begin(), bs[s].alpha.end());
      coeff.insert(coeff.end(), bs[s].contr[0].coeff.begin(), bs[s].contr[0].coeff.end());
    }
    check(lgx_set_basis(ctx_, int(bs.size()), l.data(), pure.data(), nprim.data(), atom.data(),
                        O.data(), alpha.data(), coeff.data()));
    nbf_ = int(bs.nbf());
    natoms_ = 0;
    for (int a : atom) natoms_ = std::max(natoms_, a + 1);
  }
  ~JKBuilder() {
    if (ctx_) lgx_destroy(ctx_);
  }
  JKBuilder(const JKBuilder&) = delete;
  JKBuilder& operator=(const JKBuilder&) = delete;

  /// J and K (row-major nbf x nbf) from a symmetric density D.
  lgx_jk_stats compute(const std::vector<double>& D, std::vector<double>& J,
                       std::vector<double>& K, double schwarz_thresh = 1e-12,
                       bool mixed = false, double mixed_thresh = 1e-4) {
    J.resize(size_t(nbf_) * nbf_);
    K.resize(size_t(nbf_) * nbf_);
    lgx_jk_stats st{};
    check(lgx_jk(ctx_, D.data(), J.data(), K.data(), schwarz_thresh, mixed ? LGX_MIXED : LGX_FP64,
                 mixed_thresh, &st));
    return st;
  }
  /// gradients of E_J = 1/2 sum D.J and E_K = -1/4 sum D.K, natoms x 3
  lgx_jk_stats gradient(const std::vector<double>& D, std::vector<double>& gJ,
                        std::vector<double>& gK, double schwarz_thresh = 1e-12) {
    gJ.assign(3 * size_t(natoms_), 0.0);
    gK.assign(3 * size_t(natoms_), 0.0);
    lgx_jk_stats st{};
    check(lgx_jk_grad(ctx_, D.data(), gJ.data(), gK.data(), natoms_, schwarz_thresh, &st));
    return st;
  }
  int nbf() const { return nbf_; }
  /// Operator of the J/K and gradient passes: Operator::coulomb (default),
  /// erf_coulomb or erfc_coulomb with range-separation parameter omega
  /// (the long- / short-range exchange of range-separated functionals)
  void set_operator(Operator op, double omega = 0.0) {
    const int opc = op == Operator::erf_coulomb
                        ? LGX_OP_ERF_COULOMB
                        : (op == Operator::erfc_coulomb ? LGX_OP_ERFC_COULOMB : LGX_OP_COULOMB);
    if (op != Operator::coulomb && op != Operator::erf_coulomb && op != Operator::erfc_coulomb)
      throw std::invalid_argument("JKBuilder::set_operator: unsupported operator");
    check(lgx_set_operator(ctx_, opc, omega));
  }
  /// Density-weighted screening of later J/K builds, as compute_2body_fock's
  /// `precision` argument (hartree-fock++.cc:1640-1684): quartets with
  /// max shell-block |D| * K12 * K34 below `precision` are skipped and the
  /// others' primitives screened at precision / max |D|; 0 turns it off.
  void set_fock_precision(double precision) { check(lgx_set_fock_precision(ctx_, precision)); }

 private:
  lgx_context* ctx_ = nullptr;
  int nbf_ = 0, natoms_ = 0;
  void check(lgx_status s) {
    if (s != LGX_OK) throw std::runtime_error(std::string("lgx: ") + lgx_last_error(ctx_));
  }
};

}  // namespace gb300
}  // namespace libint2

#endif
