// Test driver for the C++ drop-in headers (include/libint2.hpp): written the
// way a libint2 caller writes it (initialize, BasisSet, Engine::compute,
// compute2<...,1>, results(), lmax_exceeded, finalize), plus the batched
// JKBuilder.  Writes every shell set it computes to a binary file that the
// pytest wrapper compares with the oracle.
#include <libint2.hpp>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <limits>
#include <vector>

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::ofstream out(argv[1], std::ios::binary);
  auto put = [&](double v) { out.write(reinterpret_cast<const char*>(&v), sizeof v); };
  libint2::initialize();
  std::vector<libint2::Atom> atoms = {{8, 0.0, -0.143, 0.0}, {1, 1.638, 1.136, 0.0},
                                      {1, -1.638, 1.136, 0.0}, {8, 5.0, 0.2, 0.1},
                                      {1, 6.6, 1.4, 0.0}, {1, 3.4, 1.2, 0.3}};
  libint2::BasisSet obs("cc-pVDZ", atoms);
  put(double(obs.size()));
  libint2::Engine engine(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 0);
  const auto& buf = engine.results();
  const size_t ns = 8;  // first 8 shells: s, s, s, p, p, d on O and s, s on H
  for (size_t a = 0; a < ns; ++a)
    for (size_t b = 0; b < ns; ++b)
      for (size_t c = 0; c < ns; ++c)
        for (size_t d = 0; d < ns; ++d) {
          engine.compute(obs[a], obs[b], obs[c], obs[d]);
          const size_t n = obs[a].size() * obs[b].size() * obs[c].size() * obs[d].size();
          if (buf[0] == nullptr) {
            put(0.0);
            continue;
          }
          put(1.0);
          for (size_t i = 0; i < n; ++i) put(buf[0][i]);
        }
  // first derivatives through compute2<coulomb, xx_xx, 1>
  libint2::Engine d1(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 1);
  const size_t q1[][4] = {{5, 3, 8, 0}, {3, 5, 5, 9}, {0, 14, 5, 3}};
  for (const auto& q : q1) {
    const auto& r = d1.compute2<libint2::Operator::coulomb, libint2::BraKet::xx_xx, 1>(
        obs[q[0]], obs[q[1]], obs[q[2]], obs[q[3]]);
    const size_t n = obs[q[0]].size() * obs[q[1]].size() * obs[q[2]].size() * obs[q[3]].size();
    for (unsigned s = 0; s < d1.nshellsets(); ++s)
      for (size_t i = 0; i < n; ++i) put(r[s][i]);
  }
  // lmax_exceeded is thrown for max_l beyond the build
  bool thrown = false;
  try {
    libint2::Engine e(libint2::Operator::coulomb, 4, 5, 0);
  } catch (const libint2::Engine::lmax_exceeded&) {
    thrown = true;
  }
  put(thrown ? 1.0 : 0.0);
  // batched J/K
  libint2::gb300::JKBuilder jk(obs);
  const int nbf = jk.nbf();
  std::vector<double> D(size_t(nbf) * nbf), J, K;
  for (int i = 0; i < nbf; ++i)
    for (int j = 0; j < nbf; ++j) D[size_t(i) * nbf + j] = std::exp(-0.3 * std::abs(i - j));
  jk.compute(D, J, K, 0.0);
  for (double v : J) put(v);
  for (double v : K) put(v);
  // 3- and 2-centre integrals (density fitting): BraKet::xs_xx / xs_xs
  libint2::Engine e3(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 0,
                     std::numeric_limits<double>::epsilon(), nullptr, libint2::BraKet::xs_xx);
  libint2::Engine e3d(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 1,
                      std::numeric_limits<double>::epsilon(), nullptr, libint2::BraKet::xs_xx);
  libint2::Engine e2(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 0,
                     std::numeric_limits<double>::epsilon(), nullptr, libint2::BraKet::xs_xs);
  const size_t t3[][3] = {{5, 3, 8}, {3, 5, 14}, {0, 9, 2}};
  for (const auto& t : t3) {
    const size_t n = obs[t[0]].size() * obs[t[1]].size() * obs[t[2]].size();
    const auto& r = e3.compute(obs[t[0]], obs[t[1]], obs[t[2]]);
    for (size_t i = 0; i < n; ++i) put(r[0][i]);
    const auto& rd = e3d.compute2<libint2::Operator::coulomb, libint2::BraKet::xs_xx, 1>(
        obs[t[0]], libint2::Shell::unit(), obs[t[1]], obs[t[2]]);
    put(double(e3d.nshellsets()));
    for (unsigned s = 0; s < e3d.nshellsets(); ++s)
      for (size_t i = 0; i < n; ++i) put(rd[s][i]);
    const auto& r2 = e2.compute(obs[t[0]], obs[t[1]]);
    for (size_t i = 0; i < obs[t[0]].size() * obs[t[1]].size(); ++i) put(r2[0][i]);
  }
  // second derivatives: compute2<coulomb, xx_xx, 2>, 78 sets
  libint2::Engine d2(libint2::Operator::coulomb, obs.max_nprim(), 2, 2);
  const size_t q2[][4] = {{5, 3, 8, 0}, {3, 0, 1, 9}};
  for (const auto& q : q2) {
    const auto& r = d2.compute2<libint2::Operator::coulomb, libint2::BraKet::xx_xx, 2>(
        obs[q[0]], obs[q[1]], obs[q[2]], obs[q[3]]);
    const size_t n = obs[q[0]].size() * obs[q[1]].size() * obs[q[2]].size() * obs[q[3]].size();
    put(double(d2.nshellsets()));
    for (unsigned s = 0; s < d2.nshellsets(); ++s)
      for (size_t i = 0; i < n; ++i) put(r[s][i]);
  }
  // range-separated operator: erfc(omega r)/r with omega as the params argument
  libint2::Engine ec(libint2::Operator::erfc_coulomb, obs.max_nprim(), obs.max_l(), 0,
                     std::numeric_limits<double>::epsilon(), 0.3);
  for (const auto& q : q1) {
    const auto& r = ec.compute(obs[q[0]], obs[q[1]], obs[q[2]], obs[q[3]]);
    const size_t n = obs[q[0]].size() * obs[q[1]].size() * obs[q[2]].size() * obs[q[3]].size();
    for (size_t i = 0; i < n; ++i) put(r[0][i]);
  }
  // precomputed ShellPair data, as compute_2body_fock passes it: pairs at
  // the machine epsilon, the engine at 1e-10 (deriv 0 and 1)
  {
    const double ln_eps = std::log(std::numeric_limits<double>::epsilon());
    libint2::Engine p0(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 0, 1e-10);
    libint2::Engine p1(libint2::Operator::coulomb, obs.max_nprim(), obs.max_l(), 1, 1e-10);
    for (const auto& q : q1) {
      libint2::ShellPair sp12(obs[q[0]], obs[q[1]], ln_eps), sp34(obs[q[2]], obs[q[3]], ln_eps);
      const size_t n =
          obs[q[0]].size() * obs[q[1]].size() * obs[q[2]].size() * obs[q[3]].size();
      const auto& r0 = p0.compute2<libint2::Operator::coulomb, libint2::BraKet::xx_xx, 0>(
          obs[q[0]], obs[q[1]], obs[q[2]], obs[q[3]], &sp12, &sp34);
      put(r0[0] == nullptr ? 0.0 : 1.0);
      if (r0[0] != nullptr)
        for (size_t i = 0; i < n; ++i) put(r0[0][i]);
      const auto& r1 = p1.compute2<libint2::Operator::coulomb, libint2::BraKet::xx_xx, 1>(
          obs[q[0]], obs[q[1]], obs[q[2]], obs[q[3]], &sp12, &sp34);
      put(r1[0] == nullptr ? 0.0 : 1.0);
      if (r1[0] != nullptr)
        for (unsigned s = 0; s < p1.nshellsets(); ++s)
          for (size_t i = 0; i < n; ++i) put(r1[s][i]);
    }
  }
  libint2::finalize();
  std::cout << "ok" << std::endl;
  return 0;
}
