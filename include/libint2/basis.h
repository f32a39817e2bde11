// libint2::Atom, read_dotxyz and libint2::BasisSet for the GB300 drop-in.
//
// BasisSet(name, atoms) reads <data_path>/<name>.g94 with the G94 reader of
// liblgx (lgx_basis_load: the rules of read_g94_basis_library,
// basis.h.in:473-621 of the reference, including SP-shell splitting, the
// Gaussian Cartesian-d convention and aug- composition) and places the
// shells on the atoms (basis.h.in:134-182).  data_path(): the
// LIBINT_DATA_PATH environment variable, else the compile-time
// LGX_DATA_PATH (libint_gb300/data/basis of this repository by default).
// xyz files are read in angstrom and converted with CODATA 2018
// (atom.h:52-55).
#ifndef LGX_LIBINT2_BASIS_H
#define LGX_LIBINT2_BASIS_H

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <istream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../lgx.h"
#include "shell.h"

#ifndef LGX_DATA_PATH
#define LGX_DATA_PATH "libint_gb300/data/basis"
#endif

namespace libint2 {

struct Atom {
  int atomic_number;
  double x, y, z;
};

namespace constants {
struct codata_2018 {
  static constexpr double bohr_to_angstrom = 0.529177210903;
  static constexpr double angstrom_to_bohr = 1 / bohr_to_angstrom;
};
}  // namespace constants

/// reads an XYZ file (angstrom) into atoms in bohr (atom.h:209-211)
inline std::vector<Atom> read_dotxyz(std::istream& is,
                                     double bohr_to_angstrom =
                                         constants::codata_2018::bohr_to_angstrom) {
  static const char* sym[] = {"",  "H",  "He", "Li", "Be", "B", "C",  "N",  "O",  "F",
                              "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"};
  size_t natom = 0;
  std::string line;
  std::getline(is, line);
  std::istringstream(line) >> natom;
  std::getline(is, line);  // comment
  std::vector<Atom> atoms;
  for (size_t i = 0; i < natom; ++i) {
    std::getline(is, line);
    std::istringstream iss(line);
    std::string s;
    double x, y, z;
    iss >> s >> x >> y >> z;
    int Z = -1;
    for (int k = 1; k < int(sizeof(sym) / sizeof(sym[0])); ++k) {
      std::string t = sym[k];
      if (t.size() == s.size() &&
          std::equal(t.begin(), t.end(), s.begin(),
                     [](char a, char b) { return std::tolower(a) == std::tolower(b); }))
        Z = k;
    }
    if (Z < 0) throw std::runtime_error("read_dotxyz: unknown element " + s);
    atoms.push_back({Z, x / bohr_to_angstrom, y / bohr_to_angstrom, z / bohr_to_angstrom});
  }
  return atoms;
}

class BasisSet : public std::vector<Shell> {
 public:
  BasisSet() = default;
  BasisSet(std::string name, const std::vector<Atom>& atoms) : name_(std::move(name)) {
    std::vector<int32_t> Z;
    std::vector<double> xyz;
    for (const auto& a : atoms) {
      Z.push_back(a.atomic_number);
      xyz.insert(xyz.end(), {a.x, a.y, a.z});
    }
    const std::string dp = data_path();
    int ns = 0, np = 0;
    if (lgx_basis_load(dp.c_str(), name_.c_str(), int(Z.size()), Z.data(), xyz.data(), &ns,
                       &np, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr) !=
        LGX_OK)
      throw std::ios_base::failure("BasisSet: could not read basis " + name_ + " from " + dp);
    std::vector<int32_t> l(ns), pure(ns), nprim(ns), atom(ns);
    std::vector<double> O(3 * ns), alpha(np), coeff(np);
    lgx_basis_load(dp.c_str(), name_.c_str(), int(Z.size()), Z.data(), xyz.data(), &ns, &np,
                   l.data(), pure.data(), nprim.data(), atom.data(), O.data(), alpha.data(),
                   coeff.data());
    int off = 0;
    for (int s = 0; s < ns; ++s) {
      Shell sh(svector<double>(alpha.begin() + off, alpha.begin() + off + nprim[s]),
               {{l[s], pure[s] != 0,
                 svector<double>(coeff.begin() + off, coeff.begin() + off + nprim[s])}},
               {{O[3 * s], O[3 * s + 1], O[3 * s + 2]}}, false);
      push_back(std::move(sh));
      shell2atom_.push_back(atom[s]);
      off += nprim[s];
    }
  }
  explicit BasisSet(const std::vector<Shell>& shells) : std::vector<Shell>(shells) {
    shell2atom_.assign(shells.size(), 0);
  }

  const std::string& name() const { return name_; }
  long nbf() const {
    long n = 0;
    for (const auto& s : *this) n += long(s.size());
    return n;
  }
  size_t max_nprim() const {
    size_t n = 0;
    for (const auto& s : *this) n = std::max(n, s.nprim());
    return n;
  }
  int max_l() const {
    int l = 0;
    for (const auto& s : *this) l = std::max(l, s.contr[0].l);
    return l;
  }
  std::vector<size_t> shell2bf() const {
    std::vector<size_t> r;
    size_t o = 0;
    for (const auto& s : *this) {
      r.push_back(o);
      o += s.size();
    }
    return r;
  }
  const std::vector<long>& shell2atom_index() const { return shell2atom_; }
  /// BasisSet::shell2atom / atom2shell (basis.h.in:279-335): shell k maps to
  /// the first atom whose coordinates equal its origin exactly (-1 when none,
  /// or std::logic_error with throw_if_no_match); atom a maps to the shells
  /// whose origin equals its coordinates, in shell order.
  std::vector<long> shell2atom(const std::vector<Atom>& atoms) const {
    return shell2atom(*this, atoms, false);
  }
  std::vector<std::vector<long>> atom2shell(const std::vector<Atom>& atoms) const {
    return atom2shell(atoms, *this);
  }
  static std::vector<long> shell2atom(const std::vector<Shell>& shells,
                                      const std::vector<Atom>& atoms,
                                      bool throw_if_no_match = false) {
    std::vector<long> r;
    r.reserve(shells.size());
    for (const auto& s : shells) {
      long hit = -1;
      for (size_t a = 0; a < atoms.size() && hit < 0; ++a)
        if (s.O[0] == atoms[a].x && s.O[1] == atoms[a].y && s.O[2] == atoms[a].z) hit = long(a);
      if (hit < 0 && throw_if_no_match) throw std::logic_error("shell2atom: no matching atom found");
      r.push_back(hit);
    }
    return r;
  }
  static std::vector<std::vector<long>> atom2shell(const std::vector<Atom>& atoms,
                                                   const std::vector<Shell>& shells) {
    std::vector<std::vector<long>> r(atoms.size());
    for (size_t a = 0; a < atoms.size(); ++a)
      for (size_t k = 0; k < shells.size(); ++k)
        if (shells[k].O[0] == atoms[a].x && shells[k].O[1] == atoms[a].y &&
            shells[k].O[2] == atoms[a].z)
          r[a].push_back(long(k));
    return r;
  }
  void set_pure(bool pure) {
    for (auto& s : *this)
      for (auto& c : s.contr) c.pure = pure;
  }
  static std::string data_path() {
    if (const char* p = std::getenv("LIBINT_DATA_PATH")) return p;
    return LGX_DATA_PATH;
  }

 private:
  std::string name_;
  std::vector<long> shell2atom_;
};

inline size_t max_nprim(const std::vector<Shell>& shells) {
  size_t n = 0;
  for (const auto& s : shells) n = std::max(n, s.nprim());
  return n;
}
inline int max_l(const std::vector<Shell>& shells) {
  int l = 0;
  for (const auto& s : shells) l = std::max(l, s.contr[0].l);
  return l;
}
inline size_t nbf(const std::vector<Shell>& shells) {
  size_t n = 0;
  for (const auto& s : shells) n += s.size();
  return n;
}

}  // namespace libint2

#endif
