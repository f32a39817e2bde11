// Host utilities of liblgx: shell normalization, the G94 basis-set reader
// and the synthetic water-cluster builder.  Plain C++ (no CUDA).
#include <atomic>
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/lgx.h"

namespace {

double dfac(int n) {  // n!!, (-1)!! = 1
  double r = 1;
  for (int i = n; i > 1; i -= 2) r *= i;
  return r;
}

// Shell::do_enforce_unit_normalization (include/libint2/shell.h:891-901):
// process-wide, on by default.
std::atomic<bool> g_unit_normalization{true};

// Shell::renorm (include/libint2/shell.h:958-999): primitive normalization
// embedded into the coefficients, then (when enforced) the contraction
// rescaled to unit self-overlap.
void normalize(int l, int nprim, const double* alpha, const double* cin, double* cout) {
  const double sqrt_pi3 = 5.56832799683170784528481798212;  // pi^{3/2}
  std::vector<double> c(cin, cin + nprim);
  for (int p = 0; p < nprim; ++p) {
    if (alpha[p] == 0) continue;
    const double two_a = 2 * alpha[p];
    const double t = std::pow(two_a, l + 1) * std::sqrt(two_a);
    c[p] *= std::sqrt(std::pow(2.0, l) * t / (sqrt_pi3 * dfac(2 * l - 1)));
  }
  if (!g_unit_normalization.load()) {
    for (int p = 0; p < nprim; ++p) cout[p] = c[p];
    return;
  }
  double norm = 0;
  for (int p = 0; p < nprim; ++p)
    for (int q = 0; q <= p; ++q) {
      const double g = alpha[p] + alpha[q];
      norm += (p == q ? 1 : 2) * dfac(2 * l - 1) * sqrt_pi3 * c[p] * c[q] /
              (std::pow(2.0, l) * std::pow(g, l + 1) * std::sqrt(g));
    }
  const double f = 1 / std::sqrt(norm);
  for (int p = 0; p < nprim; ++p) cout[p] = c[p] * f;
}

struct RawShell {
  int l;
  bool pure;
  std::vector<double> alpha, coeff;
};

const char* kSymbols[] = {"",   "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",
                          "Ne", "Na", "Mg", "Al", "Si", "P",  "S",  "Cl", "Ar"};

int symbol_to_Z(const std::string& s) {
  for (int z = 1; z < int(sizeof(kSymbols) / sizeof(kSymbols[0])); ++z) {
    const char* t = kSymbols[z];
    if (s.size() == std::strlen(t)) {
      bool eq = true;
      for (size_t i = 0; i < s.size(); ++i)
        if (std::tolower(s[i]) != std::tolower(t[i])) eq = false;
      if (eq) return z;
    }
  }
  return -1;
}

int am_letter(char c) {
  switch (std::toupper(c)) {
    case 'S': return 0;
    case 'P': return 1;
    case 'D': return 2;
    case 'F': return 3;
    case 'G': return 4;
    case 'H': return 5;
    case 'I': return 6;
  }
  return -1;
}

// Gaussian's Cartesian-d convention (basis.h.in:367-385).
bool cartesian_d(const std::string& n) {
  if (n.rfind("3-21", 0) == 0 || n.rfind("4-31g", 0) == 0) return true;
  if (n.rfind("6-31", 0) == 0 && n.size() > 4 && n[4] != '1') {
    const auto g = n.find('g');
    if (g == std::string::npos) return false;
    if (g + 1 == n.size()) return true;
    if (n[g + 1] == '*' || n[g + 1] == 's') return true;
  }
  return false;
}

// G94 reader (read_g94_basis_library, basis.h.in:473-621).
bool read_g94(const std::string& file, bool force_cart_d,
              std::vector<std::vector<RawShell>>& byZ, std::string& err) {
  std::ifstream is(file);
  if (!is.good()) {
    err = "cannot open " + file;
    return false;
  }
  byZ.assign(119, {});
  std::string line;
  bool nextbasis = true, nextshell = false, first = true;
  int Z = -1;
  while (std::getline(is, line)) {
    while (!line.empty() && (line.back() == '\r' || line.back() == ' ')) line.pop_back();
    if (line.empty() || line[0] == '!') continue;
    if (line == "****") {
      if (first) continue;
      nextbasis = true;
      nextshell = false;
      continue;
    }
    std::istringstream iss(line);
    if (nextbasis) {
      nextbasis = false;
      first = false;
      std::string sym;
      iss >> sym;
      Z = symbol_to_Z(sym);
      if (Z < 0) {
        err = "unknown element " + sym + " in " + file;
        return false;
      }
      nextshell = true;
      continue;
    }
    if (nextshell) {
      std::string label;
      int nprim = 0;
      iss >> label >> nprim;
      auto read_prims = [&](int ncol, std::vector<double>& e, std::vector<double>& c1,
                            std::vector<double>& c2) {
        for (int p = 0; p < nprim; ++p) {
          std::string pl;
          while (std::getline(is, pl) && (pl.empty() || pl[0] == '!')) {
          }
          for (auto& ch : pl) {
            if (ch == 'd') ch = 'e';
            if (ch == 'D') ch = 'E';
          }
          std::istringstream ps(pl);
          double x, y, z = 0;
          ps >> x >> y;
          if (ncol == 3) ps >> z;
          e.push_back(x);
          c1.push_back(y);
          c2.push_back(z);
        }
      };
      if (label == "SP" || label == "sp") {
        RawShell s, p;
        std::vector<double> dummy;
        read_prims(3, s.alpha, s.coeff, p.coeff);
        p.alpha = s.alpha;
        s.l = 0; s.pure = false;
        p.l = 1; p.pure = false;
        byZ[Z].push_back(s);
        byZ[Z].push_back(p);
      } else {
        RawShell s;
        s.l = am_letter(label[0]);
        if (s.l < 0) {
          err = "unsupported shell label " + label;
          return false;
        }
        std::vector<double> dummy;
        read_prims(2, s.alpha, s.coeff, dummy);
        s.pure = force_cart_d ? (s.l > 2) : (s.l > 1);
        byZ[Z].push_back(s);
      }
    }
  }
  return true;
}

thread_local std::string g_host_error;

}  // namespace

extern "C" {

int lgx_enforce_unit_normalization(int flag) {
  if (flag >= 0) g_unit_normalization.store(flag != 0);
  return g_unit_normalization.load() ? 1 : 0;
}

lgx_status lgx_shell_normalize(int l, int nprim, const double* alpha,
                               const double* coeff_in, double* coeff_out) {
  if (l < 0 || nprim <= 0 || !alpha || !coeff_in || !coeff_out) return LGX_ERR_INVALID_ARG;
  normalize(l, nprim, alpha, coeff_in, coeff_out);
  return LGX_OK;
}

lgx_status lgx_basis_load(const char* data_dir, const char* name, int natoms,
                          const int32_t* Z, const double* xyz, int* nshell,
                          int* nprim_total, int32_t* l, int32_t* pure,
                          int32_t* nprim, int32_t* atom, double* origins,
                          double* alpha, double* coeff) {
  if (!data_dir || !name || natoms < 0 || !Z || !xyz || !nshell || !nprim_total)
    return LGX_ERR_INVALID_ARG;
  std::string canon(name);
  for (auto& c : canon) c = char(std::tolower(c));
  for (auto& c : canon)
    if (c == '/') c = 'I';
  const bool force_cart_d = cartesian_d(canon);
  std::vector<std::string> comps;
  if (canon.rfind("aug-cc-pv", 0) == 0 && canon.find("cabs") == std::string::npos) {
    comps.push_back(canon.substr(4));
    comps.push_back("augmentation-" + canon.substr(4));
  } else {
    comps.push_back(canon);
  }
  std::vector<std::vector<std::vector<RawShell>>> lib(comps.size());
  for (size_t i = 0; i < comps.size(); ++i) {
    std::string err;
    if (!read_g94(std::string(data_dir) + "/" + comps[i] + ".g94", force_cart_d, lib[i], err)) {
      g_host_error = err;
      return LGX_ERR_INVALID_ARG;
    }
  }
  int ns = 0, np = 0;
  for (int a = 0; a < natoms; ++a) {
    if (Z[a] < 1 || Z[a] > 118) return LGX_ERR_INVALID_ARG;
    for (auto& c : lib)
      for (auto& s : c[Z[a]]) {
        if (l) {
          l[ns] = s.l;
          pure[ns] = s.pure ? 1 : 0;
          nprim[ns] = int(s.alpha.size());
          atom[ns] = a;
          for (int x = 0; x < 3; ++x) origins[3 * ns + x] = xyz[3 * a + x];
          for (size_t p = 0; p < s.alpha.size(); ++p) alpha[np + p] = s.alpha[p];
          normalize(s.l, int(s.alpha.size()), s.alpha.data(), s.coeff.data(), coeff + np);
        }
        ++ns;
        np += int(s.alpha.size());
      }
  }
  *nshell = ns;
  *nprim_total = np;
  return LGX_OK;
}

lgx_status lgx_water_cluster(int nx, int ny, int nz, double spacing, double jitter,
                             uint64_t seed, int32_t* Z, double* xyz) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !Z || !xyz) return LGX_ERR_INVALID_ARG;
  std::mt19937_64 rng(seed);
  auto uni = [&]() { return double(rng() >> 11) * (1.0 / 9007199254740992.0); };
  const double ang2bohr = 1.0 / 0.529177210903;  // CODATA 2018 (atom.h:52-55)
  const double r = 0.96, half = 0.5 * 104.5 * M_PI / 180.0;
  const double h1[3] = {r * std::sin(half), 0.0, r * std::cos(half)};
  const double h2[3] = {-r * std::sin(half), 0.0, r * std::cos(half)};
  int m = 0;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      for (int iz = 0; iz < nz; ++iz, ++m) {
        double O[3] = {ix * spacing, iy * spacing, iz * spacing};
        for (int x = 0; x < 3; ++x) O[x] += (2 * uni() - 1) * jitter;
        // uniform random rotation from a random unit quaternion (Shoemake)
        const double u1 = uni(), u2 = uni(), u3 = uni();
        const double qx = std::sqrt(1 - u1) * std::sin(2 * M_PI * u2);
        const double qy = std::sqrt(1 - u1) * std::cos(2 * M_PI * u2);
        const double qz = std::sqrt(u1) * std::sin(2 * M_PI * u3);
        const double qw = std::sqrt(u1) * std::cos(2 * M_PI * u3);
        const double R[3][3] = {
            {1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)},
            {2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)},
            {2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)}};
        const double* hs[2] = {h1, h2};
        Z[3 * m] = 8;
        Z[3 * m + 1] = 1;
        Z[3 * m + 2] = 1;
        for (int x = 0; x < 3; ++x) xyz[9 * m + x] = O[x] * ang2bohr;
        for (int h = 0; h < 2; ++h)
          for (int x = 0; x < 3; ++x) {
            double v = O[x];
            for (int y = 0; y < 3; ++y) v += R[x][y] * hs[h][y];
            xyz[9 * m + 3 * (h + 1) + x] = v * ang2bohr;
          }
      }
  return LGX_OK;
}

const char* lgx_host_last_error(void) { return g_host_error.c_str(); }

}  // extern "C"
