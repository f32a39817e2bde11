// Test-only CPU interpreter of the per-class programs built by
// libint_gb300/csrc/lgx_program.cpp.  It executes the VRR / accumulate /
// post ops exactly as the warp kernel orders them (level by level) for one
// canonical Cartesian shell quartet and writes the canonical Cartesian shell
// sets, so tests can check the program builder against the oracle without a
// GPU.  Not part of the product.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../libint_gb300/csrc/lgx_program.h"

namespace {
// F_m(T) by the Maclaurin series in long double (test-only, slow and exact).
void boys_series(double T, int mmax, double* F) {
  const long double t = T;
  for (int m = 0; m <= mmax; ++m) {
    long double term = 1.0L / (2 * m + 1), sum = term;
    for (int i = 1; i < 5000; ++i) {
      term *= 2 * t / (2 * m + 2 * i + 1);
      sum += term;
      if (term < sum * 1e-21L) break;
    }
    F[m] = double(expl(-t) * sum);
  }
}
}  // namespace

extern "C" int interp_quartet(const int* l, const int* nprim, const double* alpha,
                              const double* coeff, const double* O, int deriv,
                              double* out) {
  lgx::ClassProgramHost P;
  try {
    P = lgx::build_class_program(l[0], l[1], l[2], l[3], deriv);
  } catch (...) {
    return -1;
  }
  std::vector<double> S(P.total_slots(), 0.0);
  const double* A = O;
  const double* B = O + 3;
  const double* C = O + 6;
  const double* D = O + 9;
  int off[4];
  off[0] = 0;
  for (int k = 1; k < 4; ++k) off[k] = off[k - 1] + nprim[k - 1];
  for (int i = 0; i < P.nacc; ++i) S[i] = 0;
  double AB2 = 0, CD2 = 0;
  for (int x = 0; x < 3; ++x) {
    AB2 += (A[x] - B[x]) * (A[x] - B[x]);
    CD2 += (C[x] - D[x]) * (C[x] - D[x]);
  }
  for (int p0 = 0; p0 < nprim[0]; ++p0)
    for (int p1 = 0; p1 < nprim[1]; ++p1)
      for (int p2 = 0; p2 < nprim[2]; ++p2)
        for (int p3 = 0; p3 < nprim[3]; ++p3) {
          const double a0 = alpha[off[0] + p0], a1 = alpha[off[1] + p1];
          const double a2 = alpha[off[2] + p2], a3 = alpha[off[3] + p3];
          const double z = a0 + a1, e = a2 + a3, g = z + e, rho = z * e / g;
          double P_[3], Q_[3], W[3];
          for (int x = 0; x < 3; ++x) {
            P_[x] = (a0 * A[x] + a1 * B[x]) / z;
            Q_[x] = (a2 * C[x] + a3 * D[x]) / e;
            W[x] = (z * P_[x] + e * Q_[x]) / g;
          }
          double PQ2 = 0;
          for (int x = 0; x < 3; ++x) PQ2 += (P_[x] - Q_[x]) * (P_[x] - Q_[x]);
          const double Kb = 5.9149671727956128778 * std::exp(-a0 * a1 / z * AB2) / z;
          const double Kk = 5.9149671727956128778 * std::exp(-a2 * a3 / e * CD2) / e;
          const double pfac = Kb * Kk / std::sqrt(g) * coeff[off[0] + p0] *
                              coeff[off[1] + p1] * coeff[off[2] + p2] * coeff[off[3] + p3];
          double F[32];
          boys_series(rho * PQ2, P.mmax, F);
          for (int m = 0; m <= P.mmax; ++m) S[P.leaf_slot0 + m] = F[m] * pfac;
          const double PA[3] = {P_[0] - A[0], P_[1] - A[1], P_[2] - A[2]};
          const double WP[3] = {W[0] - P_[0], W[1] - P_[1], W[2] - P_[2]};
          const double QC[3] = {Q_[0] - C[0], Q_[1] - C[1], Q_[2] - C[2]};
          const double WQ[3] = {W[0] - Q_[0], W[1] - Q_[1], W[2] - Q_[2]};
          const double wts[4] = {1.0, 2 * a0, 2 * a1, 2 * a3};
          const int nlev = int(P.vrr_lev.size()) - 1;
          for (int k = 0; k < nlev; ++k) {
            for (int op = P.vrr_lev[k]; op < P.vrr_lev[k + 1]; ++op) {
              const uint32_t* o = &P.vrr_ops[8 * op];
              const unsigned fl = o[6];
              const int dir = (fl >> 1) & 3, n1 = (fl >> 3) & 31, ne = (fl >> 8) & 31;
              const bool onC = fl & 1;
              const double c1 = onC ? QC[dir] : PA[dir], c2 = onC ? WQ[dir] : WP[dir];
              const double c3 = onC ? 0.5 / e : 0.5 / z, c4 = onC ? rho / e : rho / z;
              double v = c1 * S[o[1]] + c2 * S[o[2]];
              if (n1) v += n1 * c3 * (S[o[3]] - c4 * S[o[4]]);
              if (ne) v += ne * 0.5 / g * S[o[5]];
              S[o[0]] = v;
            }
            for (int op = P.acc_lev[k]; op < P.acc_lev[k + 1]; ++op) {
              const unsigned a = P.acc_ops[2 * op], w = P.acc_ops[2 * op + 1];
              S[a] += wts[w >> 30] * S[w & 0x3FFFFFFFu];
            }
          }
        }
  const double ABv[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
  const double CDv[3] = {C[0] - D[0], C[1] - D[1], C[2] - D[2]};
  const int n4 = P.ncart4;
  std::vector<double> Cset(3 * n4, 0.0);
  for (int ph = 0; ph < P.nphases; ++ph) {
    for (int k = P.phase_lev[ph]; k < P.phase_lev[ph + 1]; ++k)
      for (int op = P.post_lev[k]; op < P.post_lev[k + 1]; ++op) {
        const uint32_t* o = &P.post_ops[4 * op];
        const unsigned kind = o[3] & 15;
        const int dir = (o[3] >> 4) & 3, n = (o[3] >> 8) & 31;
        double v;
        if (kind == lgx::kHrrBra) v = S[o[1]] + ABv[dir] * S[o[2]];
        else if (kind == lgx::kHrrKet) v = S[o[1]] + CDv[dir] * S[o[2]];
        else if (kind == lgx::kDeriv) v = S[o[1]] - (n ? n * S[o[2]] : 0.0);
        else v = S[o[1]];
        S[o[0]] = v;
      }
    for (int s = 0; s < P.sets_per_phase; ++s) {
      const double* src = &S[P.cart_out + s * n4];
      if (!deriv) {
        std::memcpy(out, src, n4 * sizeof(double));
      } else {
        const int ctr = ph == 0 ? 0 : (ph == 1 ? 1 : 3);
        std::memcpy(out + size_t(ctr * 3 + s) * n4, src, n4 * sizeof(double));
        for (int i = 0; i < n4; ++i) Cset[s * n4 + i] -= src[i];
      }
    }
  }
  if (deriv)
    for (int s = 0; s < 3; ++s) std::memcpy(out + size_t(6 + s) * n4, &Cset[s * n4], n4 * sizeof(double));
  return n4;
}
