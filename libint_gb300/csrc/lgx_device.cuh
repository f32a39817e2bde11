// Device-side data structures and the Boys function of the ERI kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lgx {

// ------------------------------------------------------------------ Boys
// F_m(T) = int_0^1 u^{2m} exp(-T u^2) du.
// For T <= kBoysTmax: F_mmax by a 7-term Taylor expansion about the nearest
// grid point T_k = k/32 of a table of F_0..F_{kBoysCols-1}(T_k), then the
// stable downward recursion F_m = (2T F_{m+1} + e^{-T})/(2m+1).
// For T > kBoysTmax: F_0 = sqrt(pi/T)/2 (erf(sqrt T) == 1 to double there)
// and the upward recursion F_{m+1} = ((2m+1) F_m - e^{-T})/(2T), stable for
// 2T > 2m+1.  This is the scheme of libint's FmEval_Taylor
// (include/libint2/boys.h:519-879); the table is generated on the host from
// the Maclaurin series in extended precision.
constexpr double kBoysInvDT = 32.0;
constexpr double kBoysDT = 1.0 / 32.0;
constexpr double kBoysTmax = 33.0;
constexpr int kBoysTerms = 7;
constexpr int kBoysMaxM = 16;                         // largest mmax served
constexpr int kBoysCols = kBoysMaxM + kBoysTerms;     // 23 columns
constexpr int kBoysRows = int(kBoysTmax * 32.0) + 2;  // 1058 grid points

// Device pointer to the [kBoysRows][kBoysCols] table (set per context).
struct BoysTable {
  const double* F;
};

__device__ __forceinline__ void boys_eval(const double* __restrict__ tab,
                                          double T, int mmax,
                                          double* __restrict__ F,
                                          int stride) {
  if (T > kBoysTmax) {
    const double eT = exp(-T);
    const double rT = 1.0 / T;
    double f = 0.88622692545275801365 * sqrt(rT);
    F[0] = f;
    const double oo2T = 0.5 * rT;
    for (int m = 0; m < mmax; ++m) {
      f = ((2 * m + 1) * f - eT) * oo2T;
      F[(m + 1) * stride] = f;
    }
    return;
  }
  const int k = __double2int_rn(T * kBoysInvDT);
  const double d = T - k * kBoysDT;
  const double* row = tab + k * kBoysCols + mmax;
  // sum_{i<7} F_{mmax+i}(T_k) (-d)^i / i!   (Horner)
  double s = __ldg(row + 6);
  s = fma(s, -d * (1.0 / 6.0), __ldg(row + 5));
  s = fma(s, -d * (1.0 / 5.0), __ldg(row + 4));
  s = fma(s, -d * (1.0 / 4.0), __ldg(row + 3));
  s = fma(s, -d * (1.0 / 3.0), __ldg(row + 2));
  s = fma(s, -d * (1.0 / 2.0), __ldg(row + 1));
  s = fma(s, -d, __ldg(row + 0));
  F[mmax * stride] = s;
  if (mmax > 0) {
    const double eT = exp(-T);
    const double twoT = 2.0 * T;
    for (int m = mmax - 1; m >= 0; --m) {
      s = fma(twoT, s, eT) * (1.0 / (2 * m + 1));
      F[m * stride] = s;
    }
  }
}

// ------------------------------------------------------------ basis data
struct DevBasis {
  int nshell;
  const int* l;
  const int* pure;
  const int* nprim;
  const int* prim_off;
  const int* bf_off;
  const int* atom;
  const double* O;      // [3*nshell]
  const double* alpha;  // flattened
  const double* coeff;  // flattened, normalization embedded
};

// One primitive pair of a shell pair (s1, s2) as stored (s1 = first shell),
// with FP64 fields for the FP64 kernels and FP32 copies (centre-relative
// P, so FP32 P-Q differences keep their precision) for the FP32 kernels.
struct __align__(16) PrimPairRec {
  double P[3];
  double Kc;      // sqrt(2) pi^{5/4} exp(-rho AB^2)/gamma * c1 * c2
  double oog;     // 1/(alpha1 + alpha2)
  double ln_scr;  // ln of the pair screening factor (shell.h:1041-1059)
  double nonsph;  // Conservative screening factor
  double a1, a2;  // exponents of s1 and s2
  float fKc, fzeta, foog, fln_scr;
  float fPA1[3];  // P - O(s1)
  float fPA2[3];  // P - O(s2)
  float fa1, fa2;
  float pad[2];
};
static_assert(sizeof(PrimPairRec) == 128, "PrimPairRec layout");

// A shell pair with its primitive-pair range (pair list, shell.h:1079-1329).
struct PairRec {
  int s1, s2;       // shell indices as stored
  int pp_off, npp;  // primitive pairs [pp_off, pp_off + npp)
};

// Class program (see lgx_program.h) in device memory.
struct DevProg {
  int la, lb, lc, ld, deriv, mmax;
  int nacc, nwork, leaf_slot0;
  int nphases, sets_per_phase, ncart4, cart_out, cbuf, sph_tmp;
  int nlev, npost_lev;
  const int* vrr_lev;
  const int* acc_lev;
  const uint4* vrr_ops;  // 2 uint4 per op
  const uint2* acc_ops;
  const int* post_lev;
  const int* phase_lev;
  const uint4* post_ops;
};

// Spherical-harmonic coefficient tables, dense [l][2l+1][ncart(l)], l <= 3.
struct SphTables {
  const double* coef;  // offsets: l=0 at 0, l=1 at 1, l=2 at 1+9, l=3 at 1+9+30
};
__host__ __device__ inline int sph_off(int l) {
  return l == 0 ? 0 : (l == 1 ? 1 : (l == 2 ? 10 : 40));
}
__host__ __device__ inline int ncart_of(int l) { return (l + 1) * (l + 2) / 2; }

}  // namespace lgx
