// Boys function evaluators of the register kernels (F_0..F_MMAX at compile-
// time MMAX, times the primitive prefactor), FP64 and FP32.  The program
// kernels' runtime-mmax evaluators are boys_to_stage (lgx_warp.cuh).
#pragma once
#include "lgx_kernels.cuh"

namespace lgx {

// Boys F_0..F_MMAX(T) times the primitive prefactor pfac.
//  T <= kBoysTmax: Taylor expansion about the nearest grid point T_k = k/64
//   of the pre-divided table; every m directly when MMAX <= 2, else the top
//   m plus the downward recursion, with e^{-T} formed as the tabulated
//   e^{-T_k} (slot 7 of the m = 0 row) times the Maclaurin series of
//   e^{T_k - T} (|T_k - T| <= 1/128).
//  T > kBoysTmax (= 50): F_0 = sqrt(pi/T)/2 and the upward recursion
//   F_{m+1} = (2m+1)/(2T) F_m with the e^{-T} terms dropped; the relative
//   error of that, the regularised upper incomplete gamma Q(m+1/2, T), is
//   below 2e-16 for m <= 5 and 1.7e-15 for m = 6 at T = 50.
// FP64 evaluation once the branch and the grid point are chosen: asym
// selects the asymptotic branch; otherwise k is the grid point and md =
// T_k - T.  PF: multiply by pfac (the mixed scheme's FP32 kernels apply
// their prefactor in FP32, so they skip the FP64 products by 1).  NT: terms
// of the Taylor series and of the e^{T_k - T} series (the remainder is below
// |md|^NT/NT! of F_m: 6 terms 3.2e-16 for the FP64 kernels; 4 terms 1.6e-10
// for values that are rounded to FP32 next, whose half-ulp is 6e-8).  R32:
// 1/sqrt(T) of the asymptotic branch by one FP64 Newton step from the FP32
// estimate (relative error ~1.4e-13, again for values rounded to FP32 next)
// instead of the full-precision FP64 rsqrt.
template <int MMAX, bool PF = true, int NT = 6, bool R32 = false>
__device__ __forceinline__ void rk_boys_core(const double* __restrict__ tay, double T, bool asym,
                                             int k, double md, double pfac, double* F) {
  static_assert(NT >= 2 && NT <= 7, "the table holds 7 Taylor coefficients per m");
  static_assert(MMAX <= 6, "asymptotic branch without e^{-T} is exact to 2e-15 only for m <= 6");
  if (asym) {
    double rs;
    if constexpr (R32) {
      const double r0 = f2d_int(rsqrtf(d2f_int(T)));  // relative error <= ~3e-7
      rs = fma(0.5 * r0, fma(-(T * r0), r0, 1.0), r0);
    } else {
      rs = rsqrt(T);
    }
    const double oo2T = 0.5 * (rs * rs);
    double f = PF ? (0.88622692545275801365 * pfac) * rs : 0.88622692545275801365 * rs;
    F[0] = f;
#pragma unroll
    for (int m = 0; m < MMAX; ++m) {
      f *= (2 * m + 1) * oo2T;
      F[m + 1] = f;
    }
    return;
  }
  const double* row = tay + (k * (kBoysMaxM + 1)) * kBoysTaylorStride;
  if (MMAX <= 2) {
#pragma unroll
    for (int m = 0; m <= MMAX; ++m) {
      const double* c = row + m * kBoysTaylorStride;
      double s = __ldg(c + NT - 1);
#pragma unroll
      for (int i = NT - 2; i >= 0; --i) s = fma(s, md, __ldg(c + i));
      F[m] = PF ? s * pfac : s;
    }
  } else {
    const double* c = row + MMAX * kBoysTaylorStride;
    double s = __ldg(c + NT - 1);
#pragma unroll
    for (int i = NT - 2; i >= 0; --i) s = fma(s, md, __ldg(c + i));
    if (PF) s *= pfac;
    F[MMAX] = s;
    // e^{md} = sum_{i < NT} md^i / i!, Horner from the top term
    constexpr double inv_fact[7] = {1.0, 1.0, 0.5, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0,
                                    1.0 / 720.0};
    double e = inv_fact[NT - 1];
#pragma unroll
    for (int i = NT - 2; i >= 0; --i) e = fma(e, md, inv_fact[i]);
    const double eTp = PF ? (__ldg(row + 7) * pfac) * e : __ldg(row + 7) * e;  // pfac e^{-T}
    const double twoT = 2.0 * T;
#pragma unroll
    for (int m = MMAX - 1; m >= 0; --m) {
      s = fma(twoT, s, eTp) * (1.0 / (2 * m + 1));
      F[m] = s;
    }
  }
}

template <int MMAX>
__device__ __forceinline__ void rk_boys(const double* __restrict__ tay, double T, double pfac,
                                        double* F) {
  // nearest grid point: adding 1.5*2^52 rounds T*32 to an integer held in
  // the low mantissa bits (read back with an integer move)
  const double t32 = fma(T, kBoysInvDT, 6755399441055744.0);
  const int k = __double2loint(t32);
  const double md = fma(t32 - 6755399441055744.0, kBoysDT, -T);  // = -(T - T_k)
  rk_boys_core<MMAX>(tay, T, T > kBoysTmax, k, md, pfac, F);
}

// The mixed scheme's FP64 Boys function of an FP32 quartet, given its
// argument T = T.hi + T.lo in double-float (ds_boys_arg): the branch and the
// grid point come from T.hi; the offset md = T_k - T = (T_k - T.hi) - T.lo,
// where T_k - T.hi is exact in FP32 (T_k = k/64 and T.hi are within a
// factor 2 of each other for k >= 1, Sterbenz; 0 - T.hi for k = 0), both
// parts converted to FP64 with integer operations and subtracted in FP64;
// T itself in FP64 (one addition) for the asymptotic branch and the
// recursion.  T.hi <= 50 gives k <= 3200 < kBoysRows, and near T = 50 either
// branch is exact (the asymptotic one drops Q(m+1/2, T) < 2e-15).  The
// values are rounded to FP32 next, so the series stop at 4 terms: relative
// error below 1.6e-10 (|md| <= 1/128), 400 times under the FP32 half-ulp.
template <int MMAX>
__device__ __forceinline__ void rk_boys_b64(const double* __restrict__ tay, dsf T, double* F) {
  const bool asym = T.hi > float(kBoysTmax);
  const int k = asym ? 0 : __float2int_rn(T.hi * float(kBoysInvDT));
  const float mdh = __fadd_rn(__fmul_rn(float(k), float(kBoysDT)), -T.hi);
  const double md = f2d_int(mdh) - f2d_int(T.lo);
  if (MMAX <= 2 && !asym) {  // direct Taylor series: T itself is not needed
    rk_boys_core<MMAX, false, 4>(tay, 0.0, false, k, md, 1.0, F);
    return;
  }
  const double T64 = f2d_int(T.hi) + f2d_int(T.lo);
  rk_boys_core<MMAX, false, 4, true>(tay, T64, asym, k, md, 1.0, F);
}

template <int MMAX>
__device__ __forceinline__ void rk_boys(const float* __restrict__ tab, float T, float pfac,
                                        float* F) {
  if (T > float(kBoysTmax)) {
    const float rs = rsqrtf(T);
    const float oo2T = 0.5f * (rs * rs);
    float f = (0.886226925f * pfac) * rs;
    F[0] = f;
#pragma unroll
    for (int m = 0; m < MMAX; ++m) {
      f *= (2 * m + 1) * oo2T;  // e^{-T} < 2e-22 is below FP32 resolution
      F[m + 1] = f;
    }
    return;
  }
  const int k = __float2int_rn(T * float(kBoysInvDT));
  const float d = T - k * float(kBoysDT);
  const float* row = tab + k * kBoysCols;
  const float c3 = -d * (1.0f / 3.0f), c2 = -d * 0.5f, c1 = -d;
  float s = __ldg(row + MMAX + 3);
  s = fmaf(s, c3, __ldg(row + MMAX + 2));
  s = fmaf(s, c2, __ldg(row + MMAX + 1));
  s = fmaf(s, c1, __ldg(row + MMAX));
  s *= pfac;
  F[MMAX] = s;
  if (MMAX > 0) {
    const float eTp = __expf(-T) * pfac;
    const float twoT = 2.0f * T;
#pragma unroll
    for (int m = MMAX - 1; m >= 0; --m) {
      s = fmaf(twoT, s, eTp) * (1.0f / (2 * m + 1));
      F[m] = s;
    }
  }
}

}  // namespace lgx
