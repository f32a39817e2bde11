// Warp-cooperative Coulomb ERI kernel for sm_103a (the "program kernel"),
// included by lgx_kernels.cu (generic instances) and the generated units
// that pair it with unrolled per-class HRR / solid-harmonic stages.
//
// One warp owns one contracted shell quartet at a time (the helpers of steps
// 2-4 are also instantiated for a whole block, for the single-quartet
// kernels of lgx_kernels.cu):
//  1. primitive-quartet prologue, one primitive quartet per lane: libint's
//     screening (engine.impl.h:1313-1386), pfac, T, the Boys function and
//     the VRR geometric factors (engine.impl.h:1389-1757); survivors are
//     compacted with a ballot into a per-warp staging area.  FP32 kernels
//     evaluate it from the FP32 pair data (no FP64 instruction);
//  2. for each surviving primitive quartet the 32 lanes execute the class's
//     VRR program level by level (all ops of a level are independent) and
//     add the (e0|f0) targets into contracted accumulators (HGP contraction
//     point, src/bin/libint/dg.cc:1177-1189);
//  3. the post program (HRR, derivative rule) produces Cartesian shell sets;
//  4. a sparse Cartesian -> solid-harmonic transform per index
//     (engine.impl.h:1965-1985) and the mode-specific epilogue: libint-order
//     store with un-permutation (engine.impl.h:1988-2086), Schwarz maximum,
//     J/K digestion (hartree-fock++.cc:1709-1743) or gradient digestion
//     (hartree-fock++.cc:1909-1973).
// Integer recurrence factors are turned into T with integer operations
// (i2d_int) and FP32 sums into FP64 with f2d_int, so the FP64 pipe only
// carries FP64 arithmetic.  Slots live in shared memory when the class
// fits, else in a per-warp slice of global scratch (L1/L2 resident).  Work
// is pulled in chunks from a device counter; every loop is bounded.
#pragma once
#include "lgx_kernels.cuh"

namespace lgx {

// Per-warp table of the integer-weighted recurrence factors of the current
// primitive quartet: k/(2 zeta), k/(2 eta), k/(2(zeta+eta)) for k = 0..7.
constexpr int kKtab = 24;


template <typename T>
__device__ __forceinline__ T small_int(int n);
template <>
__device__ __forceinline__ double small_int<double>(int n) { return i2d_int(n); }
template <>
__device__ __forceinline__ float small_int<float>(int n) { return float(n); }

// An FP64 Boys value times the prefactor, as staged: FP64, or (the mixed
// scheme's FP32 kernels) rounded to FP32 first with integer operations.
__device__ __forceinline__ double boys_out(double f, double pfac) { return f * pfac; }
__device__ __forceinline__ float boys_out(double f, float pfac) { return d2f_int(f) * pfac; }

// FP64 Boys F_0..F_mmax(T) * pfac into F (runtime mmax); TO = double for the
// FP64 kernels, float for the FP32 kernels with the Boys function in FP64.
template <typename TO>
__device__ __forceinline__ void boys_to_stage(const double* __restrict__ tab,
                                              const double* __restrict__ inv_odd, double T,
                                              int mmax, TO pfac, TO* __restrict__ F) {
  if (T > kBoysTmax) {
    const double eT = exp(-T);
    const double rs = rsqrt(T);
    double f = 0.88622692545275801365 * rs;
    F[0] = boys_out(f, pfac);
    const double oo2T = 0.5 * (rs * rs);
    for (int m = 0; m < mmax; ++m) {
      f = ((2 * m + 1) * f - eT) * oo2T;
      F[m + 1] = boys_out(f, pfac);
    }
    return;
  }
  const int k = __double2int_rn(T * kBoysInvDT);
  const double d = T - k * kBoysDT;
  const double* row = tab + k * kBoysCols + mmax;
  double s = __ldg(row + 6);
  s = fma(s, -d * (1.0 / 6.0), __ldg(row + 5));
  s = fma(s, -d * (1.0 / 5.0), __ldg(row + 4));
  s = fma(s, -d * (1.0 / 4.0), __ldg(row + 3));
  s = fma(s, -d * (1.0 / 3.0), __ldg(row + 2));
  s = fma(s, -d * (1.0 / 2.0), __ldg(row + 1));
  s = fma(s, -d, __ldg(row + 0));
  F[mmax] = boys_out(s, pfac);
  if (mmax > 0) {
    const double eT = exp(-T);
    const double twoT = 2.0 * T;
    for (int m = mmax - 1; m >= 0; --m) {
      s = fma(twoT, s, eT) * __ldg(inv_odd + m);
      F[m] = boys_out(s, pfac);
    }
  }
}

// The mixed scheme's FP64 Boys function for the program kernels' FP32
// quartets (runtime mmax <= kBoysMaxM), from the double-float argument
// T = T.hi + T.lo (ds_boys_arg) and rounded to FP32 with integer operations,
// times the FP32 prefactor.  T <= 50: F_mmax by the 4-term Taylor series of
// the pre-divided table (the register kernels' rows) about T_k, e^{-T} as
// e^{-T_k} (the table's spare slot) times the 4-term series of e^{T_k - T},
// the downward recursion in FP64; relative error below 1.6e-10 before the
// rounding (|T_k - T| <= 1/128), with md = (T_k - T.hi) - T.lo exact in FP32
// for its first part (Sterbenz).  T > 50: F_0 = sqrt(pi/T)/2 and the upward
// recursion with its e^{-T} terms (they reach ~3e-8 of F_16 at T = 50).
__device__ __forceinline__ void boys_b64_stage(const double* __restrict__ tay,
                                               const double* __restrict__ inv_odd, dsf T,
                                               int mmax, float pfac, float* __restrict__ F) {
  const double T64 = f2d_int(T.hi) + f2d_int(T.lo);
  if (T.hi > float(kBoysTmax)) {
    const double eT = exp(-T64);
    // 1/sqrt(T): one FP64 Newton step from the FP32 estimate (~1.4e-13)
    const double r0 = f2d_int(rsqrtf(T.hi));
    const double rs = fma(0.5 * r0, fma(-(T64 * r0), r0, 1.0), r0);
    double f = 0.88622692545275801365 * rs;
    F[0] = d2f_int(f) * pfac;
    const double oo2T = 0.5 * (rs * rs);
    for (int m = 0; m < mmax; ++m) {
      f = ((2 * m + 1) * f - eT) * oo2T;
      F[m + 1] = d2f_int(f) * pfac;
    }
    return;
  }
  const int k = __float2int_rn(T.hi * float(kBoysInvDT));
  const float mdh = __fadd_rn(__fmul_rn(float(k), float(kBoysDT)), -T.hi);
  const double md = f2d_int(mdh) - f2d_int(T.lo);
  const double* row = tay + size_t(k) * (kBoysMaxM + 1) * kBoysTaylorStride;
  const double* c = row + mmax * kBoysTaylorStride;
  double s = __ldg(c + 3);
  s = fma(s, md, __ldg(c + 2));
  s = fma(s, md, __ldg(c + 1));
  s = fma(s, md, __ldg(c + 0));
  F[mmax] = d2f_int(s) * pfac;
  if (mmax > 0) {
    double e = 1.0 / 6.0;
    e = fma(e, md, 0.5);
    e = fma(e, md, 1.0);
    e = fma(e, md, 1.0);
    const double eT = __ldg(row + 7) * e;  // e^{-T_k} e^{T_k - T}
    const double twoT = 2.0 * T64;
    for (int m = mmax - 1; m >= 0; --m) {
      s = fma(twoT, s, eT) * __ldg(inv_odd + m);
      F[m] = d2f_int(s) * pfac;
    }
  }
}

// FP32 Boys (4-term Taylor on the same grid, FP32 recursion).
__device__ __forceinline__ void boys_to_stage(const float* __restrict__ tab, float T, int mmax,
                                              float pfac, float* __restrict__ F) {
  if (T > float(kBoysTmax)) {
    const float rs = rsqrtf(T);
    const float oo2T = 0.5f * (rs * rs);
    float f = 0.886226925f * rs;
    F[0] = f * pfac;
    for (int m = 0; m < mmax; ++m) {
      f = (2 * m + 1) * f * oo2T;
      F[m + 1] = f * pfac;
    }
    return;
  }
  const int k = __float2int_rn(T * float(kBoysInvDT));
  const float d = T - k * float(kBoysDT);
  const float* row = tab + k * kBoysCols + mmax;
  float s = __ldg(row + 3);
  s = fmaf(s, -d * (1.0f / 3.0f), __ldg(row + 2));
  s = fmaf(s, -d * 0.5f, __ldg(row + 1));
  s = fmaf(s, -d, __ldg(row + 0));
  F[mmax] = s * pfac;
  if (mmax > 0) {
    const float eT = __expf(-T);
    const float twoT = 2.0f * T;
    for (int m = mmax - 1; m >= 0; --m) {
      s = fmaf(twoT, s, eT) * (1.0f / (2 * m + 1));
      F[m] = s * pfac;
    }
  }
}

// Core integrals of the attenuated operators (libint's erf_coulomb_gm_eval
// and erfc_coulomb_gm_eval, include/libint2/boys.h:1913-1980): with
// s = omega^2 / (omega^2 + rho),
//   erf(omega r)/r :  G_m = s^{m+1/2} F_m(s T)
//   erfc(omega r)/r:  G_m = F_m(T) - s^{m+1/2} F_m(s T)
// (dG_m/dT = -G_{m+1} as for F_m, so the recurrences are unchanged).
// F holds F_m(T) * pfac for op 0 on entry; G[] is scratch of mmax+1 values.
template <typename T>
__device__ __forceinline__ void attenuate(const EriArgs& a, T Tval, T rho, int mmax, T pfac,
                                          T* __restrict__ F);
template <>
__device__ __forceinline__ void attenuate<double>(const EriArgs& a, double Tval, double rho,
                                                  int mmax, double pfac,
                                                  double* __restrict__ F) {
  if (a.op == 1 && !(a.omega2 > 0.0)) {
    for (int m = 0; m <= mmax; ++m) F[m] = 0.0;
    return;
  }
  if (a.op == 2 && !(a.omega2 > 0.0)) return;  // erfc(0) = 1: plain Coulomb
  const double s = a.omega2 / (a.omega2 + rho);
  double G[kBoysMaxM + 1];
  boys_to_stage(a.boys, a.inv_odd, Tval * s, mmax, pfac, G);
  double f = sqrt(s);
  for (int m = 0; m <= mmax; ++m, f *= s) F[m] = a.op == 1 ? f * G[m] : F[m] - f * G[m];
}
template <>
__device__ __forceinline__ void attenuate<float>(const EriArgs& a, float Tval, float rho, int mmax,
                                                 float pfac, float* __restrict__ F) {
  if (a.op == 1 && !(a.omega2 > 0.0)) {
    for (int m = 0; m <= mmax; ++m) F[m] = 0.0f;
    return;
  }
  if (a.op == 2 && !(a.omega2 > 0.0)) return;
  const float w2 = float(a.omega2);
  const float s = w2 / (w2 + rho);
  float G[kBoysMaxM + 1];
  boys_to_stage(a.boys32, Tval * s, mmax, pfac, G);
  float f = sqrtf(s);
  for (int m = 0; m <= mmax; ++m, f *= s) F[m] = a.op == 1 ? f * G[m] : F[m] - f * G[m];
}

// Quartet geometry in the kernel's precision.  FP32 differences come from
// the hi/lo float centres, so they keep FP32 relative precision.
template <typename T>
struct QuartetGeom {
  int sh[4];  // canonical shells bra1 bra2 ket1 ket2
  int bra_pp, ket_pp, nbpp, nkpp;
  bool bra_sw, ket_sw;
  T A[3], C[3];  // FP64 kernels: absolute centres of bra1 / ket1
  T AB[3], CD[3], AC[3];
  PrimScreen scr;  // primitive-screening thresholds of the quartet
};

template <typename T>
__device__ __forceinline__ void load_geom(const EriArgs& a, int bpair, int kpair, bool bsw,
                                          bool ksw, QuartetGeom<T>& g) {
  const PairRec bp = a.pairs[bpair];
  const PairRec kp = a.pairs[kpair];
  g.sh[0] = bsw ? bp.s2 : bp.s1;
  g.sh[1] = bsw ? bp.s1 : bp.s2;
  g.sh[2] = ksw ? kp.s2 : kp.s1;
  g.sh[3] = ksw ? kp.s1 : kp.s2;
  g.bra_pp = bp.pp_off;
  g.nbpp = bp.npp;
  g.ket_pp = kp.pp_off;
  g.nkpp = kp.npp;
  g.bra_sw = bsw;
  g.ket_sw = ksw;
  g.scr.prec = a.precision;
  g.scr.ln_prec = a.ln_prec;
  g.scr.fprec = a.fprecision;
  g.scr.fln_prec = a.fln_prec;
  if constexpr (sizeof(T) == 8) {
    for (int x = 0; x < 3; ++x) {
      const double A = a.basis.O[3 * g.sh[0] + x], B = a.basis.O[3 * g.sh[1] + x];
      const double C = a.basis.O[3 * g.sh[2] + x], D = a.basis.O[3 * g.sh[3] + x];
      g.A[x] = A;
      g.C[x] = C;
      g.AB[x] = A - B;
      g.CD[x] = C - D;
      g.AC[x] = A - C;
    }
  } else {
    const float* hi = a.basis.Ohi;
    const float* lo = a.basis.Olo;
    for (int x = 0; x < 3; ++x) {
      const int i0 = 3 * g.sh[0] + x, i1 = 3 * g.sh[1] + x, i2 = 3 * g.sh[2] + x,
                i3 = 3 * g.sh[3] + x;
      g.A[x] = hi[i0];
      g.C[x] = hi[i2];
      g.AB[x] = (hi[i0] - hi[i1]) + (lo[i0] - lo[i1]);
      g.CD[x] = (hi[i2] - hi[i3]) + (lo[i2] - lo[i3]);
      g.AC[x] = (hi[i0] - hi[i2]) + (lo[i0] - lo[i2]);
    }
  }
}

template <typename T>
__device__ __forceinline__ T sel3(int d, T x, T y, T z) {
  return d == 0 ? x : (d == 1 ? y : z);
}

// Prologue of one primitive quartet into the staging row st (kStage values
// of T).  Returns false if screened out.
// ATT: instantiation for the attenuated operators (a.op = erf / erfc); the
// Coulomb instantiations carry none of that code.
template <bool ATT, bool B64 = false>
__device__ __forceinline__ bool prologue(const EriArgs& a, const QuartetGeom<double>& g, int idx,
                                         double npbraket, double* st) {
  const int ib = idx / g.nkpp, ik = idx - ib * g.nkpp;
  const PrimPairRec& bp = a.pprims[g.bra_pp + ib];
  const PrimPairRec& kp = a.pprims[g.ket_pp + ik];
  if (!ln_kept(a, bp.fln_scr + kp.fln_scr, g.bra_pp + ib, g.ket_pp + ik, g.scr)) return false;
  const double zeta = bp.zeta, eta = kp.zeta;
  const double gpq = zeta + eta;
  const double rs = rsqrt(gpq);
  const double oogpq = rs * rs;
  const double pfac = bp.Kc * kp.Kc * rs;
  double mag = fabs(pfac);
  if (a.screening == 1) mag *= fmax(1.0, double(bp.fnonsph) * double(kp.fnonsph)) * npbraket;
  if (mag < g.scr.prec) return false;
  const double PQx = bp.P[0] - kp.P[0], PQy = bp.P[1] - kp.P[1], PQz = bp.P[2] - kp.P[2];
  const double rho = zeta * eta * oogpq;
  const double T = rho * fma(PQx, PQx, fma(PQy, PQy, PQz * PQz));
  if constexpr (ATT) {
    if (a.op != 1) boys_to_stage(a.boys, a.inv_odd, T, a.prog.mmax, pfac, st + kStF);
    attenuate<double>(a, T, rho, a.prog.mmax, pfac, st + kStF);
  } else {
    boys_to_stage(a.boys, a.inv_odd, T, a.prog.mmax, pfac, st + kStF);
  }
  const double ez = eta * oogpq, zz = zeta * oogpq;
  st[kStPA + 0] = bp.P[0] - g.A[0];
  st[kStPA + 1] = bp.P[1] - g.A[1];
  st[kStPA + 2] = bp.P[2] - g.A[2];
  st[kStQC + 0] = kp.P[0] - g.C[0];
  st[kStQC + 1] = kp.P[1] - g.C[1];
  st[kStQC + 2] = kp.P[2] - g.C[2];
  st[kStWP + 0] = -ez * PQx;
  st[kStWP + 1] = -ez * PQy;
  st[kStWP + 2] = -ez * PQz;
  st[kStWQ + 0] = zz * PQx;
  st[kStWQ + 1] = zz * PQy;
  st[kStWQ + 2] = zz * PQz;
  st[kStOo2z] = 0.5 * bp.oog;
  st[kStRoz] = ez;
  st[kStOo2e] = 0.5 * kp.oog;
  st[kStRoe] = zz;
  st[kStOo2ze] = 0.5 * oogpq;
  st[kStW + 0] = 2.0 * (g.bra_sw ? bp.a2 : bp.a1);
  st[kStW + 1] = 2.0 * (g.bra_sw ? bp.a1 : bp.a2);
  st[kStW + 2] = 2.0 * (g.ket_sw ? kp.a1 : kp.a2);
  return true;
}

// B64: the mixed scheme's Boys function in FP64 (kModeJKB64 /
// kModeStoreB64): T = rho |P - Q|^2 in double-float arithmetic from the
// primitive pairs' double-float records (ds_boys_arg, relative error
// ~1e-13) and F_m(T) from the FP64 evaluator (boys_b64_stage), rounded to
// FP32.
template <bool ATT, bool B64 = false>
__device__ __forceinline__ bool prologue(const EriArgs& a, const QuartetGeom<float>& g, int idx,
                                         double npbraket, float* st) {
  const int ib = idx / g.nkpp, ik = idx - ib * g.nkpp;
  const PrimPairRec& bp = a.pprims[g.bra_pp + ib];
  const PrimPairRec& kp = a.pprims[g.ket_pp + ik];
  if (!ln_kept(a, bp.fln_scr + kp.fln_scr, g.bra_pp + ib, g.ket_pp + ik, g.scr)) return false;
  const float zeta = bp.fzeta, eta = kp.fzeta;
  const float gpq = zeta + eta;
  const float rs = rsqrtf(gpq);
  const float oogpq = rs * rs;
  const float pfac = bp.fKc * kp.fKc * rs;
  const double scale =
      a.screening == 1 ? fmax(1.0, double(bp.fnonsph) * double(kp.fnonsph)) * npbraket : 1.0;
  if (!pf_kept(a, fabsf(pfac) * float(scale), scale, g.bra_pp + ib, g.ket_pp + ik, g.scr))
    return false;
  const float* PA = g.bra_sw ? bp.fPA2 : bp.fPA1;
  const float* QC = g.ket_sw ? kp.fPA2 : kp.fPA1;
  const float PQx = PA[0] - QC[0] + g.AC[0], PQy = PA[1] - QC[1] + g.AC[1],
              PQz = PA[2] - QC[2] + g.AC[2];
  const float rho = zeta * eta * oogpq;
  const float T = rho * fmaf(PQx, PQx, fmaf(PQy, PQy, PQz * PQz));
  if constexpr (B64) {
    const PrimPairJKds* bd = a.ppds + g.bra_pp + ib;
    const PrimPairJKds* kd = a.ppds + g.ket_pp + ik;
    const dsf T64 = ds_boys_arg(__ldg(&bd->hi), __ldg(&bd->lo), __ldg(&kd->hi), __ldg(&kd->lo),
                                rho, oogpq);
    boys_b64_stage(a.boys_tay, a.inv_odd, T64, a.prog.mmax, pfac, st + kStF);
  } else if constexpr (ATT) {
    if (a.op != 1) boys_to_stage(a.boys32, T, a.prog.mmax, pfac, st + kStF);
    attenuate<float>(a, T, rho, a.prog.mmax, pfac, st + kStF);
  } else {
    boys_to_stage(a.boys32, T, a.prog.mmax, pfac, st + kStF);
  }
  const float ez = eta * oogpq, zz = zeta * oogpq;
  st[kStPA + 0] = PA[0];
  st[kStPA + 1] = PA[1];
  st[kStPA + 2] = PA[2];
  st[kStQC + 0] = QC[0];
  st[kStQC + 1] = QC[1];
  st[kStQC + 2] = QC[2];
  st[kStWP + 0] = -ez * PQx;
  st[kStWP + 1] = -ez * PQy;
  st[kStWP + 2] = -ez * PQz;
  st[kStWQ + 0] = zz * PQx;
  st[kStWQ + 1] = zz * PQy;
  st[kStWQ + 2] = zz * PQz;
  st[kStOo2z] = 0.5f * bp.foog;
  st[kStRoz] = ez;
  st[kStOo2e] = 0.5f * kp.foog;
  st[kStRoe] = zz;
  st[kStOo2ze] = 0.5f * oogpq;
  st[kStW + 0] = 2.0f * (g.bra_sw ? bp.fa2 : bp.fa1);
  st[kStW + 1] = 2.0f * (g.bra_sw ? bp.fa1 : bp.fa2);
  st[kStW + 2] = 2.0f * (g.ket_sw ? kp.fa1 : kp.fa2);
  return true;
}

struct VrrOp {
  unsigned d, s1, s2, s3, s4, s5, fl;
};
__device__ __forceinline__ VrrOp load_vrr_op(const DevProg& P, int op) {
  VrrOp o;
  if (P.compact) {
    const uint4 w = __ldg(P.vrr_ops + op);
    o.d = w.x & 0xFFFFu; o.s1 = w.x >> 16;
    o.s2 = w.y & 0xFFFFu; o.s3 = w.y >> 16;
    o.s4 = w.z & 0xFFFFu; o.s5 = w.z >> 16;
    o.fl = w.w;
  } else {
    const uint4 u = __ldg(P.vrr_ops + 2 * op);
    const uint4 v = __ldg(P.vrr_ops + 2 * op + 1);
    o.d = u.x; o.s1 = u.y; o.s2 = u.z; o.s3 = u.w;
    o.s4 = v.x; o.s5 = v.y; o.fl = v.z;
  }
  return o;
}

struct PostOp {
  unsigned d, s1, s2, w;
};
__device__ __forceinline__ PostOp load_post_op(const DevProg& P, int op) {
  PostOp o;
  if (P.compact) {
    const uint2 w = __ldg(P.post_ops_c + op);
    o.d = w.x & 0xFFFFu; o.s1 = w.x >> 16;
    o.s2 = w.y & 0xFFFFu; o.w = w.y >> 16;
  } else {
    const uint4 u = __ldg(P.post_ops + op);
    o.d = u.x; o.s1 = u.y; o.s2 = u.z; o.w = u.w;
  }
  return o;
}

// Thread-group policies of the program-execution helpers below: one warp
// (the program kernel runs a quartet per warp) or the whole block (the
// single-quartet kernels of short explicit lists and caller-supplied
// primitive data, which spread one quartet's program levels over all the
// block's threads).  `lane` is the thread's rank in the group.
struct WarpGrp {
  static __device__ __forceinline__ constexpr int size() { return 32; }
  static __device__ __forceinline__ void sync() { __syncwarp(); }
};
struct BlockGrp {
  static __device__ __forceinline__ int size() { return int(blockDim.x); }
  static __device__ __forceinline__ void sync() { __syncthreads(); }
};

// Step 2 for the staged primitive quartets of `ballot` (rows of `stage`):
// the class's VRR program, level by level, and the accumulation of its
// (e0|f0) targets into the contracted slots.
template <typename T, class Grp = WarpGrp>
__device__ __forceinline__ void vrr_consume(const DevProg& P, const T* __restrict__ stage,
                                            unsigned ballot, T* __restrict__ slots,
                                            T* __restrict__ ktab, int lane) {
  while (ballot) {
    const T* st = stage + (__ffs(ballot) - 1) * kStage;
    ballot &= ballot - 1u;
    const T PAx = st[kStPA], PAy = st[kStPA + 1], PAz = st[kStPA + 2];
    const T WPx = st[kStWP], WPy = st[kStWP + 1], WPz = st[kStWP + 2];
    const T QCx = st[kStQC], QCy = st[kStQC + 1], QCz = st[kStQC + 2];
    const T WQx = st[kStWQ], WQy = st[kStWQ + 1], WQz = st[kStWQ + 2];
    const T oo2z = st[kStOo2z], roz = st[kStRoz];
    const T oo2e = st[kStOo2e], roe = st[kStRoe];
    const T oo2ze = st[kStOo2ze];
    const T w1 = st[kStW], w2 = st[kStW + 1], w3 = st[kStW + 2];
    for (int m = lane; m <= P.mmax; m += Grp::size()) slots[P.leaf_slot0 + m] = st[kStF + m];
    if (lane < kKtab)
      ktab[lane] = small_int<T>(lane & 7) * (lane < 8 ? oo2z : (lane < 16 ? oo2e : oo2ze));
    Grp::sync();
    // one VRR op: slots[d] = c1*s1 + c2*s2 [+ k1*(s3 - c4*s4)] [+ k5*s5]
    auto eval = [&](const VrrOp& o) -> T {
      const unsigned fl = o.fl;
      const int dir = (fl >> 1) & 3;
      const int n1 = (fl >> 3) & 31;
      const int ne = (fl >> 8) & 31;
      T c1, c2, c4;
      if ((fl & 1u) == 0) {
        c1 = sel3(dir, PAx, PAy, PAz);
        c2 = sel3(dir, WPx, WPy, WPz);
        c4 = roz;
      } else {
        c1 = sel3(dir, QCx, QCy, QCz);
        c2 = sel3(dir, WQx, WQy, WQz);
        c4 = roe;
      }
      T val = c1 * slots[o.s1];
      val = fma(c2, slots[o.s2], val);
      if (n1) val = fma(ktab[((fl & 1u) << 3) + n1], fma(-c4, slots[o.s4], slots[o.s3]), val);
      if (ne) val = fma(ktab[16 + ne], slots[o.s5], val);
      return val;
    };
    for (int k = 0; k < P.nlev; ++k) {
      if (k > 0) {
        // two ops per lane per step, loads first: ops of a level are
        // independent, so both may be evaluated before either is stored
        const int o1 = P.vrr_lev[k + 1];
        for (int op = P.vrr_lev[k] + lane; op < o1; op += 2 * Grp::size()) {
          const bool two = op + Grp::size() < o1;
          const VrrOp x = load_vrr_op(P, op);
          VrrOp y = x;
          if (two) y = load_vrr_op(P, op + Grp::size());
          const T vx = eval(x);
          T vy = T(0);
          if (two) vy = eval(y);
          slots[x.d] = vx;
          if (two) slots[y.d] = vy;
        }
        Grp::sync();
      }
      const int a1 = P.acc_lev[k + 1];
      for (int op = P.acc_lev[k] + lane; op < a1; op += Grp::size()) {
        const uint2 u = __ldg(P.acc_ops + op);
        const unsigned src = u.y & 0x3FFFFFFFu;
        const unsigned w = u.y >> 30;
        const T wt = w == 0 ? T(1) : (w == 1 ? w1 : (w == 2 ? w2 : w3));
        slots[u.x] = fma(wt, slots[src], slots[u.x]);
      }
      Grp::sync();
    }
  }
}

// Steps 1-2: contracted (e0|f0) accumulators in slots[0, nacc).  Returns the
// number of primitive quartets that survived screening.
template <typename T, bool ATT = false, bool B64 = false>
__device__ int contract_quartet(const EriArgs& a, const QuartetGeom<T>& g, T* __restrict__ slots,
                                T* __restrict__ stage, int lane) {
  const DevProg& P = a.prog;
  const int R = a.stage_rows;
  T* ktab = stage + R * kStage;
  for (int i = lane; i < P.nacc; i += 32) slots[i] = T(0);
  const int nq = g.nbpp * g.nkpp;
  int kept = 0;
  const double npbraket = double(nq);
  for (int base = 0; base < nq; base += R) {
    // lane r < R prepares primitive quartet base + r in its own staging row
    const int idx = base + lane;
    bool keep = false;
    if (lane < R && idx < nq)
      keep = prologue<ATT, B64>(a, g, idx, npbraket, stage + lane * kStage);
    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
    __syncwarp();
    kept += __popc(ballot);
    vrr_consume<T>(P, stage, ballot, slots, ktab, lane);
    __syncwarp();
  }
  return kept;
}

// Step 3 for one phase.
template <typename T, class Grp = WarpGrp>
__device__ void run_post_phase(const DevProg& P, int ph, const QuartetGeom<T>& g,
                               T* __restrict__ slots, int lane) {
  const T ABx = g.AB[0], ABy = g.AB[1], ABz = g.AB[2];
  const T CDx = g.CD[0], CDy = g.CD[1], CDz = g.CD[2];
  const int l0 = P.phase_lev[ph], l1 = P.phase_lev[ph + 1];
  auto eval = [&](const PostOp& o) -> T {
    const unsigned kind = o.w & 15u;
    const int dir = (o.w >> 4) & 3;
    const int n = (o.w >> 8) & 31;
    T val;
    if (kind == 0) {
      val = fma(sel3(dir, ABx, ABy, ABz), slots[o.s2], slots[o.s1]);
    } else if (kind == 1) {
      val = fma(sel3(dir, CDx, CDy, CDz), slots[o.s2], slots[o.s1]);
    } else if (kind == 2) {
      val = slots[o.s1];
      if (n) val = fma(-small_int<T>(n), slots[o.s2], val);
    } else {
      val = slots[o.s1];
    }
    return val;
  };
  for (int k = l0; k < l1; ++k) {
    const int o1 = P.post_lev[k + 1];
    for (int op = P.post_lev[k] + lane; op < o1; op += 2 * Grp::size()) {
      const bool two = op + Grp::size() < o1;
      const PostOp x = load_post_op(P, op);
      PostOp y = x;
      if (two) y = load_post_op(P, op + Grp::size());
      const T vx = eval(x);
      T vy = T(0);
      if (two) vy = eval(y);
      slots[x.d] = vx;
      if (two) slots[y.d] = vy;
    }
    Grp::sync();
  }
}

__device__ __forceinline__ double sph_coef(const EriArgs& a, int t, double*) {
  return __ldg(a.sph_cd + t);
}
__device__ __forceinline__ float sph_coef(const EriArgs& a, int t, float*) {
  return __ldg(a.sph_cf + t);
}

// Sparse Cartesian -> solid harmonics for the pure indices, ping-ponging
// between `cart` and `tmp`.  Each lane owns whole columns (all indices but
// the transformed one), so the row loops and coefficient reads are
// warp-uniform (broadcast loads).  Returns the result buffer.
template <typename T, class Grp = WarpGrp>
__device__ T* sph_transform(const EriArgs& a, const int* l, const int* pure, int* dims, T* cart,
                            T* tmp, int lane) {
  T* src = cart;
  T* dst = tmp;
  T* tag = nullptr;
  for (int k = 0; k < 4; ++k) {
    if (!pure[k]) continue;
    const int lk = l[k], np = 2 * lk + 1, nc = dims[k];
    int outer = 1, inner = 1;
    for (int t = 0; t < k; ++t) outer *= dims[t];
    for (int t = k + 1; t < 4; ++t) inner *= dims[t];
    const int ncol = outer * inner;
    for (int c = lane; c < ncol; c += Grp::size()) {
      const int o = c / inner, i = c - o * inner;
      const T* sp = src + (size_t)o * nc * inner + i;
      T* dp = dst + (size_t)o * np * inner + i;
      for (int p = 0; p < np; ++p) {
        const int t0 = __ldg(a.sph_off + lk * 9 + p), t1 = __ldg(a.sph_off + lk * 9 + p + 1);
        T v = T(0);
        for (int t = t0; t < t1; ++t)
          v = fma(sph_coef(a, t, tag), sp[__ldg(a.sph_c + t) * inner], v);
        dp[p * inner] = v;
      }
    }
    Grp::sync();
    T* x = src;
    src = dst;
    dst = x;
    dims[k] = np;
  }
  return src;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double Dval(const EriArgs& a, size_t i, double*) {
  return __ldg(a.D + i);
}
__device__ __forceinline__ float Dval(const EriArgs& a, size_t i, float*) {
  return __ldg(a.Df + i);
}
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return f2d_int(v); }

// J/K digestion of one spherical shell set V[a][b][c][d] (canonical order):
// partial sums in T, accumulated into the FP64 matrices.
template <typename T>
__device__ void digest_jk(const EriArgs& a, const QuartetGeom<T>& g, const int* dims,
                          const T* V, T deg, int lane) {
  const int n0 = dims[0], n1 = dims[1], n2 = dims[2], n3 = dims[3];
  const size_t o0 = a.basis.bf_off[g.sh[0]], o1 = a.basis.bf_off[g.sh[1]];
  const size_t o2 = a.basis.bf_off[g.sh[2]], o3 = a.basis.bf_off[g.sh[3]];
  const size_t nbf = a.nbf;
  T* tag = nullptr;
  auto v = [&](int i, int j, int k, int l) -> T { return V[((i * n1 + j) * n2 + k) * n3 + l]; };
  // J(a,b) += sum_cd D(c,d) v
  for (int e = lane; e < n0 * n1; e += 32) {
    const int i = e / n1, j = e % n1;
    T s = 0;
    for (int k = 0; k < n2; ++k)
      for (int l = 0; l < n3; ++l) s = fma(Dval(a, (o2 + k) * nbf + o3 + l, tag), v(i, j, k, l), s);
    atomicAdd(a.Jacc + (o0 + i) * nbf + o1 + j, to_f64(deg * s));
  }
  // J(c,d) += sum_ab D(a,b) v
  for (int e = lane; e < n2 * n3; e += 32) {
    const int k = e / n3, l = e % n3;
    T s = 0;
    for (int i = 0; i < n0; ++i)
      for (int j = 0; j < n1; ++j) s = fma(Dval(a, (o0 + i) * nbf + o1 + j, tag), v(i, j, k, l), s);
    atomicAdd(a.Jacc + (o2 + k) * nbf + o3 + l, to_f64(deg * s));
  }
  // K(a,c) += sum_bd D(b,d) v ; K(b,d) += sum_ac D(a,c) v
  for (int e = lane; e < n0 * n2; e += 32) {
    const int i = e / n2, k = e % n2;
    T s = 0;
    for (int j = 0; j < n1; ++j)
      for (int l = 0; l < n3; ++l) s = fma(Dval(a, (o1 + j) * nbf + o3 + l, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o0 + i) * nbf + o2 + k, to_f64(deg * s));
  }
  for (int e = lane; e < n1 * n3; e += 32) {
    const int j = e / n3, l = e % n3;
    T s = 0;
    for (int i = 0; i < n0; ++i)
      for (int k = 0; k < n2; ++k) s = fma(Dval(a, (o0 + i) * nbf + o2 + k, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o1 + j) * nbf + o3 + l, to_f64(deg * s));
  }
  // K(a,d) += sum_bc D(b,c) v ; K(b,c) += sum_ad D(a,d) v
  for (int e = lane; e < n0 * n3; e += 32) {
    const int i = e / n3, l = e % n3;
    T s = 0;
    for (int j = 0; j < n1; ++j)
      for (int k = 0; k < n2; ++k) s = fma(Dval(a, (o1 + j) * nbf + o2 + k, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o0 + i) * nbf + o3 + l, to_f64(deg * s));
  }
  for (int e = lane; e < n1 * n2; e += 32) {
    const int j = e / n2, k = e % n2;
    T s = 0;
    for (int i = 0; i < n0; ++i)
      for (int l = 0; l < n3; ++l) s = fma(Dval(a, (o0 + i) * nbf + o3 + l, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o1 + j) * nbf + o2 + k, to_f64(deg * s));
  }
}

// digest_jk with compile-time shell sizes (loops unroll; used with the
// generated post stages).
template <typename T, int N0, int N1, int N2, int N3>
__device__ __forceinline__ void digest_jk_fixed(const EriArgs& a, const QuartetGeom<T>& g,
                                                const T* __restrict__ V, T deg, int lane) {
  const size_t o0 = a.basis.bf_off[g.sh[0]], o1 = a.basis.bf_off[g.sh[1]];
  const size_t o2 = a.basis.bf_off[g.sh[2]], o3 = a.basis.bf_off[g.sh[3]];
  const size_t nbf = a.nbf;
  T* tag = nullptr;
  auto v = [&](int i, int j, int k, int l) -> T { return V[((i * N1 + j) * N2 + k) * N3 + l]; };
  for (int e = lane; e < N0 * N1; e += 32) {
    const int i = e / N1, j = e % N1;
    T s = 0;
#pragma unroll
    for (int k = 0; k < N2; ++k)
#pragma unroll
      for (int l = 0; l < N3; ++l) s = fma(Dval(a, (o2 + k) * nbf + o3 + l, tag), v(i, j, k, l), s);
    atomicAdd(a.Jacc + (o0 + i) * nbf + o1 + j, to_f64(deg * s));
  }
  for (int e = lane; e < N2 * N3; e += 32) {
    const int k = e / N3, l = e % N3;
    T s = 0;
#pragma unroll
    for (int i = 0; i < N0; ++i)
#pragma unroll
      for (int j = 0; j < N1; ++j) s = fma(Dval(a, (o0 + i) * nbf + o1 + j, tag), v(i, j, k, l), s);
    atomicAdd(a.Jacc + (o2 + k) * nbf + o3 + l, to_f64(deg * s));
  }
  for (int e = lane; e < N0 * N2; e += 32) {
    const int i = e / N2, k = e % N2;
    T s = 0;
#pragma unroll
    for (int j = 0; j < N1; ++j)
#pragma unroll
      for (int l = 0; l < N3; ++l) s = fma(Dval(a, (o1 + j) * nbf + o3 + l, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o0 + i) * nbf + o2 + k, to_f64(deg * s));
  }
  for (int e = lane; e < N1 * N3; e += 32) {
    const int j = e / N3, l = e % N3;
    T s = 0;
#pragma unroll
    for (int i = 0; i < N0; ++i)
#pragma unroll
      for (int k = 0; k < N2; ++k) s = fma(Dval(a, (o0 + i) * nbf + o2 + k, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o1 + j) * nbf + o3 + l, to_f64(deg * s));
  }
  for (int e = lane; e < N0 * N3; e += 32) {
    const int i = e / N3, l = e % N3;
    T s = 0;
#pragma unroll
    for (int j = 0; j < N1; ++j)
#pragma unroll
      for (int k = 0; k < N2; ++k) s = fma(Dval(a, (o1 + j) * nbf + o2 + k, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o0 + i) * nbf + o3 + l, to_f64(deg * s));
  }
  for (int e = lane; e < N1 * N2; e += 32) {
    const int j = e / N2, k = e % N2;
    T s = 0;
#pragma unroll
    for (int i = 0; i < N0; ++i)
#pragma unroll
      for (int l = 0; l < N3; ++l) s = fma(Dval(a, (o0 + i) * nbf + o3 + l, tag), v(i, j, k, l), s);
    atomicAdd(a.Kacc + (o1 + j) * nbf + o2 + k, to_f64(deg * s));
  }
}

// Gradient digestion (FP64): sj = sum v D_ab D_cd, sk = sum v (D_ac D_bd + D_ad D_bc)/2.
template <typename T>
__device__ void digest_grad(const EriArgs& a, const QuartetGeom<T>& g, const int* dims,
                            const T* V, double& sj, double& sk, int lane) {
  const int n0 = dims[0], n1 = dims[1], n2 = dims[2], n3 = dims[3];
  const size_t o0 = a.basis.bf_off[g.sh[0]], o1 = a.basis.bf_off[g.sh[1]];
  const size_t o2 = a.basis.bf_off[g.sh[2]], o3 = a.basis.bf_off[g.sh[3]];
  const size_t nbf = a.nbf;
  const double* D = a.D;
  double pj = 0, pk = 0;
  const int tot = n0 * n1 * n2 * n3;
  for (int e = lane; e < tot; e += 32) {
    const int l = e % n3, k = (e / n3) % n2, j = (e / (n3 * n2)) % n1, i = e / (n3 * n2 * n1);
    const double val = to_f64(V[e]);
    const double Dab = __ldg(D + (o0 + i) * nbf + o1 + j);
    const double Dcd = __ldg(D + (o2 + k) * nbf + o3 + l);
    const double Dac = __ldg(D + (o0 + i) * nbf + o2 + k);
    const double Dbd = __ldg(D + (o1 + j) * nbf + o3 + l);
    const double Dad = __ldg(D + (o0 + i) * nbf + o3 + l);
    const double Dbc = __ldg(D + (o1 + j) * nbf + o2 + k);
    pj = fma(val * Dab, Dcd, pj);
    pk = fma(val * 0.5, fma(Dac, Dbd, Dad * Dbc), pk);
  }
  sj = warp_sum(pj);
  sk = warp_sum(pk);
}

// Post-contraction policy of the generic kernel: the class's interpreted
// post program and the table-driven solid-harmonic transform.  Generated
// policies (csrc/gen/post_classes.cuh) replace both for J/K digestion with
// unrolled per-class code whose lanes own columns of the shell set.
struct PostInterp {
  static constexpr bool kGenerated = false;
};
// The same policy for the attenuated operators (erf / erfc core integrals
// in the prologue); the generated policies serve Coulomb only.
struct PostInterpAtten : PostInterp {};
template <typename Post>
struct PostAtten {
  static constexpr bool value = false;
};
template <>
struct PostAtten<PostInterpAtten> {
  static constexpr bool value = true;
};

template <typename T, int MODE, typename Post = PostInterp>
__global__ void __launch_bounds__(128) eri_warp_kernel(EriArgs a) {
  extern __shared__ double smem_d[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const DevProg& P = a.prog;
  const int stage_per_warp = (a.stage_rows * kStage + kKtab + 3) & ~3;
  T* stage = reinterpret_cast<T*>(smem_d) + wib * stage_per_warp;
  T* slots;
  if (a.global_slots) {
    const size_t gw = size_t(blockIdx.x) * wpb + wib;
    slots = reinterpret_cast<T*>(a.gscratch) + gw * size_t(a.slot_stride);
  } else {
    T* base = reinterpret_cast<T*>(smem_d) + wpb * stage_per_warp;
    slots = base + size_t(wib) * a.slot_stride;
  }
  const long long total = a.implicit ? a.bin.total : a.nitems;
  long long nchunks = 0;
  unsigned long long my_prims = 0;
  while (true) {
    long long start = 0;
    if (lane == 0) start = (long long)atomicAdd(a.counter, (unsigned long long)a.chunk);
    start = __shfl_sync(0xffffffffu, start, 0);
    if (start >= total) break;
    if (++nchunks > a.max_chunks) {  // watchdog: cannot happen for valid input
      if (lane == 0) atomicExch(a.error_flag, 1);
      break;
    }
    const long long end = min(total, start + (long long)a.chunk);
    int seg = 0;
    if (a.implicit) seg = bin_segment(a.bin, start);
    for (long long q = start; q < end; ++q) {
      int bpair, kpair, flags = 0, orig = 0;
      long long outoff = 0;
      if (a.implicit) {
        while (seg + 1 < a.bin.nseg && a.bin.seg_start[seg + 1] <= q) ++seg;
        const int j = int(q - a.bin.seg_start[seg]) + a.bin.seg_j0[seg];
        bpair = a.bin.bra_pairs[a.bin.seg_bra[seg]];
        kpair = a.bin.ket_pairs[j];
        flags = (a.pair_swap[bpair] ? 1 : 0) | (a.pair_swap[kpair] ? 2 : 0);
      } else {
        const QuartetItem it = a.items[q];
        bpair = it.bra_pair;
        kpair = it.ket_pair;
        flags = it.flags;
        outoff = it.out;
        orig = it.pad;
      }
      QuartetGeom<T> g;
      load_geom<T>(a, bpair, kpair, flags & 1, (flags >> 1) & 1, g);
      if (mode_jk(MODE) && !quartet_screen(a, g.sh, bpair, kpair, g.scr)) continue;
      const int kept =
          contract_quartet<T, PostAtten<Post>::value, mode_b64(MODE)>(a, g, slots, stage, lane);
      my_prims += kept;
      if (mode_store(MODE) && a.is_null && lane == 0) a.is_null[orig] = kept == 0 ? 1 : 0;
      if (kept == 0) {
        if (MODE == kModeSchwarz && lane == 0) a.kschwarz[outoff] = 0.0;
        continue;
      }
      const bool same_pair = (bpair == kpair);
      const int degi = (g.sh[0] == g.sh[1] ? 1 : 2) * (g.sh[2] == g.sh[3] ? 1 : 2) *
                       (same_pair ? 1 : 2);
      if constexpr (Post::kGenerated) {
        static_assert(mode_jk(MODE), "generated post stages serve the J/K digestion");
        // (e0|f0) -> (a'b'|f0) per f column, then -> (a'b'|c'd') per a'b' column
        T* bo = slots + Post::kNacc;
        Post::template bra<T>(slots, bo, g.AB, lane);
        __syncwarp();
        T* V = bo + Post::kBraOut;
        Post::template ket<T>(bo, V, g.CD, lane);
        __syncwarp();
        digest_jk_fixed<T, Post::kNA, Post::kNB, Post::kNC, Post::kND>(a, g, V,
                                                                        small_int<T>(degi), lane);
        __syncwarp();
        continue;
      }
      const int lsh[4] = {P.la, P.lb, P.lc, P.ld};
      int pure[4];
      for (int t = 0; t < 4; ++t) pure[t] = a.basis.pure[g.sh[t]];
      double cj[3] = {0, 0, 0}, ck[3] = {0, 0, 0};
      for (int ph = 0; ph < P.nphases; ++ph) {
        run_post_phase<T>(P, ph, g, slots, lane);
        for (int s = 0; s < P.sets_per_phase; ++s) {
          int dims[4] = {ncart_of(P.la), ncart_of(P.lb), ncart_of(P.lc), ncart_of(P.ld)};
          T* cart = slots + P.cart_out + s * P.ncart4;
          T* V = sph_transform<T>(a, lsh, pure, dims, cart, slots + P.sph_tmp, lane);
          const int nsph4 = dims[0] * dims[1] * dims[2] * dims[3];
          if (MODE == kModeSchwarz) {
            double mx = 0;
            for (int e = lane; e < nsph4; e += 32) mx = fmax(mx, fabs(to_f64(V[e])));
            mx = warp_max(mx);
            if (lane == 0) a.kschwarz[outoff] = sqrt(mx);
          } else if (mode_jk(MODE)) {
            digest_jk<T>(a, g, dims, V, small_int<T>(degi), lane);
          } else if (MODE == kModeGrad) {
            double sj, sk;
            digest_grad<T>(a, g, dims, V, sj, sk, lane);
            const int ctr = ph == 0 ? 0 : (ph == 1 ? 1 : 3);
            cj[s] -= sj;
            ck[s] -= sk;
            if (lane == 0) {
              const int at = a.basis.atom[g.sh[ctr]];
              atomicAdd(a.gJ + 3 * at + s, 0.5 * degi * sj);
              atomicAdd(a.gK + 3 * at + s, -0.25 * degi * sk);
            }
          } else {  // kModeStore
            const int fl = flags >> 2;
            const bool sbk = fl & 1, stb = (fl >> 1) & 1, stk = (fl >> 2) & 1;
            int perm[4];
            perm[0] = sbk ? (stk ? 3 : 2) : (stb ? 1 : 0);
            perm[1] = sbk ? (stk ? 2 : 3) : (stb ? 0 : 1);
            perm[2] = sbk ? (stb ? 1 : 0) : (stk ? 3 : 2);
            perm[3] = sbk ? (stb ? 0 : 1) : (stk ? 2 : 3);
            int tn[4];
            for (int t = 0; t < 4; ++t) tn[perm[t]] = dims[t];
            const int ctr = P.deriv ? (ph == 0 ? 0 : (ph == 1 ? 1 : 3)) : 0;
            const int ts = P.deriv ? perm[ctr] * 3 + s : 0;
            double* o = a.out + outoff + (size_t)ts * nsph4;
            T* cb = slots + P.cbuf + s * P.ncart4;
            for (int e = lane; e < nsph4; e += 32) {
              int ci[4];
              int r = e;
              ci[3] = r % dims[3]; r /= dims[3];
              ci[2] = r % dims[2]; r /= dims[2];
              ci[1] = r % dims[1]; ci[0] = r / dims[1];
              int it[4];
              for (int t = 0; t < 4; ++t) it[perm[t]] = ci[t];
              const int tidx = ((it[0] * tn[1] + it[1]) * tn[2] + it[2]) * tn[3] + it[3];
              o[tidx] = to_f64(V[e]);
              if (P.deriv) cb[e] = (ph == 0 ? T(0) : cb[e]) - V[e];
            }
            __syncwarp();
            if (P.deriv && ph == P.nphases - 1) {
              // centre C by translational invariance
              const int tsc = perm[2] * 3 + s;
              double* oc = a.out + outoff + (size_t)tsc * nsph4;
              for (int e = lane; e < nsph4; e += 32) {
                int ci[4];
                int r = e;
                ci[3] = r % dims[3]; r /= dims[3];
                ci[2] = r % dims[2]; r /= dims[2];
                ci[1] = r % dims[1]; ci[0] = r / dims[1];
                int it[4];
                for (int t = 0; t < 4; ++t) it[perm[t]] = ci[t];
                const int tidx = ((it[0] * tn[1] + it[1]) * tn[2] + it[2]) * tn[3] + it[3];
                oc[tidx] = to_f64(cb[e]);
              }
            }
          }
          __syncwarp();
        }
      }
      if (MODE == kModeGrad && lane == 0) {
        const int at = a.basis.atom[g.sh[2]];
        for (int s = 0; s < 3; ++s) {
          atomicAdd(a.gJ + 3 * at + s, 0.5 * degi * cj[s]);
          atomicAdd(a.gK + 3 * at + s, -0.25 * degi * ck[s]);
        }
      }
      __syncwarp();
    }
  }
  if (a.prim_count && lane == 0) atomicAdd(a.prim_count, my_prims);
}

// Host-side launcher and occupancy query of one kernel instance.
template <typename T, int MODE, typename Post = PostInterp>
cudaError_t launch_eri_t(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  auto k = eri_warp_kernel<T, MODE, Post>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, block, smem, st>>>(a);
  return cudaGetLastError();
}

template <typename T, int MODE, typename Post = PostInterp>
int occ_t(int block, size_t smem) {
  auto k = eri_warp_kernel<T, MODE, Post>;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem) != cudaSuccess) return 1;
  return n;
}

}  // namespace lgx
