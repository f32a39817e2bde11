// Device-side data structures and the Boys function of the ERI kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lgx {

// ------------------------------------------------------------------ Boys
// F_m(T) = int_0^1 u^{2m} exp(-T u^2) du.
// For T <= kBoysTmax: F_mmax by a Taylor expansion about the nearest grid
// point T_k = k/64 of a table of F_0..F_{kBoysCols-1}(T_k), then the
// stable downward recursion F_m = (2T F_{m+1} + e^{-T})/(2m+1).
// For T > kBoysTmax: F_0 = sqrt(pi/T)/2 (erf(sqrt T) == 1 to double there)
// and the upward recursion F_{m+1} = ((2m+1) F_m - e^{-T})/(2T), stable for
// 2T > 2m+1 (the register kernels, m <= 6, drop the e^{-T} terms, which
// are below 2e-15 relative there).  This is the scheme of libint's FmEval_Taylor
// (include/libint2/boys.h:519-879); the table is generated on the host from
// the Maclaurin series in extended precision.
constexpr double kBoysInvDT = 64.0;
constexpr double kBoysDT = 1.0 / 64.0;
constexpr double kBoysTmax = 50.0;
constexpr int kBoysTerms = 7;
constexpr int kBoysMaxM = 16;                         // largest mmax served
constexpr int kBoysCols = kBoysMaxM + kBoysTerms;     // 23 columns
constexpr int kBoysRows = int(kBoysTmax * 64.0) + 2;  // 3202 grid points

// Pre-divided Taylor table: [kBoysRows][kBoysMaxM+1][8] with
// entry i = F_{m+i}(T_k) / i! (i < 7), so that
// F_m(T_k + d) = sum_i entry_i (-d)^i by Horner without extra products;
// entry 7 of the m = 0 row holds e^{-T_k}.
constexpr int kBoysTaylorStride = 8;

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
  const float* Ohi;     // [3*nshell] float(O)
  const float* Olo;     // [3*nshell] float(O - Ohi): Ohi + Olo = O to ~1e-15
};

// float -> double with integer operations only (no FP64-pipe instruction):
// exact for normal floats; zero and subnormal inputs (|x| < 1.2e-38) give 0.
__device__ __forceinline__ double f2d_int(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (e == 0u) return __longlong_as_double((long long)sign);
  const unsigned long long exp64 = (e == 0xffu) ? 0x7ffull : (unsigned long long)(e - 127u + 1023u);
  const unsigned long long mant = (unsigned long long)(u & 0x7fffffu) << 29;
  return __longlong_as_double((long long)(sign | (exp64 << 52) | mant));
}

// double -> float, rounded to nearest even, with integer operations only
// (no FP64-pipe instruction): exact rounding for results in the normal
// float range; smaller magnitudes (|x| < 2^-126) give a signed zero and
// larger ones a signed infinity.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(u >> 63) << 31;
  const int e = int((u >> 52) & 0x7ffu) - 1023 + 127;
  const unsigned long long mant = u & 0xfffffffffffffull;
  // keep 23 of the 52 mantissa bits: add half an ulp minus one, plus the
  // lowest kept bit (ties to even); a carry out of the mantissa bumps e
  const unsigned long long r = (mant + 0xfffffffull + ((mant >> 29) & 1ull)) >> 29;
  const unsigned bits = ((unsigned)e << 23) + (unsigned)r;  // r = 2^23 carries into e
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255 || bits >= 0x7f800000u) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | bits);
}

// double(n) for a small non-negative integer n < 2^20 with integer
// operations only.
__device__ __forceinline__ double i2d_int(int n) {
  if (n <= 0) return 0.0;
  const int e = 31 - __clz(n);
  const unsigned hi = ((unsigned)(1023 + e) << 20) | ((unsigned)(n - (1 << e)) << (20 - e));
  return __hiloint2double((int)hi, 0);
}

// One primitive pair of a shell pair (s1, s2) as stored (s1 = first shell),
// with FP64 fields for the FP64 kernels and FP32 copies (centre-relative
// P, so FP32 P-Q differences keep their precision) for the FP32 kernels.
struct __align__(16) PrimPairRec {
  double P[3];
  double Kc;      // sqrt(2) pi^{5/4} exp(-rho AB^2)/gamma * c1 * c2
  double oog;     // 1/(alpha1 + alpha2)
  double zeta;    // alpha1 + alpha2
  double a1, a2;  // exponents of s1 and s2
  double ln_scr;  // ln of the pair screening factor (shell.h:1041-1059)
  float fKc, fzeta, foog, fln_scr;
  float fPA1[3];  // P - O(s1)
  float fPA2[3];  // P - O(s2)
  float fa1, fa2;
  float fnonsph;  // Conservative screening factor
  float pad;
};
static_assert(sizeof(PrimPairRec) == 128, "PrimPairRec layout");

// FP32 primitive-pair record of the J/K bins (two float4): {K c1 c2,
// zeta, 1/zeta, ln screening factor} and {P - O(first canonical centre),
// Conservative factor}.  The records of one pair class are laid out
// [depth group][primitive pair][position in the group], so the lanes that
// take consecutive ket pairs of a segment read consecutive addresses.
struct __align__(16) PrimPairJK32 {
  float4 k;
  float4 pa;
};
static_assert(sizeof(PrimPairJK32) == 32, "PrimPairJK32 layout");

// Double-float companion of a PrimPairJK32 record (same index), for the
// mixed scheme's Boys argument: the pair centre P and the exponent sum
// zeta, each as hi = the FP32 rounding of the FP64 value and lo = the FP32
// rounding of the remainder (48 significant bits: |value - hi - lo| <=
// 2^-48 |value|).
struct __align__(16) PrimPairJKds {
  float4 hi;  // P.x, P.y, P.z, zeta
  float4 lo;
};
static_assert(sizeof(PrimPairJKds) == 32, "PrimPairJKds layout");

// The double-float record of one primitive pair (centre P, exponent sum).
__device__ __forceinline__ PrimPairJKds make_jkds(double px, double py, double pz, double zeta) {
  const float hx = float(px), hy = float(py), hz = float(pz), hw = float(zeta);
  PrimPairJKds r;
  r.hi = make_float4(hx, hy, hz, hw);
  r.lo = make_float4(float(px - double(hx)), float(py - double(hy)), float(pz - double(hz)),
                     float(zeta - double(hw)));
  return r;
}

// Double-float arithmetic ("ds": value = hi + lo with |lo| <= ulp(hi)/2)
// from the error-free transformations of Knuth (two-sum), Dekker
// (fast two-sum) and the FMA two-product; __fadd_rn / __fmul_rn keep the
// compiler from contracting the steps whose rounding errors they recover.
struct dsf {
  float hi, lo;
};
__device__ __forceinline__ dsf ds_fast_two_sum(float a, float b) {  // |a| >= |b| or a = 0
  const float s = __fadd_rn(a, b);
  return {s, __fadd_rn(b, -__fadd_rn(s, -a))};
}
__device__ __forceinline__ dsf ds_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  return {s, __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb))};
}
// (two-sum also in the final normalisation: after cancellation of the
// high parts the low parts can be the larger)
__device__ __forceinline__ dsf ds_add(dsf a, dsf b) {
  const dsf s = ds_two_sum(a.hi, b.hi);
  return ds_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dsf ds_sub(dsf a, dsf b) { return ds_add(a, {-b.hi, -b.lo}); }
__device__ __forceinline__ dsf ds_mul(dsf a, dsf b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = fmaf(a.hi, b.hi, -p);
  return ds_fast_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}
__device__ __forceinline__ dsf ds_sqr(dsf a) {
  const float p = __fmul_rn(a.hi, a.hi);
  const float e = fmaf(a.hi, a.hi, -p);
  return ds_fast_two_sum(p, fmaf(2.0f * a.hi, a.lo, e));
}

// T = rho |P - Q|^2 of one primitive quartet in double-float arithmetic
// from the two pairs' double-float P and zeta (b: bra, k: ket).  rho =
// zeta eta / (zeta + eta) is the FP32 value rho0 (any estimate within
// ~1e-6) plus the correction (zeta eta - rho0 (zeta + eta)) * oogpq, the
// residual formed to 2^-46 and the correction (relative size ~1e-7) scaled
// in FP32 with the FP32 1/(zeta + eta); relative error of rho ~1e-13.  The
// representation of P (2^-48 |P|) bounds |P - Q| to ~4e-13 absolute for
// |P| <= 50 bohr; T to ~2^-44 relative beyond that.
__device__ __forceinline__ dsf ds_boys_arg(const float4& bh, const float4& bl, const float4& kh,
                                           const float4& kl, float rho0, float oogpq) {
  const dsf zb = {bh.w, bl.w}, zk = {kh.w, kl.w};
  const dsf r = ds_sub(ds_mul(zb, zk), ds_mul({rho0, 0.0f}, ds_add(zb, zk)));
  const dsf rho = ds_fast_two_sum(rho0, __fmul_rn(r.hi, oogpq));
  const dsf dx = ds_sub({bh.x, bl.x}, {kh.x, kl.x});
  const dsf dy = ds_sub({bh.y, bl.y}, {kh.y, kl.y});
  const dsf dz = ds_sub({bh.z, bl.z}, {kh.z, kl.z});
  return ds_mul(rho, ds_add(ds_add(ds_sqr(dx), ds_sqr(dy)), ds_sqr(dz)));
}

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
  // compact != 0 (every slot index < 65536): a VRR op is one uint4
  // {dst | s1<<16, s2 | s3<<16, s4 | s5<<16, flags} and a post op one uint2
  // {dst | s1<<16, s2 | word<<16}; otherwise two uint4 / one uint4 per op.
  int compact;
  const uint4* vrr_ops;
  const uint2* acc_ops;
  const int* post_lev;
  const int* phase_lev;
  const uint4* post_ops;
  const uint2* post_ops_c;
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
