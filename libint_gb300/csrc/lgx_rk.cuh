// Register-resident ERI kernel: G lanes (1, 2, 4, ..., 32) per contracted
// shell quartet.  The lanes of a group split the primitive quartets, each
// runs the prologue (screening, pfac, T, Boys, VRR factors) and the class's
// unrolled VRR with the contracted (e0|f0) accumulators in registers; the
// group then reduces the accumulators with shuffles, applies the unrolled
// HRR and solid-harmonic transform, and splits the epilogue (J/K digestion,
// store, Schwarz maximum) between its lanes.
//
// Prologue precision follows the kernel's arithmetic type T: FP64 kernels
// evaluate everything in FP64 (libint's algorithm, engine.impl.h:1306-1766);
// FP32 kernels use the FP32 copies of the primitive-pair data, with P-Q
// formed from centre-relative offsets plus the FP64 centre difference A-C
// so that it keeps FP32 relative precision.
#pragma once
#include "gen/rk_classes.cuh"
#include "lgx_boys.cuh"

namespace lgx {

// T -> double for the FP64 accumulators (integer-only for float)
__device__ __forceinline__ double rk_f64(double x) { return x; }
__device__ __forceinline__ double rk_f64(float x) { return f2d_int(x); }

// Attenuated operators (register kernels of the J/K passes): F holds
// pfac F_m(T) on entry; with s = omega^2 / (omega^2 + rho) the core
// integrals become (libint's erf_coulomb_gm_eval / erfc_coulomb_gm_eval,
// include/libint2/boys.h:1913-1980)
//   erf(omega r)/r :  s^{m+1/2} F_m(s T)
//   erfc(omega r)/r:  F_m(T) - s^{m+1/2} F_m(s T)
// (s T <= T, so the same Taylor grid serves).  omega = 0 gives zero (erf)
// and the Coulomb integrals (erfc).
template <int MMAX>
__device__ __forceinline__ void rk_attenuate(const EriArgs& a, double T, double rho, double pfac,
                                             double* F) {
  if (!(a.omega2 > 0.0)) {
    if (a.op == 1)
#pragma unroll
      for (int m = 0; m <= MMAX; ++m) F[m] = 0.0;
    return;
  }
  const double s = a.omega2 / (a.omega2 + rho);
  double G[MMAX + 1];
  rk_boys<MMAX>(a.boys_tay, T * s, pfac, G);
  double f = sqrt(s);
#pragma unroll
  for (int m = 0; m <= MMAX; ++m, f *= s) F[m] = a.op == 1 ? f * G[m] : F[m] - f * G[m];
}

template <int MMAX>
__device__ __forceinline__ void rk_attenuate(const EriArgs& a, float T, float rho, float pfac,
                                             float* F) {
  const float w2 = float(a.omega2);
  if (!(w2 > 0.0f)) {
    if (a.op == 1)
#pragma unroll
      for (int m = 0; m <= MMAX; ++m) F[m] = 0.0f;
    return;
  }
  const float s = w2 / (w2 + rho);
  float G[MMAX + 1];
  rk_boys<MMAX>(a.boys32, T * s, pfac, G);
  float f = sqrtf(s);
#pragma unroll
  for (int m = 0; m <= MMAX; ++m, f *= s) F[m] = a.op == 1 ? f * G[m] : F[m] - f * G[m];
}

template <typename T>
struct RkQuartet {
  int sh[4];
  int bra_pp, ket_pp, nbpp, nkpp;
  bool bsw, ksw;
  double A[3], C[3];  // FP64 kernels only
  T AB[3], CD[3], AC[3];
};

template <typename T>
__device__ __forceinline__ void rk_load(const EriArgs& a, int bpair, int kpair, bool bsw,
                                        bool ksw, RkQuartet<T>& q) {
  const PairRec bp = a.pairs[bpair];
  const PairRec kp = a.pairs[kpair];
  q.sh[0] = bsw ? bp.s2 : bp.s1;
  q.sh[1] = bsw ? bp.s1 : bp.s2;
  q.sh[2] = ksw ? kp.s2 : kp.s1;
  q.sh[3] = ksw ? kp.s1 : kp.s2;
  q.bra_pp = bp.pp_off;
  q.nbpp = bp.npp;
  q.ket_pp = kp.pp_off;
  q.nkpp = kp.npp;
  q.bsw = bsw;
  q.ksw = ksw;
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const double A = a.basis.O[3 * q.sh[0] + x], B = a.basis.O[3 * q.sh[1] + x];
      const double C = a.basis.O[3 * q.sh[2] + x], D = a.basis.O[3 * q.sh[3] + x];
      q.A[x] = A;
      q.C[x] = C;
      q.AB[x] = A - B;
      q.CD[x] = C - D;
      q.AC[x] = A - C;
    }
  } else {
    // FP32: differences of the hi/lo float centres keep FP32 relative
    // precision without an FP64 instruction
    const float* hi = a.basis.Ohi;
    const float* lo = a.basis.Olo;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const int i0 = 3 * q.sh[0] + x, i1 = 3 * q.sh[1] + x, i2 = 3 * q.sh[2] + x,
                i3 = 3 * q.sh[3] + x;
      q.AB[x] = (hi[i0] - hi[i1]) + (lo[i0] - lo[i1]);
      q.CD[x] = (hi[i2] - hi[i3]) + (lo[i2] - lo[i3]);
      q.AC[x] = (hi[i0] - hi[i2]) + (lo[i0] - lo[i2]);
    }
  }
}

// One primitive quartet into acc (FP64).  Returns false when screened out.
// The ln-screen runs on the FP32 copies with the FP64 values inside the
// rounding band (ln_kept) and the pfac screen compares the IEEE bit
// patterns, so neither costs an FP64 instruction outside the band.
template <class C, bool ATT>
__device__ __forceinline__ bool rk_prim(const EriArgs& a, const RkQuartet<double>& q, int ib,
                                        int ik, const PrimScreen& scr, double* acc) {
  const PrimPairRec& bp = a.pprims[q.bra_pp + ib];
  const PrimPairRec& kp = a.pprims[q.ket_pp + ik];
  if (!ln_kept(a, bp.fln_scr + kp.fln_scr, q.bra_pp + ib, q.ket_pp + ik, scr)) return false;
  const double zeta = bp.zeta, eta = kp.zeta;
  const double gpq = zeta + eta;
  const double rs = rsqrt(gpq);
  const double pfac = bp.Kc * kp.Kc * rs;
  if ((__double_as_longlong(pfac) & 0x7fffffffffffffffll) < __double_as_longlong(scr.prec))
    return false;
  const double oogpq = rs * rs;
  const double PQx = bp.P[0] - kp.P[0], PQy = bp.P[1] - kp.P[1], PQz = bp.P[2] - kp.P[2];
  const double rho = zeta * eta * oogpq;
  const double T = rho * fma(PQx, PQx, fma(PQy, PQy, PQz * PQz));
  double F[C::kMmax + 1];
  rk_boys<C::kMmax>(a.boys_tay, T, pfac, F);
  if constexpr (ATT) rk_attenuate<C::kMmax>(a, T, rho, pfac, F);
  rk::Geo<double> g;
  const double ez = eta * oogpq, zz = zeta * oogpq;
  g.PAx = bp.P[0] - q.A[0]; g.PAy = bp.P[1] - q.A[1]; g.PAz = bp.P[2] - q.A[2];
  g.QCx = kp.P[0] - q.C[0]; g.QCy = kp.P[1] - q.C[1]; g.QCz = kp.P[2] - q.C[2];
  g.WPx = -ez * PQx; g.WPy = -ez * PQy; g.WPz = -ez * PQz;
  g.WQx = zz * PQx; g.WQy = zz * PQy; g.WQz = zz * PQz;
  g.oo2z = 0.5 * bp.oog;
  g.roz = ez;
  g.oo2e = 0.5 * kp.oog;
  g.roe = zz;
  g.oo2ze = 0.5 * oogpq;
  C::template vrr<double>(F, g, acc);
  return true;
}

// FP32 primitive pair in the quartet's orientation: {K c1 c2, zeta,
// 1/zeta, ln screen} and P minus its first canonical centre.
struct PrimF32 {
  float4 k;
  float4 pa;
};

// From the coalesced J/K records (one 32-byte record, two vector loads).
__device__ __forceinline__ PrimF32 rk_rec32(const PrimPairJK32* r) {
  PrimF32 p;
  p.k = __ldg(&r->k);
  p.pa = __ldg(&r->pa);
  return p;
}

// From the general primitive-pair table (explicit quartet lists).
__device__ __forceinline__ PrimF32 rk_pp32(const PrimPairRec& r, bool sw) {
  PrimF32 p;
  p.k = make_float4(r.fKc, r.fzeta, r.foog, r.fln_scr);
  const float* PA = sw ? r.fPA2 : r.fPA1;
  p.pa = make_float4(PA[0], PA[1], PA[2], r.fnonsph);
  return p;
}

// One primitive quartet into acc (FP32).  AC = A - C of the quartet.
// bidx, kidx: the two primitive pairs' PrimPairRec indices (the FP64
// values of the screening decisions inside the rounding band).
template <class C, bool ATT>
__device__ __forceinline__ bool rk_prim(const EriArgs& a, const RkQuartet<float>& q,
                                        const PrimF32& bp, const PrimF32& kp, int bidx,
                                        int kidx, const PrimScreen& scr, float* acc) {
  if (!ln_kept(a, bp.k.w + kp.k.w, bidx, kidx, scr)) return false;
  const float zeta = bp.k.y, eta = kp.k.y;
  const float gpq = zeta + eta;
  const float rs = rsqrtf(gpq);
  const float oogpq = rs * rs;
  const float pfac = bp.k.x * kp.k.x * rs;
  if (!pf_kept(a, fabsf(pfac), 1.0, bidx, kidx, scr)) return false;
  const float PA[3] = {bp.pa.x, bp.pa.y, bp.pa.z};
  const float QC[3] = {kp.pa.x, kp.pa.y, kp.pa.z};
  const float PQx = PA[0] - QC[0] + q.AC[0], PQy = PA[1] - QC[1] + q.AC[1],
              PQz = PA[2] - QC[2] + q.AC[2];
  const float rho = zeta * eta * oogpq;
  const float T = rho * fmaf(PQx, PQx, fmaf(PQy, PQy, PQz * PQz));
  float F[C::kMmax + 1];
  rk_boys<C::kMmax>(a.boys32, T, pfac, F);
  if constexpr (ATT) rk_attenuate<C::kMmax>(a, T, rho, pfac, F);
  rk::Geo<float> g;
  const float ez = eta * oogpq, zz = zeta * oogpq;
  g.PAx = PA[0]; g.PAy = PA[1]; g.PAz = PA[2];
  g.QCx = QC[0]; g.QCy = QC[1]; g.QCz = QC[2];
  g.WPx = -ez * PQx; g.WPy = -ez * PQy; g.WPz = -ez * PQz;
  g.WQx = zz * PQx; g.WQy = zz * PQy; g.WQz = zz * PQz;
  g.oo2z = 0.5f * bp.k.z;
  g.roz = ez;
  g.oo2e = 0.5f * kp.k.z;
  g.roe = zz;
  g.oo2ze = 0.5f * oogpq;
  C::template vrr<float>(F, g, acc);
  return true;
}

// One primitive quartet into acc (FP32 VRR) with the Boys function in FP64
// (the kModeJKB64 / kModeStoreB64 kernels of the mixed scheme).  The
// screening, prefactor and VRR geometry are the FP32 ones of rk_prim above;
// the Boys argument T = rho |P - Q|^2 is formed in double-float arithmetic
// from the bins' double-float records bds / kds, or for explicit quartet
// lists (null bds / kds) from those of the primitive pairs bidx / kidx
// (ds_boys_arg: FP32 operations, relative error ~1e-13); F_m(T) comes from
// the FP64 evaluator (Taylor with the
// downward recursion and e^{-T}, or the asymptotic branch, rk_boys_b64) and
// is rounded to FP32 with integer operations before the FP32 pfac.
template <class C>
__device__ __forceinline__ bool rk_prim_b64(const EriArgs& a, const RkQuartet<float>& q,
                                            const PrimF32& bp, const PrimF32& kp,
                                            const PrimPairJKds* bds, const PrimPairJKds* kds,
                                            int bidx, int kidx, const PrimScreen& scr,
                                            float* acc) {
  if (!ln_kept(a, bp.k.w + kp.k.w, bidx, kidx, scr)) return false;
  const float zeta = bp.k.y, eta = kp.k.y;
  const float gpq = zeta + eta;
  const float rs = rsqrtf(gpq);
  const float oogpq = rs * rs;
  const float pfac = bp.k.x * kp.k.x * rs;
  if (!pf_kept(a, fabsf(pfac), 1.0, bidx, kidx, scr)) return false;
  const float PA[3] = {bp.pa.x, bp.pa.y, bp.pa.z};
  const float QC[3] = {kp.pa.x, kp.pa.y, kp.pa.z};
  const float PQx = PA[0] - QC[0] + q.AC[0], PQy = PA[1] - QC[1] + q.AC[1],
              PQz = PA[2] - QC[2] + q.AC[2];
  const float rho = zeta * eta * oogpq;
  if (!bds) {  // explicit quartet lists: the primitive pairs' own records
    bds = a.ppds + bidx;
    kds = a.ppds + kidx;
  }
  const dsf T =
      ds_boys_arg(__ldg(&bds->hi), __ldg(&bds->lo), __ldg(&kds->hi), __ldg(&kds->lo), rho, oogpq);
  double F64[C::kMmax + 1];
  rk_boys_b64<C::kMmax>(a.boys_tay, T, F64);
  float F[C::kMmax + 1];
#pragma unroll
  for (int m = 0; m <= C::kMmax; ++m) F[m] = d2f_int(F64[m]) * pfac;
  rk::Geo<float> g;
  const float ez = eta * oogpq, zz = zeta * oogpq;
  g.PAx = PA[0]; g.PAy = PA[1]; g.PAz = PA[2];
  g.QCx = QC[0]; g.QCy = QC[1]; g.QCz = QC[2];
  g.WPx = -ez * PQx; g.WPy = -ez * PQy; g.WPz = -ez * PQz;
  g.WQx = zz * PQx; g.WQy = zz * PQy; g.WQz = zz * PQz;
  g.oo2z = 0.5f * bp.k.z;
  g.roz = ez;
  g.oo2e = 0.5f * kp.k.z;
  g.roe = zz;
  g.oo2ze = 0.5f * oogpq;
  C::template vrr<float>(F, g, acc);
  return true;
}

template <typename T>
__device__ __forceinline__ T rk_shfl_xor(unsigned mask, T v, int o, int width);
template <>
__device__ __forceinline__ double rk_shfl_xor(unsigned mask, double v, int o, int width) {
  return __shfl_xor_sync(mask, v, o, width);
}
template <>
__device__ __forceinline__ float rk_shfl_xor(unsigned mask, float v, int o, int width) {
  return __shfl_xor_sync(mask, v, o, width);
}

// D value in the kernel's precision (FP32 kernels read the FP32 copy).
__device__ __forceinline__ double rk_D(const EriArgs& a, size_t i, double*) {
  return __ldg(a.D + i);
}
__device__ __forceinline__ float rk_D(const EriArgs& a, size_t i, float*) {
  return __ldg(a.Df + i);
}

// Blocks per SM the compiler has to allow for (__launch_bounds__; 0 = no
// minimum, the compiler's own register target): the measured per-class
// choice of the generator's table for the J/K kernels; otherwise 1 for the
// FP64 classes with L >= 5, where the compiler left to itself gives several
// instances 32 registers and 25-57 KB of spills per thread (local memory the
// context reserves for every resident thread), else 0.
template <typename T, int LA, int LB, int LC, int LD, int MODE, bool ATT>
constexpr int rk_min_blocks() {
  constexpr int t = ATT ? -1 : rk::min_blocks_table(sizeof(T) == 4, MODE, LA, LB, LC, LD);
  return t >= 0 ? t : (sizeof(T) == 8 && LA + LB + LC + LD >= 5 ? 1 : 0);
}

// ATT: attenuated operator (erf / erfc, EriArgs::op), J/K mode only; the
// Coulomb instances (ATT = false) carry none of its code.
template <typename T, int LA, int LB, int LC, int LD, int MODE, bool ATT = false>
__global__ void __launch_bounds__(128, (rk_min_blocks<T, LA, LB, LC, LD, MODE, ATT>()))
    rk_kernel(EriArgs a) {
  using C = rk::Cls<LA, LB, LC, LD>;
  constexpr int N0 = C::kN0, N1 = C::kN1, N2 = C::kN2, N3 = C::kN3;
  const int G = a.group;
  const int lane = threadIdx.x & 31;
  const int g = lane & (G - 1);
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  const int per_warp = 32 / G;  // quartets per warp chunk
  const long long warp_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long total = a.implicit ? a.bin.total : a.nitems;
  unsigned long long my_prims = 0;
  // Warp chunks of per_warp consecutive quartets, strided over the grid:
  // consecutive quartets share a bin segment (same bra pair, same depth).
  for (long long c = warp_id; c * per_warp < total; c += nwarps) {
    const long long c0 = c * per_warp;
    const long long qi = c0 + (lane / G);
    int seg = 0;
    if (a.implicit) {
      // One (warp-uniform) binary search per chunk; the segment starts
      // inside the chunk come from one coalesced load of the next 32
      // starts (segments are non-empty, so at most per_warp - 1 of them
      // fall inside), and each quartet's segment is seg0 plus the starts
      // at or before its offset.
      const int seg0 = bin_segment(a.bin, c0);
      const int k = seg0 + 1 + lane;
      const long long m = (k <= a.bin.nseg ? a.bin.seg_start[k] : total + 64) - c0;  // >= 1
      const unsigned starts = __reduce_or_sync(0xffffffffu, m < per_warp ? 1u << m : 0u);
      seg = seg0 + __popc(starts & ((2u << (lane / G)) - 1u));
    }
    if (qi >= total) continue;
    int bpair, kpair, flags, orig = 0;
    long long outoff = 0;
    int2 brec = make_int2(0, 0), krec = make_int2(0, 0);
    if (a.implicit) {
      const int j = int(qi - a.bin.seg_start[seg]) + a.bin.seg_j0[seg];
      const int bpos = a.bin.seg_bra[seg];
      bpair = a.bin.bra_pairs[bpos];
      kpair = a.bin.ket_pairs[j];
      if (sizeof(T) == 4 && a.jk32) {
        brec = __ldg(a.bin.bra_rec + bpos);
        krec = __ldg(a.bin.ket_rec + j);
      }
      flags = (a.pair_swap[bpair] ? 1 : 0) | (a.pair_swap[kpair] ? 2 : 0);
    } else {
      const QuartetItem it = a.items[qi];
      bpair = it.bra_pair;
      kpair = it.ket_pair;
      flags = it.flags;
      outoff = it.out;
      orig = it.pad;
    }
    RkQuartet<T> q;
    rk_load<T>(a, bpair, kpair, flags & 1, (flags >> 1) & 1, q);
    // the G lanes of a quartet agree, so a skipped quartet leaves the group
    // together
    PrimScreen scr;
    if (!quartet_screen(a, q.sh, bpair, kpair, scr) && mode_jk(MODE)) continue;
    T acc[C::kNacc];
#pragma unroll
    for (int i = 0; i < C::kNacc; ++i) acc[i] = T(0);
    const int nq = q.nbpp * q.nkpp;
    int kept = 0;
    // primitive quartets g, g+G, ... as (bra, ket) primitive pairs, stepped
    // without a division per step
    int ib = g / q.nkpp, ik = g - ib * q.nkpp;
    const int gb = G / q.nkpp, gk = G - gb * q.nkpp;
    for (int p = g; p < nq; p += G) {
      if constexpr (sizeof(T) == 4) {
        const bool rec = a.implicit && a.jk32;
        const PrimF32 bp = rec ? rk_rec32(a.jk32 + brec.x + ib * brec.y)
                               : rk_pp32(a.pprims[q.bra_pp + ib], q.bsw);
        const PrimF32 kp = rec ? rk_rec32(a.jk32 + krec.x + ik * krec.y)
                               : rk_pp32(a.pprims[q.ket_pp + ik], q.ksw);
        if constexpr (mode_b64(MODE)) {
          const PrimPairJKds* bds = rec ? a.jkds + brec.x + ib * brec.y : nullptr;
          const PrimPairJKds* kds = rec ? a.jkds + krec.x + ik * krec.y : nullptr;
          kept += rk_prim_b64<C>(a, q, bp, kp, bds, kds, q.bra_pp + ib, q.ket_pp + ik, scr, acc)
                      ? 1
                      : 0;
        } else {
          kept += rk_prim<C, ATT>(a, q, bp, kp, q.bra_pp + ib, q.ket_pp + ik, scr, acc) ? 1 : 0;
        }
      } else {
        kept += rk_prim<C, ATT>(a, q, ib, ik, scr, acc) ? 1 : 0;
      }
      ib += gb;
      ik += gk;
      if (ik >= q.nkpp) {
        ik -= q.nkpp;
        ++ib;
      }
    }
    if (G > 1) {
      for (int o = G >> 1; o > 0; o >>= 1) {
#pragma unroll
        for (int i = 0; i < C::kNacc; ++i) acc[i] += rk_shfl_xor<T>(gmask, acc[i], o, G);
        kept += __shfl_xor_sync(gmask, kept, o, G);
      }
    }
    if (g == 0) my_prims += (unsigned long long)kept;
    if (mode_store(MODE) && a.is_null && g == 0) a.is_null[orig] = kept == 0 ? 1 : 0;
    if (kept == 0) {
      if (MODE == kModeSchwarz && g == 0) a.kschwarz[outoff] = 0.0;
      continue;
    }
    T cart[C::kNcart];
    C::template hrr<T>(acc, q.AB, q.CD, cart);
    T v[C::kNsph];
    C::template sph<T>(cart, v);
    if (MODE == kModeSchwarz) {
      double mx = 0;
#pragma unroll
      for (int e = 0; e < C::kNsph; ++e) mx = fmax(mx, fabs(rk_f64(v[e])));
      if (g == 0) a.kschwarz[outoff] = sqrt(mx);
    } else if (mode_store(MODE)) {
      const int fl = flags >> 2;
      const bool sbk = fl & 1, stb = (fl >> 1) & 1, stk = (fl >> 2) & 1;
      int perm[4];
      perm[0] = sbk ? (stk ? 3 : 2) : (stb ? 1 : 0);
      perm[1] = sbk ? (stk ? 2 : 3) : (stb ? 0 : 1);
      perm[2] = sbk ? (stb ? 1 : 0) : (stk ? 3 : 2);
      perm[3] = sbk ? (stb ? 0 : 1) : (stk ? 2 : 3);
      const int dims[4] = {N0, N1, N2, N3};
      int tn[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) tn[perm[t]] = dims[t];
      double* o = a.out + outoff;
#pragma unroll
      for (int e = 0; e < C::kNsph; ++e) {
        if ((e & (G - 1)) != g) continue;
        const int ci[4] = {e / (N1 * N2 * N3), (e / (N2 * N3)) % N1, (e / N3) % N2, e % N3};
        int it[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) it[perm[t]] = ci[t];
        o[((it[0] * tn[1] + it[1]) * tn[2] + it[2]) * tn[3] + it[3]] = rk_f64(v[e]);
      }
    } else if (mode_jk(MODE)) {
      const T deg = T((q.sh[0] == q.sh[1] ? 1 : 2) * (q.sh[2] == q.sh[3] ? 1 : 2) *
                      (bpair == kpair ? 1 : 2));
      const int nbf = a.nbf;
      const size_t o0 = a.basis.bf_off[q.sh[0]], o1 = a.basis.bf_off[q.sh[1]];
      const size_t o2 = a.basis.bf_off[q.sh[2]], o3 = a.basis.bf_off[q.sh[3]];
      T* tag = nullptr;
#define V_(i, j, k, l) v[(((i) * N1 + (j)) * N2 + (k)) * N3 + (l)]
      int slot = 0;
      // J(a,b) += sum_cd D(c,d) v
      {
        T Dcd[N2 * N3];
#pragma unroll
        for (int k = 0; k < N2; ++k)
#pragma unroll
          for (int l = 0; l < N3; ++l) Dcd[k * N3 + l] = rk_D(a, (o2 + k) * nbf + o3 + l, tag);
#pragma unroll
        for (int i = 0; i < N0; ++i)
#pragma unroll
          for (int j = 0; j < N1; ++j, ++slot) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < N2; ++k)
#pragma unroll
              for (int l = 0; l < N3; ++l) s = fma(Dcd[k * N3 + l], V_(i, j, k, l), s);
            if ((slot & (G - 1)) == g) atomicAdd(a.Jacc + (o0 + i) * nbf + o1 + j, rk_f64(deg * s));
          }
      }
      // J(c,d) += sum_ab D(a,b) v
      {
        T Dab[N0 * N1];
#pragma unroll
        for (int i = 0; i < N0; ++i)
#pragma unroll
          for (int j = 0; j < N1; ++j) Dab[i * N1 + j] = rk_D(a, (o0 + i) * nbf + o1 + j, tag);
#pragma unroll
        for (int k = 0; k < N2; ++k)
#pragma unroll
          for (int l = 0; l < N3; ++l, ++slot) {
            T s = 0;
#pragma unroll
            for (int i = 0; i < N0; ++i)
#pragma unroll
              for (int j = 0; j < N1; ++j) s = fma(Dab[i * N1 + j], V_(i, j, k, l), s);
            if ((slot & (G - 1)) == g) atomicAdd(a.Jacc + (o2 + k) * nbf + o3 + l, rk_f64(deg * s));
          }
      }
      // K(a,c) += sum_bd D(b,d) v ; K(b,d) += sum_ac D(a,c) v
      {
        T Dbd[N1 * N3], Dac[N0 * N2];
#pragma unroll
        for (int j = 0; j < N1; ++j)
#pragma unroll
          for (int l = 0; l < N3; ++l) Dbd[j * N3 + l] = rk_D(a, (o1 + j) * nbf + o3 + l, tag);
#pragma unroll
        for (int i = 0; i < N0; ++i)
#pragma unroll
          for (int k = 0; k < N2; ++k) Dac[i * N2 + k] = rk_D(a, (o0 + i) * nbf + o2 + k, tag);
#pragma unroll
        for (int i = 0; i < N0; ++i)
#pragma unroll
          for (int k = 0; k < N2; ++k, ++slot) {
            T s = 0;
#pragma unroll
            for (int j = 0; j < N1; ++j)
#pragma unroll
              for (int l = 0; l < N3; ++l) s = fma(Dbd[j * N3 + l], V_(i, j, k, l), s);
            if ((slot & (G - 1)) == g) atomicAdd(a.Kacc + (o0 + i) * nbf + o2 + k, rk_f64(deg * s));
          }
#pragma unroll
        for (int j = 0; j < N1; ++j)
#pragma unroll
          for (int l = 0; l < N3; ++l, ++slot) {
            T s = 0;
#pragma unroll
            for (int i = 0; i < N0; ++i)
#pragma unroll
              for (int k = 0; k < N2; ++k) s = fma(Dac[i * N2 + k], V_(i, j, k, l), s);
            if ((slot & (G - 1)) == g) atomicAdd(a.Kacc + (o1 + j) * nbf + o3 + l, rk_f64(deg * s));
          }
      }
      // K(a,d) += sum_bc D(b,c) v ; K(b,c) += sum_ad D(a,d) v
      {
        T Dbc[N1 * N2], Dad[N0 * N3];
#pragma unroll
        for (int j = 0; j < N1; ++j)
#pragma unroll
          for (int k = 0; k < N2; ++k) Dbc[j * N2 + k] = rk_D(a, (o1 + j) * nbf + o2 + k, tag);
#pragma unroll
        for (int i = 0; i < N0; ++i)
#pragma unroll
          for (int l = 0; l < N3; ++l) Dad[i * N3 + l] = rk_D(a, (o0 + i) * nbf + o3 + l, tag);
#pragma unroll
        for (int i = 0; i < N0; ++i)
#pragma unroll
          for (int l = 0; l < N3; ++l, ++slot) {
            T s = 0;
#pragma unroll
            for (int j = 0; j < N1; ++j)
#pragma unroll
              for (int k = 0; k < N2; ++k) s = fma(Dbc[j * N2 + k], V_(i, j, k, l), s);
            if ((slot & (G - 1)) == g) atomicAdd(a.Kacc + (o0 + i) * nbf + o3 + l, rk_f64(deg * s));
          }
#pragma unroll
        for (int j = 0; j < N1; ++j)
#pragma unroll
          for (int k = 0; k < N2; ++k, ++slot) {
            T s = 0;
#pragma unroll
            for (int i = 0; i < N0; ++i)
#pragma unroll
              for (int l = 0; l < N3; ++l) s = fma(Dad[i * N3 + l], V_(i, j, k, l), s);
            if ((slot & (G - 1)) == g) atomicAdd(a.Kacc + (o1 + j) * nbf + o2 + k, rk_f64(deg * s));
          }
      }
#undef V_
    }
  }
  if (a.prim_count && my_prims) atomicAdd(a.prim_count, my_prims);
}

// Launch of one register kernel: occupancy-sized grid, capped by the work.
template <typename T, int LA, int LB, int LC, int LD, int MODE, bool ATT = false>
cudaError_t rk_launch_one(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  const int block = 128;
  auto k = rk_kernel<T, LA, LB, LC, LD, MODE, ATT>;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, block, 0) != cudaSuccess || occ < 1)
    occ = 1;
  if (a.max_bps > 0 && occ > a.max_bps) occ = a.max_bps;
  long long grid = (long long)nsm * occ;
  const long long need = (work * a.group + block - 1) / block;
  if (need < grid) grid = need < 1 ? 1 : need;
  k<<<(unsigned)grid, block, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t rk_launch(bool fp32, int mode, bool att, int la, int lb, int lc, int ld,
                      const EriArgs& a, long long work, int nsm, cudaStream_t st);
bool rk_available(bool fp32, int mode, bool att, int la, int lb, int lc, int ld);

}  // namespace lgx
