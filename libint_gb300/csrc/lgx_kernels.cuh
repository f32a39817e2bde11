// Kernel argument structures shared by the launchers (lgx_api.cu) and the
// kernels (lgx_kernels.cu).
#pragma once
#include "lgx_device.cuh"

namespace lgx {

enum KernelMode : int {
  kModeStore = 0,    // write shell sets in libint buffer order
  kModeSchwarz = 1,  // K(pair) = sqrt(max |(ab|ab)|)
  kModeJK = 2,       // digest into J/K accumulators (deriv 0)
  kModeGrad = 3,     // digest first derivatives into gJ/gK (deriv 1)
  // FP32 kernels of the mixed scheme with the Boys function in FP64: the
  // argument T = rho |P - Q|^2, F_m(T) (Taylor / asymptotic branch, e^{-T}
  // and the downward recursion) in FP64 from the FP64 pair data, then the
  // VRR / HRR / contraction in FP32; otherwise as kModeJK / kModeStore
  kModeJKB64 = 4,
  kModeStoreB64 = 5
};
__host__ __device__ constexpr bool mode_jk(int m) { return m == kModeJK || m == kModeJKB64; }
__host__ __device__ constexpr bool mode_store(int m) {
  return m == kModeStore || m == kModeStoreB64;
}
__host__ __device__ constexpr bool mode_b64(int m) {
  return m == kModeJKB64 || m == kModeStoreB64;
}

// Explicit work item: one shell quartet in canonical orientation.
struct QuartetItem {
  int bra_pair, ket_pair;  // pair-table indices
  int flags;               // bit0 bra swapped, bit1 ket swapped,
                           // bits 2..4 (swap_braket, swap_tbra, swap_tket)
  int pad;
  long long out;           // output offset (doubles) or K index (Schwarz)
};

// Implicit work: one class bin of the screened J/K quartet space as a list
// of segments.  A segment is one bra pair with a contiguous run of ket
// pairs of one contraction-depth group; segments are ordered by (bra depth
// group, ket depth group, bra pair) so consecutive quartets share their
// primitive counts.
struct BinWork {
  const int* bra_pairs;        // pair ids of the bra class (depth, K desc)
  const int* ket_pairs;        // pair ids of the ket class (depth, K desc)
  const long long* seg_start;  // [nseg+1] prefix sums of segment lengths
  const int* seg_bra;          // bra index (into bra_pairs) of each segment
  const int* seg_j0;           // first ket index (into ket_pairs)
  int nseg;
  int pad;
  long long total;
  // FP32 records (EriArgs::jk32) of list position i: jk32[rec[i].x + ip * rec[i].y]
  const int2* bra_rec;
  const int2* ket_rec;
};

// Segment containing quartet q (binary search over seg_start).
__device__ __forceinline__ int bin_segment(const BinWork& b, long long q) {
  int lo = 0, hi = b.nseg;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b.seg_start[mid] <= q) lo = mid; else hi = mid;
  }
  return lo;
}

// Staging row of one primitive quartet (the VRR inputs, libint's Libint_t
// prefactors: engine.impl.h:1389-1757), written by the kernels' prologue or,
// for caller-supplied primitive data, packed on the host.
constexpr int kStage = 36;        // values staged per primitive quartet
constexpr int kStF = 0;           // (00|00)^(m) = F_m * pfac, m <= 15
constexpr int kStMaxM = 15;
constexpr int kStPA = 16, kStWP = 19, kStQC = 22, kStWQ = 25;
constexpr int kStOo2z = 28, kStRoz = 29, kStOo2e = 30, kStRoe = 31, kStOo2ze = 32;
constexpr int kStW = 33;          // 2 alpha_A, 2 alpha_B, 2 alpha_D

// Threads of the block-cooperative single-quartet kernels (prim_set_kernel,
// eri_block_store_kernel).
constexpr int kBlockThreads = 256;

// One contracted Cartesian shell set from staged primitive quartets in the
// canonical orientation (prim_set_kernel).
struct PrimSetArgs {
  DevProg prog;
  const double* rows;   // [nrows][kStage]
  int nrows;
  int stage_rows;       // rows staged in shared memory per batch
  double AB[3], CD[3];  // canonical A - B, C - D
  int perm[4];          // canonical position k -> caller position perm[k]
  double* slots;        // global slot scratch, or nullptr for shared memory
  double* out;          // nsets x ncart(l1) ncart(l2) ncart(l3) ncart(l4), caller order
  // warp_rows: each warp contracts its own rows into its own accumulators
  // (stage and slot_stride slots per warp in shared memory), summed into
  // warp 0's before the post program; for small classes with many rows
  int warp_rows;
  int slot_stride;
};

struct EriArgs {
  DevBasis basis;
  const PairRec* pairs;
  const PrimPairRec* pprims;
  const PrimPairJKds* ppds;  // double-float P and zeta per primitive pair (pprims index)
  const PrimPairJK32* jk32;  // J/K bins: coalesced FP32 records (may be null)
  const PrimPairJKds* jkds;  // J/K bins: their double-float P and zeta (same layout)
  const unsigned char* pair_swap;  // per pair: 1 if its canonical bra1 is s2
  DevProg prog;
  const double* boys;     // [kBoysRows][kBoysCols] F_m(T_k)
  const double* boys_tay; // pre-divided Taylor table (kBoysTaylorStride)
  const float* boys32;    // FP32 copy of the Boys table
  const double* inv_odd;  // 1/(2m+1), m < 40
  // Cartesian -> solid harmonics, sparse: nonzeros of row (l, p) are
  // [sph_off[l*9+p], sph_off[l*9+p+1]) with Cartesian index sph_c[] and
  // coefficient sph_cd[] (FP64) / sph_cf[] (FP32)
  const int* sph_off;
  const int* sph_c;
  const double* sph_cd;
  const float* sph_cf;
  // screening (FP32 copies for the FP32 kernels)
  double precision, ln_prec;
  float fprecision, fln_prec;
  int screening;  // 0 Original, 1 Conservative
  // two-body operator: 0 coulomb 1/r, 1 erf(omega r)/r, 2 erfc(omega r)/r
  // (attenuated: program kernel instantiations and the ATT register kernels)
  int op;
  double omega2;  // omega^2
  // work
  const QuartetItem* items;
  long long nitems;
  BinWork bin;
  int implicit;   // 1: use bin, 0: use items
  int chunk;
  int group;           // register kernels: lanes per quartet (power of 2)
  int max_bps;         // host-side launch cap: blocks per SM (0: occupancy limit)
  unsigned long long* counter;
  // slots
  int slot_stride;     // slots per warp (elements of T)
  int stage_rows;      // program kernel: primitive quartets staged per batch (8, 16 or 32)
  int global_slots;    // 1: slots live in gscratch
  int warp_rows;       // block store kernel: each warp contracts its own primitive quartets
  void* gscratch;      // [nwarps_total][slot_stride] of T
  // outputs
  double* out;         // kModeStore
  int* is_null;        // kModeStore, per item (may be null)
  double* kschwarz;    // kModeSchwarz
  const double* D;     // kModeJK / kModeGrad
  const float* Df;     // FP32 copy of D (FP32 register kernels)
  double* Jacc;
  double* Kacc;
  double* gJ;
  double* gK;
  int nbf;
  // density-weighted screening of the J/K passes (fock_prec > 0): shell-
  // block infinity norms of D (nshell x nshell), Schwarz factor per pair
  const double* dsh;
  const double* kpair;
  double fock_prec;
  // watchdog: a bounded number of work chunks per warp
  long long max_chunks;
  int* error_flag;
  // statistics: primitive quartets computed (one atomic per thread)
  unsigned long long* prim_count;
};

// Primitive-screening thresholds of one shell quartet (Engine::set_precision:
// precision and its logarithm, with FP32 copies).
struct PrimScreen {
  double prec, ln_prec;
  float fprec, fln_prec;
};

// Primitive-quartet screening decisions that are the FP64 ones at FP32 cost
// (engine.impl.h:1306-1466: ln_scr12 + ln_scr34 > ln(precision), then
// |prefactor| >= precision).  The FP32 sum of the pairs' logarithms (|value|
// <= ~50: rounding below 1e-5) and the FP32 prefactor (below 1e-6 relative)
// decide, except inside a band around the threshold (3e-5 in the logarithm,
// 4e-6 relative in the prefactor), where the FP64 values of the two pairs'
// records (PrimPairRec bidx, kidx) decide.  A primitive quartet at the
// threshold can carry ~100x the threshold (the prefactor bounds only its
// (ss|ss) part), so with a coarse precision (density-weighted screening) an
// FP32 decision that went the other way would show in J/K.
constexpr float kLnBand = 3e-5f;
constexpr float kPfBand = 4e-6f;
__device__ __forceinline__ bool ln_kept(const EriArgs& a, float fsum, long long bidx,
                                        long long kidx, const PrimScreen& s) {
  const float dl = fsum - s.fln_prec;
  if (dl >= kLnBand) return true;
  if (dl <= -kLnBand) return false;
  return a.pprims[bidx].ln_scr + a.pprims[kidx].ln_scr > s.ln_prec;
}
// mag: the FP32 |prefactor| times scale (1, or the Conservative factor).
__device__ __forceinline__ bool pf_kept(const EriArgs& a, float mag, double scale, long long bidx,
                                        long long kidx, const PrimScreen& s) {
  if (mag >= s.fprec * (1.0f + kPfBand)) return true;
  if (mag < s.fprec * (1.0f - kPfBand)) return false;
  const PrimPairRec& b = a.pprims[bidx];
  const PrimPairRec& k = a.pprims[kidx];
  return fabs(b.Kc * k.Kc * rsqrt(b.zeta + k.zeta)) * scale >= s.prec;
}

// The thresholds of the pass, or with density-weighted screening
// (EriArgs::fock_prec > 0) those of compute_2body_fock
// (tests/hartree-fock/hartree-fock++.cc:1640-1684): Dnorm1234 = the largest
// infinity norm of the six shell blocks of D the quartet touches; the quartet
// is skipped when Dnorm1234 K12 K34 < fock_prec (returns false), else its
// primitives are screened at fock_prec / Dnorm1234 and its logarithm, both
// in FP64 as Engine::set_precision forms them (not below the precision the
// pair data were built with); the primitive decisions are then the FP64
// ones in every kernel (ln_kept, pf_kept).
__device__ __forceinline__ bool quartet_screen(const EriArgs& a, const int* sh, int bpair,
                                               int kpair, PrimScreen& s) {
  s.prec = a.precision;
  s.ln_prec = a.ln_prec;
  s.fprec = a.fprecision;
  s.fln_prec = a.fln_prec;
  if (!(a.fock_prec > 0.0)) return true;
  const int ns = a.basis.nshell;
  const double* d = a.dsh;
  const double dn = fmax(fmax(fmax(d[sh[0] * ns + sh[1]], d[sh[0] * ns + sh[2]]),
                              fmax(d[sh[1] * ns + sh[2]], d[sh[0] * ns + sh[3]])),
                         fmax(d[sh[1] * ns + sh[3]], d[sh[2] * ns + sh[3]]));
  if (dn * __ldg(a.kpair + bpair) * __ldg(a.kpair + kpair) < a.fock_prec) return false;
  const double q = a.fock_prec / dn;  // dn > 0: a zero norm failed the test above
  if (q > s.prec) {
    s.prec = q;
    s.ln_prec = log(q);
    s.fprec = __double2float_rn(q);
    s.fln_prec = __double2float_rn(s.ln_prec);
  }
  return true;
}

}  // namespace lgx
