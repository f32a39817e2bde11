// Per-angular-momentum-class "programs" for the warp-cooperative ERI kernel.
//
// For one canonical class (la>=lb, lc>=ld, la+lb<=lc+ld, libint's generated
// set, build_libint.cc:1019-1021) and derivative order, the builder
//  * forms the Obara-Saika VRR dependency DAG of every needed (e0|f0)^(0)
//    (src/bin/libint/vrr_11_twoprep_11.h:145-223,305-383: build on A first,
//    then on C with the (e-1_j 0|f-1_j 0)^(m+1) coupling term),
//  * schedules it as-soon-as-possible into levels (all nodes of a level are
//    independent, so the 32 lanes of a warp split them),
//  * assigns shared-memory slots with liveness-based reuse,
//  * emits the contraction ("accumulate") ops at the (e0|f0) point
//    (src/bin/libint/dg.cc:1177-1189), and
//  * emits the post-contraction program: HRR on the bra then the ket
//    (src/bin/libint/hrr.h:246-347), and for deriv_order 1 the Gaussian
//    derivative rule with exponent-weighted contracted sets and the
//    translational-invariance closure for centre C
//    (src/bin/libint/master_rrs_list.h:52-55).
// Op words are plain integers so the device kernel interprets them with
// warp-uniform control flow.
#pragma once
#include <cstdint>
#include <vector>

namespace lgx {

constexpr int kMaxL = 3;
// Class programs also serve one more angular momentum quantum: the
// Cartesian raised shells of the second-derivative composition.
constexpr int kMaxLInternal = kMaxL + 1;
constexpr int kMaxDeriv = 1;
constexpr int kMaxNprim = 16;

// Slots are 32-bit indices into a per-warp array of T.
// VRR op (8 words): dst, s1, s2, s3, s4, s5,
//   flags = kind(bit0: 0 build-on-A, 1 build-on-C) | dir<<1 | n1<<3 | ne<<8, 0
// value = c1*s1 + c2*s2 [+ n1*c3*(s3 - c4*s4)] [+ ne*c5*s5]
// A-build: c1=PA_i c2=WP_i c3=1/(2zeta) c4=rho/zeta
// C-build: c1=QC_j c2=WQ_j c3=1/(2eta)  c4=rho/eta  c5=1/(2(zeta+eta))
// Accumulate op (2 words): acc, src | weight<<30
//   (weight 0: 1, 1: 2*alpha_A, 2: 2*alpha_B, 3: 2*alpha_D)
// Post op (4 words): dst, s1, s2, kind | dir<<4 | n<<8
enum PostKind : uint32_t {
  kHrrBra = 0,   // dst = s1 + AB_dir * s2
  kHrrKet = 1,   // dst = s1 + CD_dir * s2
  kDeriv = 2,    // dst = s1 - n * s2   (n == 0: dst = s1)
  kCopy = 4      // dst = s1
};

struct ClassProgramHost {
  int la, lb, lc, ld, deriv, mmax, nweights;
  int nacc;          // accumulator slots [0, nacc)
  int nwork;         // work slots [nacc, nacc + nwork)
  int vrr_work;      // of which the VRR stage uses [nacc, nacc + vrr_work)
  int leaf_slot0;    // F_m * pfac written to leaf_slot0 + m
  int nphases;       // post phases: 1 (deriv 0) or 3 (centres A, B, D)
  int sets_per_phase;// Cartesian sets produced per phase: 1 or 3 (x, y, z)
  int ncart4;        // Cartesian values per set
  int cart_out;      // first slot of the sets_per_phase*ncart4 outputs
  int cbuf;          // deriv 1: 3*ncart4 slots accumulating -(dA+dB+dD)
  int sph_tmp;       // first slot of an ncart4 scratch area
  std::vector<uint32_t> vrr_ops;   // 8 words per op
  std::vector<int> vrr_lev;        // op offsets per level (size nlev+1)
  std::vector<uint32_t> acc_ops;   // 2 words per op
  std::vector<int> acc_lev;        // acc op offsets per level (size nlev+1)
  std::vector<uint32_t> post_ops;  // 4 words per op
  std::vector<int> post_lev;       // post op offsets per level, all phases
  std::vector<int> phase_lev;      // first post level of each phase (+end)
  int64_t vrr_flops = 0;           // FP operations per primitive quartet
  int64_t post_flops = 0;          // FP operations per contracted quartet
  int total_slots() const { return nacc + nwork; }
};

// Builds the program of one canonical class; throws std::runtime_error on
// invalid input.
ClassProgramHost build_class_program(int la, int lb, int lc, int ld, int deriv);

// Index of a canonical class in [0, num_classes()).
int class_index(int la, int lb, int lc, int ld);
int num_classes();

}  // namespace lgx
