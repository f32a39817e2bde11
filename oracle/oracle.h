// oracle/oracle.h -- TEST INFRASTRUCTURE ONLY.
//
// FP64 CPU restatement of libint's Coulomb ERI path (libint2::Engine
// compute2<Operator::coulomb, BraKet::xx_xx, 0|1>), used by tests/ as the
// checker of the CUDA path, by __graft_entry__.smoke() and by bench.py's
// cpu_baseline / --impl reference arm.  The product (libint_gb300/) never
// links, loads or calls it.
//
// Reference anchors (paths inside the libint tree):
//   Shell::renorm                     include/libint2/shell.h:958-999
//   ShellPair::init (Original/Cons.)  include/libint2/shell.h:1138-1256
//   Boys F_m(T) (Taylor + recursion)  include/libint2/boys.h:519-879
//   primitive-quartet data/screening  include/libint2/engine.impl.h:1306-1766
//   canonical swap / un-permutation   include/libint2/engine.impl.h:1181-1211,1988-2086
//   OS VRR                            src/bin/libint/vrr_11_twoprep_11.h:88-666
//   contraction point (e0|f0)         src/bin/libint/dg.cc:1177-1189
//   HRR                               src/bin/libint/hrr.h:246-347
//   derivative shell-set order/remap  include/libint2/deriv_map.h:170-262
//   solid harmonics (IJQC 54,83 eq15) include/libint2/solidharmonics.h:114-174
//   J/K digestion, Schwarz            tests/hartree-fock/hartree-fock++.cc:1231-1298,1574-1772
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Boys function F_m(T), m = 0..mmax (mmax <= 40).
void orc_boys(double T, int mmax, double* F);
/* Operator of every later oracle call: 0 coulomb, 1 erf(omega r)/r,
 * 2 erfc(omega r)/r (libint's erf/erfc_coulomb core integrals,
 * include/libint2/boys.h:1913-1980).  Process-wide.  Returns 0 or -1. */
int orc_set_operator(int op, double omega);

// Shell::renorm(): embeds primitive normalization and rescales the
// contraction to unit self-overlap.  coeff_out/max_ln_coeff_out: nprim each.
void orc_shell_normalize(int l, int nprim, const double* alpha,
                         const double* coeff_in, double* coeff_out,
                         double* max_ln_coeff_out);

// Real solid-harmonic coefficient of Cartesian (lx,ly,lz) in S_{l,m}
// (standard Cartesian normalization, standard m = -l..l ordering).
double orc_solid_coeff(int l, int m, int lx, int ly, int lz);

// ShellPair::init with Original (0) or Conservative (1) screening.
// Per surviving primitive pair writes P[3], K, 1/gamma, nonsph, ln_scr, p1, p2.
int orc_shellpair_init(int l1, int nprim1, const double* alpha1,
                       const double* coeff1, const double* O1, int l2,
                       int nprim2, const double* alpha2, const double* coeff2,
                       const double* O2, double ln_prec, int method, double* P,
                       double* K, double* oogamma, double* nonsph,
                       double* ln_scr, int* p1, int* p2);

// A basis: nshell shells, flattened primitive data (normalized coefficients).
typedef struct {
  int nshell;
  const int* l;         // [nshell]
  const int* pure;      // [nshell]
  const int* nprim;     // [nshell]
  const int* prim_off;  // [nshell] offset into alpha/coeff
  const int* atom;      // [nshell] atom index of the shell centre
  const double* O;      // [3*nshell]
  const double* alpha;  // flattened
  const double* coeff;  // flattened, normalization embedded
} orc_basis;

// Engine::compute(s1,s2,s3,s4) for shells given by index into the basis.
// precision: Engine::set_precision(); method: 0 Original, 1 Conservative.
// Writes nsets (1 or 12) shell sets in libint's buffer order to out.
// Returns the number of values per set, or 0 if every primitive quartet was
// screened out (libint returns results()[0] == nullptr), <0 on error.
int orc_compute_quartet(const orc_basis* bs, int s1, int s2, int s3, int s4,
                        int deriv, double precision, int method, double* out);

// As orc_compute_quartet (deriv 0 or 1) with the primitive pairs built at
// pair_precision (precomputed ShellPair data, engine.impl.h:1259-1276) and
// the primitive quartets screened at precision.
int orc_compute_quartet_pairs(const orc_basis* bs, int s1, int s2, int s3, int s4, int deriv,
                              double precision, double pair_precision, int method, double* out);

// Schwarz factors K(s1,s2) = sqrt(max|(s1 s2|s1 s2)|) (precision 0).
void orc_schwarz(const orc_basis* bs, double* K, int nthreads);

// J/K build over unique shell quartets with |K12*K34| >= schwarz_thresh,
// FP64 digestion with the 8-fold degeneracy factors.  D, J, K: nbf x nbf,
// row-major.  bf_off: [nshell] first basis function of each shell.
// Returns the number of computed (non-screened) shell quartets.
int64_t orc_jk(const orc_basis* bs, const int* bf_off, int nbf,
               const double* Kschwarz, double schwarz_thresh, const double* D,
               double* J, double* K, int nthreads);

// Per-thread J/K accumulators that persist across calls (one nbf x nbf pair
// per thread, as compute_2body_fock keeps one G per thread,
// hartree-fock++.cc:1601-1607): create, add the contributions of listed bra
// shell pairs (canonical pair indices s1 (s1+1)/2 + s2, s2 <= s1; returns
// the computed quartets and their integral count), reduce into J/K (adds
// the symmetrised sums), destroy.  ket_mask: NULL, or one flag per pair
// index restricting the ket pairs; fock_precision > 0: compute_2body_fock's
// density-weighted screening (hartree-fock++.cc:1640-1684), 0: off.
typedef struct orc_jk_acc orc_jk_acc;
orc_jk_acc* orc_jk_acc_create(int nbf, int nthreads);
void orc_jk_acc_destroy(orc_jk_acc* acc);
int64_t orc_jk_acc_pairs(orc_jk_acc* acc, const orc_basis* bs, const int* bf_off,
                         const double* Kschwarz, double schwarz_thresh, const double* D,
                         const int64_t* bra_pairs, int64_t n_bra_pairs,
                         const unsigned char* ket_mask, double fock_precision,
                         int64_t* n_integrals);
void orc_jk_acc_reduce(const orc_jk_acc* acc, double* J, double* K);

// Counts of the screened pass: unique quartets with K12 K34 >= thresh and
// their integrals (no integral is computed).
void orc_count_screened(const orc_basis* bs, const double* Kschwarz, double schwarz_thresh,
                        int64_t* n_quartets, int64_t* n_integrals);

// The benchmark configurations' synthetic water cluster (Z [3n], xyz [9n]
// bohr, atoms O, H, H per molecule) from mt19937_64(seed); 0 or -1.
int orc_water_cluster(int nx, int ny, int nz, double spacing, double jitter, uint64_t seed,
                      int* Z, double* xyz);

// As orc_jk, but only over the quartets [q_begin, q_end) of the canonical
// quartet enumeration (used to time a bounded sample); J/K accumulate.
int64_t orc_jk_sample(const orc_basis* bs, const int* bf_off, int nbf,
                      const double* Kschwarz, double schwarz_thresh,
                      const double* D, double* J, double* K, int nthreads,
                      int64_t bra_pair_begin, int64_t bra_pair_end,
                      int64_t* n_integrals);

// Nuclear gradients of E_J = 1/2 sum D J and E_K = -1/4 sum D K from
// deriv_order=1 integrals.  gJ, gK: natoms x 3.
int64_t orc_jk_grad(const orc_basis* bs, const int* bf_off, int nbf,
                    int natoms, const double* Kschwarz, double schwarz_thresh,
                    const double* D, double* gJ, double* gK, int nthreads);

#ifdef __cplusplus
}
#endif
