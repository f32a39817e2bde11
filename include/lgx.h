/* lgx.h -- C ABI of the GB300-native Coulomb ERI library (liblgx.so).
 *
 * The library computes two-electron Coulomb repulsion integrals (ERIs) over
 * contracted Gaussian shells on one NVIDIA GB300 (sm_103a), with the buffer
 * layout and conventions of libint2::Engine (Operator::coulomb and the
 * attenuated erf / erfc operators, BraKet::xx_xx, deriv_order 0, 1 and 2),
 * libint's generated per-quartet entry (libint2_build_eri*, through
 * lgx_compute_primitive_set), plus batched and fused J/K entry points.  Plain C types only; every call returns an lgx_status and never
 * aborts.  A context is bound to one CUDA device and one CUDA stream; calls
 * on one context are serialized, distinct contexts may be used from distinct
 * threads (the reference's one-Engine-per-thread model).
 *
 * Conventions shared with the reference (file:line inside the libint tree):
 *  - shells carry normalization-embedded contraction coefficients
 *    (Shell::renorm, include/libint2/shell.h:958-999);
 *  - Cartesian components in the standard order
 *    (include/libint2/cgshell_ordering.h:125-131), solid harmonics in the
 *    standard m = -l..l order (include/libint2/shgshell_ordering.h:56);
 *  - shell sets are row-major n1*n2*n3*n4 in the caller's shell order
 *    (include/libint2/engine.h:747-781); first-derivative sets come as 12
 *    sets ordered A_x,A_y,A_z,B_x,...,D_z
 *    (include/libint2/deriv_map.h:170-262, build_libint.cc:1062-1085).
 */
#ifndef LGX_H
#define LGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int lgx_status;
#define LGX_OK 0
#define LGX_ERR_INVALID_ARG 1   /* bad pointer / size / argument            */
#define LGX_ERR_CUDA 2          /* a CUDA runtime call failed                */
#define LGX_ERR_LMAX_EXCEEDED 3 /* Engine::lmax_exceeded (engine.h:893-905)  */
#define LGX_ERR_NO_BASIS 4      /* batched call before lgx_set_basis         */
#define LGX_ERR_WATCHDOG 5      /* a device-side bounded wait expired        */
#define LGX_ERR_TOO_LARGE 6     /* request exceeds a documented size limit   */
#define LGX_ERR_NO_DEVICE 7     /* no CUDA device / wrong architecture       */

/* Largest angular momentum per shell and derivative order supported
 * (deriv_order 2 through lgx_compute_shellset and
 * lgx_compute_primitive_set). */
#define LGX_MAX_L 3
#define LGX_MAX_DERIV 2
#define LGX_MAX_NPRIM 16

/* Primitive-screening methods (ScreeningMethod, shell.h:1041-1059). */
#define LGX_SCREEN_ORIGINAL 0
#define LGX_SCREEN_CONSERVATIVE 1

/* Precision modes of the batched paths.  In both mixed modes a quartet whose
 * Schwarz bound K12*K34 is below mixed_thresh runs its VRR, HRR, contraction
 * and solid-harmonic transform in FP32, every other quartet entirely in FP64,
 * and J/K are accumulated in FP64.  LGX_MIXED keeps the Boys function of
 * the FP32 quartets in FP64 (its argument T, the Taylor or asymptotic
 * branch, e^{-T} and the downward recursion; Coulomb operator);
 * LGX_MIXED_FP32_BOYS evaluates it in FP32 as well (faster, less exact). */
#define LGX_FP64 0
#define LGX_MIXED 1
#define LGX_MIXED_FP32_BOYS 2

/* Two-body operators (libint2::Operator, include/libint2/engine.h:98-184). */
#define LGX_OP_COULOMB 0       /* 1/r                                        */
#define LGX_OP_ERF_COULOMB 1   /* erf(omega r)/r  (Operator::erf_coulomb)    */
#define LGX_OP_ERFC_COULOMB 2  /* erfc(omega r)/r (Operator::erfc_coulomb)   */

typedef struct lgx_context lgx_context;

/* One contracted shell (libint2::Shell with one contraction). */
typedef struct {
  int32_t l;            /* angular momentum, 0..LGX_MAX_L                    */
  int32_t pure;         /* 1: solid harmonics, 0: Cartesian                  */
  int32_t nprim;        /* 1..LGX_MAX_NPRIM                                  */
  int32_t pad_;
  double origin[3];     /* bohr                                              */
  const double* alpha;  /* [nprim] exponents                                 */
  const double* coeff;  /* [nprim] normalization-embedded coefficients       */
} lgx_shell;

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device` (replaces libint2::initialize(),
 * include/libint2/initialize.h:76-95, plus Engine construction,
 * engine.h:502-526).  Fails with LGX_ERR_NO_DEVICE when no usable GPU. */
lgx_status lgx_create(lgx_context** ctx, int device);
/* libint2::finalize() counterpart; releases every device resource. */
lgx_status lgx_destroy(lgx_context* ctx);
/* Engine::set(Operator) + Engine::set_params(omega) (engine.h:658-700) for
 * every later call on the context (shell sets, batches, Schwarz factors,
 * J/K and gradient passes): op is one of LGX_OP_*, omega >= 0 the range-
 * separation parameter of erf/erfc (ignored for coulomb).  The attenuated
 * operators use libint's core integrals (boys.h:1913-1980) on the program
 * kernel; changing the operator drops the context's Schwarz factors and
 * quartet bins. */
lgx_status lgx_set_operator(lgx_context* ctx, int op, double omega);

/* The Boys function F_m(T) = int_0^1 u^{2m} exp(-T u^2) du, m = 0..mmax, of
 * n arguments T[i] >= 0 (HOST arrays; F is n x (mmax+1), row-major),
 * evaluated on the GPU by exactly the device function a class kernel uses:
 * variant 0 the program kernels' FP64 evaluator (mmax <= 16), 1 the
 * register kernels' FP64 evaluator (mmax <= 6), 2 and 3 their FP32
 * counterparts, 4 and 5 the LGX_MIXED scheme's FP64 evaluators of the
 * program and register kernels (4-term series, T as a double-float pair,
 * each value rounded to FP32; mmax <= 16 and <= 6), 6 the register
 * kernels' whole LGX_MIXED path from primitive-pair data: T then holds 8
 * values per argument (Pb.x, Pb.y, Pb.z, zeta, Pk.x, Pk.y, Pk.z, eta;
 * |P| <= 1e4, 1e-10 <= zeta <= 1e10) and the argument is rho |Pb - Pk|^2,
 * rho = zeta eta / (zeta + eta), formed as those kernels form it
 * (double-float records and arithmetic).  All results widened to double.
 * The batch counterpart of libint's FmEval_Taylor / FmEval_Chebyshev7
 * eval(F, T, mmax)
 * (include/libint2/boys.h:345-454,679-821), so the evaluators can be
 * checked against libint's reference values on their own. */
lgx_status lgx_boys(lgx_context* ctx, int variant, const double* T, int64_t n, int mmax,
                    double* F);

/* Device-side watchdog of the program kernels' work loops.  Each warp of a
 * program-kernel launch takes chunks of quartets from a device counter and
 * raises the context's error flag (the call then returns LGX_ERR_WATCHDOG)
 * once it would take more than a bound of chunks; by default (max_chunks
 * < 0) the bound is the launch's whole work plus slack, which a valid launch
 * never reaches.  max_chunks >= 0 replaces that bound on every later launch
 * of the context (0: a warp may take no chunk, so any program-kernel launch
 * with work trips it), so that a test can make the watchdog fire without a
 * fault or a hang: the loop ends, the flag is read and cleared, and the
 * context stays usable.  The counterpart of libint's assert-on-misuse
 * (engine.impl.h:173-174), which aborts instead. */
lgx_status lgx_set_watchdog(lgx_context* ctx, int64_t max_chunks);

/* Message of the last failed call on this context (never NULL). */
const char* lgx_last_error(const lgx_context* ctx);
/* Library version string. */
const char* lgx_version(void);

/* ------------------------------------------------------- Engine::compute */

/* Engine::compute(s1,s2,s3,s4) / compute2<coulomb,xx_xx,deriv>
 * (include/libint2/engine.impl.h:140-175,1151-2113).  `shells` are the four
 * shells in caller order; `precision` is Engine::set_precision()
 * (engine.h:809-823; <= 0 disables primitive screening); `screening` is one
 * of LGX_SCREEN_*.  On success writes *nsets (1 or 12) shell sets of
 * *nvalues doubles each, row-major in the caller's shell order, to the HOST
 * buffer `out` (capacity `out_capacity` doubles), and *is_null = 1 when every
 * primitive quartet was screened out (libint returns results()[0]==nullptr,
 * engine.impl.h:1781-1784; `out` is then untouched). */
/* deriv 2 (compute2<coulomb, xx_xx, 2>): 78 second-derivative sets in
 * libint's order (coordinate pairs c1 <= c2 over A_x..D_z, row-major,
 * CartesianDerivIterator<4>(2) of include/libint2/deriv_iter.h), for shells
 * up to LGX_MAX_L (the raised Cartesian copies of the composition reach
 * LGX_MAX_L + 1 internally). */
lgx_status lgx_compute_shellset(lgx_context* ctx, const lgx_shell shells[4],
                                int deriv, double precision, int screening,
                                double* out, size_t out_capacity, int* nsets,
                                int* nvalues, int* is_null);
/* lgx_compute_shellset (deriv 0 or 1) with the caller's precomputed
 * ShellPair data of Engine::compute2(s1, s2, s3, s4, sp12, sp34)
 * (engine.h:787-791): the reference uses a given ShellPair, instead of
 * recomputing it at the engine precision, when its ln_prec is at most
 * ln(precision) (engine.impl.h:1259-1276).  pair_ln_prec[0] / [1]: the
 * ln_prec the bra (shells 0, 1) / ket (shells 2, 3) primitive pairs are
 * screened at (ShellPair::init with `screening`, shell.h:1138-1256); the
 * primitive quartets are screened at `precision` as in
 * lgx_compute_shellset.  The caller passes ln(precision) for a pair it
 * does not supply. */
lgx_status lgx_compute_shellset_pairs(lgx_context* ctx, const lgx_shell shells[4],
                                      int deriv, double precision, int screening,
                                      const double pair_ln_prec[2], double* out,
                                      size_t out_capacity, int* nsets, int* nvalues,
                                      int* is_null);

/* ------------------------------------ generated-library entry (Libint_t) */

/* One primitive quartet of caller-computed VRR inputs, the per-primitive
 * prefactors a libint caller writes into Libint_t before
 * libint2_build_eri* (engine.impl.h:1389-1757; prep_libint2.h of the
 * reference's test_eri), for shells 1..4 = A, B, C, D in caller order with
 * primitive exponents a1..a4, zeta = a1 + a2, eta = a3 + a4,
 * rho = zeta eta / (zeta + eta), P, Q the bra / ket centres and
 * W = (zeta P + eta Q) / (zeta + eta). */
#define LGX_PRIM_MAX_M 15
typedef struct lgx_prim_quartet {
  double PA[3];        /* P - A                                              */
  double QC[3];        /* Q - C                                              */
  double WP[3];        /* W - P                                              */
  double WQ[3];        /* W - Q                                              */
  double oo2z;         /* 1 / (2 zeta)                                       */
  double oo2e;         /* 1 / (2 eta)                                        */
  double oo2ze;        /* 1 / (2 (zeta + eta))                               */
  double roz;          /* rho / zeta                                         */
  double roe;          /* rho / eta                                          */
  double two_alpha[4]; /* 2 a1 .. 2 a4 (read for derivatives only)           */
  /* (00|00)^(m) = pfac F_m(rho |PQ|^2), m = 0..l1+l2+l3+l4+deriv, with pfac
   * = 2 pi^{5/2} K_AB K_CD / (zeta eta sqrt(zeta + eta)) times the four
   * contraction coefficients (libint's LIBINT_T_SS_EREP_SS(m)) */
  double ss[LGX_PRIM_MAX_M + 1];
} lgx_prim_quartet;

/* The contracted Cartesian shell set (l1 l2|l3 l4) over `nprim` primitive
 * quartets (libint2_build_eri / libint2_build_eri1 with
 * Libint_t::contrdepth = nprim, dg.cc:1177-1189), computed on the GPU with
 * the class's VRR / HRR programs.  AB = A - B, CD = C - D.  deriv 0: one
 * set; deriv 1: 12 sets ordered A_x..D_z (all four centres; centre C by
 * translational invariance as libint's generated code does).  Sets are
 * row-major ncart(l1) ncart(l2) ncart(l3) ncart(l4) in the caller's shell
 * order and Cartesian (no solid-harmonic transform, no renormalisation:
 * the caller's (00|00)^(m) carry it), written to the HOST buffer `out`.
 * deriv 2 (libint2_build_eri2): the 78 sets in
 * libint's CartesianDerivIterator order, composed from the first-derivative
 * sets of the quartets with one shell raised (its primitives weighted by
 * 2 a_X) and lowered, which requires ss[] up to m = l1+..+l4+2. */
lgx_status lgx_compute_primitive_set(lgx_context* ctx, int l1, int l2, int l3, int l4,
                                     int deriv, const lgx_prim_quartet* prims, int nprim,
                                     const double AB[3], const double CD[3], double* out,
                                     size_t out_capacity, int* nsets, int* nvalues);

/* ----------------------------------------------------------- basis state */

/* Uploads a basis (a libint2::BasisSet, basis.h.in:134-182, flattened):
 * nshell shells, per-shell l/pure/nprim/atom index, origins [3*nshell]
 * (bohr), and the flattened exponents / normalization-embedded coefficients
 * of all shells in order.  Replaces any previous basis of the context. */
lgx_status lgx_set_basis(lgx_context* ctx, int nshell, const int32_t* l,
                         const int32_t* pure, const int32_t* nprim,
                         const int32_t* atom, const double* origins,
                         const double* alpha, const double* coeff);
/* Restricts every later J/K and gradient pass (lgx_jk*, lgx_jk_grad) to the
 * unique quartets (s1 s2|s3 s4) whose bra and ket shell pairs are both in
 * `pairs` (2*n shell indices, either order within a pair), still screened
 * by K12*K34 >= schwarz_thresh; n = 0 lifts the restriction, as does
 * lgx_set_basis.  The quartet set is the same whichever way a caller
 * enumerates bra and ket, so a CPU J/K over the same pairs (the reference's
 * compute_2body_fock loop, hartree-fock++.cc:1617-1700, with both pairs
 * drawn from the list) gives the same J and K: this is how the J/K kernels
 * are checked against a CPU implementation on bases far too large for a
 * CPU pass.  No counterpart in the reference's Engine API. */
lgx_status lgx_set_pair_subset(lgx_context* ctx, const int32_t* pairs, int64_t n);

/* Number of basis functions of the current basis. */
lgx_status lgx_basis_nbf(lgx_context* ctx, int* nbf);

/* Schwarz factors K(s1,s2) = sqrt(max |(s1 s2|s1 s2)|) for every shell pair
 * of the basis into the HOST array K [nshell*nshell] (compute_schwarz_ints,
 * tests/hartree-fock/hartree-fock++.cc:1231-1298, infinity norm). */
lgx_status lgx_schwarz(lgx_context* ctx, double* K);

/* Batched Engine::compute over an explicit quartet list: `quartets` holds
 * 4*n shell indices (caller order, HOST memory); set q is written at
 * out + offsets[q] (HOST memory, doubles) in libint's buffer order, nsets
 * consecutive sets per quartet.  `offsets` may be NULL, in which case sets
 * are packed back to back in list order.  is_null (optional, n ints)
 * receives 1 for fully screened quartets.  mode: LGX_FP64 or LGX_MIXED
 * (FP32 arithmetic for quartets whose Schwarz bound K12*K34 < mixed_thresh). */
lgx_status lgx_compute_batch(lgx_context* ctx, const int32_t* quartets,
                             int64_t n, int deriv, int mode,
                             double mixed_thresh, const int64_t* offsets,
                             double* out, size_t out_capacity,
                             int32_t* is_null);
/* lgx_compute_batch with the sets left in HBM: `d_out` (out_capacity
 * doubles) and `d_is_null` (optional, n ints) are DEVICE memory of the
 * context's GPU; quartets and offsets stay host arrays.  For callers that
 * contract the integrals on the GPU next (density fitting: the 3-centre
 * tensor and the metric), so no host copy is made.  Returns after the
 * kernels have finished. */
lgx_status lgx_compute_batch_device(lgx_context* ctx, const int32_t* quartets, int64_t n,
                                    int deriv, int mode, double mixed_thresh,
                                    const int64_t* offsets, double* d_out, size_t out_capacity,
                                    int32_t* d_is_null);

/* Statistics of one J/K (or gradient) pass. */
typedef struct {
  int64_t quartets_fp64;   /* shell quartets computed in FP64             */
  int64_t quartets_fp32;   /* shell quartets computed in FP32             */
  int64_t integrals;       /* spherical integrals computed (both modes)   */
  int64_t prim_quartets;   /* primitive quartets entering the VRR         */
  double kernel_ms;        /* device time of the integral kernels         */
  double pass_ms;          /* device time of the whole pass (incl. zeroing
                              and the final symmetrization)               */
  double flops_fp64;       /* algorithmic FP operations done in FP64      */
  double flops_fp32;       /* algorithmic FP operations done in FP32      */
  int64_t launches;        /* kernels launched by the pass                */
} lgx_jk_stats;

/* Coulomb and exchange matrices J_ab = sum_cd (ab|cd) D_cd and
 * K_ab = sum_cd (ac|bd) D_cd over all unique quartets whose Schwarz bound
 * K12*K34 >= schwarz_thresh, digested with the 8-fold degeneracy factors of
 * compute_2body_fock (hartree-fock++.cc:1628-1766) in FP64 accumulators.
 * D, J, K are nbf*nbf row-major HOST arrays (D symmetric). */
lgx_status lgx_jk(lgx_context* ctx, const double* D, double* J, double* K,
                  double schwarz_thresh, int mode, double mixed_thresh,
                  lgx_jk_stats* stats);
/* Same, with D, J, K in DEVICE memory (no host copies). */
lgx_status lgx_jk_device(lgx_context* ctx, const double* dD, double* dJ,
                         double* dK, double schwarz_thresh, int mode,
                         double mixed_thresh, lgx_jk_stats* stats);

/* Density-weighted screening of every later J/K pass on the context (lgx_jk,
 * lgx_jk_device, lgx_jk_device_noalloc), as compute_2body_fock does it
 * (tests/hartree-fock/hartree-fock++.cc:1581-1684): with Dnorm1234 the
 * largest infinity norm of the six shell blocks of D that a quartet touches
 * (compute_shellblock_norm, :939-957), a quartet that passed the Schwarz
 * test is skipped when Dnorm1234 * K12 * K34 < precision, and the others
 * have their primitives screened at precision / Dnorm1234 instead of the
 * machine epsilon (Engine::set_precision per shell set), never below the
 * epsilon the primitive-pair data are built with.  precision = 0 (the
 * default) turns it off; the gradient pass does not use it. */
lgx_status lgx_set_fock_precision(lgx_context* ctx, double precision);

/* No counterpart in the reference.  lgx_jk_device for callers that must not
 * allocate device memory while they run: code inside a region where
 * cudaMalloc is not allowed or would stall (for example while another
 * component, such as a framework's caching allocator, owns all device
 * memory), or pipelines that budget device memory up front.  The call makes
 * no cudaMalloc / cudaFree / allocating-library call: its J/K accumulators
 * and the FP32 copy of D live in one file-scope __device__ array of the
 * library, sized for nbf <= LGX_NOALLOC_MAX_NBF (768 functions: 11.25 MiB,
 * held by every GPU that loads the library until the process exits); a
 * larger basis returns LGX_ERR_TOO_LARGE.  The context's basis state (pair
 * data, Schwarz factors, quartet bins, class programs) must already exist
 * for the same schwarz_thresh / mode / mixed_thresh, i.e. after one
 * lgx_jk_device or lgx_jk call; otherwise LGX_ERR_INVALID_ARG.  The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Every call shares the one array and overwrites it (the accumulators are
 * cleared at the start of each call), so calls that overlap on the GPU
 * (two threads or contexts on one device at once) race. */
#define LGX_NOALLOC_MAX_NBF 768
lgx_status lgx_jk_device_noalloc(lgx_context* ctx, const double* dD, double* dJ,
                                 double* dK, double schwarz_thresh, int mode,
                                 double mixed_thresh, lgx_jk_stats* stats);

/* Statistics of one class launch of the last J/K or gradient pass, the
 * counterpart of libint's per-class Engine timers (LIBINT2_ENGINE_TIMERS,
 * include/libint2/engine.h:862-890), which time the primitive prologue,
 * the build and the transform per call; here one record per class bin and
 * precision of a whole pass. */
typedef struct {
  int32_t la, lb, lc, ld;  /* angular momenta of the class (canonical order)  */
  int32_t fp32;            /* 1: FP32 arithmetic, 0: FP64                     */
  int32_t kernel;          /* 0: register kernel, 1: program kernel,
                              2: program kernel with generated post stage    */
  int32_t shape;           /* lanes per quartet (kernel 0) or staging rows    */
  int32_t deriv;           /* derivative order of the pass                    */
  int64_t quartets;        /* shell quartets of the launch                    */
  int64_t prim_quartets;   /* primitive quartets entering the VRR             */
  int64_t integrals;       /* shell-set values computed (per derivative set)  */
  double flops;            /* algorithmic FP operations (FMA = 2)             */
  double ms;               /* device time of the launch (CUDA events on the
                              context's stream; -1 when not recorded)         */
  double flops_fp64;       /* of `flops`, those done in FP64 (all of them for
                              an FP64 launch; the Boys function and its
                              argument for the mixed scheme's FP32 launches) */
} lgx_launch_stats;

/* Copies up to `max` per-launch records of the last lgx_jk / lgx_jk_device
 * / lgx_jk_device_noalloc / lgx_jk_grad pass into `out` (launch order) and
 * sets *n to the number of launches of that pass.  Timings come from events
 * recorded between the launches, also when the pass replays its CUDA
 * graph. */
lgx_status lgx_last_pass_launches(lgx_context* ctx, lgx_launch_stats* out,
                                  int max, int* n);

/* Nuclear gradients of E_J = 1/2 sum D.J and E_K = -1/4 sum D.K from
 * deriv_order = 1 integrals (compute_2body_fock_deriv<1>,
 * hartree-fock++.cc:1776-2000, per-atom digestion :1909-1973).
 * gJ, gK: natoms*3 HOST arrays; natoms = 1 + max atom index of the basis. */
lgx_status lgx_jk_grad(lgx_context* ctx, const double* D, double* gJ,
                       double* gK, int natoms, double schwarz_thresh,
                       lgx_jk_stats* stats);

/* -------------------------------------------------------- host utilities */

/* Shell::do_enforce_unit_normalization (shell.h:891-901): flag 0 or 1 sets
 * whether lgx_shell_normalize and lgx_basis_load rescale each contraction to
 * unit self-overlap (process-wide, on by default, like the reference's
 * static switch); flag < 0 only queries.  Returns the setting in effect. */
int lgx_enforce_unit_normalization(int flag);

/* Shell::renorm (shell.h:958-999): coeff_out = normalization-embedded
 * coefficients for unit-normalized-primitive input coefficients (the
 * contraction renormalized to unity unless disabled above). */
lgx_status lgx_shell_normalize(int l, int nprim, const double* alpha,
                               const double* coeff_in, double* coeff_out);

/* SolidHarmonicsCoefficients::coeff (include/libint2/solidharmonics.h:
 * 114-174): the coefficient of the Cartesian component x^lx y^ly z^lz in
 * the real solid harmonic (l, m), m = -l..l, in libint's convention (all
 * Cartesian components sharing the x^l normalization), as the kernels'
 * transform uses it; 0 when lx + ly + lz != l or |m| > l. */
double lgx_solid_coeff(int l, int m, int lx, int ly, int lz);

/* BasisSet(name, atoms) with the G94 reader of basis.h.in:473-621: loads
 * `<data_dir>/<name>.g94` (name canonicalized: lower case, '*'->'_st_')
 * for natoms atoms with atomic numbers Z and positions xyz (bohr).
 * Call with l == NULL to get *nshell and *nprim_total only; then call again
 * with arrays of that size.  pure follows the reference (l > 1 unless the
 * Gaussian Cartesian-d convention applies). */
lgx_status lgx_basis_load(const char* data_dir, const char* name, int natoms,
                          const int32_t* Z, const double* xyz, int* nshell,
                          int* nprim_total, int32_t* l, int32_t* pure,
                          int32_t* nprim, int32_t* atom, double* origins,
                          double* alpha, double* coeff);

/* Synthetic water cluster: nx*ny*nz molecules, O on a grid with `spacing`
 * angstrom, each jittered by uniform(-jitter, jitter) angstrom per axis,
 * H at 0.96 A and 104.5 deg with a uniformly random orientation, from a
 * seeded mt19937_64.  Writes Z [3*n] and xyz [9*n] (bohr, CODATA 2018
 * 0.529177210903 A/bohr, atom.h:52-55), atoms ordered O,H,H per molecule. */
lgx_status lgx_water_cluster(int nx, int ny, int nz, double spacing,
                             double jitter, uint64_t seed, int32_t* Z,
                             double* xyz);

#ifdef __cplusplus
}
#endif
#endif /* LGX_H */
