/*
 * C interface of libint's generated integral library, Coulomb ERI tasks
 * eri / eri1 / eri2 (the reference's include/libint2.h with the generated
 * libint2_params.h / libint2_types.h / libint2_iface.h that
 * src/bin/libint/iface.cc:119-176,247-290,349-404,585-668 writes).  Code
 * written against libint's C API compiles unchanged against this header:
 *
 *   libint2_static_init();
 *   Libint_t erieval[contrdepth];            // one per primitive quartet
 *   libint2_init_eri(&erieval[0], max_am, 0);
 *   ... erieval[p].PA_x[0] = ...; erieval[p].LIBINT_T_SS_EREP_SS(m)[0] = ...;
 *   erieval[0].contrdepth = contrdepth;
 *   libint2_build_eri[l1][l2][l3][l4](erieval);
 *   ... erieval[0].targets[0] .. : the Cartesian shell set(s)
 *   libint2_cleanup_eri(&erieval[0]);
 *   libint2_static_cleanup();
 *
 * Every build call runs on the GPU (lgx_compute_primitive_set on a
 * process-wide context of device 0, or of the device in LGX_DEVICE): the
 * primitive records are packed into the kernels' staging layout, one warp
 * contracts them with the class's VRR / HRR programs, and the sets are
 * copied back into the Libint_t stack before the call returns.  The tables
 * hold every ordering of (l1 l2|l3 l4) up to the LIBINT2_MAX_AM_eri* limits
 * (libint's generated library holds the canonical ones only).  Build calls
 * are serialised process-wide.  A failed call (no GPU, CUDA error) fills
 * the targets with NaN and prints the reason to stderr: libint's C API has
 * no error channel.
 *
 * Deliberately alike with libint's C API (so caller code compiles
 * unchanged): the Libint_t member names of the prefactors, the
 * LIBINT_T_SS_EREP_SS(m) macro and the member it names, the function
 * names and signatures, and the LIBINT2_DEFINED / LIBINT2_PREFIXED_NAME
 * macros.  The struct layout itself is this library's own.
 */
#ifndef LGX_LIBINT2_H
#define LGX_LIBINT2_H

#include <stddef.h>

#define LIBINT2_REALTYPE double
#define LIBINT2_MAX_VECLEN 1
#define LIBINT_CONTRACTED_INTS 1
#define LIBINT_SHELL_SET_STANDARD 1
#define LIBINT_SHELL_SET LIBINT_SHELL_SET_STANDARD
#define LIBINT2_SUPPORT_ERI 1
#define LIBINT2_MAX_AM_eri 3
#define LIBINT2_MAX_AM_eri1 3
#define LIBINT2_MAX_AM_eri2 3
#define LIBINT2_MAX_AM 3
#define LIBINT_MAX_AM 4
#define LIBINT2_DERIV_ERI_ORDER 2
/* targets per build: 1, 12 or 78 shell sets */
#define LIBINT2_MAX_NTARGETS 78
/* largest m of (00|00)^(m) a build reads: 4 l_max + 2 */
#define LIBINT2_MAX_M 14

#define LIBINT2_API_PREFIX
#define LIBINT2_PREFIXED_NAME(name) lgx_prefixed_name_(LIBINT2_API_PREFIX, name)
#define lgx_prefixed_name_(prefix, name) lgx_prescanned_name_(prefix, name)
#define lgx_prescanned_name_(prefix, name) prefix##name

/* LIBINT2_DEFINED(eri, member): 1 when Libint_t has the member (the member
 * argument is macro-expanded first, so LIBINT_T_SS_EREP_SS(m) works). */
#define LIBINT2_DEFINED(taskname, symbol) lgx_defined_(taskname, symbol)
#define lgx_defined_(taskname, symbol) LIBINT2_DEFINED_##symbol

#define LIBINT_T_SS_EREP_SS(mValue) \
  _aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_##mValue

#define LGX_LIBINT_MEMBER(name) LIBINT2_REALTYPE name[LIBINT2_MAX_VECLEN];

typedef struct Libint_t {
  /* VRR / HRR prefactors of one primitive quartet (engine.impl.h:1389-1757) */
  LGX_LIBINT_MEMBER(PA_x) LGX_LIBINT_MEMBER(PA_y) LGX_LIBINT_MEMBER(PA_z)
  LGX_LIBINT_MEMBER(PB_x) LGX_LIBINT_MEMBER(PB_y) LGX_LIBINT_MEMBER(PB_z)
  LGX_LIBINT_MEMBER(QC_x) LGX_LIBINT_MEMBER(QC_y) LGX_LIBINT_MEMBER(QC_z)
  LGX_LIBINT_MEMBER(QD_x) LGX_LIBINT_MEMBER(QD_y) LGX_LIBINT_MEMBER(QD_z)
  LGX_LIBINT_MEMBER(AB_x) LGX_LIBINT_MEMBER(AB_y) LGX_LIBINT_MEMBER(AB_z)
  LGX_LIBINT_MEMBER(BA_x) LGX_LIBINT_MEMBER(BA_y) LGX_LIBINT_MEMBER(BA_z)
  LGX_LIBINT_MEMBER(CD_x) LGX_LIBINT_MEMBER(CD_y) LGX_LIBINT_MEMBER(CD_z)
  LGX_LIBINT_MEMBER(DC_x) LGX_LIBINT_MEMBER(DC_y) LGX_LIBINT_MEMBER(DC_z)
  LGX_LIBINT_MEMBER(WP_x) LGX_LIBINT_MEMBER(WP_y) LGX_LIBINT_MEMBER(WP_z)
  LGX_LIBINT_MEMBER(WQ_x) LGX_LIBINT_MEMBER(WQ_y) LGX_LIBINT_MEMBER(WQ_z)
  LGX_LIBINT_MEMBER(oo2z) LGX_LIBINT_MEMBER(oo2e) LGX_LIBINT_MEMBER(oo2ze)
  LGX_LIBINT_MEMBER(roz) LGX_LIBINT_MEMBER(roe)
  /* derivative prefactors: the build reads the four 2 alpha; the others are
   * accepted for source compatibility */
  LGX_LIBINT_MEMBER(two_alpha0_bra) LGX_LIBINT_MEMBER(two_alpha0_ket)
  LGX_LIBINT_MEMBER(two_alpha1_bra) LGX_LIBINT_MEMBER(two_alpha1_ket)
  LGX_LIBINT_MEMBER(alpha1_rho_over_zeta2) LGX_LIBINT_MEMBER(alpha2_rho_over_zeta2)
  LGX_LIBINT_MEMBER(alpha3_rho_over_eta2) LGX_LIBINT_MEMBER(alpha4_rho_over_eta2)
  LGX_LIBINT_MEMBER(alpha1_over_zetapluseta) LGX_LIBINT_MEMBER(alpha2_over_zetapluseta)
  LGX_LIBINT_MEMBER(alpha3_over_zetapluseta) LGX_LIBINT_MEMBER(alpha4_over_zetapluseta)
  LGX_LIBINT_MEMBER(rho12_over_alpha1) LGX_LIBINT_MEMBER(rho12_over_alpha2)
  LGX_LIBINT_MEMBER(rho34_over_alpha3) LGX_LIBINT_MEMBER(rho34_over_alpha4)
  /* (00|00)^(m) = pfac F_m(T), m = 0..LIBINT2_MAX_M */
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(0)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(1))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(2)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(3))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(4)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(5))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(6)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(7))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(8)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(9))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(10)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(11))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(12)) LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(13))
  LGX_LIBINT_MEMBER(LIBINT_T_SS_EREP_SS(14))
  /* results: targets[s] -> shell set s, inside stack */
  LIBINT2_REALTYPE* stack;
  LIBINT2_REALTYPE* vstack;
  LIBINT2_REALTYPE* targets[LIBINT2_MAX_NTARGETS];
  int veclen;
  /* primitive quartets of the contraction (read from element 0) */
  int contrdepth;
  /* library state: stack elements, and whether libint2_init_eri* allocated it */
  size_t lgx_stack_size;
  int lgx_owns_stack;
} Libint_t;

typedef Libint_t Libint_eri_t;
typedef Libint_t Libint_eri1_t;
typedef Libint_t Libint_eri2_t;

#define LIBINT2_DEFINED_PA_x 1
#define LIBINT2_DEFINED_PA_y 1
#define LIBINT2_DEFINED_PA_z 1
#define LIBINT2_DEFINED_PB_x 1
#define LIBINT2_DEFINED_PB_y 1
#define LIBINT2_DEFINED_PB_z 1
#define LIBINT2_DEFINED_QC_x 1
#define LIBINT2_DEFINED_QC_y 1
#define LIBINT2_DEFINED_QC_z 1
#define LIBINT2_DEFINED_QD_x 1
#define LIBINT2_DEFINED_QD_y 1
#define LIBINT2_DEFINED_QD_z 1
#define LIBINT2_DEFINED_AB_x 1
#define LIBINT2_DEFINED_AB_y 1
#define LIBINT2_DEFINED_AB_z 1
#define LIBINT2_DEFINED_BA_x 1
#define LIBINT2_DEFINED_BA_y 1
#define LIBINT2_DEFINED_BA_z 1
#define LIBINT2_DEFINED_CD_x 1
#define LIBINT2_DEFINED_CD_y 1
#define LIBINT2_DEFINED_CD_z 1
#define LIBINT2_DEFINED_DC_x 1
#define LIBINT2_DEFINED_DC_y 1
#define LIBINT2_DEFINED_DC_z 1
#define LIBINT2_DEFINED_WP_x 1
#define LIBINT2_DEFINED_WP_y 1
#define LIBINT2_DEFINED_WP_z 1
#define LIBINT2_DEFINED_WQ_x 1
#define LIBINT2_DEFINED_WQ_y 1
#define LIBINT2_DEFINED_WQ_z 1
#define LIBINT2_DEFINED_oo2z 1
#define LIBINT2_DEFINED_oo2e 1
#define LIBINT2_DEFINED_oo2ze 1
#define LIBINT2_DEFINED_roz 1
#define LIBINT2_DEFINED_roe 1
#define LIBINT2_DEFINED_two_alpha0_bra 1
#define LIBINT2_DEFINED_two_alpha0_ket 1
#define LIBINT2_DEFINED_two_alpha1_bra 1
#define LIBINT2_DEFINED_two_alpha1_ket 1
#define LIBINT2_DEFINED_alpha1_rho_over_zeta2 1
#define LIBINT2_DEFINED_alpha2_rho_over_zeta2 1
#define LIBINT2_DEFINED_alpha3_rho_over_eta2 1
#define LIBINT2_DEFINED_alpha4_rho_over_eta2 1
#define LIBINT2_DEFINED_alpha1_over_zetapluseta 1
#define LIBINT2_DEFINED_alpha2_over_zetapluseta 1
#define LIBINT2_DEFINED_alpha3_over_zetapluseta 1
#define LIBINT2_DEFINED_alpha4_over_zetapluseta 1
#define LIBINT2_DEFINED_rho12_over_alpha1 1
#define LIBINT2_DEFINED_rho12_over_alpha2 1
#define LIBINT2_DEFINED_rho34_over_alpha3 1
#define LIBINT2_DEFINED_rho34_over_alpha4 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_0 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_1 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_2 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_3 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_4 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_5 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_6 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_7 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_8 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_9 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_10 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_11 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_12 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_13 1
#define LIBINT2_DEFINED__aB_s___0__s___1___TwoPRep_s___0__s___1___Ab__up_14 1

#ifdef __cplusplus
extern "C" {
#endif

void libint2_static_init(void);
void libint2_static_cleanup(void);

/* Size of the results stack in LIBINT2_REALTYPE elements for shells up to
 * max_am (every target set of the largest class). */
size_t libint2_need_memory_eri(int max_am);
size_t libint2_need_memory_eri1(int max_am);
size_t libint2_need_memory_eri2(int max_am);
/* Sets up inteval (element 0 of the caller's array): the results stack is
 * `buf` when non-null (libint2_need_memory_* elements), else allocated. */
void libint2_init_eri(Libint_t* inteval, int max_am, void* buf);
void libint2_init_eri1(Libint_t* inteval, int max_am, void* buf);
void libint2_init_eri2(Libint_t* inteval, int max_am, void* buf);
void libint2_cleanup_eri(Libint_t* inteval);
void libint2_cleanup_eri1(Libint_t* inteval);
void libint2_cleanup_eri2(Libint_t* inteval);

/* build[l1][l2][l3][l4](inteval): the contracted Cartesian shell set(s)
 * over inteval[0 .. inteval[0].contrdepth) into inteval[0].targets. */
extern void (*libint2_build_eri[LIBINT2_MAX_AM_eri + 1][LIBINT2_MAX_AM_eri + 1]
                               [LIBINT2_MAX_AM_eri + 1][LIBINT2_MAX_AM_eri + 1])(const Libint_t*);
extern void (*libint2_build_eri1[LIBINT2_MAX_AM_eri1 + 1][LIBINT2_MAX_AM_eri1 + 1]
                                [LIBINT2_MAX_AM_eri1 + 1][LIBINT2_MAX_AM_eri1 + 1])(const Libint_t*);
extern void (*libint2_build_eri2[LIBINT2_MAX_AM_eri2 + 1][LIBINT2_MAX_AM_eri2 + 1]
                                [LIBINT2_MAX_AM_eri2 + 1][LIBINT2_MAX_AM_eri2 + 1])(const Libint_t*);

#ifdef __cplusplus
}
#endif

#endif /* LGX_LIBINT2_H */
