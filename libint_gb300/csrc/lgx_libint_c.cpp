// libint's generated-library C API (include/libint2.h): libint2_static_init
// / _cleanup, libint2_init_eri* / _need_memory_eri* / _cleanup_eri*, and
// the libint2_build_eri{,1,2}[l1][l2][l3][l4] tables (the reference's
// src/bin/libint/iface.cc:119-176,349-404 writes their generated
// counterparts).  Each build call gathers the Libint_t prefactors of its
// contrdepth primitive quartets into lgx_prim_quartet records and hands
// them to lgx_compute_primitive_set, which contracts them on the GPU; the
// shell sets land in the Libint_t stack and targets[s] points at set s.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <mutex>
#include <vector>

#include "../../include/lgx.h"
#include "../../include/libint2.h"

namespace {

std::mutex g_mu;
lgx_context* g_ctx = nullptr;
bool g_ctx_failed = false;

// Process-wide context on device LGX_DEVICE (default 0); call under g_mu.
lgx_context* context() {
  if (!g_ctx && !g_ctx_failed) {
    int dev = 0;
    if (const char* e = std::getenv("LGX_DEVICE")) dev = std::atoi(e);
    if (lgx_create(&g_ctx, dev) != LGX_OK) {
      std::fprintf(stderr, "libint2 (lgx): no usable GPU for the build functions\n");
      g_ctx = nullptr;
      g_ctx_failed = true;
    }
  }
  return g_ctx;
}

int ncart(int l) { return (l + 1) * (l + 2) / 2; }

size_t need_memory(int max_am, int ntargets) {
  if (max_am < 0) max_am = 0;
  const size_t n = size_t(ncart(max_am));
  return size_t(ntargets) * n * n * n * n;
}

void init(Libint_t* t, int max_am, void* buf, int ntargets) {
  t->stack = buf ? static_cast<double*>(buf)
                 : static_cast<double*>(std::malloc(need_memory(max_am, ntargets) * sizeof(double)));
  t->lgx_owns_stack = buf ? 0 : 1;
  t->lgx_stack_size = need_memory(max_am, ntargets);
  t->vstack = nullptr;
  for (int s = 0; s < LIBINT2_MAX_NTARGETS; ++s) t->targets[s] = nullptr;
  t->veclen = 1;
  t->contrdepth = 1;
}

void cleanup(Libint_t* t) {
  if (t->lgx_owns_stack) std::free(t->stack);
  t->stack = nullptr;
  t->lgx_owns_stack = 0;
  t->lgx_stack_size = 0;
}

// One Libint_t element -> the primitive record lgx_compute_primitive_set reads.
void gather(const Libint_t& e, lgx_prim_quartet& q) {
  q.PA[0] = e.PA_x[0]; q.PA[1] = e.PA_y[0]; q.PA[2] = e.PA_z[0];
  q.QC[0] = e.QC_x[0]; q.QC[1] = e.QC_y[0]; q.QC[2] = e.QC_z[0];
  q.WP[0] = e.WP_x[0]; q.WP[1] = e.WP_y[0]; q.WP[2] = e.WP_z[0];
  q.WQ[0] = e.WQ_x[0]; q.WQ[1] = e.WQ_y[0]; q.WQ[2] = e.WQ_z[0];
  q.oo2z = e.oo2z[0];
  q.oo2e = e.oo2e[0];
  q.oo2ze = e.oo2ze[0];
  q.roz = e.roz[0];
  q.roe = e.roe[0];
  q.two_alpha[0] = e.two_alpha0_bra[0];
  q.two_alpha[1] = e.two_alpha0_ket[0];
  q.two_alpha[2] = e.two_alpha1_bra[0];
  q.two_alpha[3] = e.two_alpha1_ket[0];
  const double* ss[LIBINT2_MAX_M + 1] = {
      e.LIBINT_T_SS_EREP_SS(0),  e.LIBINT_T_SS_EREP_SS(1),  e.LIBINT_T_SS_EREP_SS(2),
      e.LIBINT_T_SS_EREP_SS(3),  e.LIBINT_T_SS_EREP_SS(4),  e.LIBINT_T_SS_EREP_SS(5),
      e.LIBINT_T_SS_EREP_SS(6),  e.LIBINT_T_SS_EREP_SS(7),  e.LIBINT_T_SS_EREP_SS(8),
      e.LIBINT_T_SS_EREP_SS(9),  e.LIBINT_T_SS_EREP_SS(10), e.LIBINT_T_SS_EREP_SS(11),
      e.LIBINT_T_SS_EREP_SS(12), e.LIBINT_T_SS_EREP_SS(13), e.LIBINT_T_SS_EREP_SS(14)};
  for (int m = 0; m <= LGX_PRIM_MAX_M; ++m) q.ss[m] = m <= LIBINT2_MAX_M ? ss[m][0] : 0.0;
}

// build_eri{deriv}[l1][l2][l3][l4](inteval)
void build(const Libint_t* inteval, int l1, int l2, int l3, int l4, int deriv) {
  Libint_t* t = const_cast<Libint_t*>(inteval);  // libint's targets[] are mutable
  const int ns = deriv == 0 ? 1 : (deriv == 1 ? 12 : 78);
  const size_t nv = size_t(ncart(l1)) * ncart(l2) * ncart(l3) * ncart(l4);
  const int np = t->contrdepth > 0 ? t->contrdepth : 0;
  std::vector<lgx_prim_quartet> q(static_cast<size_t>(np));
  for (int p = 0; p < np; ++p) gather(inteval[p], q[size_t(p)]);
  const double AB[3] = {t->AB_x[0], t->AB_y[0], t->AB_z[0]};
  const double CD[3] = {t->CD_x[0], t->CD_y[0], t->CD_z[0]};
  const size_t cap = t->lgx_stack_size;
  lgx_status st = LGX_ERR_TOO_LARGE;
  const char* why = "shell sets larger than the stack libint2_init_eri* sized for max_am";
  if (t->stack && nv * ns <= cap) {
    std::lock_guard<std::mutex> lk(g_mu);
    lgx_context* ctx = context();
    int nsets = 0, nvalues = 0;
    st = LGX_ERR_NO_DEVICE;
    why = "no usable GPU";
    if (ctx) {
      st = lgx_compute_primitive_set(ctx, l1, l2, l3, l4, deriv, q.data(), np, AB, CD, t->stack,
                                     cap, &nsets, &nvalues);
      why = lgx_last_error(ctx);
    }
  } else if (!t->stack) {
    why = "libint2_init_eri was not called";
  }
  if (st != LGX_OK) {
    std::fprintf(stderr, "libint2 (lgx): build_eri%s[%d][%d][%d][%d] failed (%d): %s\n",
                 deriv == 0 ? "" : (deriv == 1 ? "1" : "2"), l1, l2, l3, l4, st, why);
    if (t->stack && nv * ns <= cap)
      for (size_t i = 0; i < nv * ns; ++i) t->stack[i] = std::numeric_limits<double>::quiet_NaN();
  }
  for (int s = 0; s < ns; ++s) t->targets[s] = t->stack ? t->stack + size_t(s) * nv : nullptr;
}

template <int L1, int L2, int L3, int L4, int D>
void build_fn(const Libint_t* inteval) {
  build(inteval, L1, L2, L3, L4, D);
}

}  // namespace

#define LGX_B4(D, a, b, c) \
  { &build_fn<a, b, c, 0, D>, &build_fn<a, b, c, 1, D>, &build_fn<a, b, c, 2, D>, &build_fn<a, b, c, 3, D> }
#define LGX_B3(D, a, b) { LGX_B4(D, a, b, 0), LGX_B4(D, a, b, 1), LGX_B4(D, a, b, 2), LGX_B4(D, a, b, 3) }
#define LGX_B2(D, a) { LGX_B3(D, a, 0), LGX_B3(D, a, 1), LGX_B3(D, a, 2), LGX_B3(D, a, 3) }
#define LGX_B1(D) { LGX_B2(D, 0), LGX_B2(D, 1), LGX_B2(D, 2), LGX_B2(D, 3) }

extern "C" {

void (*libint2_build_eri[LIBINT2_MAX_AM_eri + 1][LIBINT2_MAX_AM_eri + 1][LIBINT2_MAX_AM_eri + 1]
                        [LIBINT2_MAX_AM_eri + 1])(const Libint_t*) = LGX_B1(0);
void (*libint2_build_eri1[LIBINT2_MAX_AM_eri1 + 1][LIBINT2_MAX_AM_eri1 + 1][LIBINT2_MAX_AM_eri1 + 1]
                         [LIBINT2_MAX_AM_eri1 + 1])(const Libint_t*) = LGX_B1(1);
void (*libint2_build_eri2[LIBINT2_MAX_AM_eri2 + 1][LIBINT2_MAX_AM_eri2 + 1][LIBINT2_MAX_AM_eri2 + 1]
                         [LIBINT2_MAX_AM_eri2 + 1])(const Libint_t*) = LGX_B1(2);

void libint2_static_init(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  context();
}

void libint2_static_cleanup(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_ctx) lgx_destroy(g_ctx);
  g_ctx = nullptr;
  g_ctx_failed = false;
}

size_t libint2_need_memory_eri(int max_am) { return need_memory(max_am, 1); }
size_t libint2_need_memory_eri1(int max_am) { return need_memory(max_am, 12); }
size_t libint2_need_memory_eri2(int max_am) { return need_memory(max_am, 78); }
void libint2_init_eri(Libint_t* inteval, int max_am, void* buf) { init(inteval, max_am, buf, 1); }
void libint2_init_eri1(Libint_t* inteval, int max_am, void* buf) { init(inteval, max_am, buf, 12); }
void libint2_init_eri2(Libint_t* inteval, int max_am, void* buf) { init(inteval, max_am, buf, 78); }
void libint2_cleanup_eri(Libint_t* inteval) { cleanup(inteval); }
void libint2_cleanup_eri1(Libint_t* inteval) { cleanup(inteval); }
void libint2_cleanup_eri2(Libint_t* inteval) { cleanup(inteval); }

}  // extern "C"
