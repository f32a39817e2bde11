"""Caller-supplied primitive data: lgx_compute_primitive_set and libint's
generated-library C API over it (include/libint2.h: Libint_t,
LIBINT_T_SS_EREP_SS, libint2_build_eri / _eri1 / _eri2; the reference's
tests/unit/c-api.c and export/fortran/test-eri.cc call it this way), checked
against the oracle's contracted shell sets of the same raw shells
(oracle.cpp compute_quartet, pinned to the reference's eri.h brute force).
Every ordering of (l1 l2|l3 l4) is covered, canonical or not, with
contraction depths 1-2 per shell."""
import itertools
import os
import struct
import subprocess

import numpy as np
import pytest

from prim_util import oracle_sets, prim_quartets, random_shells

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-12  # relative to max(1, max |reference|), FP64 throughout


def _err(got, ref):
    scale = max(1.0, max(float(np.abs(r).max()) for r in ref))
    return max(float(np.abs(np.asarray(g).reshape(-1) - np.asarray(r).reshape(-1)).max())
               for g, r in zip(got, ref)) / scale


def _cases(rng, deriv):
    if deriv == 0:
        return list(itertools.product(range(4), repeat=4))
    if deriv == 1:
        every = list(itertools.product(range(4), repeat=4))
        pick = rng.choice(len(every), 48, replace=False)
        return [every[i] for i in pick] + [(3, 3, 3, 3), (0, 3, 1, 2), (3, 0, 0, 0)]
    every = list(itertools.product(range(4), repeat=4))
    pick = rng.choice(len(every), 24, replace=False)
    return [every[i] for i in pick] + [(2, 2, 2, 2), (0, 2, 1, 0), (1, 1, 1, 1), (3, 3, 3, 3),
                                       (3, 0, 1, 2)]


@pytest.mark.parametrize("deriv", [0, 1, 2])
def test_primitive_set_vs_oracle(lgx, deriv):
    ctx = lgx.Context(0)
    rng = np.random.default_rng(100 + deriv)
    worst = 0.0
    for ls in _cases(rng, deriv):
        sh = random_shells(rng, ls, max_depth=2)
        prims, AB, CD = prim_quartets(sh, deriv, lgx._lgx.PRIM_DTYPE)
        got = ctx.compute_primitive_set(ls, prims, AB, CD, deriv)
        ref = oracle_sets(sh, deriv)
        assert len(got) == len(ref) == {0: 1, 1: 12, 2: 78}[deriv]
        err = _err(got, ref)
        worst = max(worst, err)
        assert err < TOL, (ls, err)
    print("deriv", deriv, "worst", worst)
    ctx.close()


def test_primitive_set_errors(lgx):
    ctx = lgx.Context(0)
    rng = np.random.default_rng(7)
    sh = random_shells(rng, (1, 0, 0, 0))
    prims, AB, CD = prim_quartets(sh, 0, lgx._lgx.PRIM_DTYPE)
    with pytest.raises(lgx.LgxError) as e:
        ctx.compute_primitive_set((4, 0, 0, 0), prims, AB, CD)
    assert e.value.status == lgx._lgx.LGX_ERR_LMAX_EXCEEDED
    with pytest.raises(lgx.LgxError) as e:
        ctx.compute_primitive_set((0, 0, 4, 0), prims, AB, CD, deriv=2)
    assert e.value.status == lgx._lgx.LGX_ERR_LMAX_EXCEEDED
    # no primitive quartets: zero sets
    z = ctx.compute_primitive_set((1, 0, 0, 0), prims[:0], AB, CD)
    assert z[0].shape == (3, 1, 1, 1) and not z[0].any()
    # the context still computes
    got = ctx.compute_primitive_set((1, 0, 0, 0), prims, AB, CD)
    assert _err(got, oracle_sets(sh, 0)) < TOL
    ctx.close()


C_DRIVER = r"""
/* Fills Libint_t by member name, as libint's C callers do
 * (tests/unit/c-api.c), and calls the build tables. */
#include <libint2.h>
#include <stdio.h>
#include <stdlib.h>

#define SET_SS(m) if (LIBINT2_DEFINED(eri, LIBINT_T_SS_EREP_SS(m))) \
    e->LIBINT_T_SS_EREP_SS(m)[0] = r[21 + m];

static int ncart(int l) { return (l + 1) * (l + 2) / 2; }

int main(int argc, char** argv) {
  FILE* f = fopen(argv[1], "rb");
  FILE* g = fopen(argv[2], "wb");
  int ncase = 0;
  if (!f || !g || fread(&ncase, sizeof(int), 1, f) != 1) return 2;
  LIBINT2_PREFIXED_NAME(libint2_static_init)();
  for (int c = 0; c < ncase; ++c) {
    int h[7];
    double AB[3], CD[3];
    if (fread(h, sizeof(int), 7, f) != 7) return 3;
    if (fread(AB, sizeof(double), 3, f) != 3 || fread(CD, sizeof(double), 3, f) != 3) return 3;
    const int deriv = h[0], np = h[5], user_buf = h[6];
    Libint_t* ev = (Libint_t*)calloc((size_t)(np > 0 ? np : 1), sizeof(Libint_t));
    double* buf = NULL;
    if (deriv == 0) {
      if (user_buf) buf = (double*)malloc(libint2_need_memory_eri(LIBINT2_MAX_AM_eri) * sizeof(double));
      libint2_init_eri(&ev[0], LIBINT2_MAX_AM_eri, buf);
    } else if (deriv == 1) {
      libint2_init_eri1(&ev[0], LIBINT2_MAX_AM_eri1, 0);
    } else {
      libint2_init_eri2(&ev[0], LIBINT2_MAX_AM_eri2, 0);
    }
    for (int p = 0; p < np; ++p) {
      double r[37];
      if (fread(r, sizeof(double), 37, f) != 37) return 4;
      Libint_t* e = &ev[p];
      e->PA_x[0] = r[0]; e->PA_y[0] = r[1]; e->PA_z[0] = r[2];
      e->QC_x[0] = r[3]; e->QC_y[0] = r[4]; e->QC_z[0] = r[5];
      e->WP_x[0] = r[6]; e->WP_y[0] = r[7]; e->WP_z[0] = r[8];
      e->WQ_x[0] = r[9]; e->WQ_y[0] = r[10]; e->WQ_z[0] = r[11];
      e->oo2z[0] = r[12]; e->oo2e[0] = r[13]; e->oo2ze[0] = r[14];
      e->roz[0] = r[15]; e->roe[0] = r[16];
      e->two_alpha0_bra[0] = r[17]; e->two_alpha0_ket[0] = r[18];
      e->two_alpha1_bra[0] = r[19]; e->two_alpha1_ket[0] = r[20];
      e->AB_x[0] = AB[0]; e->AB_y[0] = AB[1]; e->AB_z[0] = AB[2];
      e->CD_x[0] = CD[0]; e->CD_y[0] = CD[1]; e->CD_z[0] = CD[2];
      SET_SS(0) SET_SS(1) SET_SS(2) SET_SS(3) SET_SS(4) SET_SS(5) SET_SS(6) SET_SS(7)
      SET_SS(8) SET_SS(9) SET_SS(10) SET_SS(11) SET_SS(12) SET_SS(13) SET_SS(14)
    }
#if LIBINT_CONTRACTED_INTS
    ev[0].contrdepth = np;
#endif
    if (deriv == 0) LIBINT2_PREFIXED_NAME(libint2_build_eri)[h[1]][h[2]][h[3]][h[4]](ev);
    else if (deriv == 1) libint2_build_eri1[h[1]][h[2]][h[3]][h[4]](ev);
    else libint2_build_eri2[h[1]][h[2]][h[3]][h[4]](ev);
    const int ns = deriv == 0 ? 1 : (deriv == 1 ? 12 : 78);
    const size_t nv = (size_t)ncart(h[1]) * ncart(h[2]) * ncart(h[3]) * ncart(h[4]);
    for (int s = 0; s < ns; ++s) fwrite(ev[0].targets[s], sizeof(double), nv, g);
    if (deriv == 0) libint2_cleanup_eri(&ev[0]);
    else if (deriv == 1) libint2_cleanup_eri1(&ev[0]);
    else libint2_cleanup_eri2(&ev[0]);
    free(buf);
    free(ev);
  }
  LIBINT2_PREFIXED_NAME(libint2_static_cleanup)();
  fclose(g);
  fclose(f);
  return 0;
}
"""


def test_libint2_c_api_vs_oracle(lgx, tmp_path):
    lgx._lgx.load()
    src = tmp_path / "capi.c"
    src.write_text(C_DRIVER)
    exe = str(tmp_path / "capi")
    libdir = os.path.join(ROOT, "libint_gb300")
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                           str(src), "-L", libdir, "-llgx", "-Wl,-rpath," + libdir, "-o", exe])
    rng = np.random.default_rng(5)
    cases = []
    for deriv, lss in ((0, [(0, 0, 0, 0), (1, 0, 1, 0), (0, 1, 2, 3), (3, 2, 1, 0), (2, 2, 2, 2),
                            (3, 3, 3, 3), (1, 1, 0, 0)]),
                       (1, [(1, 0, 0, 0), (0, 0, 1, 1), (2, 1, 0, 3), (3, 3, 2, 2)]),
                       (2, [(1, 0, 0, 0), (0, 1, 1, 0), (2, 1, 0, 2), (2, 2, 2, 2),
                            (3, 1, 0, 3)])):
        for i, ls in enumerate(lss):
            sh = random_shells(rng, ls, max_depth=2)
            prims, AB, CD = prim_quartets(sh, deriv, lgx._lgx.PRIM_DTYPE)
            cases.append((deriv, ls, sh, prims, AB, CD, int(deriv == 0 and i % 2 == 1)))
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("i", len(cases)))
        for deriv, ls, sh, prims, AB, CD, ub in cases:
            f.write(struct.pack("7i", deriv, *ls, len(prims), ub))
            f.write(np.asarray(AB, float).tobytes())
            f.write(np.asarray(CD, float).tobytes())
            rec = prims.view(np.float64).reshape(len(prims), -1)[:, :37]
            f.write(np.ascontiguousarray(rec).tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout, r.stderr)
    vals = np.fromfile(out)
    pos = 0
    worst = 0.0
    for deriv, ls, sh, prims, AB, CD, ub in cases:
        ref = oracle_sets(sh, deriv)
        n = sum(x.size for x in ref)
        got = vals[pos:pos + n]
        pos += n
        sizes = [x.size for x in ref]
        parts = np.split(got, np.cumsum(sizes)[:-1])
        err = _err(parts, ref)
        worst = max(worst, err)
        assert err < TOL, (deriv, ls, err)
    assert pos == vals.size
    print("worst", worst)
