"""Error behaviour of the boundary: the C ABI returns status codes where the
reference asserts or throws (engine.impl.h:173-174,1156-1216; exceptions
Engine::lmax_exceeded, engine.h:893-905), and the context stays usable
after every refused call."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shell(lgx, l, pure=False):
    return lgx.Shell(l, [(1.1, 1.0), (0.3, 0.5)], (0.1, -0.2, 0.3), pure=pure)


def test_lmax_exceeded(lgx):
    ctx = lgx.Context(0)
    g = _shell(lgx, 4)  # beyond LGX_MAX_L = 3
    s = _shell(lgx, 0)
    with pytest.raises(lgx.LgxError) as e:
        ctx.compute_shellset([g, s, s, s])
    assert e.value.status == lgx._lgx.LGX_ERR_LMAX_EXCEEDED
    # second derivatives: shells up to f (the composition raises them to g
    # internally), g refused
    with pytest.raises(lgx.LgxError) as e:
        ctx.compute_shellset([s, g, s, s], deriv=2)
    assert e.value.status == lgx._lgx.LGX_ERR_LMAX_EXCEEDED
    # Engine raises for max_l above the build, like Engine::lmax_exceeded
    with pytest.raises(lgx.LgxError):
        lgx.Engine(lgx.Operator.coulomb, 4, 5, 0)
    # the context still computes
    r = ctx.compute_shellset([s, s, s, s])
    assert r is not None and np.isfinite(r[0]).all()
    ctx.close()


def test_invalid_arguments(lgx):
    lib = lgx._lgx.load()
    ctx = lgx.Context(0)
    s = _shell(lgx, 1)
    arr = (lgx._lgx.LgxShell * 4)(*[s._c() for s in (s, s, s, s)])
    out = np.zeros(4)  # far too small for 81 values
    ns, nv, isnull = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    st = lib.lgx_compute_shellset(ctx._h, arr, 0, 1e-15, 0, lgx._lgx.ptr(out), out.size,
                                  ctypes.byref(ns), ctypes.byref(nv), ctypes.byref(isnull))
    assert st == lgx._lgx.LGX_ERR_TOO_LARGE
    assert b"small" in lib.lgx_last_error(ctx._h)
    st = lib.lgx_compute_shellset(ctx._h, arr, 3, 1e-15, 0, lgx._lgx.ptr(out), out.size,
                                  ctypes.byref(ns), ctypes.byref(nv), ctypes.byref(isnull))
    assert st == lgx._lgx.LGX_ERR_INVALID_ARG  # deriv 3
    # operators: unknown code, negative omega
    assert lib.lgx_set_operator(ctx._h, 7, 0.0) == lgx._lgx.LGX_ERR_INVALID_ARG
    assert lib.lgx_set_operator(ctx._h, lgx._lgx.LGX_OP_ERF_COULOMB, -1.0) == \
        lgx._lgx.LGX_ERR_INVALID_ARG
    # batched calls before a basis was uploaded
    D = np.eye(4)
    J = np.zeros((4, 4))
    K = np.zeros((4, 4))
    st = lib.lgx_jk(ctx._h, lgx._lgx.ptr(D), lgx._lgx.ptr(J), lgx._lgx.ptr(K), 1e-12, 0, 1e-4,
                    None)
    assert st == lgx._lgx.LGX_ERR_NO_BASIS
    # out-of-range shell index in a batch
    atoms = lgx.water_cluster(1, 1, 1, seed=1)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ctx.set_basis(bs)
    with pytest.raises(lgx.LgxError) as e:
        ctx.compute_batch(np.array([[0, 1, 2, len(bs)]]))
    assert e.value.status == lgx._lgx.LGX_ERR_INVALID_ARG
    # and the context still works
    out, offs, isnull = ctx.compute_batch(np.array([[0, 1, 2, 3]]))
    assert np.isfinite(out).all()
    ctx.close()


def test_cpp_facade_exceptions(lgx, tmp_path):
    # the C++ drop-in throws the reference's exception types
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "exc.cpp"
    src.write_text(r"""
#include <libint2.hpp>
#include <iostream>
int main() {
  libint2::initialize();
  int ok = 0;
  try { libint2::Engine e(libint2::Operator::coulomb, 4, 5, 0); }
  catch (const libint2::Engine::lmax_exceeded&) { ++ok; }
  try { libint2::Engine e; e.compute(libint2::Shell::unit(), libint2::Shell::unit(),
                                     libint2::Shell::unit(), libint2::Shell::unit()); }
  catch (const libint2::Engine::using_default_initialized&) { ++ok; }
  try { libint2::Engine e(libint2::Operator::overlap, 4, 2, 0); }
  catch (const std::invalid_argument&) { ++ok; }
  libint2::finalize();
  std::cout << ok << std::endl;
  return ok == 3 ? 0 : 1;
}
""")
    exe = str(tmp_path / "exc")
    lgx._lgx.load()
    subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(root, "include"), str(src),
                           "-L", os.path.join(root, "libint_gb300"), "-llgx",
                           "-Wl,-rpath," + os.path.join(root, "libint_gb300"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)


def test_watchdog_fires_and_context_recovers(lgx):
    # A bound of zero work chunks per warp makes the program kernels' bounded
    # work loops give up at their first chunk (no fault, no hang: the loop
    # ends and raises the context's error flag); the call returns
    # LGX_ERR_WATCHDOG, the flag is cleared, and with the default bound
    # restored the same context computes the same J/K as before.  cc-pVDZ
    # (dd|dd) and (dd|dp) run on the program kernel.
    atoms = lgx.water_cluster(2, 2, 1, spacing=3.0, jitter=0.2, seed=4)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    D = lgx.random_density(bs.nbf, 20, seed=5)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    J0, K0, _ = ctx.jk(D, 1e-12, lgx._lgx.LGX_FP64)
    kinds = {r["kernel"] for r in ctx.last_pass_launches()}
    assert any(k != "register" for k in kinds), kinds
    ctx.set_watchdog(0)
    with pytest.raises(lgx.LgxError) as e:
        ctx.jk(D, 1e-12, lgx._lgx.LGX_FP64)
    assert e.value.status == lgx._lgx.LGX_ERR_WATCHDOG
    ctx.set_watchdog(-1)
    J1, K1, _ = ctx.jk(D, 1e-12, lgx._lgx.LGX_FP64)
    assert np.max(np.abs(J1 - J0)) < 1e-12 and np.max(np.abs(K1 - K0)) < 1e-12
    ctx.close()
