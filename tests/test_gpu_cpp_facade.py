"""The C++ drop-in (include/libint2.hpp) compiled as a libint2 caller would
compile it, run on the GPU, and compared shell set by shell set with the
oracle (FP64, 1e-12 absolute), including first derivatives, lmax_exceeded
and the batched J/K builder."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_engine_facade(lgx, oracle_mod, tmp_path):
    lib = lgx._lgx.load()  # ensure built
    exe = str(tmp_path / "facade")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "engine_facade_test.cpp"),
                           "-L", os.path.join(ROOT, "libint_gb300"), "-llgx",
                           "-Wl,-rpath," + os.path.join(ROOT, "libint_gb300"), "-o", exe])
    outf = str(tmp_path / "out.bin")
    env = dict(os.environ, LIBINT_DATA_PATH=lgx.DATA_PATH)
    r = subprocess.run([exe, outf], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    vals = np.fromfile(outf, dtype=np.float64)
    atoms = [(8, (0.0, -0.143, 0.0)), (1, (1.638, 1.136, 0.0)), (1, (-1.638, 1.136, 0.0)),
             (8, (5.0, 0.2, 0.1)), (1, (6.6, 1.4, 0.0)), (1, (3.4, 1.2, 0.3))]
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    pos = 0
    assert int(vals[pos]) == len(bs)
    pos += 1
    worst = 0.0
    for a in range(8):
        for b in range(8):
            for c in range(8):
                for d in range(8):
                    ref = oracle_mod.compute_quartet(ob, a, b, c, d)
                    flag = vals[pos]
                    pos += 1
                    assert (flag == 0.0) == (ref is None)
                    if ref is None:
                        continue
                    n = ref[0].size
                    worst = max(worst, float(np.max(np.abs(vals[pos:pos + n] - ref[0].reshape(-1)))))
                    pos += n
    assert worst < 1e-12, worst
    for q in [(5, 3, 8, 0), (3, 5, 5, 9), (0, 14, 5, 3)]:
        ref = oracle_mod.compute_quartet(ob, *q, deriv=1)
        r = np.concatenate([x.reshape(-1) for x in ref])
        assert np.max(np.abs(vals[pos:pos + r.size] - r)) < 1e-12
        pos += r.size
    assert vals[pos] == 1.0  # lmax_exceeded thrown
    pos += 1
    nbf = bs.nbf
    J = vals[pos:pos + nbf * nbf].reshape(nbf, nbf)
    K = vals[pos + nbf * nbf:pos + 2 * nbf * nbf].reshape(nbf, nbf)
    idx = np.arange(nbf)
    D = np.exp(-0.3 * np.abs(idx[:, None] - idx[None, :]))
    Kq = oracle_mod.schwarz(ob)
    Jr, Kr, _ = oracle_mod.jk(ob, D, Kq, 0.0)
    assert np.max(np.abs(J - Jr)) < 1e-10
    assert np.max(np.abs(K - Kr)) < 1e-10
    pos += 2 * nbf * nbf
    # xs_xx (d0 and 9 derivative sets through compute2) and xs_xs, against
    # the oracle with Shell::unit() in the empty positions
    full = lgx.BasisSet(list(bs) + [lgx.Shell.unit()])
    obu = oracle_mod.OracleBasis.from_basis(full)
    u = len(bs)
    for a, c, d in [(5, 3, 8), (3, 5, 14), (0, 9, 2)]:
        ref = oracle_mod.compute_quartet(obu, a, u, c, d)[0].reshape(-1)
        assert np.max(np.abs(vals[pos:pos + ref.size] - ref)) < 1e-12
        pos += ref.size
        assert vals[pos] == 9.0
        pos += 1
        rd = oracle_mod.compute_quartet(obu, a, u, c, d, deriv=1)
        rd = np.concatenate([rd[s].reshape(-1) for s in (0, 1, 2, 6, 7, 8, 9, 10, 11)])
        assert np.max(np.abs(vals[pos:pos + rd.size] - rd)) < 1e-12
        pos += rd.size
        r2 = oracle_mod.compute_quartet(obu, a, u, c, u)[0].reshape(-1)
        assert np.max(np.abs(vals[pos:pos + r2.size] - r2)) < 1e-12
        pos += r2.size
    for q in [(5, 3, 8, 0), (3, 0, 1, 9)]:
        assert vals[pos] == 78.0
        pos += 1
        ref = np.concatenate([x.reshape(-1) for x in oracle_mod.compute_quartet(ob, *q, deriv=2)])
        assert np.max(np.abs(vals[pos:pos + ref.size] - ref)) < 1e-12
        pos += ref.size
    oracle_mod.set_operator(2, 0.3)
    try:
        for q in [(5, 3, 8, 0), (3, 5, 5, 9), (0, 14, 5, 3)]:
            ref = oracle_mod.compute_quartet(ob, *q)[0].reshape(-1)
            assert np.max(np.abs(vals[pos:pos + ref.size] - ref)) < 1e-12
            pos += ref.size
    finally:
        oracle_mod.set_operator(0)
    # compute2 with ShellPair data at the machine epsilon, engine at 1e-10
    eps = float(np.finfo(float).eps)
    for q in [(5, 3, 8, 0), (3, 5, 5, 9), (0, 14, 5, 3)]:
        for deriv in (0, 1):
            ref = oracle_mod.compute_quartet(ob, *q, deriv=deriv, precision=1e-10,
                                             pair_precision=eps)
            assert (vals[pos] == 0.0) == (ref is None)
            pos += 1
            if ref is None:
                continue
            r = np.concatenate([x.reshape(-1) for x in ref])
            assert np.max(np.abs(vals[pos:pos + r.size] - r)) < 1e-12
            pos += r.size
    assert pos == vals.size
