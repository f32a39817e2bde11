"""Host logic: the per-class VRR/HRR programs executed on the CPU by a test
interpreter (tests/cpp/program_interp.cpp) reproduce the oracle's canonical
Cartesian shell sets for every class up to (ff|ff) (deriv 0), (dd|dd) plus
f classes (deriv 1), and the internal g classes of the second-derivative
composition (deriv 1)."""
import ctypes
import itertools
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def interp(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("interp") / "libinterp.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared",
                           os.path.join(HERE, "cpp", "program_interp.cpp"),
                           os.path.join(ROOT, "libint_gb300", "csrc", "lgx_program.cpp"),
                           "-o", out])
    lib = ctypes.CDLL(out)
    lib.interp_quartet.restype = ctypes.c_int
    return lib


def canonical_classes(lmax):
    for la, lb, lc, ld in itertools.product(range(lmax + 1), repeat=4):
        if la >= lb and lc >= ld and la + lb <= lc + ld:
            yield la, lb, lc, ld


def _run(interp, oracle_mod, ls, deriv, rng):
    l = np.array(ls, np.int32)
    nprim = np.array([1 + (k + ls[k]) % 2 for k in range(4)], np.int32)
    alpha = np.concatenate([np.sort(rng.uniform(0.2, 4.0, n))[::-1] for n in nprim])
    raw = rng.uniform(0.3, 1.0, int(nprim.sum()))
    coeff = np.zeros_like(raw)
    o = 0
    for k in range(4):
        c, _ = oracle_mod.shell_normalize(ls[k], alpha[o:o + nprim[k]], raw[o:o + nprim[k]])
        coeff[o:o + nprim[k]] = c
        o += nprim[k]
    O = rng.uniform(-1, 1, 12)
    ncart = int(np.prod([(x + 1) * (x + 2) // 2 for x in ls]))
    nsets = 12 if deriv else 1
    out = np.zeros(nsets * ncart)
    P = lambda a, t=ctypes.c_double: a.ctypes.data_as(ctypes.POINTER(t))
    r = interp.interp_quartet(P(l, ctypes.c_int), P(nprim, ctypes.c_int), P(alpha), P(coeff),
                              P(O), deriv, P(out))
    assert r == ncart
    ob = oracle_mod.OracleBasis(l, np.zeros(4, np.int32), nprim, O, alpha, coeff)
    ref = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, deriv, precision=0.0)
    ref = np.concatenate([x.reshape(-1) for x in ref])
    scale = max(1.0, float(np.max(np.abs(ref))))
    return float(np.max(np.abs(out - ref))) / scale


def test_programs_deriv0(interp, oracle_mod):
    rng = np.random.default_rng(0)
    worst = max(_run(interp, oracle_mod, ls, 0, rng) for ls in canonical_classes(3))
    assert worst < 1e-13, worst


def test_programs_deriv1(interp, oracle_mod):
    rng = np.random.default_rng(1)
    classes = [c for c in canonical_classes(3) if sum(c) <= 6]
    worst = max(_run(interp, oracle_mod, ls, 1, rng) for ls in classes)
    assert worst < 1e-12, worst


def test_programs_deriv1_internal_g_classes(interp, oracle_mod):
    # the Cartesian g classes the second-derivative composition raises f
    # shells to (first derivatives of one shell raised by a quantum)
    rng = np.random.default_rng(7)
    classes = [(0, 0, 4, 0), (1, 0, 4, 1), (2, 1, 4, 0), (2, 0, 4, 2), (3, 0, 4, 1), (3, 3, 4, 3)]
    worst = max(_run(interp, oracle_mod, ls, 1, rng) for ls in classes)
    assert worst < 1e-12, worst
