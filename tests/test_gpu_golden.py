"""The CUDA path against golden shell sets from the reference's own
brute-force ERI code (independent of the oracle): every class up to (ff|ff)
at deriv 0 and up to L=5 at deriv 1, in libint's buffer order."""
import numpy as np
import pytest

from golden_util import eri_cases

pytestmark = pytest.mark.gpu


def test_engine_vs_reference_bruteforce(lgx):
    ctx = lgx.Context(0)
    worst = 0.0
    for l, pure, nprim, alpha, coeff, O, deriv, vals in eri_cases():
        shells, off = [], 0
        for k in range(4):
            n = int(nprim[k])
            shells.append(lgx.Shell.from_normalized(int(l[k]), alpha[off:off + n],
                                                    coeff[off:off + n], O[3 * k:3 * k + 3],
                                                    bool(pure[k])))
            off += n
        r = ctx.compute_shellset(shells, deriv, precision=0.0)
        got = np.concatenate([x.reshape(-1) for x in r])
        err = float(np.max(np.abs(got - vals)))
        worst = max(worst, err)
        assert err < 1e-12, (tuple(l), deriv, err)
    print("worst", worst)
    ctx.close()


def test_engine_deriv2_vs_reference_bruteforce(lgx):
    # deriv_order 2 (78 sets per quartet, shells up to f) through Engine
    from golden_util import eri_d2_cases
    worst = 0.0
    for l, pure, nprim, alpha, coeff, O, vals in eri_d2_cases():
        shells, off = [], 0
        for k in range(4):
            n = int(nprim[k])
            shells.append(lgx.Shell.from_normalized(int(l[k]), alpha[off:off + n],
                                                    coeff[off:off + n], O[3 * k:3 * k + 3],
                                                    bool(pure[k])))
            off += n
        eng = lgx.Engine(lgx.Operator.coulomb, 4, 3, 2, precision=0.0)
        assert eng.nshellsets() == 78
        r = eng.compute(*shells)
        got = np.concatenate([x.reshape(-1) for x in r])
        err = float(np.max(np.abs(got - vals)))
        worst = max(worst, err)
        assert err < 1e-12, (tuple(l), err)
    print("worst", worst)
