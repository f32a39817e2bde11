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
