"""The device Boys evaluators on their own (lgx_boys), against the reference's
FmEval_Reference<long double> values (tests/golden/boys.npz, T in [0, 1000],
m <= 16) and, on a dense grid of T, against the oracle (itself pinned to the
same fixture at 1e-14).

Bounds: FP64 evaluators 1e-14 relative (the Taylor truncation on the 1/32
grid is below 5e-17; the register evaluator's asymptotic branch drops
e^{-T} above T = 50, at most 1.7e-15 relative for m <= 6).  FP32 evaluators:
|dF_m| <= 6e-8 (1 + T) F_{m+1}(T) + 1e-6 F_m(T), where the first term is the
rounding of T to FP32 (dF_m/dT = -F_{m+1}) and the second the FP32 Taylor
step, exponential and downward recursion."""
import numpy as np
import pytest

from golden_util import load

pytestmark = pytest.mark.gpu


def _ref_dense(oracle_mod, T, mmax):
    return np.array([oracle_mod.boys(float(t), mmax) for t in T])


@pytest.mark.parametrize("variant,mmax", [(0, 16), (1, 6)])
def test_fp64_boys_vs_reference_fixture(gpu_ctx, variant, mmax):
    g = load("boys.npz")
    T = g["T"]
    ref = g["F_refld"][:, :mmax + 1]
    F = gpu_ctx.boys(T, mmax, variant)
    rel = np.abs(F - ref) / np.abs(ref)
    assert rel.max() < 1e-14, (variant, rel.max(), T[np.argmax(rel.max(1))])


@pytest.mark.parametrize("variant,mmax", [(0, 16), (1, 6)])
def test_fp64_boys_dense_vs_oracle(gpu_ctx, oracle_mod, variant, mmax):
    rng = np.random.default_rng(11)
    T = np.concatenate([rng.uniform(0, 50, 3000), rng.uniform(50, 1000, 500),
                        np.arange(0, 50.02, 1.0 / 64), [49.999999, 50.0, 50.000001]])
    ref = _ref_dense(oracle_mod, T, mmax)
    F = gpu_ctx.boys(T, mmax, variant)
    rel = np.abs(F - ref) / np.abs(ref)
    assert rel.max() < 1e-14, (variant, rel.max(), T[np.argmax(rel.max(1))])


@pytest.mark.parametrize("variant,mmax", [(2, 16), (3, 6)])
def test_fp32_boys_within_stated_bound(gpu_ctx, oracle_mod, variant, mmax):
    g = load("boys.npz")
    rng = np.random.default_rng(12)
    T = np.concatenate([g["T"], rng.uniform(0, 50, 2000), rng.uniform(50, 1000, 300)])
    ref = _ref_dense(oracle_mod, T, mmax + 1)
    F = gpu_ctx.boys(T, mmax, variant)
    bound = 6e-8 * (1.0 + T)[:, None] * ref[:, 1:] + 1e-6 * ref[:, :-1]
    err = np.abs(F - ref[:, :-1])
    assert np.all(err <= bound), float(np.max(err / bound))


def test_boys_rejects_bad_arguments(gpu_ctx, lgx):
    for T in ([-1.0], [float("nan")], [float("inf")]):
        with pytest.raises(lgx.LgxError) as e:
            gpu_ctx.boys(np.array(T), 2, 0)
        assert e.value.status == lgx._lgx.LGX_ERR_INVALID_ARG
    with pytest.raises(lgx.LgxError):
        gpu_ctx.boys(np.array([1.0]), 7, 1)  # register evaluators stop at m = 6
    assert gpu_ctx.boys(np.array([0.0]), 0, 0)[0, 0] == 1.0
