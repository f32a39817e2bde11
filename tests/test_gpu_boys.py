"""The device Boys evaluators on their own (lgx_boys), against the reference's
FmEval_Reference<long double> values (tests/golden/boys.npz, T in [0, 1000],
m <= 16) and, on a dense grid of T, against the oracle (itself pinned to the
same fixture at 1e-14).

Bounds: FP64 evaluators 1e-14 relative (the Taylor truncation on the 1/64
grid is below 3.2e-16; the register evaluator's asymptotic branch drops
e^{-T} above T = 50, at most 1.7e-15 relative for m <= 6).  FP32 evaluators:
|dF_m| <= 6e-8 (1 + T) F_{m+1}(T) + 8e-7 (mmax + 2) F_m(T) + 1e-44, where
the first term is the rounding of T to FP32 (dF_m/dT = -F_{m+1}); the second
the FP32 Taylor step, exponential and two roundings per recursion step, and
above T = 50 the 2-ulp error of rsqrtf carried (2m + 1)-fold through the
upward recursion; the third the FP32 denormal range (F_m below 1.2e-38 at
large T and m).  A float32 emulation of both evaluators stays within it
over T in [0, 2000]."""
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
    bound = 6e-8 * (1.0 + T)[:, None] * ref[:, 1:] + 8e-7 * (mmax + 2) * ref[:, :-1] + 1e-44
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


@pytest.mark.parametrize("v64,vb,mmax", [(0, 4, 16), (1, 5, 6)])
def test_mixed_scheme_boys_is_fp64_rounded_to_fp32(gpu_ctx, v64, vb, mmax):
    # the LGX_MIXED scheme's FP32 kernels take FP64 Boys values rounded to
    # nearest FP32 (integer-only conversion).  Both evaluators (program and
    # register kernels) stop the FP64 series at 4 terms (relative error
    # below 1.6e-10) and take T as a double-float pair, so their value may,
    # rarely, round to the neighbouring float32 of the FP64 evaluator's
    rng = np.random.default_rng(13)
    T = np.concatenate([load("boys.npz")["T"], rng.uniform(0, 60, 4000),
                        rng.uniform(60, 2000, 500)])
    F64 = gpu_ctx.boys(T, mmax, v64)
    Fb = gpu_ctx.boys(T, mmax, vb)
    normal = np.abs(F64) >= np.finfo(np.float32).tiny
    want = F64[normal].astype(np.float32)
    got = Fb[normal].astype(np.float32)
    ulps = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1 and np.mean(ulps == 0) > 0.999, (ulps.max(), np.mean(ulps == 0))
    assert np.all(Fb[~normal & (np.abs(F64) < 0.5 * np.finfo(np.float32).tiny)] == 0.0)


@pytest.mark.parametrize("mmax", [0, 1, 2, 4, 6])
def test_mixed_register_path_from_pair_data(gpu_ctx, oracle_mod, mmax):
    # the LGX_MIXED register kernels' whole Boys path from primitive-pair data
    # (lgx_boys variant 6): double-float records of P and zeta, the
    # double-float argument T = rho |Pb - Pk|^2, the FP64 evaluator, the FP32
    # rounding; against the oracle's F_m at the argument formed in extended
    # precision: within 1 FP32 ulp and almost always its rounding
    rng = np.random.default_rng(14 + mmax)
    n = 6000
    zb = np.exp(rng.uniform(np.log(0.05), np.log(3e4), n))
    zk = np.exp(rng.uniform(np.log(0.05), np.log(3e4), n))
    Pb = rng.uniform(-30.0, 30.0, (n, 3))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    d = np.exp(rng.uniform(np.log(1e-4), np.log(40.0), n))
    d[:50] = 0.0  # coincident centres: T = 0
    Pk = Pb + d[:, None] * u
    pairs = np.column_stack([Pb, zb, Pk, zk])
    # the argument from the same double inputs, in extended precision
    L = np.longdouble
    dd = (Pb.astype(L) - Pk.astype(L))
    T = (zb.astype(L) * zk.astype(L) / (zb.astype(L) + zk.astype(L)) * (dd * dd).sum(1))
    T = T.astype(np.float64)
    ref = _ref_dense(oracle_mod, T, mmax)
    F = gpu_ctx.boys(pairs, mmax, 6)
    normal = np.abs(ref) >= np.finfo(np.float32).tiny
    want = ref[normal].astype(np.float32)
    got = F[normal].astype(np.float32)
    ulps = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1 and np.mean(ulps == 0) > 0.999, (ulps.max(), np.mean(ulps == 0))
    assert np.all(F[~normal & (np.abs(ref) < 0.5 * np.finfo(np.float32).tiny)] == 0.0)
    assert (T > 50).sum() > 100 and (T < 1).sum() > 100  # both branches exercised
