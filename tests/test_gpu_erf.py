"""Range-separated Coulomb operators erf(omega r)/r and erfc(omega r)/r
(Operator::erf_coulomb / erfc_coulomb with omega as params) on the CUDA
path against the oracle's restatement of libint's core integrals:
shell sets at deriv 0 and 1 through Engine, the identity erf + erfc =
coulomb, and Schwarz-screened J/K builds (FP64 and mixed) with erf and erfc
(their small classes on the attenuated register kernels, the rest on the
attenuated program kernel)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = 0.4


@pytest.fixture()
def oracle_op(oracle_mod):
    yield oracle_mod
    oracle_mod.set_operator(0)


def test_engine_erf_erfc_vs_oracle(lgx, oracle_op):
    atoms = lgx.water_cluster(1, 1, 1, seed=3)
    bs = lgx.BasisSet("cc-pVTZ", atoms)          # s..f shells
    ob = oracle_op.OracleBasis.from_basis(bs)
    rng = np.random.default_rng(21)
    quads = rng.integers(0, len(bs), size=(60, 4))
    for oper, code in ((lgx.Operator.erf_coulomb, 1), (lgx.Operator.erfc_coulomb, 2)):
        oracle_op.set_operator(code, OMEGA)
        for deriv in (0, 1):
            eng = lgx.Engine(oper, bs.max_nprim(), bs.max_l(), deriv).set_params(OMEGA)
            for q in quads[: (60 if deriv == 0 else 15)]:
                r = eng.compute(*[bs[int(i)] for i in q])
                ref = oracle_op.compute_quartet(ob, *[int(i) for i in q], deriv=deriv)
                assert (r is None) == (ref is None)
                if r is None:
                    continue
                got = [r] if deriv == 0 else r
                for x, y in zip(got, ref):
                    assert np.max(np.abs(x - y)) < 1e-12, (oper, deriv, q)
    # erf + erfc = coulomb, with the three engines interleaved on one context
    e1 = lgx.Engine(lgx.Operator.erf_coulomb, bs.max_nprim(), bs.max_l()).set_params(OMEGA)
    e2 = lgx.Engine(lgx.Operator.erfc_coulomb, bs.max_nprim(), bs.max_l()).set_params(OMEGA)
    e0 = lgx.Engine(lgx.Operator.coulomb, bs.max_nprim(), bs.max_l())
    for q in quads[:20]:
        sh = [bs[int(i)] for i in q]
        a, b, c = e1.compute(*sh), e2.compute(*sh), e0.compute(*sh)
        if c is not None:
            assert np.max(np.abs(a + b - c)) < 1e-12


@pytest.mark.parametrize("oper", ["erf", "erfc"])
def test_jk_attenuated_vs_oracle(lgx, oracle_op, oper):
    atoms = lgx.water_cluster(2, 1, 1, spacing=3.0, jitter=0.2, seed=1)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_op.OracleBasis.from_basis(bs)
    D = lgx.random_density(bs.nbf, 10, seed=2)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    op, code = ((lgx.Operator.erf_coulomb, 1) if oper == "erf"
                else (lgx.Operator.erfc_coulomb, 2))
    ctx.set_operator(op, OMEGA)
    Kq = ctx.schwarz()
    oracle_op.set_operator(code, OMEGA)
    assert np.max(np.abs(Kq - oracle_op.schwarz(ob))) < 1e-12
    J, K, st = ctx.jk(D, 1e-12)
    Jr, Kr, nq = oracle_op.jk(ob, D, Kq, 1e-12)
    assert st.quartets_fp64 == nq
    assert np.max(np.abs(J - Jr)) < 1e-11 and np.max(np.abs(K - Kr)) < 1e-11
    Jm, Km, stm = ctx.jk(D, 1e-12, mode=1, mixed_thresh=1e-4)
    assert stm.quartets_fp32 > 0
    e64, em = lgx.jk_energies(D, J, K), lgx.jk_energies(D, Jm, Km)
    assert abs(e64[0] - em[0]) <= 1e-8 and abs(e64[1] - em[1]) <= 1e-8
    # back to coulomb: the context recomputes its Schwarz factors and bins
    ctx.set_operator(lgx.Operator.coulomb)
    J0, K0, _ = ctx.jk(D, 1e-12)
    oracle_op.set_operator(0)
    Jr0, Kr0, _ = oracle_op.jk(ob, D, oracle_op.schwarz(ob), 1e-12)
    assert np.max(np.abs(J0 - Jr0)) < 1e-11 and np.max(np.abs(K0 - Kr0)) < 1e-11
    ctx.close()
