"""Engine.compute on the GPU against the CPU oracle (restatement of libint's
compute2<coulomb, xx_xx, d>), shell set by shell set, in libint's buffer
order.  Tolerance: 1e-12 absolute per integral (FP64)."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rand_shell(lg, rng, l, nprim, pure):
    alpha = np.sort(rng.uniform(0.15, 6.0, nprim))[::-1]
    coeff = rng.uniform(0.2, 1.0, nprim)
    return lg.Shell(l, list(zip(alpha, coeff)), rng.uniform(-1.2, 1.2, 3), pure=pure)


def _check(lg, oracle_mod, shells, deriv, tol=TOL, precision=np.finfo(float).eps):
    bs = lg.BasisSet(list(shells))
    ob = oracle_mod.OracleBasis.from_basis(bs)
    eng = lg.Engine(lg.Operator.coulomb, 10, 3, deriv, precision=precision)
    got = eng.compute(*shells)
    ref = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, deriv, precision=precision)
    assert (got is None) == (ref is None)
    if got is None:
        return 0.0
    if deriv == 0:
        got = [got]
    err = max(float(np.max(np.abs(g - r))) for g, r in zip(got, ref))
    assert err < tol, (tuple(s.l for s in shells), deriv, err)
    return err


@pytest.mark.parametrize("deriv", [0, 1])
def test_all_classes_random_shells(lgx, oracle_mod, deriv):
    rng = np.random.default_rng(11 + deriv)
    lmax = 3 if deriv == 0 else 2
    worst = 0.0
    for ls in itertools.product(range(lmax + 1), repeat=4):
        shells = [_rand_shell(lgx, rng, l, 1 + (l + k) % 3, l > 1) for k, l in enumerate(ls)]
        worst = max(worst, _check(lgx, oracle_mod, shells, deriv))
    print("worst", worst)


def test_deriv1_f_classes(lgx, oracle_mod):
    rng = np.random.default_rng(5)
    for ls in [(3, 0, 0, 0), (0, 3, 1, 0), (3, 1, 2, 0), (2, 2, 3, 1), (3, 3, 1, 1)]:
        shells = [_rand_shell(lgx, rng, l, 1 + (l % 2), l > 1) for l in ls]
        _check(lgx, oracle_mod, shells, 1)


def test_cartesian_and_pure_p(lgx, oracle_mod):
    rng = np.random.default_rng(3)
    for pure in (False, True):
        shells = [_rand_shell(lgx, rng, l, 2, pure) for l in (1, 2, 1, 3)]
        _check(lgx, oracle_mod, shells, 0)


def test_python_binding_golden_norms(lgx):
    # python/tests/test_libint2.py:9-10,37,44-48
    s = lgx.Shell(0, [(1, 10)])
    p = lgx.Shell(1, [(1, 10)])
    eng = lgx.coulomb()
    assert abs(np.linalg.norm(eng.compute(p, p, s, s)) - 1.62867503968) < 1e-10
    basis = [s, p, s, p]
    full = eng.compute(basis, basis, basis, basis)
    assert abs(np.linalg.norm(full) - 14.7036075402) < 1e-9
    # :40-43, braket XXXS on three identical s shells: the Engine evaluates a
    # three-shell call as (a unit|c d) (engine.impl.h:159-166), = (ss|s) here
    eng3 = lgx.Engine(lgx.Operator.coulomb, braket=lgx.BraKet.XXXS)
    assert abs(np.linalg.norm(eng3.compute(s, s, s)) - 3.6563211198) < 1e-9


def test_fully_screened_returns_none(lgx):
    # two far-apart tight pairs: every primitive pair falls below precision
    s1 = lgx.Shell(0, [(50.0, 1.0)], (0, 0, 0))
    s2 = lgx.Shell(0, [(50.0, 1.0)], (20, 0, 0))
    eng = lgx.Engine(lgx.Operator.coulomb, 1, 0, 0)
    assert eng.compute(s1, s2, s1, s1) is None
    assert eng.results()[0] is None


def test_water_cc_pvdz_quartets(lgx, oracle_mod):
    atoms = lgx.water_cluster(1, 1, 1, seed=3)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    eng = lgx.Engine(lgx.Operator.coulomb, bs.max_nprim(), bs.max_l(), 0)
    rng = np.random.default_rng(0)
    for _ in range(60):
        q = [int(x) for x in rng.integers(0, len(bs), 4)]
        got = eng.compute(*[bs[i] for i in q])
        ref = oracle_mod.compute_quartet(ob, *q)
        assert np.max(np.abs(got - ref[0])) < TOL, q


@pytest.mark.parametrize("precision", [1e-10, 1e-7])
def test_coarse_precision_vs_oracle(lgx, oracle_mod, precision):
    # Engine::set_precision above the default: the primitive quartets cut by
    # the coarser threshold (engine.impl.h:1306-1766) must be the oracle's
    # ones, or the sets differ by up to ~100x the threshold
    atoms = lgx.water_cluster(1, 1, 1, seed=3)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    eng = lgx.Engine(lgx.Operator.coulomb, bs.max_nprim(), bs.max_l(), 0, precision=precision)
    rng = np.random.default_rng(1)
    for _ in range(60):
        q = [int(x) for x in rng.integers(0, len(bs), 4)]
        got = eng.compute(*[bs[i] for i in q])
        ref = oracle_mod.compute_quartet(ob, *q, precision=precision)
        assert (got is None) == (ref is None), q
        if got is not None:
            assert np.max(np.abs(got - ref[0])) < TOL, q


def test_precomputed_shellpair_data_vs_oracle(lgx, oracle_mod, gpu_ctx):
    # Engine::compute2 with ShellPair data precomputed at the machine epsilon
    # and the engine at 1e-10 (engine.impl.h:1259-1276; compute_2body_fock
    # passes such pairs, hartree-fock++.cc:1386-1425): the primitive pairs at
    # eps, the primitive quartets screened at 1e-10 -- the oracle's
    # pair_precision path
    atoms = lgx.water_cluster(1, 1, 1, seed=3)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    eps, prec = np.finfo(float).eps, 1e-10
    rng = np.random.default_rng(2)
    ndiff = 0
    for _ in range(60):
        q = [int(x) for x in rng.integers(0, len(bs), 4)]
        sh = [bs[i] for i in q]
        for deriv in (0, 1):
            got = gpu_ctx.compute_shellset(sh, deriv, prec, pair_ln_prec=(np.log(eps), np.log(eps)))
            ref = oracle_mod.compute_quartet(ob, *q, deriv, precision=prec, pair_precision=eps)
            assert (got is None) == (ref is None), q
            if got is None:
                continue
            assert max(float(np.max(np.abs(g - r))) for g, r in zip(got, ref)) < TOL, (q, deriv)
            plain = gpu_ctx.compute_shellset(sh, deriv, prec)
            if plain is None or max(float(np.max(np.abs(g - p))) for g, p in zip(got, plain)) > 0:
                ndiff += 1
    print("sets that differ from pairs built at the engine precision:", ndiff)
    # both at the engine precision: the plain call exactly
    sh = [bs[i] for i in (3, 1, 4, 0)]
    a = gpu_ctx.compute_shellset(sh, 0, prec, pair_ln_prec=(np.log(prec), np.log(prec)))
    b = gpu_ctx.compute_shellset(sh, 0, prec)
    assert (a is None and b is None) or np.array_equal(a[0], b[0])


def test_compute_2body_fock_vs_oracle(lgx, oracle_mod):
    # the binding's Engine.compute_2body_fock(D, basis) (python/src/libint2/
    # engine.cc:230-279) through one GPU J/K pass: G = 2J - K
    atoms = lgx.water_cluster(1, 1, 1, seed=3)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    D = lgx.random_density(bs.nbf, 5, seed=4)
    G = lgx.Engine(lgx.Operator.coulomb).compute_2body_fock(D, bs)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    J, K, _ = oracle_mod.jk(ob, D, oracle_mod.schwarz(ob), 0.0)
    assert np.max(np.abs(G - (2 * J - K))) < 1e-11
