"""The CPU oracle against golden fixtures produced by the reference's own
code (brute-force ERIs of src/bin/test_eri/eri.h, FmEval_Reference2,
Shell::renorm, SolidHarmonicsCoefficients, DerivMapGenerator).  Thresholds
follow tests/unit/test-2body.cc:304-322: absolute 5e-14 or relative 1e-9,
tightened to a plain 1e-12 absolute (the parity bar of this project)."""
import numpy as np

from golden_util import eri_cases, load


def test_boys_vs_reference(oracle_mod):
    g = load("boys.npz")
    worst = 0.0
    for T, ref in zip(g["T"], g["F_refld"]):
        F = oracle_mod.boys(float(T), len(ref) - 1)
        worst = max(worst, float(np.max(np.abs(F - ref))))
    assert worst < 1e-14, worst


def test_solid_harmonics_vs_reference(oracle_mod):
    g = load("solid.npz")
    for (l, m, lx, ly, lz), c in zip(g["idx"], g["coeff"]):
        assert abs(oracle_mod.solid_coeff(int(l), int(m), int(lx), int(ly), int(lz)) - c) < 1e-13


def test_shell_normalization_vs_reference(oracle_mod):
    g = load("shells.npz")
    for l, a, cin, cout in zip(g["l"], g["alpha"], g["cin"], g["cout"]):
        c, _ = oracle_mod.shell_normalize(int(l), a, cin)
        np.testing.assert_allclose(c, cout, rtol=1e-13, atol=0)


def test_eri_shellsets_vs_reference_bruteforce(oracle_mod):
    worst = 0.0
    for l, pure, nprim, alpha, coeff, O, deriv, vals in eri_cases():
        ob = oracle_mod.OracleBasis(l, pure, nprim, O, alpha, coeff)
        r = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, deriv, precision=0.0)
        got = np.concatenate([x.reshape(-1) for x in r])
        err = float(np.max(np.abs(got - vals)))
        worst = max(worst, err)
        assert err < 1e-12, (tuple(l), deriv, err)
    print("worst", worst)


def test_eri3c_2c_shellsets_vs_reference_bruteforce(oracle_mod):
    # 3-centre (a 1|c d) and 2-centre (a 1|c 1) sets with Shell::unit()
    from golden_util import eri3c_cases
    for l, pure, nprim, alpha, coeff, O, deriv, rank, vals in eri3c_cases():
        ob = oracle_mod.OracleBasis(l, pure, nprim, O, alpha, coeff)
        r = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, deriv, precision=0.0)
        got = np.concatenate([x.reshape(-1) for x in r])
        err = float(np.max(np.abs(got - vals)))
        assert err < 1e-12, (tuple(l), rank, deriv, err)


def test_deriv2_shellsets_vs_reference_bruteforce(oracle_mod):
    # deriv_order 2: 78 sets per quartet, order = CartesianDerivIterator<4>(2)
    from golden_util import eri_d2_cases
    g = load("eri_d2.npz")
    assert [(int(a), int(b)) for a, b in zip(g["c1"], g["c2"])] == \
        [(c1, c2) for c1 in range(12) for c2 in range(c1, 12)]
    for l, pure, nprim, alpha, coeff, O, vals in eri_d2_cases():
        ob = oracle_mod.OracleBasis(l, pure, nprim, O, alpha, coeff)
        r = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, 2, precision=0.0)
        got = np.concatenate([x.reshape(-1) for x in r])
        assert np.max(np.abs(got - vals)) < 1e-12, tuple(l)


def test_derivative_order_and_map(oracle_mod):
    g = load("derivmap.npz")
    # sets ordered A_x, A_y, A_z, B_x, ..., D_z
    assert list(g["order"]) == list(range(12))
    # the remap used by the oracle/kernels: canonical centre k -> target
    # centre perm[k] (engine.impl.h:1181-1211 swaps)
    for sbk in range(2):
        for stb in range(2):
            for stk in range(2):
                perm = [
                    (3 if stk else 2) if sbk else (1 if stb else 0),
                    (2 if stk else 3) if sbk else (0 if stb else 1),
                    (1 if stb else 0) if sbk else (3 if stk else 2),
                    (0 if stb else 1) if sbk else (2 if stk else 3),
                ]
                for s in range(12):
                    assert g["map"][sbk, stb, stk, s] == perm[s // 3] * 3 + s % 3


def _random_quartet_basis(oracle_mod, rng):
    shells = []
    for l in rng.integers(0, 4, 4):
        n = int(rng.integers(1, 3))
        a = rng.uniform(0.2, 3.0, n)
        c, _ = oracle_mod.shell_normalize(int(l), a, rng.uniform(0.3, 1.0, n))
        shells.append((int(l), int(l > 1), a, c, rng.uniform(-1, 1, 3)))
    return oracle_mod.OracleBasis(np.array([s[0] for s in shells], np.int32),
                                  np.array([s[1] for s in shells], np.int32),
                                  np.array([len(s[2]) for s in shells], np.int32),
                                  np.concatenate([s[4] for s in shells]),
                                  np.concatenate([s[2] for s in shells]),
                                  np.concatenate([s[3] for s in shells]))


def test_attenuated_operators_identities(oracle_mod):
    # erf + erfc = coulomb; erf(omega -> large) -> coulomb; and the closed
    # form of two normalized s Gaussians under erf(omega r)/r:
    # (pi/a)^{3/2} (pi/g)^{3/2} erf(mu R)/R, 1/mu^2 = 1/a + 1/g + 1/omega^2
    import math
    rng = np.random.default_rng(5)
    try:
        for t in range(20):
            ob = _random_quartet_basis(oracle_mod, rng)
            d = int(t % 3 == 0)
            oracle_mod.set_operator(0)
            c = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, d, precision=0.0)
            oracle_mod.set_operator(1, 0.7)
            e = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, d, precision=0.0)
            oracle_mod.set_operator(2, 0.7)
            f = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, d, precision=0.0)
            oracle_mod.set_operator(1, 1e4)
            big = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, d, precision=0.0)
            for x, y, z, w in zip(c, e, f, big):
                assert np.max(np.abs(x - (y + z))) < 1e-13
                assert np.max(np.abs(x - w)) < 1e-7
        a, g, w = 1.1, 0.7, 0.4
        ca = oracle_mod.shell_normalize(0, np.array([a]), np.array([1.0]))[0][0]
        cg = oracle_mod.shell_normalize(0, np.array([g]), np.array([1.0]))[0][0]
        A, C = np.zeros(3), np.array([0.3, -0.2, 0.5])
        z = np.zeros(4, np.int32)
        ob = oracle_mod.OracleBasis(z, z, np.ones(4, np.int32), np.concatenate([A, A, C, A]),
                                    np.array([a, 0.0, g, 0.0]), np.array([ca, 1.0, cg, 1.0]))
        oracle_mod.set_operator(1, w)
        v = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, precision=0.0)[0].item()
        R = np.linalg.norm(A - C)
        mu = 1 / math.sqrt(1 / a + 1 / g + 1 / w ** 2)
        ref = (math.pi / a) ** 1.5 * (math.pi / g) ** 1.5 * ca * cg * math.erf(mu * R) / R
        assert abs(v - ref) < 1e-13 * abs(ref)
    finally:
        oracle_mod.set_operator(0)


def test_python_binding_golden_norms(oracle_mod):
    # the reference's python/tests/test_libint2.py:9-10,37-48: norms of
    # (pp|ss), of every quartet of [s, p, s, p], and of the three-shell
    # braket XXXS on s = Shell(0, [(1, 10)]) at the origin, which libint's
    # Engine evaluates as (a unit|c d) (engine.impl.h:159-166)
    import libint_gb300 as lg
    s = lg.Shell(0, [(1, 10)])
    p = lg.Shell(1, [(1, 10)])
    u = lg.Shell.unit()
    ob = oracle_mod.OracleBasis.from_basis(lg.BasisSet([s, p, u]))
    pp_ss = oracle_mod.compute_quartet(ob, 1, 1, 0, 0, precision=1e-15)[0]
    assert abs(np.linalg.norm(pp_ss) - 1.62867503968) < 1e-10
    idx = [0, 1, 0, 1]
    sq = 0.0
    for a in idx:
        for b in idx:
            for c in idx:
                for d in idx:
                    r = oracle_mod.compute_quartet(ob, a, b, c, d, precision=1e-15)
                    sq += float(np.sum(r[0] ** 2)) if r is not None else 0.0
    assert abs(np.sqrt(sq) - 14.7036075402) < 1e-9
    s_u_ss = oracle_mod.compute_quartet(ob, 0, 2, 0, 0, precision=1e-15)[0]
    assert abs(np.linalg.norm(s_u_ss) - 3.6563211198) < 1e-9
