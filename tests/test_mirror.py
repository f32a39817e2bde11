"""Host logic of the Python mirror of the reference's pybind11 module
(python/src/libint2/libint2.cc, engine.cc), without a GPU: Shell
coefficients of normalized primitives, Operator.rank, the XXXS braket name,
and Engine.compute_2body_fock against the binding's own quartet loop, with
the J/K supplied by the oracle through a stand-in context."""
import numpy as np
import pytest


def test_shell_coeffs_normalized(lgx):
    # Shell::coeff_normalized (shell.h:915-928): one primitive of a unit-
    # normalized shell has coefficient 1; a contraction keeps its ratios
    assert np.allclose(lgx.Shell(1, [(1.0, 10.0)]).coeffs_normalized, [1.0], rtol=1e-14)
    s = lgx.Shell(2, [(2.0, 0.3), (0.5, 0.7)])
    r = np.array(s.coeffs_normalized) / np.array([0.3, 0.7])
    assert abs(r[0] - r[1]) < 1e-14 * r[0]
    assert lgx.Shell.unit().coeffs_normalized == [1.0]


def test_operator_rank_and_braket_names(lgx):
    assert lgx.Operator.rank(lgx.Operator.coulomb) == 2
    assert lgx.BraKet.XXXS is lgx.BraKet.xs_xx
    e = lgx.Engine(lgx.Operator.coulomb, braket=lgx.BraKet.XXXS)
    assert e.braket_rank() == 3 and e.nshellsets() == 1


class _OracleContext:
    """Stand-in for Context: J and K from the oracle."""

    def __init__(self, oracle_mod):
        self.o = oracle_mod
        self.calls = []

    def set_operator(self, oper, omega=0.0):
        self.calls.append(("op", oper, omega))

    def set_basis(self, bs):
        self.bs = bs
        self.calls.append(("basis", len(bs)))

    def jk(self, D, schwarz_thresh=1e-12, mode=0, mixed_thresh=1e-4):
        ob = self.o.OracleBasis.from_basis(self.bs)
        J, K, _ = self.o.jk(ob, D, self.o.schwarz(ob), schwarz_thresh)
        return J, K, None


def _binding_fock(oracle_mod, bs, D):
    # the binding's compute_2body_fock loop (engine.cc:241-279), restated
    ob = oracle_mod.OracleBasis.from_basis(bs)
    bf, n, ns = bs.shell2bf(), bs.nbf, len(bs)
    sz = [s.size() for s in bs]
    f = np.zeros((n, n))
    for P in range(ns):
        for Q in range(P + 1):
            for R in range(ns):
                for S in range(R + 1):
                    r = oracle_mod.compute_quartet(ob, P, Q, R, S)
                    if r is None:
                        continue
                    v = r[0].reshape(sz[P], sz[Q], sz[R], sz[S])
                    v = v * ((0.5 if P == Q else 1.0) * (0.5 if R == S else 1.0))
                    p_, q_, r_, s_ = (slice(bf[X], bf[X] + sz[X]) for X in (P, Q, R, S))
                    f[p_, q_] += 4 * np.einsum("pqrs,rs->pq", v, D[r_, s_])
                    f[p_, s_] -= 0.5 * np.einsum("pqrs,qr->ps", v, D[q_, r_])
                    f[p_, r_] -= 0.5 * np.einsum("pqrs,qs->pr", v, D[q_, s_])
                    f[q_, r_] -= 0.5 * np.einsum("pqrs,ps->qr", v, D[p_, s_])
                    f[q_, s_] -= 0.5 * np.einsum("pqrs,pr->qs", v, D[p_, r_])
    return f + f.T


def test_compute_2body_fock_matches_binding_loop(lgx, oracle_mod):
    atoms = [(1, (0.0, 0.0, 0.0)), (1, (0.0, 0.0, 1.4))]
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    D = lgx.random_density(bs.nbf, 1, seed=5)
    ctx = _OracleContext(oracle_mod)
    G = lgx.Engine(lgx.Operator.coulomb, context=ctx).compute_2body_fock(D, bs)
    assert ("basis", len(bs)) in ctx.calls
    ref = _binding_fock(oracle_mod, bs, D)
    assert np.max(np.abs(G - ref)) < 1e-12 * max(1.0, np.abs(ref).max())
    with pytest.raises(NotImplementedError):
        lgx.Engine(lgx.Operator.coulomb, deriv_order=1, context=ctx).compute_2body_fock(D, bs)


def test_solid_harmonics_coefficients_vs_reference(lgx):
    # the binding's SolidHarmonicsCoefficients.coefficient against the
    # reference's own coefficients (tests/golden/solid.npz)
    from golden_util import load
    g = load("solid.npz")
    for (l, m, lx, ly, lz), c in zip(g["idx"], g["coeff"]):
        got = lgx.SolidHarmonicsCoefficients.coefficient(int(l), int(m), int(lx), int(ly), int(lz))
        assert abs(got - c) < 1e-13, (l, m, lx, ly, lz)
    assert lgx.SolidHarmonicsCoefficients.coefficient(2, 3, 2, 0, 0) == 0.0   # |m| > l
    assert lgx.SolidHarmonicsCoefficients.coefficient(2, 0, 1, 0, 0) == 0.0   # sum != l


class _OracleShellsetContext(_OracleContext):
    """Stand-in for Context: shell sets from the oracle."""

    def compute_shellset(self, shells, deriv=0, precision=0.0, screening=0):
        import libint_gb300 as lg
        ob = self.o.OracleBasis.from_basis(lg.BasisSet(list(shells)))
        return self.o.compute_quartet(ob, 0, 1, 2, 3, deriv=deriv, precision=precision)


def test_compute_over_basis_sets_all_ranks(lgx, oracle_mod):
    # Engine.compute(basis, ...) for xx_xx, xs_xx, xs_xs: full arrays whose
    # blocks are the shell sets (the binding's compute2/3/4 over BasisSet)
    atoms = [(1, (0.0, 0.0, 0.0)), (1, (0.0, 0.0, 1.4))]
    obs = lgx.BasisSet("cc-pVDZ", atoms)
    aux = list(lgx.BasisSet("cc-pVDZ-jkfit", atoms))[:4]
    ctx = _OracleShellsetContext(oracle_mod)
    for bk, args in ((lgx.BraKet.xs_xs, (aux, aux)), (lgx.BraKet.xs_xx, (aux, obs, obs)),
                     (lgx.BraKet.xx_xx, (list(obs)[:3],) * 4)):
        eng = lgx.Engine(lgx.Operator.coulomb, braket=bk, context=ctx)
        full = eng.compute(*args)
        sizes = [[s.size() for s in X] for X in args]
        assert full.shape == tuple(sum(x) for x in sizes)
        # one block against a direct shell-set call
        blk = eng.compute(*[X[1] for X in args])
        sl = tuple(slice(x[0], x[0] + x[1]) for x in sizes)
        assert np.array_equal(full[sl], blk)
    # (P|Q) symmetric, (P|ab) symmetric in a, b
    V = lgx.Engine(lgx.Operator.coulomb, braket=lgx.BraKet.xs_xs, context=ctx).compute(aux, aux)
    assert np.allclose(V, V.T, atol=1e-13)
    B = lgx.Engine(lgx.Operator.coulomb, braket=lgx.BraKet.xs_xx, context=ctx).compute(aux, obs, obs)
    assert np.allclose(B, B.transpose(0, 2, 1), atol=1e-13)


def test_reference_python_test_core(lgx):
    # the reference's python/tests/test_libint2.py test_core against the
    # mirror: 6-31G water has 9 shells; the basis-wide pure setter and a
    # per-shell pure write through basis[i]
    h2o = [(8, [0.0, -0.07579, 0.0]), (1, [0.86681, 0.60144, 0.0]),
           (1, [-0.86681, 0.60144, 0.0])]
    assert lgx.MAX_AM > 0
    basis = lgx.BasisSet("6-31g", h2o)
    assert len(basis) == 9
    basis.pure = False
    pure = [False] * len(basis)
    assert [s.pure for s in basis] == pure
    basis[0].pure = True
    pure[0] = True
    assert [s.pure for s in basis] == pure
