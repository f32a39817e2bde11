"""Batched and fused paths on the GPU against the oracle: Schwarz factors,
explicit quartet batches (FP64 and mixed), J/K digestion with Schwarz
screening, and deriv_order=1 gradient digestion (against the oracle and
central finite differences)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def water2(lgx, oracle_mod):
    atoms = lgx.water_cluster(2, 1, 1, spacing=3.0, jitter=0.2, seed=1)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    D = lgx.random_density(bs.nbf, 10, seed=2)
    return atoms, bs, ob, D


def test_schwarz_matches_oracle(lgx, oracle_mod, water2):
    _, bs, ob, _ = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    K = ctx.schwarz()
    Kref = oracle_mod.schwarz(ob)
    assert np.max(np.abs(K - Kref)) < 1e-12
    ctx.close()


def test_batch_fp64_vs_oracle(lgx, oracle_mod, water2):
    _, bs, ob, _ = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    rng = np.random.default_rng(4)
    q = rng.integers(0, len(bs), size=(400, 4))
    out, offs, isnull = ctx.compute_batch(q)
    worst = 0.0
    for i, quad in enumerate(q):
        ref = oracle_mod.compute_quartet(ob, *[int(x) for x in quad])
        if ref is None:
            assert isnull[i] == 1
            continue
        n = ref[0].size
        worst = max(worst, float(np.max(np.abs(out[offs[i]:offs[i] + n] - ref[0].reshape(-1)))))
    assert worst < 1e-12, worst
    ctx.close()


def test_batch_deriv1_vs_oracle(lgx, oracle_mod, water2):
    _, bs, ob, _ = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    rng = np.random.default_rng(5)
    q = rng.integers(0, len(bs), size=(60, 4))
    out, offs, isnull = ctx.compute_batch(q, deriv=1)
    for i, quad in enumerate(q):
        ref = oracle_mod.compute_quartet(ob, *[int(x) for x in quad], deriv=1)
        if ref is None:
            continue
        ref = np.concatenate([r.reshape(-1) for r in ref])
        assert np.max(np.abs(out[offs[i]:offs[i] + ref.size] - ref)) < 1e-12
    ctx.close()


def test_batch_mixed_error_bound(lgx, oracle_mod, water2):
    _, bs, ob, _ = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    K = ctx.schwarz()
    rng = np.random.default_rng(6)
    q = rng.integers(0, len(bs), size=(400, 4))
    out, offs, _ = ctx.compute_batch(q, mode=1, mixed_thresh=1e-4)
    for i, quad in enumerate(q):
        a, b, c, d = [int(x) for x in quad]
        ref = oracle_mod.compute_quartet(ob, a, b, c, d)
        if ref is None:
            continue
        err = np.max(np.abs(out[offs[i]:offs[i] + ref[0].size] - ref[0].reshape(-1)))
        bound = K[a, b] * K[c, d]
        # FP64 quartets keep the FP64 tolerance; FP32 ones stay far below the bound
        assert err < (1e-12 if bound >= 1e-4 else max(1e-12, 1e-5 * bound)), (quad, err, bound)
    ctx.close()


@pytest.mark.parametrize("thresh", [0.0, 1e-12])
def test_jk_fp64_vs_oracle(lgx, oracle_mod, water2, thresh):
    _, bs, ob, D = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    J, K, st = ctx.jk(D, schwarz_thresh=thresh)
    Kq = oracle_mod.schwarz(ob)
    Jr, Kr, nq = oracle_mod.jk(ob, D, Kq, thresh)
    assert st.quartets_fp64 == nq
    assert np.max(np.abs(J - Jr)) < 1e-11
    assert np.max(np.abs(K - Kr)) < 1e-11
    ej, ek = lgx.jk_energies(D, J, K)
    ejr, ekr = lgx.jk_energies(D, Jr, Kr)
    assert abs(ej - ejr) < 1e-11 and abs(ek - ekr) < 1e-11
    ctx.close()


def test_jk_brute_force_definition(lgx, oracle_mod):
    # J_ab = sum_cd (ab|cd) D_cd, K_ab = sum_cd (ac|bd) D_cd from the full tensor
    atoms = lgx.water_cluster(1, 1, 1, seed=9)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    D = lgx.random_density(bs.nbf, 5, seed=3)
    n = bs.nbf
    off = bs.shell2bf()
    G = np.zeros((n, n, n, n))
    for a in range(len(bs)):
        for b in range(len(bs)):
            for c in range(len(bs)):
                for d in range(len(bs)):
                    r = oracle_mod.compute_quartet(ob, a, b, c, d)
                    if r is None:
                        continue
                    na, nb, nc, nd = r[0].shape
                    G[off[a]:off[a] + na, off[b]:off[b] + nb,
                      off[c]:off[c] + nc, off[d]:off[d] + nd] = r[0]
    Jb = np.einsum("abcd,cd->ab", G, D)
    Kb = np.einsum("acbd,cd->ab", G, D)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    J, K, _ = ctx.jk(D, schwarz_thresh=0.0)
    assert np.max(np.abs(J - Jb)) < 1e-11
    assert np.max(np.abs(K - Kb)) < 1e-11
    ctx.close()


def test_jk_mixed_energy_error(lgx, water2):
    _, bs, _, D = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    J64, K64, _ = ctx.jk(D, 1e-12)
    Jm, Km, st = ctx.jk(D, 1e-12, mode=1, mixed_thresh=1e-4)
    assert st.quartets_fp32 > 0
    e64 = lgx.jk_energies(D, J64, K64)
    em = lgx.jk_energies(D, Jm, Km)
    assert abs(e64[0] - em[0]) <= 1e-8 and abs(e64[1] - em[1]) <= 1e-8
    ctx.close()


def test_gradient_vs_oracle_and_fd(lgx, oracle_mod, water2):
    atoms, bs, ob, D = water2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    natoms = len(atoms)
    gJ, gK, _ = ctx.jk_grad(D, natoms, 1e-12)
    Kq = oracle_mod.schwarz(ob)
    gJr, gKr, _ = oracle_mod.jk_grad(ob, D, Kq, natoms, 1e-12)
    assert np.max(np.abs(gJ - gJr)) < 1e-10
    assert np.max(np.abs(gK - gKr)) < 1e-10
    # translational invariance of the two-electron energies
    assert np.max(np.abs(gJ.sum(axis=0))) < 1e-9
    # central finite differences, h = 1e-4 bohr, on two coordinates
    h = 1e-4
    for (at, x) in [(0, 0), (4, 2)]:
        e = []
        for sgn in (+1, -1):
            moved = [lgx.Atom(Z, xyz) for Z, xyz in atoms]
            xyz = list(moved[at][1]); xyz[x] += sgn * h
            moved[at] = lgx.Atom(moved[at][0], xyz)
            bsm = lgx.BasisSet("cc-pVDZ", moved)
            c2 = lgx.Context(0)
            c2.set_basis(bsm)
            Jm, Km, _ = c2.jk(D, 0.0)
            e.append(lgx.jk_energies(D, Jm, Km))
            c2.close()
        fdJ = (e[0][0] - e[1][0]) / (2 * h)
        fdK = (e[0][1] - e[1][1]) / (2 * h)
        assert abs(fdJ - gJ[at, x]) < 1e-6, (fdJ, gJ[at, x])
        assert abs(fdK - gK[at, x]) < 1e-6, (fdK, gK[at, x])
    ctx.close()


@pytest.fixture(scope="module")
def water_tz(lgx, oracle_mod):
    atoms = lgx.water_cluster(1, 1, 1, seed=4)
    bs = lgx.BasisSet("cc-pVTZ", atoms)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    D = lgx.random_density(bs.nbf, 5, seed=5)
    return atoms, bs, ob, D


@pytest.mark.parametrize("variant", ["tuned", "interpreted_post"])
def test_jk_tz_vs_oracle(lgx, oracle_mod, water_tz, monkeypatch, variant):
    # cc-pVTZ reaches the f classes: (ff|ff) and the other L > 6 classes run
    # on the program kernel, with the generated post stages unless disabled
    if variant == "interpreted_post":
        monkeypatch.setenv("LGX_DISABLE_POST", "1")
    else:  # tune every class bin, however small
        monkeypatch.setenv("LGX_TUNE_MIN", "1")
    _, bs, ob, D = water_tz
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    J, K, st = ctx.jk(D, schwarz_thresh=1e-12)
    Kq = oracle_mod.schwarz(ob)
    Jr, Kr, nq = oracle_mod.jk(ob, D, Kq, 1e-12)
    assert st.quartets_fp64 == nq
    assert np.max(np.abs(J - Jr)) < 1e-11
    assert np.max(np.abs(K - Kr)) < 1e-11
    # a second pass reuses the tuned variants and gives the same result
    J2, K2, _ = ctx.jk(D, schwarz_thresh=1e-12)
    assert np.max(np.abs(J2 - J)) < 1e-12 and np.max(np.abs(K2 - K)) < 1e-12
    Jm, Km, stm = ctx.jk(D, 1e-12, mode=1, mixed_thresh=1e-4)
    assert stm.quartets_fp32 > 0
    e64 = lgx.jk_energies(D, J, K)
    em = lgx.jk_energies(D, Jm, Km)
    assert abs(e64[0] - em[0]) <= 1e-8 and abs(e64[1] - em[1]) <= 1e-8
    ctx.close()


def test_jk_graph_replay_matches_eager(lgx, water2, monkeypatch):
    # the second pass with the same settings replays the captured CUDA graph;
    # it must see the new density and match a pass without graphs
    _, bs, _, D = water2
    D2 = lgx.random_density(bs.nbf, 10, seed=7)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    for mode in (0, 1):
        ctx.jk(D, 1e-12, mode=mode)                   # eager, then captured
        J2, K2, st = ctx.jk(D2, 1e-12, mode=mode)     # graph replay
        assert st.pass_ms > 0 and st.integrals > 0
        monkeypatch.setenv("LGX_GRAPHS", "0")
        ref = lgx.Context(0)
        ref.set_basis(bs)
        Jr, Kr, _ = ref.jk(D2, 1e-12, mode=mode)
        ref.close()
        monkeypatch.delenv("LGX_GRAPHS")
        assert np.max(np.abs(J2 - Jr)) < 1e-12 and np.max(np.abs(K2 - Kr)) < 1e-12
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_density_weighted_screening_vs_oracle(lgx, oracle_mod, mode):
    # compute_2body_fock's density-weighted screening (lgx_set_fock_precision)
    # against the oracle's restatement of it, on a density whose shell blocks
    # span many orders of magnitude so that the screening skips quartets
    atoms = lgx.water_cluster(2, 2, 2, spacing=3.0, jitter=0.2, seed=31)
    bs = lgx.BasisSet("cc-pVDZ", atoms)
    rng = np.random.default_rng(32)
    D = lgx.random_density(bs.nbf, 40, seed=33)
    D *= np.exp(rng.uniform(-14, 0, bs.nbf))[:, None]
    D = 0.5 * (D + D.T)
    fock = 1e-10
    ob = oracle_mod.OracleBasis.from_basis(bs)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    K = ctx.schwarz()
    ns = len(bs)
    acc = oracle_mod.JKAccumulator(ob.nbf)
    acc.add_pairs(ob, D, K, 1e-12, np.arange(ns * (ns + 1) // 2), fock_precision=fock)
    Jo, Ko = acc.reduce()
    acc.close()
    J0, K0, _ = ctx.jk(D, 1e-12, mode=mode)
    ctx.set_fock_precision(fock)
    J, Kx, _ = ctx.jk(D, 1e-12, mode=mode)
    J2, K2, _ = ctx.jk(D, 1e-12, mode=mode)  # the replayed pass graph
    ctx.set_fock_precision(0.0)
    J3, K3, _ = ctx.jk(D, 1e-12, mode=mode)
    ctx.close()
    # both sides screen alike, the FP64 kernels with the FP64 thresholds
    # fock / Dnorm1234 and its logarithm (a primitive quartet at the
    # threshold can carry ~100x the threshold, so FP32 decisions would show
    # here at ~1e-8); the mixed pass's FP32 quartets decide in FP32 and
    # carry their FP32 arithmetic error
    tol = 1e-11 if mode == 0 else 1e-8
    assert np.max(np.abs(J - Jo)) < tol and np.max(np.abs(Kx - Ko)) < tol
    assert np.array_equal(J, J2) or np.max(np.abs(J - J2)) < 1e-12
    # screening changes the result, and switching it off restores the plain pass
    assert np.max(np.abs(J - J0)) > 0
    assert np.max(np.abs(J3 - J0)) < 1e-12 and np.max(np.abs(K3 - K0)) < 1e-12
    eo, e = lgx.jk_energies(D, Jo, Ko), lgx.jk_energies(D, J, Kx)
    assert abs(eo[0] - e[0]) < 1e-8 and abs(eo[1] - e[1]) < 1e-8
