"""Parity at the sizes of the five benchmark configurations (seeded synthetic
water clusters, O on a grid with 3.0 A spacing, +-0.2 A jitter, random
orientation; cc-pVDZ / cc-pVTZ from the reference's basis library).

1. (H2O)4 cc-pVDZ, every unique shell quartet at deriv 0, FP64, no Schwarz
   screening: each integral against the oracle at 1e-12 absolute.
2. (H2O)32 cc-pVDZ, Schwarz 1e-12, batched FP64: J and K (a D-weighted sum
   of every screened integral) against the oracle's J/K over the same
   screened quartets, and a random sample of screened quartets integral by
   integral at 1e-12.
3. (H2O)32 cc-pVDZ mixed (FP32 where K12*K34 < 1e-4): J/K energy errors
   against the FP64 pass at or below 1e-8 Eh, and the integral error of
   sampled FP32 quartets against the oracle within the mixed-precision bound.
4. cc-pVTZ (up to f, contraction depths 1-8): (H2O)4 on a 2x2x1 grid, FP64
   J/K against the oracle and the mixed energy error (the (H2O)64 case itself
   is the benchmark workload; an FP64 oracle pass over it takes hours).
5. (H2O)16 cc-pVDZ deriv_order=1: sampled derivative shell sets against the
   oracle, translational invariance of the gradients, and central finite
   differences (h = 1e-4 bohr) of the J/K energies on three coordinates.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 2024


def cluster(lgx, grid, basis):
    atoms = lgx.water_cluster(*grid, spacing=3.0, jitter=0.2, seed=SEED)
    bs = lgx.BasisSet(basis, atoms)
    nwat = grid[0] * grid[1] * grid[2]
    D = lgx.random_density(bs.nbf, 5 * nwat, seed=SEED + 1)
    return atoms, bs, D


def unique_quartets(ns):
    """Canonical unique quartets (a>=b, c>=d, (ab)>=(cd)) of ns shells."""
    a, b = np.tril_indices(ns)
    pairs = np.stack([a, b], 1)
    i, j = np.tril_indices(len(pairs))
    return np.concatenate([pairs[i], pairs[j]], 1).astype(np.int32)


def set_sizes(bs, q):
    sz = np.array([s.size() for s in bs], np.int64)
    return sz[q[:, 0]] * sz[q[:, 1]] * sz[q[:, 2]] * sz[q[:, 3]]


def screened_sample(K, n, thresh, rng, lo=None, hi=None):
    """n random unique quartets with K12*K34 >= thresh (and, when given,
    lo <= K12*K34 < hi)."""
    ns = K.shape[0]
    a, b = np.tril_indices(ns)
    kp = K[a, b]
    out = []
    while sum(len(x) for x in out) < n:
        i = rng.integers(0, len(a), 4 * n)
        j = rng.integers(0, len(a), 4 * n)
        i, j = np.maximum(i, j), np.minimum(i, j)
        bound = kp[i] * kp[j]
        keep = bound >= thresh
        if lo is not None:
            keep &= (bound >= lo) & (bound < hi)
        out.append(np.stack([a[i], b[i], a[j], b[j]], 1)[keep])
    return np.concatenate(out)[:n].astype(np.int32)


def compare_batch(lgx, oracle_mod, ctx, ob, bs, q, deriv=0, mode=0, tol=1e-12, bound=None):
    out, offs, isnull = ctx.compute_batch(q, deriv=deriv, mode=mode)
    nv = set_sizes(bs, q) * (12 if deriv else 1)
    ref, risnull = oracle_mod.compute_batch(ob, q, offs, int(nv.sum()), deriv=deriv)
    assert np.array_equal(isnull, risnull)
    diff = np.abs(out[:nv.sum()] - ref[:nv.sum()])
    if bound is None:
        worst = float(diff.max()) if diff.size else 0.0
        assert worst < tol, worst
        return worst
    # per-quartet tolerance (mixed precision): tol(bound of the quartet)
    owner = np.repeat(np.arange(len(q)), nv)
    per = np.zeros(len(q))
    np.maximum.at(per, owner, diff)
    lim = np.array([tol(x) for x in bound])
    assert np.all(per < lim), (per[per >= lim][:5], bound[per >= lim][:5])
    return float(per.max())


def test_config1_h2o4_every_unique_quartet_fp64(lgx, oracle_mod):
    _, bs, _ = cluster(lgx, (2, 2, 1), "cc-pVDZ")
    ob = oracle_mod.OracleBasis.from_basis(bs)
    q = unique_quartets(len(bs))
    assert len(q) == 692076 and int(set_sizes(bs, q).sum()) == 11272220
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    compare_batch(lgx, oracle_mod, ctx, ob, bs, q)
    # offsets = NULL packs the sets in list order: identical to the explicit
    # prefix-sum offsets the Python binding passes (a long list, so the host
    # grouping runs on several threads and fixes the packed offsets per chunk)
    import ctypes
    out, offs, _ = ctx.compute_batch(q)
    packed = np.full(out.size, np.nan)
    lib = lgx._lgx.load()
    qc = np.ascontiguousarray(q, np.int32)
    st = lib.lgx_compute_batch(ctx._h, lgx._lgx.ptr(qc, ctypes.c_int32), len(qc), 0, 0, 1e-4,
                               None, lgx._lgx.ptr(packed), packed.size, None)
    assert st == 0
    assert np.array_equal(packed, out)
    ctx.close()


@pytest.fixture(scope="module")
def h2o32(lgx, oracle_mod):
    atoms, bs, D = cluster(lgx, (4, 4, 2), "cc-pVDZ")
    ob = oracle_mod.OracleBasis.from_basis(bs)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    K = ctx.schwarz()
    yield bs, ob, D, ctx, K
    ctx.close()


def test_config2_h2o32_fp64_jk_and_sampled_quartets(lgx, oracle_mod, h2o32):
    bs, ob, D, ctx, K = h2o32
    assert np.max(np.abs(K - oracle_mod.schwarz(ob))) < 1e-12
    J, Kx, st = ctx.jk(D, 1e-12)
    Jr, Kr, nq = oracle_mod.jk(ob, D, K, 1e-12)
    assert st.quartets_fp64 == nq and st.quartets_fp32 == 0
    assert np.max(np.abs(J - Jr)) < 1e-10
    assert np.max(np.abs(Kx - Kr)) < 1e-10
    e, er = lgx.jk_energies(D, J, Kx), lgx.jk_energies(D, Jr, Kr)
    assert abs(e[0] - er[0]) < 1e-9 and abs(e[1] - er[1]) < 1e-10
    q = screened_sample(K, 200000, 1e-12, np.random.default_rng(11))
    compare_batch(lgx, oracle_mod, ctx, ob, bs, q)


@pytest.mark.parametrize("mode", [1, 2])  # LGX_MIXED (FP64 Boys), LGX_MIXED_FP32_BOYS
def test_config3_h2o32_mixed_errors(lgx, oracle_mod, h2o32, mode):
    bs, ob, D, ctx, K = h2o32
    J64, K64, _ = ctx.jk(D, 1e-12)
    Jm, Km, st = ctx.jk(D, 1e-12, mode=mode, mixed_thresh=1e-4)
    assert st.quartets_fp32 > 5 * st.quartets_fp64 > 0
    e64, em = lgx.jk_energies(D, J64, K64), lgx.jk_energies(D, Jm, Km)
    assert abs(e64[0] - em[0]) <= 1e-8 and abs(e64[1] - em[1]) <= 1e-8
    # FP32 quartets (bound < 1e-4): error far below the bound; FP64 ones exact
    rng = np.random.default_rng(12)
    q32 = screened_sample(K, 100000, 1e-12, rng, lo=1e-12, hi=1e-4)
    q64 = screened_sample(K, 20000, 1e-4, rng)
    a, b, c, d = q32.T
    compare_batch(lgx, oracle_mod, ctx, ob, bs, q32, mode=mode,
                  tol=lambda x: max(1e-12, 1e-5 * x), bound=K[a, b] * K[c, d])
    compare_batch(lgx, oracle_mod, ctx, ob, bs, q64, mode=mode)


def test_config4_tz_h2o4_fp64_and_mixed(lgx, oracle_mod):
    _, bs, D = cluster(lgx, (2, 2, 1), "cc-pVTZ")
    assert bs.max_l() == 3 and bs.max_nprim() == 8
    ob = oracle_mod.OracleBasis.from_basis(bs)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    Kq = ctx.schwarz()
    J, K, st = ctx.jk(D, 1e-12)
    Jr, Kr, nq = oracle_mod.jk(ob, D, Kq, 1e-12)
    assert st.quartets_fp64 == nq
    assert np.max(np.abs(J - Jr)) < 1e-10 and np.max(np.abs(K - Kr)) < 1e-10
    Jm, Km, stm = ctx.jk(D, 1e-12, mode=1, mixed_thresh=1e-4)
    assert stm.quartets_fp32 > 0
    e64, em = lgx.jk_energies(D, J, K), lgx.jk_energies(D, Jm, Km)
    assert abs(e64[0] - em[0]) <= 1e-8 and abs(e64[1] - em[1]) <= 1e-8
    # the (ff|ff)-containing classes, integral by integral
    q = screened_sample(Kq, 20000, 1e-12, np.random.default_rng(13))
    compare_batch(lgx, oracle_mod, ctx, ob, bs, q)
    ctx.close()


def test_config5_h2o16_gradients(lgx, oracle_mod):
    atoms, bs, D = cluster(lgx, (4, 2, 2), "cc-pVDZ")
    ob = oracle_mod.OracleBasis.from_basis(bs)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    Kq = ctx.schwarz()
    # derivative shell sets, integral by integral
    q = screened_sample(Kq, 20000, 1e-12, np.random.default_rng(14))
    compare_batch(lgx, oracle_mod, ctx, ob, bs, q, deriv=1)
    natoms = len(atoms)
    gJ, gK, st = ctx.jk_grad(D, natoms, 0.0)
    assert gJ.shape == (48, 3)
    assert np.max(np.abs(gJ.sum(axis=0))) < 1e-8 and np.max(np.abs(gK.sum(axis=0))) < 1e-8
    h = 1e-4
    c2 = lgx.Context(0)
    for at, x in [(0, 0), (17, 1), (46, 2)]:
        e = []
        for sgn in (+1, -1):
            moved = [lgx.Atom(Z, xyz) for Z, xyz in atoms]
            xyz = list(moved[at][1])
            xyz[x] += sgn * h
            moved[at] = lgx.Atom(moved[at][0], xyz)
            c2.set_basis(lgx.BasisSet("cc-pVDZ", moved))
            Jm, Km, _ = c2.jk(D, 0.0)
            e.append(lgx.jk_energies(D, Jm, Km))
        fdJ = (e[0][0] - e[1][0]) / (2 * h)
        fdK = (e[0][1] - e[1][1]) / (2 * h)
        assert abs(fdJ - gJ[at, x]) < 2e-6, (at, x, fdJ, gJ[at, x])
        assert abs(fdK - gK[at, x]) < 2e-6, (at, x, fdK, gK[at, x])
    c2.close()
    ctx.close()
