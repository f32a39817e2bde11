"""Parity at the target configuration, (H2O)64 cc-pVTZ on a 4x4x4 grid with
Schwarz 1e-12 (3712 functions; 1.95e10 screened quartets, far beyond an FP64
CPU pass), against the FP64 oracle:

1. Quartets sampled from every class bin of the screened pass (up to 1000
   per (bra pair class, ket pair class) bin, about 50k in all) through the
   batched entry in FP64, each integral at 1e-12 absolute.
2. The J/K kernels of the benchmarked pass (lgx_jk_device) restricted to a
   seeded subset of 3000 significant shell pairs (every screened quartet
   whose bra and ket pairs are both in the subset, lgx_set_pair_subset)
   against the oracle's J/K over the same quartets: FP64 J and K at 1e-10
   per element, and the mixed pass's Coulomb and exchange energies within
   1e-8 Eh of the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 2024
THRESH = 1e-12


@pytest.fixture(scope="module")
def target(lgx, oracle_mod):
    atoms = lgx.water_cluster(4, 4, 4, spacing=3.0, jitter=0.2, seed=SEED)
    bs = lgx.BasisSet("cc-pVTZ", atoms)
    D = lgx.random_density(bs.nbf, 5 * 64, seed=SEED + 1)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    K = oracle_mod.schwarz(ob)
    return bs, D, ob, K


def _pair_class(l1, l2):
    hi, lo = np.maximum(l1, l2), np.minimum(l1, l2)
    return hi * (hi + 1) // 2 + lo


def test_target_sampled_quartets_every_bin(lgx, oracle_mod, target):
    bs, D, ob, K = target
    assert bs.nbf == 3712
    ns = len(bs)
    a, b = np.tril_indices(ns)
    kp = K[a, b]
    sig = kp * K.max() >= THRESH
    a, b, kp = a[sig], b[sig], kp[sig]
    cls = _pair_class(ob.l[a], ob.l[b])
    rng = np.random.default_rng(7)
    picks = []
    nbins = 0
    for x in range(10):
        for y in range(x, 10):
            ix, iy = np.flatnonzero(cls == x), np.flatnonzero(cls == y)
            if len(ix) == 0 or len(iy) == 0:
                continue
            got = []
            for _ in range(20):  # rejection sampling of screened quartets of the bin
                i = rng.choice(ix, 20000)
                j = rng.choice(iy, 20000)
                ok = kp[i] * kp[j] >= THRESH
                got.append(np.stack([i[ok], j[ok]], 1))
                if sum(len(g) for g in got) >= 1000:
                    break
            g = np.unique(np.concatenate(got), axis=0)[:1000]
            if len(g):
                nbins += 1
                picks.append(g)
    p = np.concatenate(picks)
    q = np.stack([a[p[:, 0]], b[p[:, 0]], a[p[:, 1]], b[p[:, 1]]], 1).astype(np.int32)
    assert nbins == 55 and len(q) >= 45000, (nbins, len(q))
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    out, offs, isnull = ctx.compute_batch(q)
    ref, rnull = oracle_mod.compute_batch(ob, q, offs, len(out))
    np.testing.assert_array_equal(isnull, rnull)
    err = np.max(np.abs(out - ref))
    assert err < 1e-12, err
    ctx.close()


def _subset(ob, K, n, seed):
    import bench
    return bench.sample_pairs(ob, K, THRESH, n, seed)


def test_target_jk_pair_subset_vs_oracle(lgx, oracle_mod, target):
    torch = pytest.importorskip("torch")
    bs, D, ob, K = target
    pairs = _subset(ob, K, 3000, 31)
    acc = oracle_mod.JKAccumulator(ob.nbf)
    nq, nint = acc.add_pairs(ob, D, K, THRESH, pairs, ket_subset=True)
    Jo, Ko = acc.reduce()
    acc.close()
    EJo, EKo = lgx.jk_energies(D, Jo, Ko)
    s1 = np.floor((np.sqrt(8.0 * pairs + 1) - 1) / 2).astype(np.int64)
    s1 -= (s1 * (s1 + 1) // 2 > pairs)
    s1 += ((s1 + 1) * (s1 + 2) // 2 <= pairs)
    s2 = pairs - s1 * (s1 + 1) // 2
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    ctx.set_pair_subset(np.stack([s1, s2], 1))
    dD = torch.tensor(D, device="cuda")
    dJ, dK = torch.empty_like(dD), torch.empty_like(dD)
    st = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), THRESH, lgx._lgx.LGX_FP64)
    assert st.quartets_fp64 == nq and st.integrals == nint
    J, Kx = dJ.cpu().numpy(), dK.cpu().numpy()
    assert np.max(np.abs(J - Jo)) < 1e-10 and np.max(np.abs(Kx - Ko)) < 1e-10
    st = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), THRESH, lgx._lgx.LGX_MIXED,
                       1e-4)
    assert st.quartets_fp32 > 0 and st.quartets_fp64 + st.quartets_fp32 == nq
    EJ, EK = lgx.jk_energies(D, dJ.cpu().numpy(), dK.cpu().numpy())
    assert abs(EJ - EJo) <= 1e-8 and abs(EK - EKo) <= 1e-8, (EJ - EJo, EK - EKo)
    # lifting the restriction brings the whole screened pass back
    ctx.set_pair_subset(None)
    st = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), THRESH, lgx._lgx.LGX_MIXED,
                       1e-4)
    assert st.quartets_fp64 + st.quartets_fp32 == oracle_mod.count_screened(ob, K, THRESH)[0]
    ctx.close()
