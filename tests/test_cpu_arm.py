"""The CPU side of the benchmark, without a GPU: the oracle's own inputs (G94
reader, water cluster, density) reproduce the reference's BasisSet and the
product's loader bit for bit; the screened-pass counter equals a brute-force
enumeration; the pair-subset digestion covers each quartet of the subset
once; and the reference arm runs without loading any part of liblgx.so."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from golden_util import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_basis_matches_reference_basisset(oracle_mod):
    from oracle import inputs
    g = load("basis.npz")
    atoms = [(int(z), g["xyz"][3 * i:3 * i + 3]) for i, z in enumerate(g["Z"])]
    for name in ("cc-pVDZ", "cc-pVTZ"):
        key = name.lower().replace("-", "")
        ob = inputs.load_basis(name, atoms)
        np.testing.assert_array_equal(ob.l, g[key + "_l"])
        np.testing.assert_array_equal(ob.pure, g[key + "_pure"])
        np.testing.assert_array_equal(ob.nprim, g[key + "_nprim"])
        np.testing.assert_array_equal(ob.O, g[key + "_O"])
        np.testing.assert_array_equal(ob.alpha, g[key + "_alpha"])
        np.testing.assert_allclose(ob.coeff, g[key + "_coeff"], rtol=1e-14, atol=0)


@pytest.mark.parametrize("grid,name", [((2, 2, 1), "cc-pVDZ"), ((1, 1, 2), "cc-pVTZ"),
                                       ((1, 1, 1), "aug-cc-pVDZ"), ((1, 1, 1), "6-31G")])
def test_oracle_inputs_equal_product_loader(oracle_mod, lgx, grid, name):
    from oracle import inputs
    a1 = inputs.water_cluster(*grid, spacing=3.0, jitter=0.2, seed=2024)
    a2 = lgx.water_cluster(*grid, spacing=3.0, jitter=0.2, seed=2024)
    assert [z for z, _ in a1] == [z for z, _ in a2]
    np.testing.assert_array_equal(np.array([x for _, x in a1]), np.array([x for _, x in a2]))
    ob = inputs.load_basis(name, a1)
    bs = lgx.BasisSet(name, a2)
    for f in ("l", "pure", "nprim", "atom"):
        np.testing.assert_array_equal(getattr(ob, f), np.asarray(getattr(bs, f)))
    np.testing.assert_array_equal(ob.O, bs.origins)
    np.testing.assert_array_equal(ob.alpha, bs.alpha)
    np.testing.assert_array_equal(ob.coeff, bs.coeff)
    np.testing.assert_array_equal(inputs.random_density(ob.nbf, 7, seed=3),
                                  lgx.random_density(bs.nbf, 7, seed=3))


def _small(oracle_mod):
    from oracle import inputs
    atoms = inputs.water_cluster(2, 1, 1, spacing=3.0, jitter=0.2, seed=9)
    ob = inputs.load_basis("cc-pVDZ", atoms)
    K = oracle_mod.schwarz(ob)
    D = inputs.random_density(ob.nbf, 10, seed=10)
    return ob, K, D


def test_count_screened_equals_enumeration(oracle_mod):
    ob, K, D = _small(oracle_mod)
    ns = ob.nshell
    for thresh in (0.0, 1e-12, 1e-6):
        nq = nint = 0
        for s1 in range(ns):
            for s2 in range(s1 + 1):
                for s3 in range(s1 + 1):
                    for s4 in range((s2 if s3 == s1 else s3) + 1):
                        if K[s1, s2] * K[s3, s4] >= thresh:
                            nq += 1
                            nint += int(ob.nfunc[s1] * ob.nfunc[s2] * ob.nfunc[s3] *
                                        ob.nfunc[s4])
        assert oracle_mod.count_screened(ob, K, thresh) == (nq, nint)


def test_pair_subset_digestion_is_the_sub_basis_jk(oracle_mod):
    # quartets whose pairs both lie among the shells X are exactly the
    # quartets of the basis restricted to X: the subset J/K must equal the
    # full J/K of that sub-basis, embedded
    ob, K, D = _small(oracle_mod)
    X = np.array([0, 2, 3, 7, 12, 13, 16, 20])
    s1, s2 = np.meshgrid(X, X, indexing="ij")
    keep = s1 >= s2
    pairs = np.sort(s1[keep].astype(np.int64) * (s1[keep] + 1) // 2 + s2[keep])
    acc = oracle_mod.JKAccumulator(ob.nbf, 2)
    acc.add_pairs(ob, D, K, 1e-12, pairs, ket_subset=True)
    J, Kx = acc.reduce()
    acc.close()
    sub = oracle_mod.OracleBasis(ob.l[X], ob.pure[X], ob.nprim[X],
                                 ob.O.reshape(-1, 3)[X],
                                 np.concatenate([ob.alpha[ob.prim_off[s]:ob.prim_off[s] +
                                                          ob.nprim[s]] for s in X]),
                                 np.concatenate([ob.coeff[ob.prim_off[s]:ob.prim_off[s] +
                                                          ob.nprim[s]] for s in X]))
    bf = np.concatenate([np.arange(ob.bf_off[s], ob.bf_off[s] + ob.nfunc[s]) for s in X])
    Js, Ks, _ = oracle_mod.jk(sub, D[np.ix_(bf, bf)], K[np.ix_(X, X)], 1e-12)
    np.testing.assert_allclose(J[np.ix_(bf, bf)], Js, rtol=0, atol=1e-13)
    np.testing.assert_allclose(Kx[np.ix_(bf, bf)], Ks, rtol=0, atol=1e-13)
    other = np.setdiff1d(np.arange(ob.nbf), bf)
    assert np.all(J[np.ix_(other, other)] == 0) and np.all(Kx[np.ix_(other, other)] == 0)


def test_accumulator_matches_full_jk(oracle_mod):
    ob, K, D = _small(oracle_mod)
    ns = ob.nshell
    acc = oracle_mod.JKAccumulator(ob.nbf, 3)
    allp = np.arange(ns * (ns + 1) // 2)
    acc.add_pairs(ob, D, K, 1e-12, allp[::2])
    acc.add_pairs(ob, D, K, 1e-12, allp[1::2])
    J, Kx = acc.reduce()
    acc.close()
    Jf, Kf, _ = oracle_mod.jk(ob, D, K, 1e-12)
    np.testing.assert_allclose(J, Jf, rtol=0, atol=1e-13)
    np.testing.assert_allclose(Kx, Kf, rtol=0, atol=1e-13)


def test_sample_pairs_fixed_and_stratified(oracle_mod):
    import bench
    ob, K, _ = _small(oracle_mod)
    a = bench.sample_pairs(ob, K, 1e-12, 40, 5)
    b = bench.sample_pairs(ob, K, 1e-12, 40, 5)
    np.testing.assert_array_equal(a, b)
    assert len(np.unique(a)) == len(a) and abs(len(a) - 40) <= 12
    ns = ob.nshell
    s1, s2 = np.tril_indices(ns)
    cls = np.maximum(ob.l[s1], ob.l[s2]) * 8 + np.minimum(ob.l[s1], ob.l[s2])
    assert set(np.unique(cls[a])) == set(np.unique(cls))  # every pair class drawn


def test_reference_arm_loads_no_gpu_library():
    # bench.py --impl reference on the smallest workload, in its own
    # process: one JSON line, and liblgx.so never mapped into the process
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--workload', "
        "'h2o4_cc-pvdz', '--steps', '2', '--warmup', '1']\n"
        "import bench\n"
        "rc = bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "sys.stderr.write('LGX_LOADED=%d\\n' % ('liblgx' in maps))\n"
        "sys.exit(rc)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    assert "LGX_LOADED=0" in r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["dtype"] == "f64"
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["integrals_per_pass"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1


def test_oracle_density_screening_matches_direct_loop(oracle_mod):
    # compute_2body_fock's density-weighted screening restated in a plain
    # loop (hartree-fock++.cc:1640-1684): the accumulator with fock_precision
    # must give the same J/K
    from oracle import inputs
    atoms = inputs.water_cluster(2, 1, 1, spacing=3.0, jitter=0.2, seed=21)
    ob = inputs.load_basis("cc-pVDZ", atoms)
    K = oracle_mod.schwarz(ob)
    rng = np.random.default_rng(22)
    D = inputs.random_density(ob.nbf, 10, seed=23)
    D *= np.exp(rng.uniform(-12, 0, ob.nbf))[:, None]  # a wide range of block norms
    D = 0.5 * (D + D.T)
    fock = 1e-9
    ns = ob.nshell
    off, nf = ob.bf_off, ob.nfunc
    Dsh = np.array([[np.abs(D[off[a]:off[a] + nf[a], off[b]:off[b] + nf[b]]).max()
                     for b in range(ns)] for a in range(ns)])
    J = np.zeros_like(D); Kx = np.zeros_like(D)
    eps = np.finfo(float).eps
    nq = skipped = 0
    for s1 in range(ns):
        for s2 in range(s1 + 1):
            for s3 in range(s1 + 1):
                for s4 in range((s2 if s3 == s1 else s3) + 1):
                    if K[s1, s2] * K[s3, s4] < 1e-12:
                        continue
                    d = max(Dsh[s1, s2], Dsh[s1, s3], Dsh[s2, s3], Dsh[s1, s4], Dsh[s2, s4],
                            Dsh[s3, s4])
                    if d * K[s1, s2] * K[s3, s4] < fock:
                        skipped += 1
                        continue
                    nq += 1
                    # pairs precomputed at the machine epsilon, quartets screened at
                    # fock / Dnorm1234 (hartree-fock++.cc:1386-1425,1681-1684)
                    v = oracle_mod.compute_quartet(ob, s1, s2, s3, s4, precision=max(eps, fock / d),
                                                   pair_precision=eps)
                    if v is None:
                        continue
                    v = v[0]
                    deg = ((1 if s1 == s2 else 2) * (1 if s3 == s4 else 2) *
                           (1 if (s1 == s3 and s2 == s4) else 2))
                    a = slice(off[s1], off[s1] + nf[s1]); b = slice(off[s2], off[s2] + nf[s2])
                    c = slice(off[s3], off[s3] + nf[s3]); e = slice(off[s4], off[s4] + nf[s4])
                    w = deg * v
                    J[a, b] += np.einsum("ijkl,kl->ij", w, D[c, e])
                    J[c, e] += np.einsum("ijkl,ij->kl", w, D[a, b])
                    Kx[a, c] += np.einsum("ijkl,jl->ik", w, D[b, e])
                    Kx[b, e] += np.einsum("ijkl,ik->jl", w, D[a, c])
                    Kx[a, e] += np.einsum("ijkl,jk->il", w, D[b, c])
                    Kx[b, c] += np.einsum("ijkl,il->jk", w, D[a, e])
    J = 0.25 * (J + J.T)
    Kx = 0.125 * (Kx + Kx.T)
    assert skipped > 0 and nq > 0
    acc = oracle_mod.JKAccumulator(ob.nbf, 2)
    got_nq, _ = acc.add_pairs(ob, D, K, 1e-12, np.arange(ns * (ns + 1) // 2), fock_precision=fock)
    Jo, Ko = acc.reduce()
    acc.close()
    assert got_nq == nq
    np.testing.assert_allclose(Jo, J, rtol=0, atol=1e-13)
    np.testing.assert_allclose(Ko, Kx, rtol=0, atol=1e-13)
