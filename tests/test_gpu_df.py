"""Three- and two-centre Coulomb integrals (BraKet::xs_xx, xs_xs), the
integrals of density fitting, on the CUDA path:

* Engine(braket=XSXX / XSXS).compute(a, c, d) / compute(a, c) at deriv 0 and
  1 against the reference's brute-force sets with Shell::unit() in the empty
  positions (tests/golden/eri3c.npz), in libint's order (derivative sets of
  the real centres only: 9 and 6);
* the batched path: the 3-centre tensor (P|ab) and the 2-centre metric (P|Q)
  of (H2O)2 cc-pVDZ with the cc-pVDZ-jkfit fitting basis through
  lgx_compute_batch, with a unit shell appended to the context's basis,
  against the oracle; and the density-fitted Coulomb energy close to the
  exact one.
"""
import numpy as np
import pytest

from golden_util import eri3c_cases

pytestmark = pytest.mark.gpu

SETS = {3: [0, 1, 2, 6, 7, 8, 9, 10, 11], 2: [0, 1, 2, 6, 7, 8]}


def test_engine_xs_xx_xs_xs_vs_reference_bruteforce(lgx):
    worst = 0.0
    for l, pure, nprim, alpha, coeff, O, deriv, rank, vals in eri3c_cases():
        shells, off = [], 0
        for k in range(4):
            n = int(nprim[k])
            shells.append(lgx.Shell.from_normalized(int(l[k]), alpha[off:off + n],
                                                    coeff[off:off + n], O[3 * k:3 * k + 3],
                                                    bool(pure[k])))
            off += n
        bk = lgx.BraKet.XSXX if rank == 3 else lgx.BraKet.XSXS
        eng = lgx.Engine(lgx.Operator.coulomb, 10, 3, deriv, precision=0.0, braket=bk)
        args = [shells[0], shells[2], shells[3]] if rank == 3 else [shells[0], shells[2]]
        r = eng.compute(*args)
        assert eng.nshellsets() == (3 * rank if deriv else 1)
        nv = int(np.prod([s.size() for s in args]))
        ref = vals.reshape(12 if deriv else 1, nv)
        if deriv:
            ref = ref[SETS[rank]]
            got = np.stack([x.reshape(-1) for x in r])
        else:
            got = r.reshape(1, -1)
            assert r.shape == tuple(s.size() for s in args)
        err = float(np.max(np.abs(got - ref)))
        worst = max(worst, err)
        assert err < 1e-12, (tuple(l), rank, deriv, err)
    print("worst", worst)


def test_df_tensors_batched_vs_oracle(lgx, oracle_mod):
    atoms = lgx.water_cluster(2, 1, 1, spacing=3.0, jitter=0.2, seed=8)
    obs = lgx.BasisSet("cc-pVDZ", atoms)
    dfbs = lgx.BasisSet("cc-pVDZ-jkfit", atoms)
    # one context basis: orbital shells, fitting shells, then the unit shell
    full = lgx.BasisSet(list(obs) + list(dfbs) + [lgx.Shell.unit()])
    full.atom_of_shell = obs.atom_of_shell + dfbs.atom_of_shell + [0]
    ns, na, u = len(obs), len(dfbs), len(obs) + len(dfbs)
    ctx = lgx.Context(0)
    ctx.set_basis(full)
    a, b = np.tril_indices(ns)
    P = np.arange(ns, ns + na)
    q3 = np.array([(p, u, i, j) for p in P for i, j in zip(a, b)], np.int32)
    q2 = np.array([(p, u, r, u) for p in P for r in P if r <= p], np.int32)
    ob = oracle_mod.OracleBasis.from_basis(full)
    sz = np.array([s.size() for s in full], np.int64)
    import torch
    for q in (q3, q2):
        out, offs, isnull = ctx.compute_batch(q)
        nv = sz[q[:, 0]] * sz[q[:, 1]] * sz[q[:, 2]] * sz[q[:, 3]]
        ref, risnull = oracle_mod.compute_batch(ob, q, offs, int(nv.sum()))
        assert np.array_equal(isnull, risnull)
        assert np.max(np.abs(out[:nv.sum()] - ref[:nv.sum()])) < 1e-12
        # the same sets left in HBM (lgx_compute_batch_device): bit-identical
        d = torch.full((int(nv.sum()),), float("nan"), dtype=torch.float64, device="cuda")
        dn = torch.full((len(q),), -1, dtype=torch.int32, device="cuda")
        offs_d = ctx.compute_batch_device(q, d.data_ptr(), d.numel(), d_is_null=dn.data_ptr())
        assert np.array_equal(offs_d, offs)
        assert np.array_equal(d.cpu().numpy(), out[:nv.sum()])
        assert np.array_equal(dn.cpu().numpy(), isnull)
    # assemble (P|ab) and (P|Q); DF Coulomb energy vs the exact one
    nbf, naux = obs.nbf, dfbs.nbf
    off_o, off_a = obs.shell2bf(), dfbs.shell2bf()
    B = np.zeros((naux, nbf, nbf))
    out, offs, _ = ctx.compute_batch(q3)
    for k, (p, _, i, j) in enumerate(q3):
        n = (sz[p], sz[i], sz[j])
        blk = out[offs[k]:offs[k] + np.prod(n)].reshape(n)
        pa, ia, ja = off_a[p - ns], off_o[i], off_o[j]
        B[pa:pa + n[0], ia:ia + n[1], ja:ja + n[2]] = blk
        B[pa:pa + n[0], ja:ja + n[2], ia:ia + n[1]] = blk.transpose(0, 2, 1)
    V = np.zeros((naux, naux))
    out, offs, _ = ctx.compute_batch(q2)
    for k, (p, _, r, _) in enumerate(q2):
        n = (sz[p], sz[r])
        blk = out[offs[k]:offs[k] + np.prod(n)].reshape(n)
        pa, ra = off_a[p - ns], off_a[r - ns]
        V[pa:pa + n[0], ra:ra + n[1]] = blk
        V[ra:ra + n[1], pa:pa + n[0]] = blk.T
    assert np.linalg.eigvalsh(V).min() > 0  # Coulomb metric is positive definite
    D = lgx.random_density(nbf, 10, seed=9)
    gamma = np.einsum("pab,ab->p", B, D)
    Jdf = np.einsum("pab,p->ab", B, np.linalg.solve(V, gamma))
    c2 = lgx.Context(0)
    c2.set_basis(obs)
    J, K, _ = c2.jk(D, 0.0)
    ej, ejdf = 0.5 * np.sum(D * J), 0.5 * np.sum(D * Jdf)
    # robust fitting: the DF Coulomb energy is a lower bound, close to exact
    assert ejdf <= ej + 1e-10 and (ej - ejdf) / ej < 1e-3, (ej, ejdf)
    c2.close()
    ctx.close()
