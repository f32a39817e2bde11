"""System-level pin of the oracle: the reference's own Hartree-Fock golden
values reproduced with the oracle's J/K (and its deriv_order=1 gradient
digestion) plus one-body integrals and an SCF in the harness.

* aug-cc-pVDZ rotated water: E = -76.003354058439 within 5e-12 and the
  2-body forces F2 within 1e-9 (tests/hartree-fock/hartree-fock++-validate.py);
* the 2-body Hessian H2 (45 values, 1e-9) from the oracle's deriv_order 2;
* 6-31G water of python/tests/test_hf.py: its energy to 7 decimals.
"""
import numpy as np

import hf_util


def test_aug_cc_pvdz_energy_and_2body_forces(lgx, oracle_mod):
    from oracle import scf
    atoms, bs, g = hf_util.rotated_water(lgx)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    S, H, enuc, nocc = hf_util.core(bs, atoms)
    Kq = oracle_mod.schwarz(ob)
    E, D, _, _, _ = scf.rhf(S, H, nocc, lambda D: oracle_mod.jk(ob, D, Kq, 0.0)[:2], enuc)
    assert abs(E - float(g["rot_energy"])) < float(g["rot_energy_tol"]), E
    # F2 = sum_ab D_ab dG_ab/dx with G = 2J - K, i.e. 4 (dE_J + dE_K)
    gJ, gK, _ = oracle_mod.jk_grad(ob, D, Kq, len(atoms), 0.0)
    F2 = 4.0 * (gJ + gK)
    assert np.max(np.abs(F2 - g["rot_F2"])) < float(g["rot_F2_tol"]), F2


def test_631g_energy(lgx, oracle_mod):
    from oracle import scf
    atoms, bs, g = hf_util.water_631g(lgx)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    S, H, enuc, nocc = hf_util.core(bs, atoms)
    Kq = oracle_mod.schwarz(ob)
    E = scf.rhf_plain(S, H, nocc, lambda D: oracle_mod.jk(ob, D, Kq, 0.0)[:2], enuc)
    assert hf_util.places_ok(E, float(g["h2o631_energy"]), int(g["h2o631_places"])), E


def test_aug_cc_pvdz_2body_hessian(lgx, oracle_mod):
    from oracle import scf
    atoms, bs, g = hf_util.rotated_water(lgx)
    ob = oracle_mod.OracleBasis.from_basis(bs)
    S, H, enuc, nocc = hf_util.core(bs, atoms)
    Kq = oracle_mod.schwarz(ob)
    E, D, _, _, _ = scf.rhf(S, H, nocc, lambda D: oracle_mod.jk(ob, D, Kq, 0.0)[:2], enuc)
    quads = hf_util.unique_quartets(len(bs))
    q = np.array([x[:4] for x in quads], np.int32)
    sz = np.array([s.size() for s in bs], np.int64)
    nv = sz[q[:, 0]] * sz[q[:, 1]] * sz[q[:, 2]] * sz[q[:, 3]] * 78
    offs = np.zeros(len(q), np.int64)
    offs[1:] = np.cumsum(nv)[:-1]
    out, isnull = oracle_mod.compute_batch(ob, q, offs, int(nv.sum()), deriv=2)
    index = {tuple(x[:4]): i for i, x in enumerate(quads)}

    def sets_of(a, b, c, d):
        i = index[(a, b, c, d)]
        return None if isnull[i] else out[offs[i]:offs[i] + nv[i]]

    H2 = hf_util.hessian_2body(bs, atoms, D, sets_of)
    assert np.max(np.abs(H2 - H2.T)) < 1e-10
    diff = np.max(np.abs(hf_util.upper(H2) - g["rot_H2_upper"]))
    assert diff < float(g["rot_H2_tol"]), diff
