"""The reference's Hartree-Fock golden values with the GPU J/K path doing
every two-electron step (Schwarz-screened J/K builds through lgx_jk, the
2-body forces through lgx_jk_grad): aug-cc-pVDZ rotated water energy within
5e-12 and 2-body forces within 1e-9 (hartree-fock++-validate.py), the 6-31G
energy of python/tests/test_hf.py to 7 decimals, the mixed-precision J/K
converging to the same energy within 1e-8, and the 2-body Hessian H2 (45
values, 1e-9) from the GPU's deriv_order 2 shell sets."""
import numpy as np
import pytest

import hf_util

pytestmark = pytest.mark.gpu


def test_aug_cc_pvdz_energy_and_2body_forces_gpu(lgx):
    from oracle import scf
    atoms, bs, g = hf_util.rotated_water(lgx)
    S, H, enuc, nocc = hf_util.core(bs, atoms)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    E, D, _, _, it = scf.rhf(S, H, nocc, lambda D: ctx.jk(D, 0.0)[:2], enuc)
    assert abs(E - float(g["rot_energy"])) < float(g["rot_energy_tol"]), E
    gJ, gK, _ = ctx.jk_grad(D, len(atoms), 0.0)
    F2 = 4.0 * (gJ + gK)
    assert np.max(np.abs(F2 - g["rot_F2"])) < float(g["rot_F2_tol"]), F2
    # mixed precision (FP32 for quartets with K12*K34 < 1e-4) with the
    # default Schwarz threshold: same SCF energy within 1e-8
    Em, _, _, _, _ = scf.rhf(S, H, nocc, lambda D: ctx.jk(D, 1e-12, mode=1,
                                                          mixed_thresh=1e-4)[:2], enuc)
    assert abs(Em - float(g["rot_energy"])) < 1e-8, Em
    ctx.close()


def test_631g_energy_gpu(lgx):
    from oracle import scf
    atoms, bs, g = hf_util.water_631g(lgx)
    S, H, enuc, nocc = hf_util.core(bs, atoms)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    E = scf.rhf_plain(S, H, nocc, lambda D: ctx.jk(D, 0.0)[:2], enuc)
    assert hf_util.places_ok(E, float(g["h2o631_energy"]), int(g["h2o631_places"])), E
    ctx.close()


def test_aug_cc_pvdz_2body_hessian_gpu(lgx):
    from oracle import scf
    atoms, bs, g = hf_util.rotated_water(lgx)
    S, H, enuc, nocc = hf_util.core(bs, atoms)
    ctx = lgx.Context(0)
    ctx.set_basis(bs)
    E, D, _, _, _ = scf.rhf(S, H, nocc, lambda D: ctx.jk(D, 0.0)[:2], enuc)
    eng = lgx.Engine(lgx.Operator.coulomb, bs.max_nprim(), bs.max_l(), 2, context=ctx)

    def sets_of(a, b, c, d):
        return eng.compute(bs[a], bs[b], bs[c], bs[d])

    H2 = hf_util.hessian_2body(bs, atoms, D, sets_of)
    diff = np.max(np.abs(hf_util.upper(H2) - g["rot_H2_upper"]))
    assert diff < float(g["rot_H2_tol"]), diff
    ctx.close()
