"""Shared set-up of the Hartree-Fock checks: the molecules and golden values
of the reference's HF tests (tests/golden/hf.npz, made by
tests/golden/make_golden.py) and the one-body part from oracle/onebody.py."""
import numpy as np

from golden_util import load

BOHR_TO_ANGSTROM = 0.529177210903  # CODATA 2018, include/libint2/atom.h:52-55


def rotated_water(lgx):
    """h2o_rotated.xyz in bohr, aug-cc-pVDZ without unit renormalization of
    the contractions (hartree-fock++.cc:281), and the golden values."""
    g = load("hf.npz")
    atoms = [(int(z), tuple(float(x) / BOHR_TO_ANGSTROM for x in xyz))
             for z, xyz in zip(g["rot_Z"], g["rot_xyz_angstrom"])]
    prev = lgx.Shell.do_enforce_unit_normalization(False)
    try:
        bs = lgx.BasisSet(str(g["rot_basis"]), atoms)
    finally:
        lgx.Shell.do_enforce_unit_normalization(True)
    assert prev is False
    return atoms, bs, g


def water_631g(lgx):
    g = load("hf.npz")
    atoms = [(int(z), tuple(float(x) for x in xyz))
             for z, xyz in zip(g["h2o631_Z"], g["h2o631_xyz_bohr"])]
    return atoms, lgx.BasisSet(str(g["h2o631_basis"]), atoms), g


def core(bs, atoms):
    from oracle import onebody
    S, T, V = onebody.one_body(bs, atoms)
    return S, T + V, onebody.nuclear_repulsion(atoms), sum(a[0] for a in atoms) // 2


def places_ok(value, ref, places):
    return round(abs(value - ref), places) == 0  # unittest's assertAlmostEqual
