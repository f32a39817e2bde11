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


def unique_quartets(ns):
    """Canonical unique shell quartets a>=b, c>=d, (ab)>=(cd) with their
    8-fold degeneracy factors (hartree-fock++.cc:1628-1700)."""
    out = []
    for a in range(ns):
        for b in range(a + 1):
            for c in range(a + 1):
                for d in range(c + 1 if c < a else b + 1):
                    deg = (1 if a == b else 2) * (1 if c == d else 2) * (1 if (a, b) == (c, d) else 2)
                    out.append((a, b, c, d, deg))
    return out


def hessian_2body(bs, atoms, D, sets_of):
    """H2 = sum_ab D_ab d2G_ab/dx dy with G = 2J - K (compute_2body_fock_deriv<2>,
    hartree-fock++.cc:763-776): per unique quartet
    deg * [2 D_ab D_cd - (D_ac D_bd + D_ad D_bc)/2] * d2(ab|cd), the 78 sets
    (coordinate pairs c1 <= c2 of the quartet's centres, row-major) mapped to
    atom coordinates.  sets_of(a, b, c, d) -> 78 arrays or None."""
    n = 3 * len(atoms)
    H = np.zeros((n, n))
    off = bs.shell2bf()
    s2a = bs.atom_of_shell
    pairs = [(c1, c2) for c1 in range(12) for c2 in range(c1, 12)]
    for a, b, c, d, deg in unique_quartets(len(bs)):
        r = sets_of(a, b, c, d)
        if r is None:
            continue
        sl = [slice(off[s], off[s] + bs[s].size()) for s in (a, b, c, d)]
        W = 2.0 * np.einsum("ij,kl->ijkl", D[sl[0], sl[1]], D[sl[2], sl[3]]) - 0.5 * (
            np.einsum("ik,jl->ijkl", D[sl[0], sl[2]], D[sl[1], sl[3]]) +
            np.einsum("il,jk->ijkl", D[sl[0], sl[3]], D[sl[1], sl[2]]))
        vals = deg * np.tensordot(np.asarray(r).reshape(78, -1), W.reshape(-1), axes=1)
        ctr = (a, b, c, d)
        for (c1, c2), v in zip(pairs, vals):
            p = 3 * s2a[ctr[c1 // 3]] + c1 % 3
            q = 3 * s2a[ctr[c2 // 3]] + c2 % 3
            H[p, q] += v
            if c1 != c2:
                H[q, p] += v
    return H


def upper(H):
    return np.array([H[r, c] for r in range(H.shape[0]) for c in range(r, H.shape[0])])
