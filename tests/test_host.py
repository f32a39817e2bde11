"""Host-side logic of the product (no GPU calls): the C-ABI library loads and
exports every entry point include/lgx.h declares; the G94 basis reader and
shell normalization reproduce the reference's BasisSet; the water-cluster
builder is deterministic and geometrically right."""
import os
import re

import numpy as np

from golden_util import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(lgx):
    lib = lgx._lgx.load()
    header = open(os.path.join(ROOT, "include", "lgx.h")).read()
    names = set(re.findall(r"\b(lgx_[a-z0-9_]+)\s*\(", header))
    assert names, "no declarations found"
    for n in sorted(names):
        assert hasattr(lib, n), n
        assert n in lgx._lgx.SIGNATURES, n
    assert lib.lgx_version().decode().startswith("lgx")


def test_basis_matches_reference_basisset(lgx):
    g = load("basis.npz")
    atoms = [(int(z), g["xyz"][3 * i:3 * i + 3]) for i, z in enumerate(g["Z"])]
    for name in ("cc-pVDZ", "cc-pVTZ"):
        key = name.lower().replace("-", "")
        bs = lgx.BasisSet(name, atoms)
        np.testing.assert_array_equal(bs.l, g[key + "_l"])
        np.testing.assert_array_equal(bs.pure, g[key + "_pure"])
        np.testing.assert_array_equal(bs.nprim, g[key + "_nprim"])
        np.testing.assert_allclose(bs.origins, g[key + "_O"], rtol=0, atol=0)
        np.testing.assert_allclose(bs.alpha, g[key + "_alpha"], rtol=0, atol=0)
        np.testing.assert_allclose(bs.coeff, g[key + "_coeff"], rtol=1e-14, atol=0)


def test_shell_normalization_matches_reference(lgx):
    g = load("shells.npz")
    for l, a, cin, cout in zip(g["l"], g["alpha"], g["cin"], g["cout"]):
        s = lgx.Shell(int(l), list(zip(a, cin)))
        np.testing.assert_allclose(s.coeff, cout, rtol=1e-13)


def test_water_cluster_geometry(lgx):
    atoms = lgx.water_cluster(2, 2, 1, spacing=3.0, jitter=0.2, seed=42)
    again = lgx.water_cluster(2, 2, 1, spacing=3.0, jitter=0.2, seed=42)
    assert atoms == again
    other = lgx.water_cluster(2, 2, 1, spacing=3.0, jitter=0.2, seed=43)
    assert atoms != other
    a2b = 1 / 0.529177210903
    for m in range(4):
        O = np.array(atoms[3 * m][1]); H1 = np.array(atoms[3 * m + 1][1])
        H2 = np.array(atoms[3 * m + 2][1])
        assert atoms[3 * m][0] == 8 and atoms[3 * m + 1][0] == 1
        assert abs(np.linalg.norm(H1 - O) - 0.96 * a2b) < 1e-12
        ang = np.degrees(np.arccos(np.dot(H1 - O, H2 - O) /
                                   (np.linalg.norm(H1 - O) * np.linalg.norm(H2 - O))))
        assert abs(ang - 104.5) < 1e-9
        grid = np.array([(m // 2) * 3.0, (m % 2) * 3.0, 0.0]) * a2b
        assert np.all(np.abs(O - grid) <= 0.2 * a2b + 1e-12)


def test_basis_sizes_of_the_configurations(lgx):
    # (H2O)n with cc-pVDZ: 12 shells / 24 functions per water; cc-pVTZ 22 / 58
    a = lgx.water_cluster(2, 1, 1)
    dz = lgx.BasisSet("cc-pVDZ", a)
    tz = lgx.BasisSet("cc-pVTZ", a)
    assert (len(dz), dz.nbf, dz.max_nprim(), dz.max_l()) == (24, 48, 8, 2)
    assert (len(tz), tz.nbf, tz.max_nprim(), tz.max_l()) == (44, 116, 8, 3)


def test_random_density_is_psd(lgx):
    D = lgx.random_density(40, 7, seed=1)
    assert np.allclose(D, D.T)
    w = np.linalg.eigvalsh(D)
    assert w.min() > -1e-12 and np.sum(w > 1e-10) == 7
