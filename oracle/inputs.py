"""Inputs of the oracle's CPU runs, built without the GPU library.

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's CPU arms (the
``--impl reference`` arm and ``cpu_baseline``), so that those arms load no
part of liblgx.so.  The product package has its own loader
(lgx_basis_load) and cluster generator (lgx_water_cluster); a CPU test checks
that both give the same basis and geometry.

* ``read_g94`` restates libint's G94 basis-library reader,
  BasisSet::read_g94_basis_library (include/libint2/basis.h.in:473-621):
  '!' comments and empty lines skipped, '****' separates elements (a
  leading '****' is the older EMSL header), an element line then shell
  lines ``<label> <nprim> <scale>``, Fortran 'D' exponents, SP shells split
  into an s and a p shell, and d and higher shells pure (solid harmonics)
  unless the basis uses Cartesian d (f and higher stay pure).
* ``load_basis`` follows BasisSet(name, atoms) (basis.h.in:134-182,
  canonicalize_name / the aug-cc-pVXZ split into the base set plus its
  "augmentation-" file): for each atom in order, the shells of its element,
  centred on the atom, with Shell::renorm applied (the oracle's
  orc_shell_normalize, shell.h:958-999).
* ``water_cluster`` wraps the oracle's restatement of the configurations'
  cluster construction (orc_water_cluster), ``random_density`` the
  configurations' density D = C C^T.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import oracle

_HERE = os.path.dirname(os.path.abspath(__file__))
DATA_DIR = os.path.join(os.path.dirname(_HERE), "libint_gb300", "data", "basis")

_SYMBOLS = ["", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si",
            "P", "S", "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni",
            "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"]
_AM = "SPDFGHIKLMNOQRTUVWXYZ"


def _element_z(sym: str) -> int:
    for z, s in enumerate(_SYMBOLS):
        if z and s.lower() == sym.lower():
            return z
    raise ValueError("unknown element symbol %r" % sym)


def _am_of_label(label: str) -> int:
    c = label[0].upper()
    if c == "J":  # Gaussian's labels skip J: I=6, J=7, then K=8, L=9, ...
        return 7
    l = _AM.index(c)
    return l + 1 if l >= 7 else l


def cartesian_d(canon: str) -> bool:
    """Pople bases whose d shells are Cartesian (3-21G, 4-31G, 6-31G*,
    6-31G**; not 6-311G), as libint's BasisSet decides from the name."""
    if canon.startswith("3-21") or canon.startswith("4-31g"):
        return True
    if canon.startswith("6-31") and len(canon) > 4 and canon[4] != "1":
        g = canon.find("g")
        if g < 0:
            return False
        return g + 1 == len(canon) or canon[g + 1] in "*s"
    return False


def read_g94(path: str, force_cartesian_d: bool = False):
    """{Z: [(l, pure, alpha[], coeff[]), ...]} from a Gaussian-94 library file."""
    shells = {}
    with open(path) as f:
        lines = [ln.rstrip("\r\n ") for ln in f]
    i = 0
    nextbasis, nextshell, first = True, False, True
    Z = None
    while i < len(lines):
        line = lines[i]
        i += 1
        if not line or line[0] == "!":
            continue
        if line == "****":
            if first:
                continue
            nextbasis, nextshell = True, False
            continue
        if nextbasis:
            nextbasis, first = False, False
            Z = _element_z(line.split()[0])
            shells.setdefault(Z, [])
            nextshell = True
            continue
        if nextshell:
            tok = line.split()
            label, nprim = tok[0], int(tok[1])
            rows = []
            while len(rows) < nprim:
                pl = lines[i]
                i += 1
                if not pl or pl[0] == "!":
                    continue
                rows.append([float(x.replace("D", "E").replace("d", "e")) for x in pl.split()])
            alpha = np.array([r[0] for r in rows])
            if label in ("SP", "sp"):
                shells[Z].append((0, False, alpha, np.array([r[1] for r in rows])))
                shells[Z].append((1, False, alpha.copy(), np.array([r[2] for r in rows])))
            else:
                l = _am_of_label(label)
                pure = l > 2 if force_cartesian_d else l > 1
                shells[Z].append((l, pure, alpha, np.array([r[1] for r in rows])))
    return shells


def canonical_name(name: str) -> str:
    return name.lower().replace("/", "I")


def load_basis(name: str, atoms, data_dir: str | None = None) -> "oracle.OracleBasis":
    """BasisSet(name, atoms) as an OracleBasis (normalised contractions)."""
    canon = canonical_name(name)
    comps = [canon]
    if canon.startswith("aug-cc-pv") and "cabs" not in canon:
        comps = [canon[4:], "augmentation-" + canon[4:]]
    force = cartesian_d(canon)
    libs = [read_g94(os.path.join(data_dir or DATA_DIR, c + ".g94"), force) for c in comps]
    l, pure, nprim, atom, O, alpha, coeff = [], [], [], [], [], [], []
    for ia, (Z, xyz) in enumerate(atoms):
        for lib in libs:
            for (sl, spure, sa, sc) in lib.get(int(Z), []):
                cn, _ = oracle.shell_normalize(sl, sa, sc)
                l.append(sl); pure.append(1 if spure else 0); nprim.append(len(sa))
                atom.append(ia); O.extend(float(v) for v in xyz)
                alpha.extend(sa); coeff.extend(cn)
    return oracle.OracleBasis(l, pure, nprim, O, alpha, coeff, atom)


def water_cluster(nx, ny, nz, spacing=3.0, jitter=0.2, seed=0):
    """[(Z, (x, y, z))] in bohr: the configurations' water cluster."""
    n = nx * ny * nz
    Z = np.zeros(3 * n, np.int32)
    xyz = np.zeros(9 * n)
    lib = oracle._lib()
    lib.orc_water_cluster.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_uint64,
                                      ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_double)]
    if lib.orc_water_cluster(nx, ny, nz, spacing, jitter, seed,
                             Z.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                             xyz.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) != 0:
        raise ValueError("orc_water_cluster: bad arguments")
    return [(int(Z[i]), tuple(xyz[3 * i:3 * i + 3])) for i in range(3 * n)]


def random_density(nbf: int, nocc: int, seed: int = 0) -> np.ndarray:
    """D = C C^T, C of shape nbf x nocc with entries N(0, 1)/sqrt(nbf) from
    numpy's default_rng(seed): the configurations' density."""
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((nbf, nocc)) / np.sqrt(nbf)
    return C @ C.T
