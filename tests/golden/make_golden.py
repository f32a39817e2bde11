"""Generates the golden fixtures in tests/golden/ from the reference's own
code, compiled in place by oracle/ref/build_ref.sh into oracle/_ref/libref.so
(libint2::Shell::renorm, SolidHarmonicsCoefficients::coeff,
FmEval_Reference2, BasisSet, DerivMapGenerator and the brute-force ERI of
src/bin/test_eri/eri.h).  Run where the reference tree exists, naming it
in LGX_REFERENCE_ROOT:

    LGX_REFERENCE_ROOT=<libint tree> python tests/golden/make_golden.py

Outputs (numpy .npz, committed):
  boys.npz        F_m(T) from FmEval_Reference2 and FmEval_Reference<long double>
  solid.npz       solid-harmonic coefficients, l <= 4
  shells.npz      normalized coefficients of random shells (Shell::renorm)
  basis.npz       BasisSet("cc-pVDZ"/"cc-pVTZ") for one water
  derivmap.npz    first-derivative shell-set order and bra/ket-swap map
  eri.npz         brute-force contracted shell sets, d0 and d1, many classes
  eri3c.npz       brute-force 3-centre (a 1|c d) and 2-centre (a 1|c 1) shell
                  sets, d0 and d1 (1 = Shell::unit(), exponent 0), same layout
                  as eri.npz plus the braket rank
  eri_d2.npz      brute-force second-derivative (deriv_order 2) shell sets, 78
                  per quartet in libint's order (CartesianDerivIterator<4>(2)),
                  shells up to f, with that order as coordinate pairs
  hf.npz          system-level golden values of the reference's Hartree-Fock
                  tests, read as text: the rotated-water geometry
                  (tests/hartree-fock/h2o_rotated.xyz) with the aug-cc-pVDZ
                  energy and 2-body forces its validator checks
                  (hartree-fock++-validate.py), and the water geometry and
                  6-31G energy of python/tests/test_hf.py

    python tests/golden/make_golden.py --hf-only    # hf.npz alone
    python tests/golden/make_golden.py --eri3c-only # eri3c.npz alone
    python tests/golden/make_golden.py --d2-only    # eri_d2.npz alone
"""
import ctypes
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402

P = lambda a, t=ctypes.c_double: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731


def main():
    oracle.build_ref()
    ref = oracle.ref_lib()
    assert ref is not None, "reference build missing"
    rng = np.random.default_rng(20240601)

    # Boys
    T = np.concatenate([np.linspace(0, 40, 801), [45, 60, 80, 117, 118, 150, 300, 1000]])
    mmax = 16
    F2 = np.zeros((len(T), mmax + 1))
    Fld = np.zeros((len(T), mmax + 1))
    for i, t in enumerate(T):
        ref.ref_boys_reference2(float(t), mmax, P(F2[i]))
        if t < 117:
            ref.ref_boys_reference_ld(float(t), mmax, P(Fld[i]))
        else:
            Fld[i] = F2[i]
    np.savez_compressed(os.path.join(HERE, "boys.npz"), T=T, F_ref2=F2, F_refld=Fld)

    # solid harmonics
    rows = []
    for l in range(5):
        for m in range(-l, l + 1):
            for lx in range(l, -1, -1):
                for ly in range(l - lx, -1, -1):
                    rows.append((l, m, lx, ly, l - lx - ly,
                                 ref.ref_solid_coeff(l, m, lx, ly, l - lx - ly)))
    rows = np.array(rows)
    np.savez_compressed(os.path.join(HERE, "solid.npz"), idx=rows[:, :5].astype(np.int32),
                        coeff=rows[:, 5])

    # shell normalization
    L, A, Cin, Cout = [], [], [], []
    for k in range(40):
        l = k % 5
        n = 1 + k % 4
        a = np.sort(rng.uniform(0.05, 50.0, n))[::-1].copy()
        c = rng.uniform(-1, 1, n)
        co = np.zeros(n)
        ml = np.zeros(n)
        ref.ref_shell_normalize(l, 0, n, P(a), P(c), P(co), P(ml))
        L.append(l); A.append(a); Cin.append(c); Cout.append(co)
    np.savez_compressed(os.path.join(HERE, "shells.npz"), l=np.array(L, np.int32),
                        alpha=np.array(A, dtype=object), cin=np.array(Cin, dtype=object),
                        cout=np.array(Cout, dtype=object), allow_pickle=True)

    # BasisSet for one water (bohr)
    Z = np.array([8, 1, 1], np.int32)
    xyz = np.array([0.0, -0.143, 0.0, 1.638, 1.136, 0.0, -1.638, 1.136, 0.0])
    out = {"Z": Z, "xyz": xyz}
    for name in ("cc-pVDZ", "cc-pVTZ"):
        ns = ref.ref_basis(name.encode(), 3, P(Z, ctypes.c_int), P(xyz), None, None, None,
                           None, None, None, 0)
        l = np.zeros(ns, np.int32); pure = np.zeros(ns, np.int32); npr = np.zeros(ns, np.int32)
        O = np.zeros(3 * ns); al = np.zeros(400); co = np.zeros(400)
        ref.ref_basis(name.encode(), 3, P(Z, ctypes.c_int), P(xyz), P(l, ctypes.c_int),
                      P(pure, ctypes.c_int), P(npr, ctypes.c_int), P(O), P(al), P(co), 400)
        m = int(npr.sum())
        key = name.lower().replace("-", "")
        out[key + "_l"] = l; out[key + "_pure"] = pure; out[key + "_nprim"] = npr
        out[key + "_O"] = O; out[key + "_alpha"] = al[:m]; out[key + "_coeff"] = co[:m]
    np.savez_compressed(os.path.join(HERE, "basis.npz"), **out)

    # derivative order and map
    order = np.zeros(12, np.int32)
    ref.ref_deriv_order1(P(order, ctypes.c_int))
    dmap = np.zeros((2, 2, 2, 12), np.int32)
    for a, b, c, s in itertools.product(range(2), range(2), range(2), range(12)):
        dmap[a, b, c, s] = ref.ref_deriv_map1(a, b, c, s)
    np.savez_compressed(os.path.join(HERE, "derivmap.npz"), order=order, map=dmap)

    # brute-force shell sets
    cases = []
    for ls in itertools.product(range(4), repeat=4):
        cases.append((ls, 0))
    for ls in itertools.product(range(3), repeat=4):
        if sum(ls) <= 5:
            cases.append((ls, 1))
    recs = {"l": [], "pure": [], "nprim": [], "alpha": [], "coeff": [], "O": [], "deriv": [],
            "values": [], "offset": []}
    off = 0
    vals = []
    for ls, d in cases:
        shells = []
        for k, l in enumerate(ls):
            n = 1 if (l == 3 or sum(ls) > 7) else (2 if l > 0 else 3)
            a = np.sort(rng.uniform(0.15, 5.0, n))[::-1].copy()
            c = rng.uniform(0.2, 1.0, n)
            cn, _ = oracle.shell_normalize(l, a, c)
            pure = 1 if l > 1 else 0
            shells.append((l, pure, a, cn, rng.uniform(-1.2, 1.2, 3)))
        r = oracle.ref_eri_shellset(ref, shells, d)
        v = np.concatenate([x.reshape(-1) for x in r])
        recs["l"].append(ls); recs["pure"].append([s[1] for s in shells])
        recs["nprim"].append([len(s[2]) for s in shells])
        recs["alpha"].append(np.concatenate([s[2] for s in shells]))
        recs["coeff"].append(np.concatenate([s[3] for s in shells]))
        recs["O"].append(np.concatenate([s[4] for s in shells]))
        recs["deriv"].append(d)
        recs["offset"].append(off)
        vals.append(v)
        off += v.size
    maxp = max(len(a) for a in recs["alpha"])
    alpha = np.zeros((len(cases), maxp)); coeff = np.zeros((len(cases), maxp))
    for i in range(len(cases)):
        alpha[i, :len(recs["alpha"][i])] = recs["alpha"][i]
        coeff[i, :len(recs["coeff"][i])] = recs["coeff"][i]
    np.savez_compressed(os.path.join(HERE, "eri.npz"), l=np.array(recs["l"], np.int32),
                        pure=np.array(recs["pure"], np.int32),
                        nprim=np.array(recs["nprim"], np.int32), alpha=alpha, coeff=coeff,
                        O=np.array(recs["O"]), deriv=np.array(recs["deriv"], np.int32),
                        offset=np.array(recs["offset"], np.int64),
                        values=np.concatenate(vals))
    print("cases", len(cases), "values", off)


def eri3c_fixtures():
    """3- and 2-centre shell sets from the reference's brute-force eri.h with
    unit shells (l = 0, exponent 0, coefficient 1, at the origin) in the
    empty positions, as Engine::compute does for xs_xx / xs_xs
    (engine.impl.h:140-175)."""
    oracle.build_ref()
    ref = oracle.ref_lib()
    assert ref is not None, "reference build missing"
    rng = np.random.default_rng(20240602)
    unit = (0, 0, np.array([0.0]), np.array([1.0]), np.zeros(3))
    cases = []
    for la, lc, ld in itertools.product(range(4), repeat=3):
        cases.append(((la, 0, lc, ld), 3, 0))
        if la + lc + ld <= 5:
            cases.append(((la, 0, lc, ld), 3, 1))
    for la, lc in itertools.product(range(4), repeat=2):
        cases.append(((la, 0, lc, 0), 2, 0))
        cases.append(((la, 0, lc, 0), 2, 1))
    recs = {"l": [], "pure": [], "nprim": [], "alpha": [], "coeff": [], "O": [], "deriv": [],
            "rank": [], "offset": []}
    off, vals = 0, []
    for ls, rank, d in cases:
        shells = []
        for k, l in enumerate(ls):
            if k == 1 or (rank == 2 and k == 3):
                shells.append(unit)
                continue
            n = 1 if l == 3 else (2 if l > 0 else 3)
            a = np.sort(rng.uniform(0.15, 5.0, n))[::-1].copy()
            c = rng.uniform(0.2, 1.0, n)
            cn, _ = oracle.shell_normalize(l, a, c)
            shells.append((l, 1 if l > 1 else 0, a, cn, rng.uniform(-1.2, 1.2, 3)))
        r = oracle.ref_eri_shellset(ref, shells, d)
        v = np.concatenate([x.reshape(-1) for x in r])
        recs["l"].append(ls); recs["pure"].append([s[1] for s in shells])
        recs["nprim"].append([len(s[2]) for s in shells])
        recs["alpha"].append(np.concatenate([s[2] for s in shells]))
        recs["coeff"].append(np.concatenate([s[3] for s in shells]))
        recs["O"].append(np.concatenate([s[4] for s in shells]))
        recs["deriv"].append(d); recs["rank"].append(rank)
        recs["offset"].append(off)
        vals.append(v)
        off += v.size
    maxp = max(len(a) for a in recs["alpha"])
    alpha = np.zeros((len(cases), maxp)); coeff = np.zeros((len(cases), maxp))
    for i in range(len(cases)):
        alpha[i, :len(recs["alpha"][i])] = recs["alpha"][i]
        coeff[i, :len(recs["coeff"][i])] = recs["coeff"][i]
    np.savez_compressed(os.path.join(HERE, "eri3c.npz"), l=np.array(recs["l"], np.int32),
                        pure=np.array(recs["pure"], np.int32),
                        nprim=np.array(recs["nprim"], np.int32), alpha=alpha, coeff=coeff,
                        O=np.array(recs["O"]), deriv=np.array(recs["deriv"], np.int32),
                        rank=np.array(recs["rank"], np.int32),
                        offset=np.array(recs["offset"], np.int64), values=np.concatenate(vals))


def eri_d2_fixtures():
    """Second-derivative shell sets from the reference's brute-force eri.h
    (any derivative order, via CartesianDerivIterator<4>(2))."""
    oracle.build_ref()
    ref = oracle.ref_lib()
    assert ref is not None, "reference build missing"
    rng = np.random.default_rng(20240603)
    c1, c2 = oracle.ref_deriv_order2(ref)
    cases = [(0, 0, 0, 0), (1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1), (1, 1, 0, 0),
             (1, 0, 1, 0), (0, 1, 0, 1), (1, 1, 1, 1), (2, 0, 0, 0), (0, 2, 1, 0), (2, 1, 0, 1),
             (1, 0, 2, 1), (2, 2, 0, 0), (0, 0, 2, 2), (2, 1, 1, 2),
             # f shells (the composition raises them to g)
             (3, 0, 0, 0), (0, 1, 3, 0), (3, 1, 0, 2), (2, 3, 3, 1)]
    recs = {"l": [], "pure": [], "nprim": [], "alpha": [], "coeff": [], "O": [], "offset": []}
    off, vals = 0, []
    for t, ls in enumerate(cases):
        shells = []
        for k, l in enumerate(ls):
            n = 2 if (l < 2 and sum(ls) <= 3) else 1
            a = np.sort(rng.uniform(0.2, 3.0, n))[::-1].copy()
            c = rng.uniform(0.3, 1.0, n)
            cn, _ = oracle.shell_normalize(l, a, c)
            shells.append((l, (1 if l > 1 else 0) if t % 2 else 0, a, cn, rng.uniform(-1.0, 1.0, 3)))
        r = oracle.ref_eri_shellset(ref, shells, 2)
        v = np.concatenate([x.reshape(-1) for x in r])
        recs["l"].append(ls); recs["pure"].append([s[1] for s in shells])
        recs["nprim"].append([len(s[2]) for s in shells])
        recs["alpha"].append(np.concatenate([s[2] for s in shells]))
        recs["coeff"].append(np.concatenate([s[3] for s in shells]))
        recs["O"].append(np.concatenate([s[4] for s in shells]))
        recs["offset"].append(off)
        vals.append(v)
        off += v.size
    maxp = max(len(a) for a in recs["alpha"])
    alpha = np.zeros((len(cases), maxp)); coeff = np.zeros((len(cases), maxp))
    for i in range(len(cases)):
        alpha[i, :len(recs["alpha"][i])] = recs["alpha"][i]
        coeff[i, :len(recs["coeff"][i])] = recs["coeff"][i]
    np.savez_compressed(os.path.join(HERE, "eri_d2.npz"), l=np.array(recs["l"], np.int32),
                        pure=np.array(recs["pure"], np.int32),
                        nprim=np.array(recs["nprim"], np.int32), alpha=alpha, coeff=coeff,
                        O=np.array(recs["O"]), offset=np.array(recs["offset"], np.int64),
                        values=np.concatenate(vals), c1=c1, c2=c2)


# the libint source tree whose test files hold the HF golden values
REFERENCE = os.environ.get("LGX_REFERENCE_ROOT", "")
SYMBOL_Z = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "Ne": 10}


def _floats_after(text, name):
    """The list literal assigned to `name` in a Python source text."""
    import re
    m = re.search(r"^%s\s*=\s*\[([^\]]*)\]" % re.escape(name), text, re.M)
    return [float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]


def _scalar_after(text, name):
    import re
    m = re.search(r"^%s\s*=\s*([-+0-9.eE]+)" % re.escape(name), text, re.M)
    return float(m.group(1))


def hf_fixtures(root=REFERENCE):
    if not root or not os.path.isdir(root):
        sys.exit("hf fixtures: set LGX_REFERENCE_ROOT to the libint source tree")
    import re
    hf = os.path.join(root, "tests", "hartree-fock")
    with open(os.path.join(hf, "h2o_rotated.xyz")) as f:
        lines = f.read().splitlines()
    nat = int(lines[0].split()[0])
    Z, xyz = [], []
    for ln in lines[2:2 + nat]:
        t = ln.split()
        Z.append(SYMBOL_Z[t[0]])
        xyz.append([float(v) for v in t[1:4]])
    with open(os.path.join(hf, "hartree-fock++-validate.py")) as f:
        val = f.read()
    eref = _floats_after(val, "eref")[0]
    etol = _scalar_after(val, "etol")
    F2 = _floats_after(val, "F2ref")
    F2tol = _scalar_after(val, "F2tol")
    H2 = _floats_after(val, "H2ref")
    H2tol = _scalar_after(val, "H2tol")
    with open(os.path.join(root, "python", "tests", "test_hf.py")) as f:
        py = f.read()
    m = re.search(r"h2o\s*=\s*\[(.*?)\n\]", py, re.S)
    atoms631 = re.findall(r"\(\s*(\d+)\s*,\s*\[([^\]]*)\]\s*\)", m.group(1))
    Z631 = [int(a) for a, _ in atoms631]
    xyz631 = [[float(v) for v in b.split(",")] for _, b in atoms631]
    e631 = float(re.search(r"assertAlmostEqual\(rhf\.energy\(\),\s*([-0-9.]+)\)", py).group(1))
    np.savez(os.path.join(HERE, "hf.npz"),
             rot_Z=np.array(Z, np.int32), rot_xyz_angstrom=np.array(xyz),
             rot_basis="aug-cc-pVDZ", rot_energy=eref, rot_energy_tol=etol,
             rot_F2=np.array(F2).reshape(nat, 3), rot_F2_tol=F2tol,
             rot_H2_upper=np.array(H2), rot_H2_tol=H2tol,
             h2o631_Z=np.array(Z631, np.int32), h2o631_xyz_bohr=np.array(xyz631),
             h2o631_basis="6-31G", h2o631_energy=e631, h2o631_places=7)


if __name__ == "__main__" and "--hf-only" in sys.argv:
    hf_fixtures()
elif __name__ == "__main__" and "--eri3c-only" in sys.argv:
    eri3c_fixtures()
elif __name__ == "__main__" and "--d2-only" in sys.argv:
    eri_d2_fixtures()
elif __name__ == "__main__":
    hf_fixtures()
    eri3c_fixtures()
    eri_d2_fixtures()
    main()
