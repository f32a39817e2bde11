"""The oracle against the reference's own code compiled live in this
container (oracle/_ref); skipped where the reference tree is absent."""
import itertools

import numpy as np
import pytest


def test_shellpair_init_matches_reference(oracle_mod, ref_lib):
    import ctypes
    P = lambda a, t=ctypes.c_double: a.ctypes.data_as(ctypes.POINTER(t))
    rng = np.random.default_rng(7)
    for method in (0, 1):
        for _ in range(20):
            n1, n2 = rng.integers(1, 5, 2)
            l1, l2 = rng.integers(0, 4, 2)
            a1 = rng.uniform(0.1, 20, n1); a2 = rng.uniform(0.1, 20, n2)
            c1 = rng.uniform(0.01, 2, n1); c2 = rng.uniform(0.01, 2, n2)
            O1 = rng.uniform(-3, 3, 3); O2 = rng.uniform(-3, 3, 3)
            ln_prec = np.log(1e-10)
            mine = oracle_mod.shellpair_init(int(l1), a1, c1, O1, int(l2), a2, c2, O2, ln_prec,
                                             method)
            n = n1 * n2
            Pr = np.zeros(3 * n); K = np.zeros(n); oog = np.zeros(n); ns = np.zeros(n)
            ls = np.zeros(n); p1 = np.zeros(n, np.int32); p2 = np.zeros(n, np.int32)
            AB = np.zeros(3)
            l = np.array([l1, l2], np.int32); npr = np.array([n1, n2], np.int32)
            cnt = ref_lib.ref_shellpair_init(P(l, ctypes.c_int), P(npr, ctypes.c_int), P(a1),
                                             P(c1), P(O1), P(a2), P(c2), P(O2),
                                             ctypes.c_double(ln_prec), method, P(Pr), P(K),
                                             P(oog), P(ns), P(ls), P(p1, ctypes.c_int),
                                             P(p2, ctypes.c_int), P(AB))
            assert cnt == len(mine["K"])
            np.testing.assert_allclose(mine["K"], K[:cnt], rtol=1e-14)
            np.testing.assert_allclose(mine["ln_scr"], ls[:cnt], rtol=1e-13, atol=1e-13)
            np.testing.assert_allclose(mine["nonsph"], ns[:cnt], rtol=1e-13)
            np.testing.assert_array_equal(mine["p1"], p1[:cnt])


def test_eri_random_classes_live(oracle_mod, ref_lib):
    rng = np.random.default_rng(3)
    for ls in itertools.product([0, 1, 2], repeat=4):
        if rng.random() > 0.25:
            continue
        shells = []
        for l in ls:
            a = rng.uniform(0.2, 3, 2)
            c, _ = oracle_mod.shell_normalize(l, a, rng.uniform(0.3, 1, 2))
            shells.append((l, 1 if l > 1 else 0, a, c, rng.uniform(-1, 1, 3)))
        ref = oracle_mod.ref_eri_shellset(ref_lib, shells, 0)[0]
        ob = oracle_mod.OracleBasis([s[0] for s in shells], [s[1] for s in shells], [2] * 4,
                                    np.concatenate([s[4] for s in shells]),
                                    np.concatenate([s[2] for s in shells]),
                                    np.concatenate([s[3] for s in shells]))
        got = oracle_mod.compute_quartet(ob, 0, 1, 2, 3, 0, precision=0.0)[0]
        assert np.max(np.abs(got - ref)) < 1e-13
