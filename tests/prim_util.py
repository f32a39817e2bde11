"""Caller side of libint's generated-library API, for the tests of
lgx_compute_primitive_set and include/libint2.h: the per-primitive-quartet
prefactors a libint caller computes before libint2_build_eri*
(engine.impl.h:1389-1757; the reference's test driver prep_libint2.h
writes the same quantities), from raw primitive shells (exponents and
coefficients used as given, no normalization), with the oracle's Boys
function."""
import numpy as np

from oracle import oracle

TWO_PI_25 = 2.0 * np.pi ** 2.5


def random_shells(rng, ls, max_depth=2, spread=1.2):
    """Four raw shells (l, alphas, coeffs, origin) with 1..max_depth primitives."""
    out = []
    for l in ls:
        n = int(rng.integers(1, max_depth + 1))
        a = np.sort(rng.uniform(0.3, 3.0, n))[::-1].copy()
        c = rng.uniform(0.4, 1.2, n)
        out.append((int(l), a, c, rng.uniform(-spread, spread, 3)))
    return out


def prim_quartets(shells, deriv, dtype):
    """(records of dtype, AB, CD): one record per primitive quartet, in the
    p0 p1 p2 p3 nesting of libint's callers."""
    (l1, a1s, c1s, A), (l2, a2s, c2s, B), (l3, a3s, c3s, C), (l4, a4s, c4s, D) = shells
    mmax = l1 + l2 + l3 + l4 + deriv
    recs = []
    for a1, c1 in zip(a1s, c1s):
        for a2, c2 in zip(a2s, c2s):
            for a3, c3 in zip(a3s, c3s):
                for a4, c4 in zip(a4s, c4s):
                    z, e = a1 + a2, a3 + a4
                    P = (a1 * A + a2 * B) / z
                    Q = (a3 * C + a4 * D) / e
                    rho = z * e / (z + e)
                    W = (z * P + e * Q) / (z + e)
                    K1 = np.exp(-a1 * a2 / z * np.dot(A - B, A - B))
                    K2 = np.exp(-a3 * a4 / e * np.dot(C - D, C - D))
                    pfac = TWO_PI_25 * K1 * K2 / (z * e * np.sqrt(z + e)) * c1 * c2 * c3 * c4
                    F = oracle.boys(float(rho * np.dot(P - Q, P - Q)), mmax)
                    r = np.zeros((), dtype)
                    r["PA"], r["QC"], r["WP"], r["WQ"] = P - A, Q - C, W - P, W - Q
                    r["oo2z"], r["oo2e"], r["oo2ze"] = 0.5 / z, 0.5 / e, 0.5 / (z + e)
                    r["roz"], r["roe"] = rho / z, rho / e
                    r["two_alpha"] = [2 * a1, 2 * a2, 2 * a3, 2 * a4]
                    ss = np.zeros(dtype["ss"].shape)
                    ss[:mmax + 1] = pfac * np.asarray(F)[:mmax + 1]
                    r["ss"] = ss
                    recs.append(r)
    return np.array(recs, dtype=dtype), A - B, C - D


def oracle_sets(shells, deriv):
    """The oracle's contracted Cartesian shell sets of the same raw shells
    (1, 12 or 78 sets, caller order)."""
    L = np.array([s[0] for s in shells], np.int32)
    ob = oracle.OracleBasis(L, np.zeros(4, np.int32),
                            np.array([len(s[1]) for s in shells], np.int32),
                            np.concatenate([s[3] for s in shells]),
                            np.concatenate([s[1] for s in shells]),
                            np.concatenate([s[2] for s in shells]))
    return oracle.compute_quartet(ob, 0, 1, 2, 3, deriv=deriv, precision=0.0)
