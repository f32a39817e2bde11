"""One-body integrals (overlap, kinetic energy, nuclear attraction) in FP64
numpy, for the Hartree-Fock check of the J/K path.

TEST INFRASTRUCTURE ONLY (like the rest of oracle/): the RHF energy and
force golden values of the reference's HF driver (hartree-fock++.cc) need
the core Hamiltonian, which is outside the ERI path.  These matrices stand
in for libint's Engine with Operator::overlap / kinetic / nuclear
(include/libint2/engine.h:98-184; compute_1body_ints, hartree-fock++.cc
:1108-1170), restated from the published Obara-Saika recursions (S. Obara
and A. Saika, J. Chem. Phys. 84, 3963 (1986); T. Helgaker, P. Jorgensen and
J. Olsen, Molecular Electronic-Structure Theory, 9.3):

  overlap, per axis:  S_{i+1,j} = X_PA S_{ij} + (i S_{i-1,j} + j S_{i,j-1}) / 2p
                      S_{i,j+1} = X_PB S_{ij} + (i S_{i-1,j} + j S_{i,j-1}) / 2p
  kinetic, per axis:  T_ij = -2 b^2 S_{i,j+2} + b (2j+1) S_ij - j(j-1)/2 S_{i,j-2}
  nuclear attraction: Theta^(m)_{a+1_i,0} = PA_i Theta^(m)_{a0} - PC_i Theta^(m+1)_{a0}
                        + a_i/2p (Theta^(m)_{a-1_i,0} - Theta^(m+1)_{a-1_i,0}),
                      Theta^(m)_{00} = 2 pi/p K_AB F_m(p |PC|^2),
                      then (a|b+1_i) = (a+1_i|b) + AB_i (a|b) on contracted values.

Shells are taken as they are (normalization embedded in the coefficients,
libint's standard Cartesian normalization: every component shares the x^l
factor); pure shells are transformed with the same real solid-harmonic
coefficients the ERI oracle uses (solidharmonics.h:114-174, m = -l..l).
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle


def _comps(l):
    return [(lx, ly, l - lx - ly) for lx in range(l, -1, -1) for ly in range(l - lx, -1, -1)]


def _sph(l):
    cs = _comps(l)
    M = np.zeros((2 * l + 1, len(cs)))
    for p in range(2 * l + 1):
        for c, (lx, ly, lz) in enumerate(cs):
            M[p, c] = oracle.solid_coeff(l, p - l, lx, ly, lz)
    return M


def _prim_pairs(sa, sb):
    a = np.repeat(sa.alpha, len(sb.alpha))
    b = np.tile(sb.alpha, len(sa.alpha))
    c = np.repeat(sa.coeff, len(sb.alpha)) * np.tile(sb.coeff, len(sa.alpha))
    p = a + b
    A, B = np.asarray(sa.O, float), np.asarray(sb.O, float)
    P = (a[:, None] * A + b[:, None] * B) / p[:, None]
    AB2 = float(np.dot(A - B, A - B))
    K = np.exp(-a * b / p * AB2)
    return a, b, c, p, P, A, B, K


def _overlap_1d(imax, jmax, PA, PB, oo2p):
    S = [[None] * (jmax + 1) for _ in range(imax + 1)]
    one = np.ones_like(PA)
    S[0][0] = one
    for i in range(imax + 1):
        for j in range(jmax + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                v = PA * S[i - 1][j]
                if i > 1:
                    v = v + (i - 1) * oo2p * S[i - 2][j]
                if j > 0:
                    v = v + j * oo2p * S[i - 1][j - 1]
            else:
                v = PB * S[i][j - 1]
                if j > 1:
                    v = v + (j - 1) * oo2p * S[i][j - 2]
            S[i][j] = v
    return S


def _overlap_kinetic_pair(sa, sb):
    a, b, c, p, P, A, B, K = _prim_pairs(sa, sb)
    la, lb = sa.l, sb.l
    oo2p = 0.5 / p
    pref = c * K * (np.pi / p) ** 1.5
    S1 = [_overlap_1d(la, lb + 2, P[:, x] - A[x], P[:, x] - B[x], oo2p) for x in range(3)]

    def T1(x, i, j):
        t = -2.0 * b * b * S1[x][i][j + 2] + b * (2 * j + 1) * S1[x][i][j]
        if j > 1:
            t = t - 0.5 * j * (j - 1) * S1[x][i][j - 2]
        return t

    ca, cb = _comps(la), _comps(lb)
    S = np.zeros((len(ca), len(cb)))
    T = np.zeros((len(ca), len(cb)))
    for u, ea in enumerate(ca):
        for v, eb in enumerate(cb):
            sx, sy, sz = (S1[x][ea[x]][eb[x]] for x in range(3))
            S[u, v] = np.sum(pref * sx * sy * sz)
            T[u, v] = np.sum(pref * (T1(0, ea[0], eb[0]) * sy * sz + sx * T1(1, ea[1], eb[1]) * sz
                                     + sx * sy * T1(2, ea[2], eb[2])))
    return S, T


def _boys_vec(T, mmax):
    return np.array([oracle.boys(float(t), mmax) for t in T])  # (n, mmax+1)


def _nuclear_pair(sa, sb, charges):
    a, b, c, p, P, A, B, K = _prim_pairs(sa, sb)
    la, lb = sa.l, sb.l
    L = la + lb
    oo2p = 0.5 / p
    PA = P - A
    out = {}
    for Z, C in charges:
        C = np.asarray(C, float)
        PC = P - C
        F = _boys_vec(p * np.sum(PC * PC, axis=1), L)
        base = (-Z) * c * (2.0 * np.pi / p) * K
        memo = {}

        def th(e, m):
            key = (e, m)
            if key in memo:
                return memo[key]
            if e == (0, 0, 0):
                v = base * F[:, m]
            else:
                i = 0 if e[0] else (1 if e[1] else 2)
                em = list(e)
                em[i] -= 1
                em = tuple(em)
                v = PA[:, i] * th(em, m) - PC[:, i] * th(em, m + 1)
                if em[i] > 0:
                    e2 = list(em)
                    e2[i] -= 1
                    e2 = tuple(e2)
                    v = v + em[i] * oo2p * (th(e2, m) - th(e2, m + 1))
            memo[key] = v
            return v

        for l in range(la, L + 1):
            for e in _comps(l):
                out[e] = out.get(e, 0.0) + float(np.sum(th(e, 0)))
    # horizontal transfer on contracted values: (a|b+1_i) = (a+1_i|b) + AB_i (a|b)
    AB = np.asarray(sa.O, float) - np.asarray(sb.O, float)
    hr = {(ea, (0, 0, 0)): out[ea] for l in range(la, L + 1) for ea in _comps(l)}

    def h(ea, eb):
        key = (ea, eb)
        if key in hr:
            return hr[key]
        i = 0 if eb[0] else (1 if eb[1] else 2)
        ebm = list(eb)
        ebm[i] -= 1
        eap = list(ea)
        eap[i] += 1
        v = h(tuple(eap), tuple(ebm)) + AB[i] * h(ea, tuple(ebm))
        hr[key] = v
        return v

    ca, cb = _comps(la), _comps(lb)
    V = np.zeros((len(ca), len(cb)))
    for u, ea in enumerate(ca):
        for v, eb in enumerate(cb):
            V[u, v] = h(ea, eb)
    return V


def _to_sph(M, sa, sb):
    if sa.pure and sa.l > 0:
        M = _sph(sa.l) @ M
    if sb.pure and sb.l > 0:
        M = M @ _sph(sb.l).T
    return M


def one_body(basis, atoms):
    """Overlap S, kinetic T and nuclear attraction V (point nuclei of
    `atoms`, (Z, xyz) in bohr) over a libint_gb300.BasisSet, nbf x nbf."""
    off = basis.shell2bf()
    n = basis.nbf
    S = np.zeros((n, n)); T = np.zeros((n, n)); V = np.zeros((n, n))
    charges = [(float(Z), xyz) for Z, xyz in atoms]
    for i, sa in enumerate(basis):
        for j, sb in enumerate(basis[:i + 1]):
            s, t = _overlap_kinetic_pair(sa, sb)
            v = _nuclear_pair(sa, sb, charges)
            blocks = [_to_sph(x, sa, sb) for x in (s, t, v)]
            ra = slice(off[i], off[i] + sa.size())
            rb = slice(off[j], off[j] + sb.size())
            for M, blk in zip((S, T, V), blocks):
                M[ra, rb] = blk
                M[rb, ra] = blk.T
    return S, T, V


def nuclear_repulsion(atoms):
    e = 0.0
    for i in range(len(atoms)):
        for j in range(i):
            r = math.dist(atoms[i][1], atoms[j][1])
            e += atoms[i][0] * atoms[j][0] / r
    return e


def nuclear_repulsion_gradient(atoms):
    g = np.zeros((len(atoms), 3))
    for i in range(len(atoms)):
        for j in range(len(atoms)):
            if i == j:
                continue
            d = np.subtract(atoms[i][1], atoms[j][1])
            r = np.linalg.norm(d)
            g[i] -= atoms[i][0] * atoms[j][0] * d / r ** 3
    return g
