"""Closed-shell Hartree-Fock driver for the system-level check of the J/K
path.

TEST INFRASTRUCTURE ONLY: restates the SCF of the reference's
tests/hartree-fock/hartree-fock++.cc (main, :209-520): core-Hamiltonian
guess, density D = C_occ C_occ^T, Fock matrix F = H + G with G = 2J - K
(compute_2body_fock, :1574-1772), energy E = sum D (H + F) + E_nuc (:478),
DIIS on the commutator FDS - SDF (libint2/diis.h), converged when the
energy change and the commutator are both below `conv` (:411-515).  The
J/K builder is a callable, so the same driver runs on the GPU path
(libint_gb300.Context.jk) and on the CPU oracle.
"""
from __future__ import annotations

import numpy as np


def rhf(S, H, nocc, jk, enuc=0.0, conv=1e-12, maxiter=100, ndiis=8):
    """Returns (E_total, D, C, orbital energies, iterations).  jk(D) -> (J, K)."""
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T

    def diag(F):
        e, Ct = np.linalg.eigh(X.T @ F @ X)
        C = X @ Ct
        return e, C

    eps, C = diag(H)
    D = C[:, :nocc] @ C[:, :nocc].T
    E = 0.0
    errs, focks = [], []
    for it in range(1, maxiter + 1):
        J, K = jk(D)
        F = H + 2.0 * J - K
        E_last, E = E, float(np.sum(D * (H + F)))
        err = F @ D @ S - S @ D @ F
        rms = float(np.sqrt(np.mean(err * err)))
        if it > 1 and abs(E - E_last) < conv and rms < conv:
            return E + enuc, D, C, eps, it
        errs.append(err)
        focks.append(F)
        errs, focks = errs[-ndiis:], focks[-ndiis:]
        Fx = F
        if len(errs) > 1:
            n = len(errs)
            B = -np.ones((n + 1, n + 1))
            B[n, n] = 0.0
            for i in range(n):
                for j in range(n):
                    B[i, j] = np.sum(errs[i] * errs[j])
            rhs = np.zeros(n + 1)
            rhs[n] = -1.0
            c = np.linalg.lstsq(B, rhs, rcond=None)[0][:n]
            Fx = sum(ci * Fi for ci, Fi in zip(c, focks))
        eps, C = diag(Fx)
        D = C[:, :nocc] @ C[:, :nocc].T
    raise RuntimeError("SCF did not converge in %d iterations (rms %.2e)" % (maxiter, rms))


def rhf_plain(S, H, nocc, jk, enuc=0.0, iterations=30, tol=1e-6):
    """The undamped SCF of the reference's python/tests/test_hf.py:53-100
    (RHF.converge): generalized eigenproblem F C = S C e, no DIIS, energy
    sum D_new (H + F) after each diagonalization, stop when it changes by
    less than `tol`.  Its energy is only converged to about `tol`, so this
    restatement (same guess, same steps) is what reproduces that test's
    golden value to its 7 decimals."""
    import scipy.linalg

    def density(F):
        _, C = scipy.linalg.eigh(F, S)
        return C[:, :nocc] @ C[:, :nocc].T

    D = density(H)
    ehf = None
    for _ in range(iterations):
        J, K = jk(D)
        F = H + 2.0 * J - K
        prev = ehf or 0.0
        D = density(F)
        ehf = float(np.sum(D * (H + F)))
        if abs(prev - ehf) < tol:
            break
    return enuc + ehf
