"""libint_gb300 -- GB300-native Coulomb ERIs with libint2's interface.

Host-side mirror of the reference's Python/C++ interface for the Coulomb
ERI path (python/src/libint2/libint2.cc, include/libint2/engine.h): Shell,
BasisSet, Atom, Operator, BraKet, ScreeningMethod, Engine with
compute(s1, s2, s3, s4) returning libint's buffer order, plus the batched
J/K and gradient passes.  All arithmetic runs in liblgx.so on the GPU.
"""
from __future__ import annotations

import ctypes
import enum
import os
from typing import Iterable, Sequence

import numpy as np

from . import _lgx
from ._lgx import LgxError

__all__ = ["Shell", "BasisSet", "Atom", "Operator", "BraKet", "ScreeningMethod",
           "Engine", "Context", "coulomb", "initialize", "finalize", "water_cluster",
           "LgxError", "MAX_AM", "DATA_PATH"]

MAX_AM = 3
DATA_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis")
BOHR_TO_ANGSTROM = 0.529177210903  # CODATA 2018 (include/libint2/atom.h:52-55)


class Operator(enum.Enum):
    """libint2::Operator (engine.h:98-184): coulomb, and the attenuated
    erf_coulomb / erfc_coulomb (params = omega)."""
    coulomb = 2
    erf_coulomb = 16
    erfc_coulomb = 17

    @staticmethod
    def rank(op) -> int:
        """libint2::rank(Operator) (the binding's Operator.rank): the number
        of electrons the operator couples, 2 for every operator here."""
        return 2


_OP_CODE = {Operator.coulomb: _lgx.LGX_OP_COULOMB, Operator.erf_coulomb: _lgx.LGX_OP_ERF_COULOMB,
            Operator.erfc_coulomb: _lgx.LGX_OP_ERFC_COULOMB}


class BraKet(enum.Enum):
    """libint2::BraKet (engine.h:188-206; binding names XXXX, XSXX, XSXS,
    XXXS): four-centre xx_xx, and the three- and two-centre xs_xx / xs_xs
    that the reference computes with Shell.unit() in the empty positions.
    The binding's XXXS is an alias of the three-centre braket here: libint's
    Engine evaluates every three-shell call as (a unit|c d)
    (engine.impl.h:159-166), and the binding's own test expects that value
    (python/tests/test_libint2.py:40-43)."""
    XXXX = 1
    xx_xx = 1
    XSXX = 3
    xs_xx = 3
    XXXS = 3
    XSXS = 4
    xs_xs = 4


_BRAKET_RANK = {BraKet.xx_xx: 4, BraKet.xs_xx: 3, BraKet.xs_xs: 2}
# derivative sets of the real centres within the 12 four-centre sets
_DERIV_SETS = {4: list(range(12)), 3: [0, 1, 2, 6, 7, 8, 9, 10, 11], 2: [0, 1, 2, 6, 7, 8]}


class ScreeningMethod(enum.IntEnum):
    """libint2::ScreeningMethod (shell.h:1041-1059), primitive screening."""
    Original = 0
    Conservative = 1


def _ncart(l):
    return (l + 1) * (l + 2) // 2


class Shell:
    """libint2::Shell with one contraction.  `primitives` are
    (exponent, coefficient) pairs with coefficients of unit-normalized
    primitives; normalization is embedded on construction (Shell::renorm,
    shell.h:958-999).  Python-binding defaults: center at the origin,
    pure=True (python/src/libint2/libint2.cc:155-160)."""

    def __init__(self, L: int, primitives: Sequence[tuple], center=(0.0, 0.0, 0.0),
                 pure: bool = True, embed_normalization: bool = True):
        self.l = int(L)
        self.alpha = np.ascontiguousarray([float(a) for a, _ in primitives])
        c_in = np.ascontiguousarray([float(c) for _, c in primitives])
        self._coeffs_in = c_in.copy()
        if embed_normalization:
            out = np.zeros_like(c_in)
            _lgx.check(_lgx.load().lgx_shell_normalize(self.l, len(c_in), _lgx.ptr(self.alpha),
                                                        _lgx.ptr(c_in), _lgx.ptr(out)),
                       None, "lgx_shell_normalize")
            self.coeff = out
        else:
            self.coeff = c_in
        self.O = np.asarray(center, dtype=float).reshape(3).copy()
        self.pure = bool(pure)

    @staticmethod
    def do_enforce_unit_normalization(flag=None) -> bool:
        """Shell::do_enforce_unit_normalization (shell.h:891-901): reports,
        or sets when flag is given, whether new shells (and basis sets) have
        their contractions rescaled to unit self-overlap; process-wide."""
        return bool(_lgx.load().lgx_enforce_unit_normalization(-1 if flag is None else int(bool(flag))))

    @classmethod
    def unit(cls):
        """Shell::unit() (shell.h:904-914): exponent 0, coefficient 1, at the
        origin; the placeholder of the 3- and 2-centre brakets."""
        return cls.from_normalized(0, [0.0], [1.0], (0.0, 0.0, 0.0), False)

    @classmethod
    def from_normalized(cls, L, alpha, coeff, center, pure):
        s = cls.__new__(cls)
        s.l = int(L)
        s.alpha = np.ascontiguousarray(alpha, dtype=float)
        s.coeff = np.ascontiguousarray(coeff, dtype=float)
        s._coeffs_in = None
        s.O = np.asarray(center, dtype=float).reshape(3).copy()
        s.pure = bool(pure)
        return s

    def size(self) -> int:
        return 2 * self.l + 1 if self.pure else _ncart(self.l)

    def nprim(self) -> int:
        return len(self.alpha)

    @property
    def coeffs(self):
        return list(self.coeff)

    @property
    def coeffs_normalized(self):
        """Coefficients of unit-normalized primitives (Shell::coeff_normalized,
        shell.h:915-928): the embedded coefficients times the inverse
        primitive normalization sqrt(pi^{3/2} (2l-1)!! / (2^l (2a)^{l+3/2}));
        a zero exponent (the unit shell) keeps its coefficient."""
        l = self.l
        dfact = float(np.prod(np.arange(2 * l - 1, 0, -2))) if l > 0 else 1.0
        a2 = 2.0 * self.alpha
        out = self.coeff.copy()
        nz = a2 > 0
        out[nz] = self.coeff[nz] * np.sqrt(np.pi ** 1.5 * dfact / (2.0 ** l * a2[nz] ** (l + 1.5)))
        return list(out)

    def move(self, center):
        self.O = np.asarray(center, dtype=float).reshape(3).copy()
        return self

    def _c(self) -> _lgx.LgxShell:
        r = _lgx.LgxShell()
        r.l = self.l
        r.pure = 1 if self.pure else 0
        r.nprim = len(self.alpha)
        for x in range(3):
            r.origin[x] = self.O[x]
        r.alpha = _lgx.ptr(self.alpha)
        r.coeff = _lgx.ptr(self.coeff)
        return r

    def __repr__(self):
        return "Shell(l=%d, pure=%s, nprim=%d, O=%s)" % (self.l, self.pure, self.nprim(),
                                                         list(self.O))


class Atom(tuple):
    """(Z, [x, y, z]) in bohr, like libint2::Atom."""

    def __new__(cls, Z, xyz):
        return super().__new__(cls, (int(Z), tuple(float(v) for v in xyz)))


class BasisSet(list):
    """libint2::BasisSet: shells on atoms from a G94 library file
    (basis.h.in:134-182, read_g94_basis_library :473-621)."""

    def __init__(self, name_or_shells, atoms=None, data_path: str | None = None):
        if atoms is None:
            super().__init__(name_or_shells)
            self.name = None
            self.atom_of_shell = [0] * len(self)
            return
        super().__init__()
        self.name = name_or_shells
        Z = np.ascontiguousarray([int(a[0]) for a in atoms], dtype=np.int32)
        xyz = np.ascontiguousarray([list(a[1]) for a in atoms], dtype=float).reshape(-1)
        lib = _lgx.load()
        ns, np_ = ctypes.c_int(0), ctypes.c_int(0)
        dpath = (data_path or os.environ.get("LIBINT_DATA_PATH") or DATA_PATH).encode()
        st = lib.lgx_basis_load(dpath, self.name.encode(), len(Z), _lgx.ptr(Z, ctypes.c_int32),
                                _lgx.ptr(xyz), ctypes.byref(ns), ctypes.byref(np_),
                                None, None, None, None, None, None, None)
        _lgx.check(st, None, "lgx_basis_load(%s)" % self.name)
        n, m = ns.value, np_.value
        l = np.zeros(n, np.int32); pure = np.zeros(n, np.int32); nprim = np.zeros(n, np.int32)
        atom = np.zeros(n, np.int32); O = np.zeros(3 * n); alpha = np.zeros(m); coeff = np.zeros(m)
        I = ctypes.c_int32
        st = lib.lgx_basis_load(dpath, self.name.encode(), len(Z), _lgx.ptr(Z, I), _lgx.ptr(xyz),
                                ctypes.byref(ns), ctypes.byref(np_), _lgx.ptr(l, I),
                                _lgx.ptr(pure, I), _lgx.ptr(nprim, I), _lgx.ptr(atom, I),
                                _lgx.ptr(O), _lgx.ptr(alpha), _lgx.ptr(coeff))
        _lgx.check(st, None, "lgx_basis_load(%s)" % self.name)
        off = 0
        for s in range(n):
            k = int(nprim[s])
            self.append(Shell.from_normalized(int(l[s]), alpha[off:off + k], coeff[off:off + k],
                                              O[3 * s:3 * s + 3], bool(pure[s])))
            off += k
        self.atom_of_shell = [int(a) for a in atom]

    # flattened views used by the C ABI and the oracle
    @property
    def l(self):
        return np.array([s.l for s in self], np.int32)

    @property
    def pure(self):
        return np.array([1 if s.pure else 0 for s in self], np.int32)

    @pure.setter
    def pure(self, flag):
        for s in self:
            s.pure = bool(flag)

    @property
    def nprim(self):
        return np.array([s.nprim() for s in self], np.int32)

    @property
    def origins(self):
        return np.concatenate([s.O for s in self]) if len(self) else np.zeros(0)

    @property
    def alpha(self):
        return np.concatenate([s.alpha for s in self]) if len(self) else np.zeros(0)

    @property
    def coeff(self):
        return np.concatenate([s.coeff for s in self]) if len(self) else np.zeros(0)

    @property
    def atom(self):
        return np.array(self.atom_of_shell, np.int32)

    @property
    def nbf(self) -> int:
        return int(sum(s.size() for s in self))

    def shell2bf(self):
        out, o = [], 0
        for s in self:
            out.append(o)
            o += s.size()
        return out

    functions = property(shell2bf)

    def max_nprim(self):
        return max(s.nprim() for s in self)

    def max_l(self):
        return max(s.l for s in self)


def water_cluster(nx, ny, nz, spacing=3.0, jitter=0.2, seed=0):
    """(H2O)_{nx*ny*nz} on a grid (angstrom spacing, uniform jitter), random
    orientations, 0.96 A / 104.5 deg; atoms in bohr as [(Z, (x, y, z))]."""
    n = nx * ny * nz
    Z = np.zeros(3 * n, np.int32)
    xyz = np.zeros(9 * n)
    _lgx.check(_lgx.load().lgx_water_cluster(nx, ny, nz, spacing, jitter, seed,
                                             _lgx.ptr(Z, ctypes.c_int32), _lgx.ptr(xyz)),
               None, "lgx_water_cluster")
    return [Atom(int(Z[i]), xyz[3 * i:3 * i + 3]) for i in range(3 * n)]


class Context:
    """One GPU context (lgx_context): basis state, batched and J/K passes."""

    def __init__(self, device: int = 0):
        self._lib = _lgx.load()
        h = ctypes.c_void_p()
        st = self._lib.lgx_create(ctypes.byref(h), int(device))
        if st != _lgx.LGX_OK:
            raise LgxError(st, "lgx_create failed (no usable sm_100+ CUDA device?)")
        self._h = h
        self.basis = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lgx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        _lgx.check(st, self._h, what)

    def set_operator(self, oper: Operator = Operator.coulomb, omega: float = 0.0):
        """Operator of every later call (lgx_set_operator): coulomb, or
        erf_coulomb / erfc_coulomb with range-separation parameter omega."""
        self._check(self._lib.lgx_set_operator(self._h, _OP_CODE[Operator(oper)], float(omega)),
                    "lgx_set_operator")

    def boys(self, T, mmax: int, variant: int = 0):
        """F_0..F_mmax(T) for an array of T from the device evaluator
        `variant` (lgx_boys: 0/1 FP64 program/register kernel, 2/3 FP32,
        4/5 FP64 rounded to FP32; 6: T is an (n, 8) array of pair data
        Pb.xyz, zeta, Pk.xyz, eta, the mixed register kernels' whole path)."""
        T = np.ascontiguousarray(T, np.float64)
        n = T.shape[0] if int(variant) == 6 else T.size
        T = T.reshape(-1)
        F = np.zeros((n, int(mmax) + 1))
        self._check(self._lib.lgx_boys(self._h, int(variant), _lgx.ptr(T), n, int(mmax),
                                       _lgx.ptr(F)), "lgx_boys")
        return F

    def set_fock_precision(self, precision: float = 0.0):
        """Density-weighted screening of later J/K passes (lgx_set_fock_precision):
        skip quartets with Dnorm1234 K12 K34 < precision and screen the
        primitives of the rest at precision / Dnorm1234, as the reference's
        compute_2body_fock does; 0 turns it off."""
        self._check(self._lib.lgx_set_fock_precision(self._h, float(precision)),
                    "lgx_set_fock_precision")

    def set_watchdog(self, max_chunks: int = -1):
        """Bound on the work chunks a program-kernel warp may take per launch
        before the call fails with LGX_ERR_WATCHDOG (lgx_set_watchdog);
        a negative value restores the default bound derived from each
        launch's work, 0 trips on any program-kernel launch with work."""
        self._check(self._lib.lgx_set_watchdog(self._h, int(max_chunks)), "lgx_set_watchdog")

    # ------------------------------------------------------------ engine
    def compute_shellset(self, shells, deriv=0, precision=np.finfo(float).eps,
                         screening=ScreeningMethod.Original, pair_ln_prec=None):
        """One shell set (list of nsets arrays, or None when fully screened).
        pair_ln_prec: None, or (bra, ket) ln_prec of caller-precomputed
        ShellPair data (lgx_compute_shellset_pairs; deriv 0 or 1)."""
        arr = (_lgx.LgxShell * 4)(*[s._c() for s in shells])
        nsets = {0: 1, 1: 12, 2: 78}[int(deriv)]
        nv = int(np.prod([s.size() for s in shells]))
        out = np.zeros(nsets * nv)
        ns, nvals, isnull = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        if pair_ln_prec is None:
            st = self._lib.lgx_compute_shellset(self._h, arr, int(deriv), float(precision),
                                                int(screening), _lgx.ptr(out), out.size,
                                                ctypes.byref(ns), ctypes.byref(nvals),
                                                ctypes.byref(isnull))
        else:
            pl = np.asarray(pair_ln_prec, dtype=np.float64).reshape(2)
            st = self._lib.lgx_compute_shellset_pairs(self._h, arr, int(deriv), float(precision),
                                                      int(screening), _lgx.ptr(pl),
                                                      _lgx.ptr(out), out.size, ctypes.byref(ns),
                                                      ctypes.byref(nvals), ctypes.byref(isnull))
        self._check(st, "lgx_compute_shellset")
        if isnull.value:
            return None
        shape = tuple(s.size() for s in shells)
        return [out[i * nv:(i + 1) * nv].reshape(shape) for i in range(ns.value)]

    def compute_primitive_set(self, ls, prims, AB, CD, deriv=0):
        """Contracted Cartesian shell set(s) (l1 l2|l3 l4) from caller-computed
        primitive quartets (libint2_build_eri / _eri1 / _eri2 with Libint_t
        prefactors): `prims` is an array of dtype PRIM_DTYPE, AB = A - B,
        CD = C - D.  Returns the 1 / 12 / 78 sets in the caller's shell
        order, each shaped (ncart(l1), ncart(l2), ncart(l3), ncart(l4))."""
        ls = [int(x) for x in ls]
        prims = np.ascontiguousarray(prims, dtype=_lgx.PRIM_DTYPE)
        nsets = {0: 1, 1: 12, 2: 78}[int(deriv)]
        shape = tuple((l + 1) * (l + 2) // 2 for l in ls)
        nv = int(np.prod(shape))
        out = np.zeros(nsets * nv)
        AB = np.ascontiguousarray(AB, dtype=float)
        CD = np.ascontiguousarray(CD, dtype=float)
        ns, nvals = ctypes.c_int(), ctypes.c_int()
        st = self._lib.lgx_compute_primitive_set(
            self._h, ls[0], ls[1], ls[2], ls[3], int(deriv),
            prims.ctypes.data_as(ctypes.POINTER(_lgx.LgxPrimQuartet)), len(prims),
            _lgx.ptr(AB), _lgx.ptr(CD), _lgx.ptr(out), out.size, ctypes.byref(ns),
            ctypes.byref(nvals))
        self._check(st, "lgx_compute_primitive_set")
        return [out[i * nv:(i + 1) * nv].reshape(shape) for i in range(ns.value)]

    # ------------------------------------------------------------- basis
    def set_basis(self, basis: BasisSet):
        I = ctypes.c_int32
        self._arrs = (basis.l, basis.pure, basis.nprim, basis.atom, basis.origins,
                      basis.alpha, basis.coeff)
        l, pure, nprim, atom, O, alpha, coeff = self._arrs
        st = self._lib.lgx_set_basis(self._h, len(basis), _lgx.ptr(l, I), _lgx.ptr(pure, I),
                                     _lgx.ptr(nprim, I), _lgx.ptr(atom, I), _lgx.ptr(O),
                                     _lgx.ptr(alpha), _lgx.ptr(coeff))
        self._check(st, "lgx_set_basis")
        self.basis = basis

    def set_pair_subset(self, pairs=None):
        """Restrict later J/K and gradient passes to quartets whose bra and ket
        shell pairs both come from `pairs` (n x 2 shell indices);
        None or an empty list lifts the restriction (lgx_set_pair_subset)."""
        p = np.ascontiguousarray(np.zeros((0, 2)) if pairs is None else pairs,
                                 np.int32).reshape(-1, 2)
        self._check(self._lib.lgx_set_pair_subset(self._h, _lgx.ptr(p, ctypes.c_int32),
                                                  len(p)), "lgx_set_pair_subset")

    def schwarz(self):
        n = len(self.basis)
        K = np.zeros((n, n))
        self._check(self._lib.lgx_schwarz(self._h, _lgx.ptr(K)), "lgx_schwarz")
        return K

    def compute_batch(self, quartets, deriv=0, mode=_lgx.LGX_FP64, mixed_thresh=1e-4):
        q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
        if q.size and (q.min() < 0 or q.max() >= len(self.basis)):
            raise LgxError(_lgx.LGX_ERR_INVALID_ARG, "quartet shell index out of range")
        sizes = np.array([s.size() for s in self.basis], np.int64)
        nv = sizes[q[:, 0]] * sizes[q[:, 1]] * sizes[q[:, 2]] * sizes[q[:, 3]] * (12 if deriv else 1)
        offs = np.zeros(len(q), np.int64)
        if len(q):
            offs[1:] = np.cumsum(nv)[:-1]
        out = np.zeros(int(nv.sum()) if len(q) else 1)
        isnull = np.zeros(max(len(q), 1), np.int32)
        st = self._lib.lgx_compute_batch(self._h, _lgx.ptr(q, ctypes.c_int32), len(q), int(deriv),
                                         int(mode), float(mixed_thresh),
                                         _lgx.ptr(offs, ctypes.c_int64), _lgx.ptr(out),
                                         out.size, _lgx.ptr(isnull, ctypes.c_int32))
        self._check(st, "lgx_compute_batch")
        return out, offs, isnull[:len(q)]

    def compute_batch_device(self, quartets, d_out, out_capacity, deriv=0, mode=_lgx.LGX_FP64,
                             mixed_thresh=1e-4, offsets=None, d_is_null=0):
        """compute_batch with the sets left in device memory: d_out is the
        address of out_capacity doubles on the context's GPU (e.g. a torch
        tensor's data_ptr()), d_is_null optionally that of len(quartets)
        int32.  Returns the offsets (computed as in compute_batch when not
        given)."""
        q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
        if q.size and (q.min() < 0 or q.max() >= len(self.basis)):
            raise LgxError(_lgx.LGX_ERR_INVALID_ARG, "quartet shell index out of range")
        if offsets is None:
            sizes = np.array([s.size() for s in self.basis], np.int64)
            nv = (sizes[q[:, 0]] * sizes[q[:, 1]] * sizes[q[:, 2]] * sizes[q[:, 3]] *
                  (12 if deriv else 1))
            offsets = np.zeros(len(q), np.int64)
            if len(q):
                offsets[1:] = np.cumsum(nv)[:-1]
        offsets = np.ascontiguousarray(offsets, np.int64)
        st = self._lib.lgx_compute_batch_device(self._h, _lgx.ptr(q, ctypes.c_int32), len(q),
                                                int(deriv), int(mode), float(mixed_thresh),
                                                _lgx.ptr(offsets, ctypes.c_int64),
                                                ctypes.c_void_p(int(d_out)), int(out_capacity),
                                                ctypes.c_void_p(int(d_is_null) or None))
        self._check(st, "lgx_compute_batch_device")
        return offsets

    def jk(self, D, schwarz_thresh=1e-12, mode=_lgx.LGX_FP64, mixed_thresh=1e-4):
        n = self.basis.nbf
        D = np.ascontiguousarray(D, dtype=float)
        J = np.zeros((n, n)); K = np.zeros((n, n))
        stats = _lgx.LgxJkStats()
        st = self._lib.lgx_jk(self._h, _lgx.ptr(D), _lgx.ptr(J), _lgx.ptr(K),
                              float(schwarz_thresh), int(mode), float(mixed_thresh),
                              ctypes.byref(stats))
        self._check(st, "lgx_jk")
        return J, K, stats

    def jk_device(self, dD, dJ, dK, schwarz_thresh=1e-12, mode=_lgx.LGX_FP64,
                  mixed_thresh=1e-4):
        """D/J/K given as device pointers (ints), e.g. torch tensor data_ptr()."""
        stats = _lgx.LgxJkStats()
        st = self._lib.lgx_jk_device(self._h, ctypes.c_void_p(dD), ctypes.c_void_p(dJ),
                                     ctypes.c_void_p(dK), float(schwarz_thresh), int(mode),
                                     float(mixed_thresh), ctypes.byref(stats))
        self._check(st, "lgx_jk_device")
        return stats

    def jk_device_noalloc(self, dD, dJ, dK, schwarz_thresh=1e-12, mode=_lgx.LGX_FP64,
                          mixed_thresh=1e-4):
        """jk_device without device allocation during the call (see
        lgx_jk_device_noalloc in include/lgx.h for the limits and the
        preparation it needs)."""
        stats = _lgx.LgxJkStats()
        st = self._lib.lgx_jk_device_noalloc(self._h, ctypes.c_void_p(dD), ctypes.c_void_p(dJ),
                                             ctypes.c_void_p(dK), float(schwarz_thresh),
                                             int(mode), float(mixed_thresh), ctypes.byref(stats))
        self._check(st, "lgx_jk_device_noalloc")
        return stats

    def jk_grad(self, D, natoms=None, schwarz_thresh=1e-12):
        if natoms is None:
            natoms = int(max(self.basis.atom_of_shell)) + 1
        D = np.ascontiguousarray(D, dtype=float)
        gJ = np.zeros((natoms, 3)); gK = np.zeros((natoms, 3))
        stats = _lgx.LgxJkStats()
        st = self._lib.lgx_jk_grad(self._h, _lgx.ptr(D), _lgx.ptr(gJ), _lgx.ptr(gK),
                                   int(natoms), float(schwarz_thresh), ctypes.byref(stats))
        self._check(st, "lgx_jk_grad")
        return gJ, gK, stats

    _KERNELS = {0: "register", 1: "program", 2: "program+generated-post"}

    def last_pass_launches(self):
        """Per-launch records of the last J/K or gradient pass (launch
        order): class, precision, kernel, quartets, primitive quartets,
        algorithmic FLOPs and device time (ms) of each class launch."""
        n = ctypes.c_int()
        self._check(self._lib.lgx_last_pass_launches(self._h, None, 0, ctypes.byref(n)),
                    "lgx_last_pass_launches")
        arr = (_lgx.LgxLaunchStats * max(1, n.value))()
        self._check(self._lib.lgx_last_pass_launches(self._h, arr, n.value, ctypes.byref(n)),
                    "lgx_last_pass_launches")
        out = []
        for r in arr[:n.value]:
            out.append({"class": (r.la, r.lb, r.lc, r.ld), "fp32": bool(r.fp32),
                        "kernel": self._KERNELS.get(r.kernel, str(r.kernel)), "shape": r.shape,
                        "deriv": r.deriv, "quartets": r.quartets,
                        "prim_quartets": r.prim_quartets, "integrals": r.integrals,
                        "flops": r.flops, "flops_fp64": r.flops_fp64, "ms": r.ms})
        return out


_DEFAULT_CTX = None


def _default_context() -> Context:
    global _DEFAULT_CTX
    if _DEFAULT_CTX is None:
        _DEFAULT_CTX = Context(0)
    return _DEFAULT_CTX


def initialize(device: int = 0):
    """libint2::initialize() (initialize.h:76-95): creates the GPU context."""
    global _DEFAULT_CTX
    if _DEFAULT_CTX is None:
        _DEFAULT_CTX = Context(device)


def finalize():
    global _DEFAULT_CTX
    if _DEFAULT_CTX is not None:
        _DEFAULT_CTX.close()
        _DEFAULT_CTX = None


class Engine:
    """libint2::Engine for Operator.coulomb / BraKet.xx_xx (engine.h:444-1064).

    compute(s1, s2, s3, s4) returns the shell set in libint's buffer order
    (row-major, caller's shell order), or None when every primitive quartet
    was screened out; results() holds the last nshellsets() sets.
    """

    def __init__(self, oper: Operator = Operator.coulomb, max_nprim: int = 10,
                 max_l: int = MAX_AM, deriv_order: int = 0,
                 precision: float = float(np.finfo(float).eps), braket=None,
                 screening: ScreeningMethod = ScreeningMethod.Original,
                 context: Context | None = None):
        if oper not in _OP_CODE:
            raise NotImplementedError("only Operator coulomb, erf_coulomb, erfc_coulomb")
        if braket not in (None, BraKet.xx_xx, BraKet.xs_xx, BraKet.xs_xs):
            raise NotImplementedError("only BraKet xx_xx, xs_xx and xs_xs are implemented")
        if max_l > MAX_AM:
            raise LgxError(_lgx.LGX_ERR_LMAX_EXCEEDED, "max_l exceeds LGX_MAX_L")
        if deriv_order not in (0, 1, 2):
            raise NotImplementedError("deriv_order must be 0, 1 or 2")
        if deriv_order == 2 and braket not in (None, BraKet.xx_xx):
            raise NotImplementedError("deriv_order 2 is implemented for BraKet.xx_xx")
        self.oper = oper
        self.braket = braket or BraKet.xx_xx
        self.max_nprim = max_nprim
        self.max_l = max_l
        self.deriv_order = deriv_order
        self.screening = screening
        self.set_precision(precision)
        self._ctx = context
        self._results = [None]
        self._omega = 0.0

    def set_params(self, omega: float):
        """Engine::set_params: omega of erf_coulomb / erfc_coulomb."""
        if not omega >= 0:
            raise ValueError("omega must be >= 0")
        self._omega = float(omega)
        return self

    def set_precision(self, prec: float):
        self._precision = max(float(prec), 0.0)
        return self

    def precision(self):
        return self._precision

    def set(self, screening: ScreeningMethod):
        self.screening = ScreeningMethod(screening)
        return self

    def braket_rank(self):
        return _BRAKET_RANK[self.braket]

    def nshellsets(self):
        if self.deriv_order == 2:
            return 78
        return 3 * self.braket_rank() if self.deriv_order else 1

    def results(self):
        return self._results

    def compute(self, *shells):
        """compute(s1, s2, s3, s4) for xx_xx, (s1, s2, s3) for xs_xx,
        (s1, s2) for xs_xs (the binding's compute2/3/4, engine.cc:165-202);
        arrays shaped by the given shells, None when screened out."""
        rank = self.braket_rank()
        if len(shells) != rank:
            raise ValueError("compute: %s takes %d shells" % (self.braket.name, rank))
        if all(isinstance(s, (BasisSet, list)) for s in shells):
            return self._compute_basis(*shells)
        for s in shells:
            if s.l > self.max_l:
                raise LgxError(_lgx.LGX_ERR_LMAX_EXCEEDED, "lmax_exceeded")
        full = list(shells)
        if rank == 3:
            full = [shells[0], Shell.unit(), shells[1], shells[2]]
        elif rank == 2:
            full = [shells[0], Shell.unit(), shells[1], Shell.unit()]
        ctx = self._ctx or _default_context()
        ctx.set_operator(self.oper, self._omega)  # contexts are shared between engines
        r = ctx.compute_shellset(full, self.deriv_order, self._precision, self.screening)
        if r is not None:
            shape = tuple(s.size() for s in shells)
            sel = [0] if self.deriv_order == 0 else (
                _DERIV_SETS[rank] if self.deriv_order == 1 else range(78))
            r = [r[i].reshape(shape) for i in sel]
        self._results = r if r is not None else [None] * self.nshellsets()
        if r is None:
            return None
        return r[0] if self.deriv_order == 0 else r

    def compute_2body_fock(self, D, basis):
        """The binding's Engine.compute_2body_fock(D, basis)
        (python/src/libint2/engine.cc:230-279): the closed-shell two-body
        Fock matrix G = 2J - K of density D over `basis` (J_ab = sum_cd
        (ab|cd) D_cd, K_ab = sum_cd (ac|bd) D_cd, which is what the binding's
        quartet loop accumulates), for this engine's operator and omega,
        from one J/K pass on the GPU with every quartet (no Schwarz
        screening, as the binding's loop)."""
        if self.braket != BraKet.xx_xx or self.deriv_order != 0:
            raise NotImplementedError("compute_2body_fock: BraKet.xx_xx and deriv_order 0")
        bs = basis if isinstance(basis, BasisSet) else BasisSet(list(basis))
        ctx = self._ctx or _default_context()
        ctx.set_operator(self.oper, self._omega)
        ctx.set_basis(bs)
        J, K, _ = ctx.jk(np.asarray(D, dtype=float), 0.0)
        return 2.0 * J - K

    def _compute_basis(self, *bases):
        """The binding's compute over basis sets (parallel_compute,
        engine.cc:146-157): the full array (nbf of each argument), block by
        block from the shell sets (first set for derivatives); screened-out
        blocks are zero."""
        import itertools
        nb = [sum(s.size() for s in X) for X in bases]
        out = np.zeros(nb)
        offs = [np.cumsum([0] + [s.size() for s in X]) for X in bases]
        for idx in itertools.product(*[range(len(X)) for X in bases]):
            r = self.compute(*[X[i] for X, i in zip(bases, idx)])
            if r is None:
                continue
            blk = r if self.deriv_order == 0 else r[0]
            out[tuple(slice(offs[k][i], offs[k][i + 1]) for k, i in enumerate(idx))] = blk
        return out


class SolidHarmonicsCoefficients:
    """libint2.SolidHarmonicsCoefficients of the binding (libint2.cc:255-261):
    coefficient(l, m, lx, ly, lz) of the Cartesian component x^lx y^ly z^lz
    in the real solid harmonic (l, m) (solidharmonics.h:114-174), the set
    the kernels' transform uses (lgx_solid_coeff)."""

    @staticmethod
    def coefficient(l, m, lx, ly, lz) -> float:
        return float(_lgx.load().lgx_solid_coeff(int(l), int(m), int(lx), int(ly), int(lz)))


def coulomb() -> Engine:
    """The reference binding's coulomb() factory: precision 1e-15
    (python/src/libint2/libint2.cc:50-55)."""
    return Engine(Operator.coulomb, precision=1e-15)


def random_density(nbf: int, nocc: int, seed: int = 0) -> np.ndarray:
    """Synthetic symmetric positive semidefinite density D = C C^T, C of shape
    nbf x nocc with entries N(0, 1)/sqrt(nbf) from numpy's default_rng(seed)."""
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((nbf, nocc)) / np.sqrt(nbf)
    return C @ C.T


def jk_energies(D, J, K):
    """E_J = 1/2 sum D.J and E_K = -1/4 sum D.K."""
    return 0.5 * float(np.sum(D * J)), -0.25 * float(np.sum(D * K))
