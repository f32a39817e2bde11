"""ctypes wrapper of the FP64 CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's cpu_baseline / ``--impl reference`` arm, always as the checker
or the timed CPU baseline.  The product package never imports it.

The oracle restates libint's ``Engine::compute2<coulomb, xx_xx, d>`` (see
oracle/oracle.h for the file:line anchors into the libint tree).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(_HERE, "_ref", "libref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile oracle/oracle.cpp into oracle/liboracle.so (gcc, OpenMP)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call(["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC",
                           "-shared", src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref(reference_root: str | None = None) -> str | None:
    """Compile the reference's own headers into oracle/_ref/libref.so when the
    reference tree is present (development container only).  The tree is
    `reference_root`, else $LGX_REFERENCE_ROOT, else the default location
    that oracle/ref/build_ref.sh knows; the recipe skips quietly when the
    tree is absent (as on a GPU machine)."""
    root = reference_root or os.environ.get("LGX_REFERENCE_ROOT")
    cmd = ["bash", os.path.join(_HERE, "ref", "build_ref.sh")] + ([root] if root else [])
    subprocess.check_call(cmd)
    return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None


class _Basis(ctypes.Structure):
    _fields_ = [("nshell", ctypes.c_int), ("l", _ip), ("pure", _ip),
                ("nprim", _ip), ("prim_off", _ip), ("atom", _ip),
                ("O", _dp), ("alpha", _dp), ("coeff", _dp)]


def _lib():
    global _LIB
    try:
        return _LIB
    except NameError:
        pass
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.orc_boys.argtypes = [ctypes.c_double, ctypes.c_int, _dp]
    lib.orc_solid_coeff.restype = ctypes.c_double
    lib.orc_solid_coeff.argtypes = [ctypes.c_int] * 5
    lib.orc_compute_quartet.restype = ctypes.c_int
    lib.orc_jk.restype = ctypes.c_int64
    lib.orc_jk_sample.restype = ctypes.c_int64
    lib.orc_jk_grad.restype = ctypes.c_int64
    _LIB = lib
    return lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


class OracleBasis:
    """Flattened basis (shell arrays) handed to the oracle."""

    def __init__(self, l, pure, nprim, origins, alpha, coeff, atom=None):
        self.l = np.ascontiguousarray(l, dtype=np.int32)
        self.pure = np.ascontiguousarray(pure, dtype=np.int32)
        self.nprim = np.ascontiguousarray(nprim, dtype=np.int32)
        self.O = np.ascontiguousarray(origins, dtype=np.float64).reshape(-1)
        self.alpha = np.ascontiguousarray(alpha, dtype=np.float64)
        self.coeff = np.ascontiguousarray(coeff, dtype=np.float64)
        n = len(self.l)
        self.atom = (np.zeros(n, np.int32) if atom is None else
                     np.ascontiguousarray(atom, dtype=np.int32))
        self.prim_off = np.zeros(n, np.int32)
        if n:
            self.prim_off[1:] = np.cumsum(self.nprim)[:-1]
        self.nfunc = np.where(self.pure == 1, 2 * self.l + 1,
                              (self.l + 1) * (self.l + 2) // 2).astype(np.int32)
        self.bf_off = np.zeros(n, np.int32)
        if n:
            self.bf_off[1:] = np.cumsum(self.nfunc)[:-1]
        self.nbf = int(self.nfunc.sum())
        self._c = _Basis(n, _ptr(self.l, ctypes.c_int), _ptr(self.pure, ctypes.c_int),
                         _ptr(self.nprim, ctypes.c_int), _ptr(self.prim_off, ctypes.c_int),
                         _ptr(self.atom, ctypes.c_int), _ptr(self.O, ctypes.c_double),
                         _ptr(self.alpha, ctypes.c_double), _ptr(self.coeff, ctypes.c_double))

    @classmethod
    def from_basis(cls, bs):
        """From any object exposing the flattened arrays of libint_gb300.BasisSet."""
        return cls(bs.l, bs.pure, bs.nprim, bs.origins, bs.alpha, bs.coeff, bs.atom)

    @property
    def nshell(self):
        return len(self.l)


def boys(T: float, mmax: int) -> np.ndarray:
    F = np.zeros(mmax + 1)
    _lib().orc_boys(float(T), int(mmax), _ptr(F, ctypes.c_double))
    return F


OP_COULOMB, OP_ERF_COULOMB, OP_ERFC_COULOMB = 0, 1, 2


def set_operator(op: int = OP_COULOMB, omega: float = 0.0):
    """Operator of every later oracle call (process-wide): coulomb, or
    erf/erfc(omega r)/r with libint's core integrals."""
    lib = _lib()
    lib.orc_set_operator.argtypes = [ctypes.c_int, ctypes.c_double]
    lib.orc_set_operator.restype = ctypes.c_int
    if lib.orc_set_operator(int(op), float(omega)) != 0:
        raise ValueError("oracle: bad operator")


def solid_coeff(l, m, lx, ly, lz) -> float:
    return _lib().orc_solid_coeff(l, m, lx, ly, lz)


def shell_normalize(l, alpha, coeff):
    alpha = np.ascontiguousarray(alpha, np.float64)
    coeff = np.ascontiguousarray(coeff, np.float64)
    out = np.zeros_like(coeff)
    mln = np.zeros_like(coeff)
    _lib().orc_shell_normalize(ctypes.c_int(l), ctypes.c_int(len(alpha)),
                               _ptr(alpha, ctypes.c_double), _ptr(coeff, ctypes.c_double),
                               _ptr(out, ctypes.c_double), _ptr(mln, ctypes.c_double))
    return out, mln


def shellpair_init(l1, a1, c1, O1, l2, a2, c2, O2, ln_prec, method=0):
    a1 = np.ascontiguousarray(a1, np.float64); c1 = np.ascontiguousarray(c1, np.float64)
    a2 = np.ascontiguousarray(a2, np.float64); c2 = np.ascontiguousarray(c2, np.float64)
    O1 = np.ascontiguousarray(O1, np.float64); O2 = np.ascontiguousarray(O2, np.float64)
    n = len(a1) * len(a2)
    P = np.zeros(3 * n); K = np.zeros(n); oog = np.zeros(n); ns = np.zeros(n); ls = np.zeros(n)
    p1 = np.zeros(n, np.int32); p2 = np.zeros(n, np.int32)
    d = ctypes.c_double
    cnt = _lib().orc_shellpair_init(
        l1, len(a1), _ptr(a1, d), _ptr(c1, d), _ptr(O1, d), l2, len(a2), _ptr(a2, d),
        _ptr(c2, d), _ptr(O2, d), ctypes.c_double(ln_prec), method, _ptr(P, d), _ptr(K, d),
        _ptr(oog, d), _ptr(ns, d), _ptr(ls, d), _ptr(p1, ctypes.c_int), _ptr(p2, ctypes.c_int))
    return dict(P=P[:3 * cnt].reshape(-1, 3), K=K[:cnt], oogamma=oog[:cnt],
                nonsph=ns[:cnt], ln_scr=ls[:cnt], p1=p1[:cnt], p2=p2[:cnt])


def compute_quartet(basis: OracleBasis, s1, s2, s3, s4, deriv=0,
                    precision=np.finfo(float).eps, method=0, pair_precision=0.0):
    """Engine::compute(s1,s2,s3,s4): list of nsets arrays (n1,n2,n3,n4), or
    None when every primitive quartet was screened out.  pair_precision > 0
    builds the primitive pairs at that precision (a caller's precomputed
    ShellPair data) and screens only the primitive quartets at precision."""
    n = [int(basis.nfunc[s]) for s in (s1, s2, s3, s4)]
    nsets = {0: 1, 1: 12, 2: 78}[deriv]
    out = np.zeros(nsets * int(np.prod(n)))
    if pair_precision > 0:
        r = _lib().orc_compute_quartet_pairs(ctypes.byref(basis._c), s1, s2, s3, s4, deriv,
                                             ctypes.c_double(precision),
                                             ctypes.c_double(pair_precision), method,
                                             _ptr(out, ctypes.c_double))
    else:
        r = _lib().orc_compute_quartet(ctypes.byref(basis._c), s1, s2, s3, s4, deriv,
                                       ctypes.c_double(precision), method,
                                       _ptr(out, ctypes.c_double))
    if r < 0:
        raise ValueError("oracle: bad arguments")
    if r == 0:
        return None
    return [out[i * r:(i + 1) * r].reshape(n) for i in range(nsets)]


def compute_batch(basis: OracleBasis, quartets, offsets, total, deriv=0,
                  precision=np.finfo(float).eps, method=0, nthreads=0):
    """Engine::compute over an explicit quartet list (n x 4 shell indices),
    OpenMP over quartets; set q lands at out[offsets[q]:...] as in
    lgx_compute_batch.  Returns (out, is_null)."""
    q = np.ascontiguousarray(quartets, np.int32).reshape(-1, 4)
    offs = np.ascontiguousarray(offsets, np.int64)
    out = np.zeros(max(1, int(total)))
    isnull = np.zeros(max(1, len(q)), np.int32)
    lib = _lib()
    lib.orc_compute_batch.argtypes = [ctypes.POINTER(_Basis), _ip, ctypes.c_int64, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int64), _dp, _ip, ctypes.c_int]
    r = lib.orc_compute_batch(ctypes.byref(basis._c), _ptr(q, ctypes.c_int), len(q), deriv,
                              precision, method, _ptr(offs, ctypes.c_int64),
                              _ptr(out, ctypes.c_double), _ptr(isnull, ctypes.c_int), nthreads)
    if r < 0:
        raise ValueError("oracle: bad arguments")
    return out, isnull[:len(q)]


def schwarz(basis: OracleBasis, nthreads=0) -> np.ndarray:
    K = np.zeros((basis.nshell, basis.nshell))
    _lib().orc_schwarz(ctypes.byref(basis._c), _ptr(K, ctypes.c_double), nthreads)
    return K


def jk(basis: OracleBasis, D, Kschwarz, thresh=1e-12, nthreads=0):
    nbf = basis.nbf
    D = np.ascontiguousarray(D, np.float64)
    J = np.zeros((nbf, nbf)); K = np.zeros((nbf, nbf))
    nq = _lib().orc_jk(ctypes.byref(basis._c), _ptr(basis.bf_off, ctypes.c_int), nbf,
                       _ptr(np.ascontiguousarray(Kschwarz), ctypes.c_double),
                       ctypes.c_double(thresh), _ptr(D, ctypes.c_double),
                       _ptr(J, ctypes.c_double), _ptr(K, ctypes.c_double), nthreads)
    return J, K, int(nq)


def jk_sample(basis: OracleBasis, D, Kschwarz, thresh, pair_begin, pair_end,
              nthreads=0):
    """J/K contributions of bra shell pairs [pair_begin, pair_end) of the
    canonical enumeration; returns (J, K, n_quartets, n_integrals)."""
    nbf = basis.nbf
    D = np.ascontiguousarray(D, np.float64)
    J = np.zeros((nbf, nbf)); K = np.zeros((nbf, nbf))
    nint = ctypes.c_int64(0)
    nq = _lib().orc_jk_sample(ctypes.byref(basis._c), _ptr(basis.bf_off, ctypes.c_int), nbf,
                              _ptr(np.ascontiguousarray(Kschwarz), ctypes.c_double),
                              ctypes.c_double(thresh), _ptr(D, ctypes.c_double),
                              _ptr(J, ctypes.c_double), _ptr(K, ctypes.c_double), nthreads,
                              ctypes.c_int64(pair_begin), ctypes.c_int64(pair_end),
                              ctypes.byref(nint))
    return J, K, int(nq), int(nint.value)


class JKAccumulator:
    """Per-thread J/K accumulators kept across calls (orc_jk_acc_*): add the
    contributions of listed bra shell pairs, then reduce once, as the
    reference's compute_2body_fock keeps one G per thread."""

    def __init__(self, nbf: int, nthreads: int = 0):
        lib = _lib()
        lib.orc_jk_acc_create.restype = ctypes.c_void_p
        lib.orc_jk_acc_create.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.orc_jk_acc_destroy.argtypes = [ctypes.c_void_p]
        lib.orc_jk_acc_pairs.restype = ctypes.c_int64
        lib.orc_jk_acc_pairs.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Basis), _ip, _dp,
                                         ctypes.c_double, _dp,
                                         ctypes.POINTER(ctypes.c_int64), ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_double,
                                         ctypes.POINTER(ctypes.c_int64)]
        lib.orc_jk_acc_reduce.argtypes = [ctypes.c_void_p, _dp, _dp]
        self._lib = lib
        self.nbf = int(nbf)
        self._h = lib.orc_jk_acc_create(self.nbf, int(nthreads))
        if not self._h:
            raise ValueError("orc_jk_acc_create failed")

    def add_pairs(self, basis: OracleBasis, D, Kschwarz, thresh, pairs, ket_subset=False,
                  fock_precision=0.0):
        """Adds the quartets of bra pairs `pairs` (canonical pair indices
        s1 (s1 + 1) / 2 + s2, s2 <= s1) with every ket pair up to the bra, or
        with `ket_subset` only the kets among `pairs` (each unordered quartet
        of the subset once), with compute_2body_fock's density-weighted
        screening when fock_precision > 0; returns (n_quartets, n_integrals)."""
        D = np.ascontiguousarray(D, np.float64)
        Ks = np.ascontiguousarray(Kschwarz, np.float64)
        p = np.ascontiguousarray(pairs, np.int64)
        mask = None
        if ket_subset:
            ns = basis.nshell
            mask = np.zeros(ns * (ns + 1) // 2, np.uint8)
            mask[p] = 1
        nint = ctypes.c_int64(0)
        nq = self._lib.orc_jk_acc_pairs(self._h, ctypes.byref(basis._c),
                                        _ptr(basis.bf_off, ctypes.c_int),
                                        _ptr(Ks, ctypes.c_double), ctypes.c_double(thresh),
                                        _ptr(D, ctypes.c_double), _ptr(p, ctypes.c_int64),
                                        len(p), None if mask is None else mask.ctypes.data,
                                        ctypes.c_double(fock_precision), ctypes.byref(nint))
        if nq < 0:
            raise ValueError("orc_jk_acc_pairs: bad arguments")
        return int(nq), int(nint.value)

    def reduce(self):
        J = np.zeros((self.nbf, self.nbf)); K = np.zeros((self.nbf, self.nbf))
        self._lib.orc_jk_acc_reduce(self._h, _ptr(J, ctypes.c_double), _ptr(K, ctypes.c_double))
        return J, K

    def close(self):
        if self._h:
            self._lib.orc_jk_acc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def count_screened(basis: OracleBasis, Kschwarz, thresh):
    """(unique quartets, integrals) of the Schwarz-screened pass."""
    lib = _lib()
    lib.orc_count_screened.argtypes = [ctypes.POINTER(_Basis), _dp, ctypes.c_double,
                                       ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64)]
    nq, ni = ctypes.c_int64(0), ctypes.c_int64(0)
    Ks = np.ascontiguousarray(Kschwarz, np.float64)
    lib.orc_count_screened(ctypes.byref(basis._c), _ptr(Ks, ctypes.c_double),
                           ctypes.c_double(thresh), ctypes.byref(nq), ctypes.byref(ni))
    return int(nq.value), int(ni.value)


def jk_grad(basis: OracleBasis, D, Kschwarz, natoms, thresh=1e-12, nthreads=0):
    D = np.ascontiguousarray(D, np.float64)
    gJ = np.zeros((natoms, 3)); gK = np.zeros((natoms, 3))
    nq = _lib().orc_jk_grad(ctypes.byref(basis._c), _ptr(basis.bf_off, ctypes.c_int),
                            basis.nbf, natoms,
                            _ptr(np.ascontiguousarray(Kschwarz), ctypes.c_double),
                            ctypes.c_double(thresh), _ptr(D, ctypes.c_double),
                            _ptr(gJ, ctypes.c_double), _ptr(gK, ctypes.c_double), nthreads)
    return gJ, gK, int(nq)


# ------------------------------------------------------------------ reference
def ref_lib():
    """The reference's own code compiled in place (oracle/_ref/libref.so), or
    None when it has not been built (e.g. away from the reference tree)."""
    if not os.path.exists(REF_LIB_PATH):
        return None
    lib = ctypes.CDLL(REF_LIB_PATH)
    lib.ref_solid_coeff.restype = ctypes.c_double
    lib.ref_solid_coeff.argtypes = [ctypes.c_int] * 5
    lib.ref_boys_reference2.argtypes = [ctypes.c_double, ctypes.c_int, _dp]
    lib.ref_boys_reference_ld.argtypes = [ctypes.c_double, ctypes.c_int, _dp]
    lib.ref_boys_taylor.argtypes = [ctypes.c_double, ctypes.c_int, _dp]
    return lib


def ref_deriv_order2(lib):
    """(c1, c2) coordinate pairs (0..11, c1 <= c2) of libint's 78
    second-derivative shell sets, from the reference's CartesianDerivIterator."""
    c1 = np.zeros(78, np.int32)
    c2 = np.zeros(78, np.int32)
    n = lib.ref_deriv_order2(_ptr(c1, ctypes.c_int), _ptr(c2, ctypes.c_int))
    assert n == 78
    return c1, c2


def ref_eri_shellset(lib, shells, deriv=0):
    """Brute-force shell set from the reference's eri.h.  shells: 4 tuples
    (l, pure, alpha, coeff_normalized, origin)."""
    l = np.array([s[0] for s in shells], np.int32)
    pure = np.array([s[1] for s in shells], np.int32)
    nprim = np.array([len(s[2]) for s in shells], np.int32)
    alpha = np.concatenate([np.asarray(s[2], float) for s in shells])
    coeff = np.concatenate([np.asarray(s[3], float) for s in shells])
    O = np.concatenate([np.asarray(s[4], float) for s in shells])
    n = [(2 * s[0] + 1) if s[1] else (s[0] + 1) * (s[0] + 2) // 2 for s in shells]
    nsets = {0: 1, 1: 12, 2: 78}[deriv]
    out = np.zeros(nsets * int(np.prod(n)))
    lib.ref_eri_shellset(_ptr(l, ctypes.c_int), _ptr(pure, ctypes.c_int),
                         _ptr(nprim, ctypes.c_int), _ptr(alpha, ctypes.c_double),
                         _ptr(coeff, ctypes.c_double), _ptr(O, ctypes.c_double),
                         deriv, _ptr(out, ctypes.c_double))
    m = int(np.prod(n))
    return [out[i * m:(i + 1) * m].reshape(n) for i in range(nsets)]
