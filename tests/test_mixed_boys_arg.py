"""The double-float arithmetic that forms the mixed scheme's Boys argument
T = rho |P - Q|^2 (ds_boys_arg in libint_gb300/csrc/lgx_device.cuh),
restated step by step in numpy float32 with the FMA emulated in float64
(the product of two float32 values is exact there), against the argument in
extended precision.  This pins the numerical design -- 48-bit records of P
and zeta, the residual correction of the FP32 rho, the error-free sums and
products -- on the CPU: the relative error of T stays near 1e-13 except
where T itself is tiny, and its effect on F_m(T) stays far below the FP32
half-ulp the mixed scheme rounds to.  The device code itself is checked
against the oracle by tests/test_gpu_boys.py (lgx_boys variant 6)."""
import numpy as np

f32, f64 = np.float32, np.float64


def _add(a, b):
    return (a.astype(f32) + b.astype(f32)).astype(f32)


def _mul(a, b):
    return (a.astype(f32) * b.astype(f32)).astype(f32)


def _fma(a, b, c):
    return (a.astype(f64) * b.astype(f64) + c.astype(f64)).astype(f32)


def _fast_two_sum(a, b):
    s = _add(a, b)
    return s, _add(b, -_add(s, -a))


def _two_sum(a, b):
    s = _add(a, b)
    bb = _add(s, -a)
    return s, _add(_add(a, -_add(s, -bb)), _add(b, -bb))


def _ds_add(a, b):
    s = _two_sum(a[0], b[0])
    return _two_sum(s[0], _add(s[1], _add(a[1], b[1])))


def _ds_sub(a, b):
    return _ds_add(a, (-b[0], -b[1]))


def _ds_mul(a, b):
    p = _mul(a[0], b[0])
    e = _fma(a[0], b[0], -p)
    return _fast_two_sum(p, _fma(a[0], b[1], _fma(a[1], b[0], e)))


def _ds_sqr(a):
    p = _mul(a[0], a[0])
    e = _fma(a[0], a[0], -p)
    return _fast_two_sum(p, _fma(f32(2) * a[0], a[1], e))


def _split(x):
    h = x.astype(f32)
    return h, (x - h.astype(f64)).astype(f32)


def test_double_float_boys_argument_accuracy():
    rng = np.random.default_rng(1)
    n = 100000
    zb = np.exp(rng.uniform(np.log(0.05), np.log(3e4), n))
    zk = np.exp(rng.uniform(np.log(0.05), np.log(3e4), n))
    Pb = rng.uniform(-30.0, 30.0, (n, 3))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    d = np.exp(rng.uniform(np.log(1e-4), np.log(40.0), n))
    Pk = Pb + d[:, None] * u
    zbs, zks = _split(zb), _split(zk)
    # the FP32 prologue's rho and 1/(zeta + eta) (rsqrt correctly rounded here)
    oog = _mul(*(2 * [(1.0 / np.sqrt(_add(zbs[0], zks[0]).astype(f64))).astype(f32)]))
    rho0 = _mul(_mul(zbs[0], zks[0]), oog)
    r = _ds_sub(_ds_mul(zbs, zks), _ds_mul((rho0, np.zeros(n, f32)), _ds_add(zbs, zks)))
    rho = _fast_two_sum(rho0, _mul(r[0], oog))
    acc = None
    for c in range(3):
        s = _ds_sqr(_ds_sub(_split(Pb[:, c]), _split(Pk[:, c])))
        acc = s if acc is None else _ds_add(acc, s)
    T = _ds_mul(rho, acc)
    Tds = T[0].astype(f64) + T[1].astype(f64)
    L = np.longdouble
    Tref = (zb.astype(L) * zk.astype(L) / (zb.astype(L) + zk.astype(L))
            * ((Pb.astype(L) - Pk.astype(L)) ** 2).sum(1))
    rel = np.abs((Tds - Tref) / Tref).astype(f64)
    Tr = Tref.astype(f64)
    assert np.median(rel) < 1e-12
    # the 48-bit records of P bound the error where |P - Q| is small
    assert rel[Tr > 1e-3].max() < 1e-9
    # effect on F_m(T): |dF_m / F_m| <= T |dT / T| min(1, (m + 1/2) / T), m <= 6
    dF = Tr * rel * np.minimum(1.0, 6.5 / np.maximum(Tr, 1e-300))
    assert dF.max() < 1e-9  # against the FP32 half-ulp 6e-8
