"""Generates libint_gb300/csrc/gen/rk_classes.cuh: unrolled, register-resident
per-class device code for the thread-per-quartet ERI kernels.

For each canonical class (la>=lb, lc>=ld, la+lb<=lc+ld) it emits
  vrr<T>(F, geo, acc): Obara-Saika VRR on A then C
      (src/bin/libint/vrr_11_twoprep_11.h:145-223,305-383), straight-line,
      each needed (e0|f0)^(m) computed once, targets added into acc[]
      (the HGP contraction point, src/bin/libint/dg.cc:1177-1189);
  hrr<T>(acc, AB, CD, cart): HRR on the bra then the ket
      (src/bin/libint/hrr.h:246-347) into the Cartesian shell set;
  sph<T>(cart, out): Cartesian -> real solid harmonics for every l>=2 index
      (solidharmonics.h:282-463 applied index by index, coefficients of
      Schlegel & Frisch IJQC 54, 83 (1995) eq. 15, the coefficient set of
      solidharmonics.h:114-174).
Nodes are emitted in depth-first post-order from the targets, which keeps
the live set (registers) small.

usage: python libint_gb300/codegen/gen_rk.py [OUT]
"""
from __future__ import annotations

import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DEFAULT = os.path.join(os.path.dirname(HERE), "csrc", "gen", "rk_classes.cuh")

# classes compiled into register kernels: total angular momentum <= RK_MAX_L
# for the J/K digestion kernels, <= RK_MAX_L_STORE for store / Schwarz
RK_MAX_L = 6
RK_MAX_L_STORE = 4
LMAX = 3
# (precision, mode, class limit, attenuated operator) variants; the
# attenuated (erf / erfc) register kernels serve the J/K passes only
# (the kModeJKB64 / kModeStoreB64 FP32 kernels evaluate the Boys function in
# FP64: the mixed scheme's FP32 quartets)
VARIANTS = [("double", "kModeJK", RK_MAX_L, False), ("float", "kModeJK", RK_MAX_L, False),
            ("float", "kModeJKB64", RK_MAX_L, False),
            ("double", "kModeStore", RK_MAX_L_STORE, False),
            ("double", "kModeSchwarz", RK_MAX_L_STORE, False),
            ("float", "kModeStore", RK_MAX_L_STORE, False),
            ("float", "kModeStoreB64", RK_MAX_L_STORE, False),
            ("double", "kModeJK", RK_MAX_L, True), ("float", "kModeJK", RK_MAX_L, True)]
N_UNITS = 24  # instantiation translation units (compiled in parallel)

# __launch_bounds__ minimum blocks per SM of the J/K register kernels (0: the
# compiler's own register target), per (precision, mode, class).  Kernels not
# listed get 1 for FP64 classes with L >= 5 (left to itself the compiler
# gives several of them 32 registers and 25-57 KB of spills per thread; with
# 1 their serial (H2O)64 cc-pVTZ launches ran 14-29% faster), else 0.  The
# listed ones: the spill-free settings that beat the compiler's choice by
# 7-11% in a sweep of 0, 1, 3, 4, 6, 8 over tuned serial passes of
# (H2O)64 cc-pVTZ.  Caps that make the FP32 kernels spill were faster in
# serial passes but slower inside the graph pass, where the spills compete
# for L2 with the concurrent launches ((ps|ps) of the mixed scheme at 8:
# 434 GB of DRAM traffic and +40% time), so none is listed.
MIN_BLOCKS = {
    ("float", "kModeJK", (1, 0, 3, 0)): 4,
    ("float", "kModeJK", (2, 0, 2, 0)): 4,
    ("float", "kModeJKB64", (0, 0, 3, 3)): 3,
}
MODE_IDS = {"kModeStore": 0, "kModeSchwarz": 1, "kModeJK": 2, "kModeJKB64": 4,
            "kModeStoreB64": 5}


def comps(l):
    return [(lx, ly, l - lx - ly) for lx in range(l, -1, -1) for ly in range(l - lx, -1, -1)]


def first_dir(c):
    return 0 if c[0] else (1 if c[1] else 2)


def sh(c, i, d):
    c = list(c)
    c[i] += d
    return tuple(c)


def ncart(l):
    return (l + 1) * (l + 2) // 2


def rk_classes(lmax_total=None):
    lmax_total = RK_MAX_L if lmax_total is None else lmax_total
    out = []
    for la in range(LMAX + 1):
        for lb in range(la + 1):
            for lc in range(LMAX + 1):
                for ld in range(lc + 1):
                    if la + lb <= lc + ld and la + lb + lc + ld <= lmax_total:
                        out.append((la, lb, lc, ld))
    return out


# ------------------------------------------------------------- solid harmonics
def _fac(n):
    return math.factorial(n) if n >= 0 else 0


def _dfac(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def _binom(n, k):
    return math.comb(n, k) if 0 <= k <= n else 0


def solid_coeff(l, m, lx, ly, lz):
    am = abs(m)
    if (lx + ly - am) % 2:
        return 0.0
    j = (lx + ly - am) // 2
    if j < 0:
        return 0.0
    i = am - lx
    if (m >= 0) != (abs(i) % 2 == 0):
        return 0.0
    pf = math.sqrt(_fac(2 * lx) * _fac(2 * ly) * _fac(2 * lz) / _fac(2 * l) * _fac(l - am) /
                   _fac(l) / _fac(l + am) / (_fac(lx) * _fac(ly) * _fac(lz)))
    pf /= 2 ** l
    # (-1)^(i/2) resp. (-1)^((i-1)/2); the exponents are exact integers here
    e = (i - 1) // 2 if m < 0 else i // 2
    pf *= -1 if e % 2 else 1
    s = 0.0
    for ii in range(j, (l - am) // 2 + 1):
        t = _binom(l, ii) * _binom(ii, j) * (-1) ** ii * _fac(2 * (l - ii)) / _fac(l - am - 2 * ii)
        s1 = 0.0
        for k in range(0, min(j, lx // 2) + 1):
            if lx - 2 * k <= am:
                s1 += _binom(j, k) * _binom(am, lx - 2 * k) * (-1) ** k
        s += t * s1
    s *= math.sqrt(_dfac(2 * l - 1) / (_dfac(2 * lx - 1) * _dfac(2 * ly - 1) * _dfac(2 * lz - 1)))
    return pf * s if m == 0 else math.sqrt(2.0) * pf * s


def sph_matrix(l):
    return [[solid_coeff(l, p - l, *c) for c in comps(l)] for p in range(2 * l + 1)]


def lit(x):
    r = repr(float(x))
    return "T(%s)" % r


# ------------------------------------------------------------------- emitter
class Emitter:
    def __init__(self):
        self.lines = []
        self.n = 0

    def tmp(self, expr):
        name = "t%d" % self.n
        self.n += 1
        self.lines.append("    const T %s = %s;" % (name, expr))
        return name


def gen_class(la, lb, lc, ld):
    L = la + lb + lc + ld
    mmax = L
    targets = [(e, f) for le in range(la, la + lb + 1) for e in comps(le)
               for lf in range(lc, lc + ld + 1) for f in comps(lf)]
    acc_index = {t: k for k, t in enumerate(targets)}
    em = Emitter()
    names = {}
    xyz = "xyz"
    used_n = set()

    def node(e, f, m):
        key = (e, f, m)
        if key in names:
            return names[key]
        if sum(e) == 0 and sum(f) == 0:
            names[key] = "F[%d]" % m
            return names[key]
        if sum(f) > 0:
            j = first_dir(f)
            f1 = sh(f, j, -1)
            a = node(e, f1, m)
            b = node(e, f1, m + 1)
            expr = "fma(g.WQ%s, %s, g.QC%s * %s)" % (xyz[j], b, xyz[j], a)
            if f1[j] > 0:
                f2 = sh(f1, j, -1)
                c = node(e, f2, m)
                d = node(e, f2, m + 1)
                used_n.add(("e", f1[j]))
                expr = "fma(oo2e_%d, fma(-g.roe, %s, %s), %s)" % (f1[j], d, c, expr)
            if e[j] > 0:
                x = node(sh(e, j, -1), f1, m + 1)
                used_n.add(("ze", e[j]))
                expr = "fma(oo2ze_%d, %s, %s)" % (e[j], x, expr)
        else:
            i = first_dir(e)
            e1 = sh(e, i, -1)
            a = node(e1, f, m)
            b = node(e1, f, m + 1)
            expr = "fma(g.WP%s, %s, g.PA%s * %s)" % (xyz[i], b, xyz[i], a)
            if e1[i] > 0:
                e2 = sh(e1, i, -1)
                c = node(e2, f, m)
                d = node(e2, f, m + 1)
                used_n.add(("z", e1[i]))
                expr = "fma(oo2z_%d, fma(-g.roz, %s, %s), %s)" % (e1[i], d, c, expr)
        names[key] = em.tmp(expr)
        return names[key]

    body = []
    for t, k in acc_index.items():
        v = node(t[0], t[1], 0)
        em.lines.append("    acc[%d] += %s;" % (k, v))
    pre = []
    for kind, n in sorted(used_n):
        if kind == "z":
            pre.append("    const T oo2z_%d = T(%d) * g.oo2z;" % (n, n))
        elif kind == "e":
            pre.append("    const T oo2e_%d = T(%d) * g.oo2e;" % (n, n))
        else:
            pre.append("    const T oo2ze_%d = T(%d) * g.oo2ze;" % (n, n))
    vrr_body = pre + em.lines
    vrr_flops = sum(l.count("fma(") * 2 + l.count(" * ") for l in em.lines) + len(acc_index)

    # ---------------- HRR
    hem = Emitter()
    hnames = {}

    def bra(a, b, f):
        key = ("b", a, b, f)
        if key in hnames:
            return hnames[key]
        if sum(b) == 0:
            hnames[key] = "acc[%d]" % acc_index[(a, f)]
            return hnames[key]
        i = first_dir(b)
        s1 = bra(sh(a, i, 1), sh(b, i, -1), f)
        s2 = bra(a, sh(b, i, -1), f)
        hnames[key] = hem.tmp("fma(AB[%d], %s, %s)" % (i, s2, s1))
        return hnames[key]

    def ket(a, b, c, d):
        key = ("k", a, b, c, d)
        if key in hnames:
            return hnames[key]
        if sum(d) == 0:
            return bra(a, b, c)
        j = first_dir(d)
        s1 = ket(a, b, sh(c, j, 1), sh(d, j, -1))
        s2 = ket(a, b, c, sh(d, j, -1))
        hnames[key] = hem.tmp("fma(CD[%d], %s, %s)" % (j, s2, s1))
        return hnames[key]

    o = 0
    for a in comps(la):
        for b in comps(lb):
            for c in comps(lc):
                for d in comps(ld):
                    v = ket(a, b, c, d)
                    hem.lines.append("    cart[%d] = %s;" % (o, v))
                    o += 1
    hrr_flops = sum(l.count("fma(") * 2 for l in hem.lines)
    ncart4 = o

    # ---------------- solid harmonics (l >= 2 indices)
    ls = [la, lb, lc, ld]
    dims = [ncart(l) for l in ls]
    cur = ["cart[%d]" % i for i in range(ncart4)]
    sem = Emitter()
    sph_flops = 0
    for k in range(4):
        if ls[k] < 2:
            continue
        M = sph_matrix(ls[k])
        npure = 2 * ls[k] + 1
        outer = int(math.prod(dims[:k]))
        inner = int(math.prod(dims[k + 1:]))
        nxt = []
        for oo in range(outer):
            for p in range(npure):
                for ii in range(inner):
                    terms = [(M[p][c], cur[(oo * dims[k] + c) * inner + ii])
                             for c in range(dims[k]) if M[p][c] != 0.0]
                    expr = "%s * %s" % (lit(terms[0][0]), terms[0][1])
                    for cf, src in terms[1:]:
                        expr = "fma(%s, %s, %s)" % (lit(cf), src, expr)
                    sph_flops += 2 * len(terms) - 1
                    nxt.append(sem.tmp(expr))
        cur = nxt
        dims[k] = npure
    nsph4 = len(cur)
    for i, v in enumerate(cur):
        sem.lines.append("    out[%d] = %s;" % (i, v))

    key = "%d, %d, %d, %d" % (la, lb, lc, ld)
    s = []
    s.append("template <>\nstruct Cls<%s> {" % key)
    s.append("  static constexpr int kMmax = %d, kNacc = %d, kNcart = %d, kNsph = %d;" %
             (mmax, len(acc_index), ncart4, nsph4))
    s.append("  static constexpr int kN0 = %d, kN1 = %d, kN2 = %d, kN3 = %d;" % tuple(dims))
    s.append("  static constexpr int kVrrFlops = %d, kHrrFlops = %d, kSphFlops = %d;" %
             (vrr_flops, hrr_flops, sph_flops))
    s.append("  template <typename T>\n  static __device__ __forceinline__ void vrr(const T* F, "
             "const Geo<T>& g, T* acc) {")
    s.extend(vrr_body)
    s.append("  }")
    s.append("  template <typename T>\n  static __device__ __forceinline__ void hrr(const T* acc, "
             "const T* AB, const T* CD, T* cart) {")
    s.extend(hem.lines)
    s.append("  }")
    s.append("  template <typename T>\n  static __device__ __forceinline__ void sph(const T* cart, "
             "T* out) {")
    s.extend(sem.lines)
    s.append("  }")
    s.append("};")
    return "\n".join(s)


def _write_if_changed(path, text):
    if os.path.exists(path) and open(path).read() == text:
        return
    with open(path, "w") as f:
        f.write(text)


def _cost(c):
    la, lb, lc, ld = c
    return (la + lb + lc + ld + 1) ** 4


def write_units(gen_dir):
    """Instantiation units: each defines the launchers of a share of the
    (precision, mode, class) kernels; rk_dispatch.cu maps run-time
    (precision, mode, class) to them.  Returns the unit file names."""
    items = []
    for prec, mode, lmax, att in VARIANTS:
        for c in rk_classes(lmax):
            items.append((prec, mode, att, c))
    items.sort(key=lambda it: -_cost(it[3]))
    units = [[] for _ in range(N_UNITS)]
    load = [0] * N_UNITS
    for it in items:  # greedy balance by estimated code size
        k = load.index(min(load))
        units[k].append(it)
        load[k] += _cost(it[3])
    names = []
    decls = []
    for k, u in enumerate(units):
        name = "rk_unit_%02d.cu" % k
        names.append(name)
        lines = ["// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.",
                 '#include "../lgx_rk.cuh"', "", "namespace lgx {"]
        for prec, mode, att, c in u:
            fn = "rk_launch_%s_%s%s_%d%d%d%d" % (prec[0], mode[5:].lower(), "_att" if att else "",
                                                 *c)
            decls.append((prec, mode, att, c, fn))
            lines.append("cudaError_t %s(const EriArgs& a, long long work, int nsm, "
                         "cudaStream_t st) {" % fn)
            lines.append("  return rk_launch_one<%s, %d, %d, %d, %d, %s, %s>(a, work, nsm, st);" %
                         (prec, *c, mode, "true" if att else "false"))
            lines.append("}")
        lines.append("}  // namespace lgx")
        _write_if_changed(os.path.join(gen_dir, name), "\n".join(lines) + "\n")
    d = ["// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.",
         "// Run-time dispatch of the register kernels.", '#include "../lgx_rk.cuh"', "",
         "namespace lgx {"]
    for prec, mode, att, c, fn in decls:
        d.append("cudaError_t %s(const EriArgs& a, long long work, int nsm, cudaStream_t st);" % fn)
    d.append("")
    d.append("// Launches the register kernel of (precision, mode, operator, class);")
    d.append("// returns cudaErrorNotSupported when that kernel is not compiled.")
    d.append("cudaError_t rk_launch(bool fp32, int mode, bool att, int la, int lb, int lc, int ld, "
             "const EriArgs& a, long long work, int nsm, cudaStream_t st) {")
    d.append("  const int key = ((((att ? 1 : 0) * 2 + (fp32 ? 1 : 0)) * 8 + mode) * 4096) + "
             "((la * 8 + lb) * 8 + lc) * 8 + ld;")
    d.append("  switch (key) {")
    for prec, mode, att, c, fn in sorted(decls, key=lambda x: x[4]):
        mode_id = {"kModeStore": 0, "kModeSchwarz": 1, "kModeJK": 2, "kModeJKB64": 4,
                   "kModeStoreB64": 5}[mode]
        key = ((((1 if att else 0) * 2 + (1 if prec == "float" else 0)) * 8 + mode_id) * 4096) + \
            ((c[0] * 8 + c[1]) * 8 + c[2]) * 8 + c[3]
        d.append("    case %d: return %s(a, work, nsm, st);" % (key, fn))
    d.append("  }")
    d.append("  return cudaErrorNotSupported;")
    d.append("}")
    d.append("")
    d.append("bool rk_available(bool fp32, int mode, bool att, int la, int lb, int lc, int ld) {")
    d.append("  const int L = la + lb + lc + ld;")
    d.append("  if (att) return mode == kModeJK && L <= %d;" % RK_MAX_L)
    d.append("  if (mode == kModeJK) return L <= %d;" % RK_MAX_L)
    d.append("  if (mode == kModeJKB64) return fp32 && L <= %d;" % RK_MAX_L)
    d.append("  if (mode == kModeStoreB64) return fp32 && L <= %d;" % RK_MAX_L_STORE)
    d.append("  if (mode == kModeStore) return L <= %d;" % RK_MAX_L_STORE)
    d.append("  if (mode == kModeSchwarz) return !fp32 && L <= %d;" % RK_MAX_L_STORE)
    d.append("  return false;")
    d.append("}")
    d.append("}  // namespace lgx")
    _write_if_changed(os.path.join(gen_dir, "rk_dispatch.cu"), "\n".join(d) + "\n")
    return names + ["rk_dispatch.cu"]


def main(out=OUT_DEFAULT):
    os.makedirs(os.path.dirname(out), exist_ok=True)
    parts = ["// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.",
             "// Unrolled per-class VRR / HRR / solid-harmonic code for the",
             "// register-resident ERI kernels (see gen_rk.py for the recurrences).",
             "#pragma once", '#include "../lgx_rk_common.cuh"', "", "namespace lgx {",
             "namespace rk {", "", "template <int LA, int LB, int LC, int LD>", "struct Cls;", ""]
    classes = rk_classes()
    for c in classes:
        parts.append(gen_class(*c))
        parts.append("")
    parts.append("// __launch_bounds__ minimum blocks per SM of the listed register kernels")
    parts.append("// (gen_rk.py MIN_BLOCKS); -1: not listed.")
    parts.append("constexpr int min_blocks_table(bool fp32, int mode, int la, int lb, int lc, "
                 "int ld) {")
    parts.append("  switch (((fp32 ? 1 : 0) * 8 + mode) * 4096 + ((la * 8 + lb) * 8 + lc) * 8 + "
                 "ld) {")
    for (prec, mode, c), v in sorted(MIN_BLOCKS.items()):
        key = ((1 if prec == "float" else 0) * 8 + MODE_IDS[mode]) * 4096 + \
            ((c[0] * 8 + c[1]) * 8 + c[2]) * 8 + c[3]
        parts.append("    case %d: return %d;  // %s %s (%d%d|%d%d)" % (key, v, prec, mode, *c))
    parts.append("    default: return -1;")
    parts.append("  }")
    parts.append("}")
    parts.append("")
    parts.append("}  // namespace rk")
    parts.append("}  // namespace lgx")
    text = "\n".join(parts) + "\n"
    _write_if_changed(out, text)
    return write_units(os.path.dirname(out))


if __name__ == "__main__":
    print("\n".join(main(sys.argv[1] if len(sys.argv) > 1 else OUT_DEFAULT)))
