"""Generates the unrolled post-contraction stages of the program kernel for
the J/K classes above the register-kernel limit (csrc/gen/post_classes.cuh,
csrc/gen/post_unit_XX.cu, csrc/gen/post_dispatch.cu).

For a canonical class (la, lb, lc, ld) the contracted (e0|f0) set, laid out
as the class program builds it (e-shell block, f-shell block, e-major;
lgx_program.cpp), is turned into the solid-harmonic shell set in two
column-parallel stages of one warp:
  bra<T>: lane = one ket function f of shells lc..lc+ld; HRR on the bra
      (a b| = (a+1_i b-1_i| + AB_i (a b-1_i|, src/bin/libint/hrr.h:246-347)
      and the solid-harmonic transform of a and b, all in registers;
      writes (a'b'|f) with f fastest (conflict-free stores);
  ket<T>: lane = one bra function pair a'b'; HRR on the ket and the
      transform of c and d (Schlegel & Frisch eq. 15 coefficients, the set of
      solidharmonics.h:114-174); writes V[a'][b'][c'][d'].
Every step is warp-synchronous only at the stage boundary, and no op stream
is read: the per-class code replaces the interpreted post program and the
table-driven transform for these classes.

usage: python libint_gb300/codegen/gen_post.py
"""
from __future__ import annotations

import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from gen_rk import (LMAX, RK_MAX_L, Emitter, _write_if_changed, comps, first_dir,  # noqa: E402
                    lit, ncart, sh, sph_matrix)

GEN_DIR = os.path.join(os.path.dirname(HERE), "csrc", "gen")
N_UNITS = 8


def post_classes():
    """J/K classes served by the program kernel (above the register kernels)."""
    out = []
    for la in range(LMAX + 1):
        for lb in range(la + 1):
            for lc in range(LMAX + 1):
                for ld in range(lc + 1):
                    if la + lb <= lc + ld and la + lb + lc + ld > RK_MAX_L:
                        out.append((la, lb, lc, ld))
    return out


def nsph(l):
    return 2 * l + 1 if l >= 2 else ncart(l)


def transform(em, vals, dims, ls, which):
    """Solid-harmonic transform of the indices in `which` (l >= 2) of the
    row-major value list vals[dims]; returns (values, dims)."""
    cur = list(vals)
    dims = list(dims)
    for k in which:
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
                    nxt.append(em.tmp(expr))
        cur = nxt
        dims[k] = npure
    return cur, dims


def gen_class(la, lb, lc, ld):
    ls = [la, lb, lc, ld]
    # contracted-set layout of the class program (deriv 0)
    off = {}
    n = 0
    for le in range(la, la + lb + 1):
        for lf in range(lc, lc + ld + 1):
            off[(le, lf)] = n
            n += ncart(le) * ncart(lf)
    nacc = n
    fshells = list(range(lc, lc + ld + 1))
    foff = {}
    nf = 0
    for lf in fshells:
        foff[lf] = nf
        nf += ncart(lf)
    nfp = nf if nf % 2 else nf + 1  # odd column stride: conflict-free ket loads
    na, nb, nc, nd = (nsph(l) for l in ls)
    nab = na * nb
    ncd = nc * nd

    # ---------------- bra stage (lane = f column)
    em = Emitter()
    inputs = {}
    for le in range(la, la + lb + 1):
        for ie, e in enumerate(comps(le)):
            inputs[e] = "x%d_%d" % (le, ie)
            em.lines.append("      const T %s = acc[b%d + %d * s];" % (inputs[e], le, ie))
    memo = {}

    def bra(a, b):
        key = (a, b)
        if key in memo:
            return memo[key]
        if sum(b) == 0:
            return inputs[a]
        i = first_dir(b)
        s1 = bra(sh(a, i, 1), sh(b, i, -1))
        s2 = bra(a, sh(b, i, -1))
        memo[key] = em.tmp("fma(AB[%d], %s, %s)" % (i, s2, s1))
        return memo[key]

    cart = [bra(a, b) for a in comps(la) for b in comps(lb)]
    vals, _ = transform(em, cart, [ncart(la), ncart(lb)], [la, lb], [0, 1])
    assert len(vals) == nab
    for k, v in enumerate(vals):
        em.lines.append("      bo[%d * kNFP + col] = %s;" % (k, v))
    sel = []
    for idx, lf in enumerate(fshells):
        lo, hi = foff[lf], foff[lf] + ncart(lf)
        assigns = " ".join("b%d = %d + (col - %d);" % (le, off[(le, lf)], lo)
                           for le in range(la, la + lb + 1))
        cond = "col < %d" % hi
        if idx == 0:
            sel.append("      if (%s) { s = %d; %s }" % (cond, ncart(lf), assigns))
        elif idx < len(fshells) - 1:
            sel.append("      else if (%s) { s = %d; %s }" % (cond, ncart(lf), assigns))
        else:
            sel.append("      else { s = %d; %s }" % (ncart(lf), assigns))
    if len(fshells) == 1:
        sel = ["      { s = %d; %s }" % (ncart(fshells[0]), " ".join(
            "b%d = %d + col;" % (le, off[(le, fshells[0])]) for le in range(la, la + lb + 1)))]
    bdecl = "      int s, %s;" % ", ".join("b%d" % le for le in range(la, la + lb + 1))
    bra_body = [bdecl] + sel + em.lines

    # ---------------- ket stage (lane = a'b' column)
    kem = Emitter()
    kin = {}
    for lf in fshells:
        for i_, f in enumerate(comps(lf)):
            kin[f] = "y%d_%d" % (lf, i_)
            kem.lines.append("      const T %s = src[%d];" % (kin[f], foff[lf] + i_))
    kmemo = {}

    def ket(c, d):
        key = (c, d)
        if key in kmemo:
            return kmemo[key]
        if sum(d) == 0:
            return kin[c]
        j = first_dir(d)
        s1 = ket(sh(c, j, 1), sh(d, j, -1))
        s2 = ket(c, sh(d, j, -1))
        kmemo[key] = kem.tmp("fma(CD[%d], %s, %s)" % (j, s2, s1))
        return kmemo[key]

    kcart = [ket(c, d) for c in comps(lc) for d in comps(ld)]
    kvals, _ = transform(kem, kcart, [ncart(lc), ncart(ld)], [lc, ld], [0, 1])
    assert len(kvals) == ncd
    for k, v in enumerate(kvals):
        kem.lines.append("      dst[%d] = %s;" % (k, v))

    key = "%d, %d, %d, %d" % (la, lb, lc, ld)
    s = ["template <>", "struct PostGen<%s> {" % key,
         "  static constexpr bool kGenerated = true;",
         "  static constexpr int kNacc = %d, kNF = %d, kNFP = %d;" % (nacc, nf, nfp),
         "  static constexpr int kNA = %d, kNB = %d, kNC = %d, kND = %d;" % (na, nb, nc, nd),
         "  static constexpr int kBraOut = %d, kV = %d;" % (nab * nfp, nab * ncd),
         "  static constexpr int kSlots = kNacc + kBraOut + kV;",
         "  template <typename T>",
         "  static __device__ __forceinline__ void bra(const T* __restrict__ acc, "
         "T* __restrict__ bo, const T* AB, int lane) {",
         "    for (int col = lane; col < kNF; col += 32) {"]
    s += bra_body
    s += ["    }", "  }",
          "  template <typename T>",
          "  static __device__ __forceinline__ void ket(const T* __restrict__ bo, "
          "T* __restrict__ V, const T* CD, int lane) {",
          "    for (int col = lane; col < kNA * kNB; col += 32) {",
          "      const T* src = bo + col * kNFP;",
          "      T* dst = V + col * (kNC * kND);"]
    s += kem.lines
    s += ["    }", "  }", "};"]
    return "\n".join(s)


def _cost(c):
    return (sum(c) + 1) ** 3


def main():
    os.makedirs(GEN_DIR, exist_ok=True)
    classes = post_classes()
    parts = ["// GENERATED by libint_gb300/codegen/gen_post.py -- do not edit.",
             "// Unrolled post-contraction stages (HRR + solid harmonics) of the",
             "// program kernel for the J/K classes above the register kernels.",
             "#pragma once", '#include "../lgx_warp.cuh"', "", "namespace lgx {", "",
             "template <int LA, int LB, int LC, int LD>", "struct PostGen;", ""]
    for c in classes:
        parts.append(gen_class(*c))
        parts.append("")
    parts.append("}  // namespace lgx")
    _write_if_changed(os.path.join(GEN_DIR, "post_classes.cuh"), "\n".join(parts) + "\n")

    # (precision, mode): FP64, FP32, and FP32 with the FP64 Boys function of
    # the mixed scheme
    variants = (("double", "kModeJK"), ("float", "kModeJK"), ("float", "kModeJKB64"))
    items = [(v, c) for c in classes for v in variants]
    items.sort(key=lambda it: -_cost(it[1]))
    units = [[] for _ in range(N_UNITS)]
    load = [0] * N_UNITS
    for it in items:
        k = load.index(min(load))
        units[k].append(it)
        load[k] += _cost(it[1])
    names = []
    decls = []
    for k, u in enumerate(units):
        name = "post_unit_%02d.cu" % k
        names.append(name)
        lines = ["// GENERATED by libint_gb300/codegen/gen_post.py -- do not edit.",
                 '#include "post_classes.cuh"', "", "namespace lgx {"]
        for (prec, mode), c in u:
            tag = "%s%s_%d%d%d%d" % (prec[0], "b" if mode == "kModeJKB64" else "", *c)
            decls.append((prec, mode, c, tag))
            post = "PostGen<%d, %d, %d, %d>" % c
            lines.append("cudaError_t post_launch_%s(const EriArgs& a, int grid, int block, "
                         "size_t smem, cudaStream_t st) {" % tag)
            lines.append("  return launch_eri_t<%s, %s, %s>(a, grid, block, smem, st);" %
                         (prec, mode, post))
            lines.append("}")
            lines.append("int post_occ_%s(int block, size_t smem) {" % tag)
            lines.append("  return occ_t<%s, %s, %s>(block, smem);" % (prec, mode, post))
            lines.append("}")
        lines.append("}  // namespace lgx")
        _write_if_changed(os.path.join(GEN_DIR, name), "\n".join(lines) + "\n")

    d = ["// GENERATED by libint_gb300/codegen/gen_post.py -- do not edit.",
         "// Run-time dispatch of the program kernels with generated post stages.",
         '#include "../lgx_kernels.cuh"', "", "namespace lgx {"]
    for prec, mode, c, tag in decls:
        d.append("cudaError_t post_launch_%s(const EriArgs& a, int grid, int block, size_t smem, "
                 "cudaStream_t st);" % tag)
        d.append("int post_occ_%s(int block, size_t smem);" % tag)
    d.append("")

    def ckey(c):
        return ((c[0] * 8 + c[1]) * 8 + c[2]) * 8 + c[3]

    def vkey(prec, mode):
        return (4096 if prec == "float" else 0) + (8192 if mode == "kModeJKB64" else 0)

    d.append("// Launches the J/K program kernel of (precision, mode, class) with its")
    d.append("// generated post stage; cudaErrorNotSupported when there is none.")
    d.append("cudaError_t post_launch(bool fp32, int mode, int la, int lb, int lc, int ld, "
             "const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {")
    d.append("  switch ((fp32 ? 4096 : 0) + (mode == kModeJKB64 ? 8192 : 0) + "
             "((la * 8 + lb) * 8 + lc) * 8 + ld) {")
    for prec, mode, c, tag in decls:
        d.append("    case %d: return post_launch_%s(a, grid, block, smem, st);" %
                 (vkey(prec, mode) + ckey(c), tag))
    d.append("  }")
    d.append("  return cudaErrorNotSupported;")
    d.append("}")
    d.append("")
    d.append("int post_blocks_per_sm(bool fp32, int mode, int la, int lb, int lc, int ld, "
             "int block, size_t smem) {")
    d.append("  switch ((fp32 ? 4096 : 0) + (mode == kModeJKB64 ? 8192 : 0) + "
             "((la * 8 + lb) * 8 + lc) * 8 + ld) {")
    for prec, mode, c, tag in decls:
        d.append("    case %d: return post_occ_%s(block, smem);" %
                 (vkey(prec, mode) + ckey(c), tag))
    d.append("  }")
    d.append("  return 0;")
    d.append("}")
    d.append("")
    d.append("// Contracted-set size and the slots the generated post stage needs")
    d.append("// (accumulators + bra-stage output + shell set); false if none.")
    d.append("bool post_info(int la, int lb, int lc, int ld, int* nacc, int* slots) {")
    d.append("  switch (((la * 8 + lb) * 8 + lc) * 8 + ld) {")
    for c in classes:
        info = gen_sizes(*c)
        d.append("    case %d: *nacc = %d; *slots = %d; return true;" % (ckey(c), *info))
    d.append("  }")
    d.append("  return false;")
    d.append("}")
    d.append("}  // namespace lgx")
    _write_if_changed(os.path.join(GEN_DIR, "post_dispatch.cu"), "\n".join(d) + "\n")
    return names + ["post_dispatch.cu"]


def gen_sizes(la, lb, lc, ld):
    nacc = sum(ncart(le) * ncart(lf) for le in range(la, la + lb + 1)
               for lf in range(lc, lc + ld + 1))
    nf = sum(ncart(lf) for lf in range(lc, lc + ld + 1))
    nfp = nf if nf % 2 else nf + 1
    nab = nsph(la) * nsph(lb)
    return nacc, nacc + nab * nfp + nab * nsph(lc) * nsph(ld)


if __name__ == "__main__":
    print("\n".join(main()))
