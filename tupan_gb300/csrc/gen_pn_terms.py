"""Generate tg_pn_terms.cuh: straight-line CUDA for the post-Newtonian pair terms.

One-time generator, run with the reference tree's root in TUPAN_REF:

    python tupan_gb300/csrc/gen_pn_terms.py $TUPAN_REF/tupan/lib/src/pn_terms.h

The post-Newtonian two-body accelerations (1PN, 2PN, 2.5PN, 3PN and 3.5PN
terms of the harmonic-coordinate equations of motion) are a fixed table of
rational coefficients; the reference states them in
tupan/lib/src/pn_terms.h:126-567 (p2p_pn2/4/5/6/7).  This script reads those
expressions, expands every `a` and `b` factor with sympy into monomials over
ten pair invariants, groups the monomials by their mass/distance prefactor
(im^p jm^q inv_r^k) and emits a templated device function that evaluates each
group as prefactor * (linear combination of velocity monomials).  Powers and
products of the invariants are computed once and shared between groups.  The
generated header is committed; the build never needs the reference tree.
"""
import re
import sys
from collections import defaultdict

import sympy as sp

BASE = ["im", "jm", "inv_r", "iv2", "jv2", "ivjv", "niv", "njv", "nv", "v2"]
MASSY = ("im", "jm", "inv_r")
VELO = ("iv2", "jv2", "ivjv", "niv", "njv", "nv", "v2")
# tag -> (c power, min order, extra factor folded into the term)
ORDERS = [("2", 2, 2, None), ("4", 4, 4, None), ("5", 5, 5, "im*inv_r"),
          ("6", 6, 6, None), ("7", 7, 7, "im*inv_r")]
PI2 = 9.869604401089358


def expressions(text, tag):
    body = text[text.index("p2p_pn%s(" % tag):]
    out = {}
    for comp in ("a", "b"):
        m = re.search(r"pn%s->%s\s*=(.*?);" % (tag, comp), body, re.S)
        out[comp] = m.group(1)
    return out


def to_sympy(src, syms):
    src = re.sub(r"//[^\n]*", "", src)
    src = re.sub(r"\b_(\d+)_(\d+)\b", r"sp.Rational(\1,\2)", src)
    derived = {"im2": "im**2", "jm2": "jm**2", "imjm": "(im*jm)", "jv4": "jv2**2",
               "iv4": "iv2**2", "ivjvivjv": "ivjv**2", "niv2": "niv**2",
               "njv2": "njv**2", "nivnjv": "(niv*njv)", "nvnv": "nv**2",
               "inv_r2": "inv_r**2"}
    for k, v in derived.items():
        src = re.sub(r"\b%s\b" % k, v, src)
    src = "(" + " ".join(src.split()) + ")"
    env = dict(syms)
    env["sp"] = sp
    env["PI2"] = sp.Symbol("PI2")
    return eval(src, env)


def pow_name(var, k):
    return var if k == 1 else "%s_%d" % (var, k)


def mono_name(exps, names):
    parts = [pow_name(n, e) for n, e in zip(names, exps) if e]
    return "_x_".join(parts) if parts else None


def main(path):
    text = open(path).read()
    syms = {n: sp.Symbol(n) for n in BASE}
    groups_by_order = []
    powers = defaultdict(int)           # var -> max power needed
    products = {}                        # name -> list of (var, k)
    for tag, cpow, minord, extra in ORDERS:
        ex = expressions(text, tag)
        comp_groups = {}
        for comp in ("a", "b"):
            e = to_sympy(ex[comp], syms)
            if extra:
                e = e * to_sympy(extra, syms)
            poly = sp.Poly(sp.expand(e), *[syms[n] for n in BASE])
            groups = defaultdict(list)
            for monom, coeff in poly.terms():
                mexp = monom[:3]
                vexp = monom[3:]
                c = float(coeff.subs(sp.Symbol("PI2"), PI2))
                groups[mexp].append((c, vexp))
                for n, k in zip(BASE, monom):
                    powers[n] = max(powers[n], k)
            comp_groups[comp] = groups
        groups_by_order.append((tag, cpow, minord, comp_groups))

    out = []
    w = out.append
    w("// Generated by tupan_gb300/csrc/gen_pn_terms.py -- do not edit.")
    w("// Post-Newtonian pair factors A (along r) and B (along v) of the")
    w("// two-body equations of motion, orders 1, 2, 2.5, 3, 3.5 PN, as in")
    w("// tupan/lib/src/pn_terms.h:126-567 (same coefficients, own evaluation).")
    w("#pragma once")
    w("namespace tg {")
    w("template <class T>")
    w("__device__ __forceinline__ void pn_factors(unsigned long order,")
    w("    T im, T jm, T inv_r, T iv2, T jv2, T ivjv, T niv, T njv, T nv, T v2,")
    w("    T inv2, T inv4, T inv5, T inv6, T inv7, T &A, T &B)")
    w("{")
    w("    A = T(0); B = T(0);")
    w("    if (order < 2) return;")
    # power ladders
    for n in BASE:
        for k in range(2, powers[n] + 1):
            w("    const T %s = %s * %s;" % (pow_name(n, k), pow_name(n, k - 1), n))
    invmap = {2: "inv2", 4: "inv4", 5: "inv5", 6: "inv6", 7: "inv7"}
    declared = set()

    def need_product(exps, names, indent):
        nm = mono_name(exps, names)
        if nm is None or nm in declared:
            return nm
        factors = [pow_name(n, e) for n, e in zip(names, exps) if e]
        if len(factors) == 1:
            return factors[0]
        # build incrementally from the first factors
        prev = factors[0]
        for i in range(1, len(factors)):
            cur = "_x_".join(factors[:i + 1])
            if cur not in declared:
                w("%sconst T %s = %s * %s;" % (indent, cur, prev, factors[i]))
                declared.add(cur)
            prev = cur
        return nm

    for tag, cpow, minord, comp_groups in groups_by_order:
        w("    if (order >= %dul) {" % minord)
        declared.clear()   # products are block-scoped; the compiler merges repeats
        for comp in ("a", "b"):
            w("        T %s%s = T(0);" % (comp, tag))
            for mexp, terms in sorted(comp_groups[comp].items()):
                mname = need_product(mexp, MASSY, "        ")
                # velocity polynomial of this group
                acc = "v%s%s_%s" % (comp, tag, "_".join(str(x) for x in mexp))
                first = True
                for c, vexp in terms:
                    vname = need_product(vexp, VELO, "        ")
                    cs = "T(%.17g)" % c
                    if first:
                        expr = cs if vname is None else "%s * %s" % (cs, vname)
                        w("        T %s = %s;" % (acc, expr))
                        first = False
                    else:
                        if vname is None:
                            w("        %s += %s;" % (acc, cs))
                        else:
                            w("        %s = fma(%s, %s, %s);" % (acc, cs, vname, acc))
                if mname is None:
                    w("        %s%s += %s;" % (comp, tag, acc))
                else:
                    w("        %s%s = fma(%s, %s, %s%s);" % (comp, tag, mname, acc, comp, tag))
        w("        A = fma(%s, a%s, A);" % (invmap[cpow], tag))
        w("        B = fma(%s, b%s, B);" % (invmap[cpow], tag))
        w("    }")
    w("}")
    w("}  // namespace tg")
    dst = __file__.replace("gen_pn_terms.py", "tg_pn_terms.cuh")
    open(dst, "w").write("\n".join(out) + "\n")
    print("wrote", dst, len(out), "lines")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: %s <reference root>/tupan/lib/src/pn_terms.h" % sys.argv[0])
    main(sys.argv[1])
