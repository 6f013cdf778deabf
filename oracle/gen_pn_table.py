"""Generate oracle/pn_table.h: the post-Newtonian pair terms as monomial tables.

TEST INFRASTRUCTURE (one-time generator for the oracle's data).  Run here,
with the reference tree's root in TUPAN_REF:

    python oracle/gen_pn_table.py $TUPAN_REF/tupan/lib/src/pn_terms.h

It reads the reference's PN expressions (tupan/lib/src/pn_terms.h:126-567:
p2p_pn2, p2p_pn4, p2p_pn5, p2p_pn6, p2p_pn7), expands each `a` and `b`
polynomial with sympy into a sum of monomials over ten base variables, and
writes them as a C table.  The oracle evaluates the table generically
(tupan_oracle.c: pn_eval), which is a different evaluation structure from the
reference's nested forms: same polynomial, independent rounding.  The table is
the physics (coefficients of the 1, 2, 2.5, 3 and 3.5 PN two-body equations of
motion) and has to be alike; the output is committed so the GPU machine, which
has no reference tree, can build the oracle.
"""
import re
import sys

import sympy as sp

BASE = ["im", "jm", "inv_r", "iv2", "jv2", "ivjv", "niv", "njv", "nv", "v2"]
ENUM = ["PN_IM", "PN_JM", "PN_IR", "PN_IV2", "PN_JV2", "PN_IVJV",
        "PN_NIV", "PN_NJV", "PN_NV", "PN_V2"]
# order tag -> (c power, minimum clight.order that enables it, extra factor)
ORDERS = {"2": (2, 2, None), "4": (4, 4, None), "5": (5, 5, "im*inv_r"),
          "6": (6, 6, None), "7": (7, 7, "im*inv_r")}


def expressions(text, tag):
    """Return the C source of pn<tag>->a and pn<tag>->b."""
    body = text[text.index("p2p_pn%s(" % tag):]
    out = {}
    for comp in ("a", "b"):
        m = re.search(r"pn%s->%s\s*=(.*?);" % (tag, comp), body, re.S)
        out[comp] = m.group(1)
    return out


def to_sympy(src, syms):
    src = re.sub(r"//[^\n]*", "", src)
    src = re.sub(r"\b_(\d+)_(\d+)\b", r"sp.Rational(\1,\2)", src)
    derived = {
        "im2": "im**2", "jm2": "jm**2", "imjm": "(im*jm)", "jv4": "jv2**2",
        "iv4": "iv2**2", "ivjvivjv": "ivjv**2", "niv2": "niv**2",
        "njv2": "njv**2", "nivnjv": "(niv*njv)", "nvnv": "nv**2",
        "inv_r2": "inv_r**2",
    }
    for k, v in derived.items():
        src = re.sub(r"\b%s\b" % k, v, src)
    src = "(" + " ".join(src.split()) + ")"
    env = dict(syms)
    env["sp"] = sp
    env["PI2"] = sp.Symbol("PI2")
    return eval(src, env)


def main(path):
    text = open(path).read()
    syms = {n: sp.Symbol(n) for n in BASE}
    PI2 = 9.869604401089358
    lines = []
    lines.append("/* Generated by oracle/gen_pn_table.py -- do not edit. */")
    lines.append("/* TEST INFRASTRUCTURE: PN two-body terms as monomial tables. */")
    lines.append("#ifndef PN_TABLE_H\n#define PN_TABLE_H")
    lines.append("enum { %s, PN_NVAR };" % ", ".join(ENUM))
    lines.append("struct pn_mono { double c; unsigned char e[PN_NVAR]; };")
    lines.append("struct pn_order { unsigned long min_order; int cpow; "
                 "const struct pn_mono *a; int na; const struct pn_mono *b; int nb; };")
    tabs = []
    for tag, (cpow, minord, extra) in ORDERS.items():
        ex = expressions(text, tag)
        for comp in ("a", "b"):
            e = to_sympy(ex[comp], syms)
            if extra:
                e = e * to_sympy(extra, syms)
            e = sp.expand(e)
            poly = sp.Poly(e, *[syms[n] for n in BASE])
            name = "pn%s_%s" % (tag, comp)
            rows = []
            for monom, coeff in poly.terms():
                cval = float(coeff.subs(sp.Symbol("PI2"), PI2))
                rows.append("  {%.17g, {%s}}" % (cval, ",".join(str(k) for k in monom)))
            lines.append("static const struct pn_mono %s[] = {\n%s\n};" % (name, ",\n".join(rows)))
            tabs.append((name, len(rows)))
        lines.append("")
    lines.append("#define PN_NORDERS 5")
    lines.append("static const struct pn_order pn_orders[PN_NORDERS] = {")
    k = 0
    for tag, (cpow, minord, extra) in ORDERS.items():
        (na_name, na), (nb_name, nb) = tabs[k], tabs[k + 1]
        k += 2
        lines.append("  {%dul, %d, %s, %d, %s, %d}," % (minord, cpow, na_name, na, nb_name, nb))
    lines.append("};")
    lines.append("#endif")
    out = __file__.replace("gen_pn_table.py", "pn_table.h")
    open(out, "w").write("\n".join(lines) + "\n")
    print("wrote", out, [t for t in tabs])


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: %s <reference root>/tupan/lib/src/pn_terms.h" % sys.argv[0])
    main(sys.argv[1])
