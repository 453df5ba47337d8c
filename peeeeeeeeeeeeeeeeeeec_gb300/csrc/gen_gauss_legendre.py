"""Generate gauss_legendre_table.h: Gauss-Legendre nodes and weights on [-1, 1].

The nodes are the roots of the Legendre polynomial P_n, found to 40 digits by
sympy; the weights are w_i = 2 / ((1 - x_i^2) P_n'(x_i)^2).  Each value is
rounded once to binary64 and written as a C99 hex-float literal, so the table
is exact and identical on every compiler.  Orders: 2 3 4 5 6 8 10 12 16 (the
set the reference tabulates in quadrature.c:94-313).

Run:  python gen_gauss_legendre.py > gauss_legendre_table.h
"""
import sympy as sp

ORDERS = [2, 3, 4, 5, 6, 8, 10, 12, 16]


def rule(n):
    x = sp.symbols("x")
    p = sp.legendre_poly(n, x, polys=True)
    dp = p.diff(x)
    roots = sorted(sp.Poly(p).nroots(n=40, maxsteps=400))
    nodes, weights = [], []
    for r in roots:
        r = sp.Float(0) if abs(r) < sp.Float("1e-30") else r
        nodes.append(float(r))
        weights.append(float(2 / ((1 - r ** 2) * dp.eval(r) ** 2)))
    # exact mirror symmetry, as in any tabulated rule
    for i in range(n // 2):
        nodes[n - 1 - i] = -nodes[i]
        weights[n - 1 - i] = weights[i]
    return nodes, weights


def main():
    print("/* Generated by gen_gauss_legendre.py; do not edit. */")
    print("#ifndef PEEC_GB300_GAUSS_LEGENDRE_TABLE_H")
    print("#define PEEC_GB300_GAUSS_LEGENDRE_TABLE_H")
    print("/* Row r holds order GL_ORDERS[r]; unused slots are 0. */")
    print("#define GL_NUM_ORDERS %d" % len(ORDERS))
    print("static const int GL_ORDERS[GL_NUM_ORDERS] = {%s};" % ", ".join(map(str, ORDERS)))
    xs, ws = [], []
    for n in ORDERS:
        x, w = rule(n)
        xs.append(x + [0.0] * (16 - n))
        ws.append(w + [0.0] * (16 - n))
    for name, tab in (("GL_NODES", xs), ("GL_WEIGHTS", ws)):
        print("static const double %s[GL_NUM_ORDERS][16] = {" % name)
        for row in tab:
            print("    {" + ", ".join(v.hex() if v != 0 else "0.0" for v in row) + "},")
        print("};")
    print("#endif")


if __name__ == "__main__":
    main()
