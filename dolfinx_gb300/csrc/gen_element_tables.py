"""Generate element_tables.h: exact reference tensors of Lagrange P1/P2 on
the reference tetrahedron, emitted as straight-line CUDA device code.

Run from the package root:  python dolfinx_gb300/csrc/gen_element_tables.py

The element matrix of a(u,v) = \\int kappa grad u.grad v + k2 u v on an
affine tetrahedron is
    A_ij = sum_{a<=b} G_ab Shat_ab[i][j] + k2 |detJ| M[i][j],
    G_ab = kappa |detJ| sum_m K_am K_bm,   K = J^{-1},
with Shat_aa = S_aa, Shat_ab = S_ab + S_ba (a<b) and
S_ab[i][j] = \\int_ref d_a phi_i d_b phi_j dX. Only non-zero terms are
emitted, so the FP64 operation count per element is minimal (FP64 is the
scarce resource on GB300). Basis and dof order follow Basix (vertices,
then edges (2,3),(1,3),(1,2),(0,3),(0,2),(0,1)).
"""

import os

import sympy as sp

X, Y, Z = sp.symbols("X Y Z")
LAM = [1 - X - Y - Z, X, Y, Z]
EDGES = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]
# G component order: 00, 11, 22, 01, 02, 12
GAB = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def basis(deg):
    if deg == 1:
        return list(LAM)
    return [LAM[i] * (2 * LAM[i] - 1) for i in range(4)] + [4 * LAM[a] * LAM[b] for a, b in EDGES]


def integ(f):
    return sp.integrate(sp.integrate(sp.integrate(sp.expand(f), (Z, 0, 1 - X - Y)), (Y, 0, 1 - X)),
                        (X, 0, 1))


def lit(c):
    c = sp.nsimplify(c)
    return "(%s)" % sp.N(c, 20) if c.q == 1 else "(%d.0/%d.0)" % (c.p, c.q)


def gen(deg):
    phi = basis(deg)
    nd = len(phi)
    d = [[sp.diff(p, v) for v in (X, Y, Z)] for p in phi]
    S = {(a, b): [[integ(d[i][a] * d[j][b]) for j in range(nd)] for i in range(nd)]
         for a in range(3) for b in range(3)}
    M = [[integ(phi[i] * phi[j]) for j in range(nd)] for i in range(nd)]
    F = [[integ(phi[i] * LAM[p]) for p in range(4)] for i in range(nd)]
    W = [integ(phi[i]) for i in range(nd)]
    out = []
    out.append("// Upper triangle (row-major, i <= j) of the P%d stiffness + mass element" % deg)
    out.append("// matrix: A[k] for k = packed index of (i, j); G per GAB order.")
    out.append("template <bool MASS>")
    out.append("__device__ __forceinline__ void tet_p%d_poisson_upper(const double* G, double mk2,"
               " double* A)\n{" % deg)
    k = 0
    nterms = 0
    mass = []
    for i in range(nd):
        for j in range(i, nd):
            terms = []
            for g, (a, b) in enumerate(GAB):
                c = S[a, b][i][j] + (S[b, a][i][j] if a != b else 0)
                if c != 0:
                    terms.append("%s * G[%d]" % (lit(c), g))
            nterms += len(terms)
            expr = " + ".join(terms) if terms else "0.0"
            out.append("  A[%d] = %s;" % (k, expr))
            mass.append("    A[%d] += mk2 * %s;" % (k, lit(M[i][j])))
            k += 1
    out.append("  if constexpr (MASS)\n  {")
    out.extend(mass)
    out.append("  }")
    out.append("}")
    out.append("// %d stiffness terms" % nterms)
    out.append("// Source tensor F[i][p] = int_ref phi_i lambda_p (P1 coefficient).")
    out.append("__device__ __forceinline__ void tet_p%d_source(const double* f, double adet,"
               " double* b)\n{" % deg)
    for i in range(nd):
        terms = ["%s * f[%d]" % (lit(F[i][p]), p) for p in range(4) if F[i][p] != 0]
        out.append("  b[%d] = adet * (%s);" % (i, " + ".join(terms)))
    out.append("}")
    out.append("// int_ref phi_i (body force with a constant vector).")
    out.append("__constant__ double kTetP%dIntegral[%d] = {%s};"
               % (deg, nd, ", ".join(lit(w) for w in W)))
    return "\n".join(out)


def gen_p2_gradients():
    """Reference gradients of the P2 basis at the 4-point degree-2 rule
    (barycentric (a,b,b,b) and permutations, weights 1/24)."""
    a = (5 + 3 * sp.sqrt(5)) / 20
    b = (5 - sp.sqrt(5)) / 20
    phi = basis(2)
    d = [[sp.diff(p, v) for v in (X, Y, Z)] for p in phi]
    rows = []
    for q in range(4):
        lam = [b, b, b, b]
        lam[q] = a
        pt = {X: lam[1], Y: lam[2], Z: lam[3]}
        vals = []
        for i in range(10):
            vals.append("{%s}" % ", ".join("%.17g" % float(sp.N(d[i][k].subs(pt), 30))
                                           for k in range(3)))
        rows.append("  {%s}" % ", ".join(vals))
    return ("// P2 reference gradients at the 4-point rule, [q][i][X,Y,Z]; weight 1/24 each.\n"
            "__constant__ double kP2GradQ4[4][10][3] = {\n%s};\n" % ",\n".join(rows))


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    body = [
        "// Generated by gen_element_tables.py -- do not edit by hand.",
        "// Exact reference tensors for Lagrange P1/P2 on the reference tetrahedron.",
        "#pragma once",
        "",
        gen(1),
        "",
        gen(2),
        "",
        gen_p2_gradients(),
    ]
    with open(os.path.join(here, "element_tables.h"), "w") as fh:
        fh.write("\n".join(body))


if __name__ == "__main__":
    main()
