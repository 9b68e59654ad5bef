"""Generate tests/golden/p2_reference_matrices.json.

Exact (sympy, rational arithmetic) stiffness and mass matrices of the H1P1 and
H1P2 bases on the reference triangle and tetrahedron, with the basis order of
src/fedefs/h1_p1.jl:64-75 and src/fedefs/h1_p2.jl:134-165.  These are
known-answer values independent of any quadrature rule; the oracle's FP64
assembly on a single reference cell must reproduce them.

Run:  python tests/golden/make_golden.py
"""
import json
import os

import sympy as sp


def bases(dim, fe):
    x = sp.symbols("x0:%d" % dim)
    r = 1 - sum(x)
    if fe == 1:
        return x, [r] + list(x)
    if dim == 2:
        return x, [2 * r * (r - sp.Rational(1, 2)), 2 * x[0] * (x[0] - sp.Rational(1, 2)),
                   2 * x[1] * (x[1] - sp.Rational(1, 2)), 4 * r * x[0], 4 * x[0] * x[1], 4 * x[1] * r]
    return x, [2 * r * (r - sp.Rational(1, 2)), 2 * x[0] * (x[0] - sp.Rational(1, 2)),
               2 * x[1] * (x[1] - sp.Rational(1, 2)), 2 * x[2] * (x[2] - sp.Rational(1, 2)),
               4 * r * x[0], 4 * r * x[1], 4 * r * x[2], 4 * x[0] * x[1], 4 * x[0] * x[2], 4 * x[1] * x[2]]


def integrate_simplex(expr, x):
    if len(x) == 2:
        return sp.integrate(sp.integrate(expr, (x[1], 0, 1 - x[0])), (x[0], 0, 1))
    return sp.integrate(sp.integrate(sp.integrate(expr, (x[2], 0, 1 - x[0] - x[1])), (x[1], 0, 1 - x[0])),
                        (x[0], 0, 1))


def main():
    out = {}
    for dim in (2, 3):
        for fe in (1, 2):
            x, phi = bases(dim, fe)
            n = len(phi)
            K = [[sp.nsimplify(integrate_simplex(sum(sp.diff(phi[a], v) * sp.diff(phi[b], v) for v in x), x))
                  for b in range(n)] for a in range(n)]
            M = [[integrate_simplex(phi[a] * phi[b], x) for b in range(n)] for a in range(n)]
            out[f"P{fe}_{dim}d_stiffness"] = {"dim": dim, "fe": fe, "kind": "stiffness",
                                             "exact": [[str(v) for v in row] for row in K],
                                             "matrix": [[float(v) for v in row] for row in K]}
            out[f"P{fe}_{dim}d_mass"] = {"dim": dim, "fe": fe, "kind": "mass",
                                        "exact": [[str(v) for v in row] for row in M],
                                        "matrix": [[float(v) for v in row] for row in M]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "p2_reference_matrices.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
