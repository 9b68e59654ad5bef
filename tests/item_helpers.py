"""Test data of the ItemIntegrator tests: the reference's exact test
polynomials (test/runtests.jl:38-78, exact_function2D / exact_function3D:
vector fields whose components are sums of x_k^p with fixed coefficients) as
polynomial data records (component, coefficient, e1, e2, e3), their gradients
(component-major, the layout of the Gradient operator), and a point
evaluator for interpolation."""
import numpy as np

# (component, coefficient, exponent vector / p) of exact_function{2,3}D(p): a
# term (c, a, k) stands for a * x_k^p; k = -1 is the constant a
_EXACT = {
    2: [(0, 1.0, 0), (0, 2.0, 1), (0, 1.0, -1), (1, 3.0, 0), (1, -1.0, 1), (1, -1.0, -1)],
    3: [(0, 2.0, 2), (0, -1.0, 1), (0, -1.0, -1), (1, 1.0, 0), (1, 2.0, 1), (1, 1.0, -1),
        (2, 3.0, 0), (2, -1.0, 1), (2, -1.0, -1)],
}


def exact_terms(dim, p):
    """Polynomial records of exact_function{dim}D(p) (dim components)."""
    out = []
    for c, a, k in _EXACT[dim]:
        e = [0.0, 0.0, 0.0]
        if k >= 0:
            e[k] = float(p)
        out.append((c, a, *e))
    return np.array(out)


def exact_gradient_terms(dim, p):
    """Records of the gradient: component c*dim + j = d/dx_j of component c."""
    out = []
    for c, a, k in _EXACT[dim]:
        if k < 0 or p == 0:
            continue
        e = [0.0, 0.0, 0.0]
        e[k] = float(p - 1)
        out.append((c * dim + k, a * p, *e))
    return np.array(out)


def exact_eval(dim, p, x):
    """Values of exact_function{dim}D(p) at points x (m, dim) -> (m, dim)."""
    y = np.zeros((x.shape[0], dim))
    for c, a, k in _EXACT[dim]:
        y[:, c] += a * (x[:, k] ** p if k >= 0 else 1.0)
    return y
