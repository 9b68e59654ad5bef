// Quadrature rules and reference-element basis tables (host side).
//
// Quadrature: src/quadrature.jl (Triangle2D :173-194, Tetrahedron3D :268-325,
// Gauss :506-525, Stroud conical product :528-562).  Basis derivatives are
// computed with forward-mode dual numbers in the operation order ForwardDiff
// uses (value*partials products as  vy*px + vx*py), so the tables agree with
// the reference's _prepare_derivatives (src/feevaluator.jl:235-293) to the
// last bit wherever the inputs do.  This file must be compiled without FMA
// contraction (-ffp-contract=off), as Julia evaluates `a*b + c` unfused.
#include <cmath>
#include <cstring>

#include "grmp_internal.h"

namespace {

// Golub-Welsch: eigenvalues (ascending) and first eigenvector components of a
// symmetric tridiagonal matrix, by cyclic Jacobi rotations.
void tridiag_eig(int n, const double *diag, const double *off, double *ev, double *v1) {
    double a[16][16], v[16][16];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            a[i][j] = 0.0;
            v[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int i = 0; i < n; i++) a[i][i] = diag[i];
    for (int i = 0; i + 1 < n; i++) a[i][i + 1] = a[i + 1][i] = off[i];
    for (int sweep = 0; sweep < 100; sweep++) {
        double s2 = 0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) s2 += a[p][q] * a[p][q];
        if (s2 < 1e-300) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                if (std::fabs(a[p][q]) < 1e-300) continue;
                double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double x = a[k][p], y = a[k][q];
                    a[k][p] = c * x - s * y;
                    a[k][q] = s * x + c * y;
                }
                for (int k = 0; k < n; k++) {
                    double x = a[p][k], y = a[q][k];
                    a[p][k] = c * x - s * y;
                    a[q][k] = s * x + c * y;
                }
                for (int k = 0; k < n; k++) {
                    double x = v[k][p], y = v[k][q];
                    v[k][p] = c * x - s * y;
                    v[k][q] = s * x + c * y;
                }
            }
    }
    int idx[16];
    for (int i = 0; i < n; i++) idx[i] = i;
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (a[idx[j]][idx[j]] < a[idx[i]][idx[i]]) std::swap(idx[i], idx[j]);
    for (int i = 0; i < n; i++) {
        ev[i] = a[idx[i]][idx[i]];
        double nrm = 0;
        for (int k = 0; k < n; k++) nrm += v[k][idx[i]] * v[k][idx[i]];
        v1[i] = v[0][idx[i]] / std::sqrt(nrm);
    }
}

int stroud(int order, double (*x)[3], double *w) {
    int n = order / 2 + 1;
    double dg[16] = {0}, of[16], r[16], a[16], s[16], b[16], v1[16];
    for (int i = 1; i < n; i++) of[i - 1] = i / std::sqrt(4.0 * i * i - 1.0);
    tridiag_eig(n, dg, of, r, v1);
    for (int i = 0; i < n; i++) a[i] = 2.0 * v1[i] * v1[i];
    for (int i = 1; i <= n; i++) dg[i - 1] = -1.0 / (4.0 * i * i - 1.0);
    for (int i = 1; i < n; i++) of[i - 1] = std::sqrt((double)(i + 1) * i) / (2.0 * (i + 1) - 1.0);
    tridiag_eig(n, dg, of, s, v1);
    for (int i = 0; i < n; i++) b[i] = 2.0 * v1[i] * v1[i];
    for (int i = 0; i < n; i++) {
        r[i] = 0.5 * r[i] + 0.5;
        s[i] = 0.5 * s[i] + 0.5;
        a[i] = 0.5 * a[i];
        b[i] = 0.5 * b[i];
    }
    int q = 0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++, q++) {
            x[q][0] = s[j] * 1.0 - r[i] * (s[j] - 1.0) * 0.0;
            x[q][1] = s[j] * 0.0 - r[i] * (s[j] - 1.0) * 1.0;
            x[q][2] = 0.0;
            w[q] = a[i] * b[j];
        }
    return q;
}

// ------------------------------------------------------------------ duals
struct D {
    double v, d[3];
};
inline D var(double x, int j) {
    D r{x, {0, 0, 0}};
    r.d[j] = 1.0;
    return r;
}
inline D mul(D x, D y) {
    D r;
    r.v = x.v * y.v;
    for (int i = 0; i < 3; i++) r.d[i] = y.v * x.d[i] + x.v * y.d[i];
    return r;
}
inline D scal(double c, D x) {
    D r;
    r.v = c * x.v;
    for (int i = 0; i < 3; i++) r.d[i] = c * x.d[i];
    return r;
}
inline D subc(D x, double c) {
    D r = x;
    r.v = x.v - c;
    return r;
}
inline D csub(double c, D x) {
    D r;
    r.v = c - x.v;
    for (int i = 0; i < 3; i++) r.d[i] = -x.d[i];
    return r;
}
inline D sub(D x, D y) {
    D r;
    r.v = x.v - y.v;
    for (int i = 0; i < 3; i++) r.d[i] = x.d[i] - y.d[i];
    return r;
}

// Scalar basis functions (one component).  H1P1: src/fedefs/h1_p1.jl:64-75;
// H1P2: src/fedefs/h1_p2.jl:134-165; H1BR (2D): the P1 functions followed by
// the three face bubbles, src/fedefs/h1v_br.jl:117-130.
int scalar_basis(int fe, int dim, const D *x, D *o) {
    if (fe == GRMP_FE_H1P1 || fe == GRMP_FE_H1BR) {
        D r = csub(1.0, x[0]);
        for (int j = 1; j < dim; j++) r = sub(r, x[j]);
        o[0] = r;
        for (int j = 0; j < dim; j++) o[1 + j] = x[j];
        if (fe == GRMP_FE_H1P1) return dim + 1;
        if (dim == 3) {
            // face bubbles of the faces [0,1,2], [0,1,3], [1,2,3], [0,2,3]
            // (src/fedefs/h1v_br.jl:221-233), products left to right
            o[4] = mul(mul(scal(60.0, x[0]), r), x[1]);
            o[5] = mul(mul(scal(60.0, r), x[0]), x[2]);
            o[6] = mul(mul(scal(60.0, x[0]), x[1]), x[2]);
            o[7] = mul(mul(scal(60.0, r), x[1]), x[2]);
            return 8;
        }
        o[3] = mul(scal(6.0, x[0]), r);
        o[4] = mul(scal(6.0, x[1]), x[0]);
        o[5] = mul(scal(6.0, r), x[1]);
        return 6;
    }
    if (fe == GRMP_FE_H1P2 && dim == 2) {
        D r = sub(csub(1.0, x[0]), x[1]);
        o[0] = mul(scal(2.0, r), subc(r, 0.5));
        o[1] = mul(scal(2.0, x[0]), subc(x[0], 0.5));
        o[2] = mul(scal(2.0, x[1]), subc(x[1], 0.5));
        o[3] = mul(scal(4.0, r), x[0]);
        o[4] = mul(scal(4.0, x[0]), x[1]);
        o[5] = mul(scal(4.0, x[1]), r);
        return 6;
    }
    if (fe == GRMP_FE_H1P2 && dim == 3) {
        D r = sub(sub(csub(1.0, x[0]), x[1]), x[2]);
        o[0] = mul(scal(2.0, r), subc(r, 0.5));
        o[1] = mul(scal(2.0, x[0]), subc(x[0], 0.5));
        o[2] = mul(scal(2.0, x[1]), subc(x[1], 0.5));
        o[3] = mul(scal(2.0, x[2]), subc(x[2], 0.5));
        o[4] = mul(scal(4.0, r), x[0]);
        o[5] = mul(scal(4.0, r), x[1]);
        o[6] = mul(scal(4.0, r), x[2]);
        o[7] = mul(scal(4.0, x[0]), x[1]);
        o[8] = mul(scal(4.0, x[0]), x[2]);
        o[9] = mul(scal(4.0, x[1]), x[2]);
        return 10;
    }
    if (fe == GRMP_FE_L2P0) {
        o[0] = D{1.0, {0, 0, 0}};
        return 1;
    }
    return 0;
}

}  // namespace

int grmp_fe_polyorder(int fe, int dim) {
    switch (fe) {
        case GRMP_FE_H1P1: return 1;
        case GRMP_FE_H1P2: return 2;
        case GRMP_FE_H1BR: return dim == 2 ? 2 : 3;
        case GRMP_FE_L2P0: return 0;
        case GRMP_FE_HDIVRT0: return 1;
        case GRMP_FE_HDIVBDM1: return 1;
    }
    return -1;
}

int grmp_fe_nb(int fe, int dim) {
    switch (fe) {
        case GRMP_FE_H1P1: return dim + 1;
        case GRMP_FE_H1P2: return dim == 2 ? 6 : 10;
        case GRMP_FE_H1BR: return dim == 2 ? 6 : 8;
        case GRMP_FE_L2P0: return 1;
    }
    return 0;
}

int grmp_fe_ldofs(int fe, int dim, int ncomp) {
    switch (fe) {
        case GRMP_FE_H1P1: return (dim + 1) * ncomp;
        case GRMP_FE_H1P2: return (dim == 2 ? 6 : 10) * ncomp;
        case GRMP_FE_H1BR: return dim == 2 ? 9 : 16;
        case GRMP_FE_L2P0: return ncomp;
        case GRMP_FE_HDIVRT0: return dim + 1;
    }
    return 0;
}

int grmp_quadrature(int dim, int order, double (*x)[3], double *w) {
    std::memset(x, 0, sizeof(double) * 3 * GRMP_MAXQ);
    if (order < 0) order = 0;
    if (dim == 2) {
        if (order <= 1) {
            x[0][0] = x[0][1] = 1.0 / 3.0;
            w[0] = 1.0;
            return 1;
        }
        if (order == 2) {
            x[0][0] = 0.5; x[0][1] = 0.5;
            x[1][0] = 0.0; x[1][1] = 0.5;
            x[2][0] = 0.5; x[2][1] = 0.0;
            w[0] = w[1] = w[2] = 1.0 / 3.0;
            return 3;
        }
        if (order <= 20) return stroud(order, x, w);   // orders 8, 12-14 use the reference's symmetric tables
        return 0;
    }
    if (dim == 3) {
        if (order <= 1) {
            x[0][0] = x[0][1] = x[0][2] = 0.25;
            w[0] = 1.0;
            return 1;
        }
        if (order == 2) {
            const double a = 0.1381966011250105, b = 0.5854101966249685;
            const double p[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
            for (int i = 0; i < 4; i++) {
                for (int k = 0; k < 3; k++) x[i][k] = p[i][k];
                w[i] = 0.25;
            }
            return 4;
        }
        if (order == 3) {
            const double p[5][3] = {{1.0 / 4, 1.0 / 4, 1.0 / 4}, {1.0 / 2, 1.0 / 6, 1.0 / 6}, {1.0 / 6, 1.0 / 6, 1.0 / 6},
                                    {1.0 / 6, 1.0 / 6, 1.0 / 2}, {1.0 / 6, 1.0 / 2, 1.0 / 6}};
            const double ww[5] = {-4.0 / 5, 9.0 / 20, 9.0 / 20, 9.0 / 20, 9.0 / 20};
            for (int i = 0; i < 5; i++) {
                for (int k = 0; k < 3; k++) x[i][k] = p[i][k];
                w[i] = ww[i];
            }
            return 5;
        }
        if (order == 4) {
            const double c = 0.2500000000000000, d = 0.7857142857142857, e = 0.0714285714285714,
                         f = 0.1005964238332008, g = 0.3994035761667992;
            const double p[11][3] = {{c, c, c}, {d, e, e}, {e, e, e}, {e, e, d}, {e, d, e}, {f, g, g},
                                     {g, f, g}, {g, g, f}, {g, f, f}, {f, g, f}, {f, f, g}};
            const double w1 = -0.0789333333333333, w2 = 0.0457333333333333, w3 = 0.1493333333333333;
            const double ww[11] = {w1, w2, w2, w2, w2, w3, w3, w3, w3, w3, w3};
            for (int i = 0; i < 11; i++) {
                for (int k = 0; k < 3; k++) x[i][k] = p[i][k];
                w[i] = ww[i];
            }
            return 11;
        }
        return 0;
    }
    return 0;
}

int grmp_tables(int dim, int fe, int order, RefTables *t) {
    std::memset(t, 0, sizeof(RefTables));
    t->dim = dim;
    t->nq = grmp_quadrature(dim, order, t->xref, t->w);
    if (t->nq == 0) return GRMP_ERR_UNSUPPORTED;
    for (int q = 0; q < t->nq; q++) {
        D x[3], o[GRMP_MAX_LDOFS];
        for (int j = 0; j < dim; j++) x[j] = var(t->xref[q][j], j);
        int nb = scalar_basis(fe, dim, x, o);
        if (nb == 0) return GRMP_ERR_UNSUPPORTED;
        t->nb = nb;
        for (int a = 0; a < nb; a++) {
            t->vals[q][a] = o[a].v;
            for (int j = 0; j < dim; j++) t->derivs[q][a][j] = o[a].d[j];
        }
    }
    return GRMP_OK;
}

extern "C" int grmp_reference_tables(int dim, int fe_kind, int order, int *nq, int *nb, double *xref, double *w,
                                     double *vals, double *derivs) {
    if (dim != 2 && dim != 3) return GRMP_ERR_INVALID_ARG;
    static RefTables t;   // large; host-only query
    static std::mutex m;
    std::lock_guard<std::mutex> lk(m);
    int rc = grmp_tables(dim, fe_kind, order, &t);
    if (rc) return rc;
    if (nq) *nq = t.nq;
    if (nb) *nb = t.nb;
    for (int q = 0; q < t.nq; q++) {
        if (xref)
            for (int k = 0; k < 3; k++) xref[3 * q + k] = t.xref[q][k];
        if (w) w[q] = t.w[q];
        for (int a = 0; a < t.nb; a++) {
            if (vals) vals[q * t.nb + a] = t.vals[q][a];
            if (derivs)
                for (int j = 0; j < dim; j++) derivs[(q * t.nb + a) * dim + j] = t.derivs[q][a][j];
        }
    }
    return GRMP_OK;
}
