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

// Symmetric rules of Zhang, Cui and Liu ("A set of symmetric quadrature rules
// on triangles and tetrahedra", J. Comput. Math. 27 (2009) 89-96) with the
// orbit constants and the point order of src/quadrature.jl:332-499: the
// reference takes them for triangles of order 8 and 12-14 and for
// tetrahedra of order 5-8 (and, with a warning, above 8).
int symmetric_triangle(int order, double (*x)[3], double *w) {
    double w3;
    const double *a21, *w21, (*a111)[2], *w111;
    int n21, n111;
    static const double a21_8[3] = {.1705693077517602066222935014914645, .0505472283170309754584235505965989,
                                    .4592925882927231560288155144941693};
    static const double w21_8[3] = {.1032173705347182502817915502921290, .0324584976231980803109259283417806,
                                    .0950916342672846247938961043885843};
    static const double a111_8[1][2] = {{.2631128296346381134217857862846436, .0083947774099576053372138345392944}};
    static const double w111_8[1] = {.0272303141744349942648446900739089};
    static const double a21_14[7] = {.0099797608064584324152935295820524, .4799778935211883898105528650883899,
                                     .1538119591769669000000000000000000, .0740234771169878100000000000000000,
                                     .1303546825033300000000000000000000, .2306172260266531342996053700983831,
                                     .4223320834191478241144087137913939};
    static const double w21_14[7] = {.0017351512297252675680618638808094, .0261637825586145217778288591819783,
                                     .0039197292424018290965208275701454, .0122473597569408660972869899262505,
                                     .0281996285032579601073663071515657, .0508870871859594852960348275454540,
                                     .0504534399016035991910208971341189};
    static const double a111_14[4][2] = {{.7862373859346610033296221140330900, .1906163600319009042461432828653034},
                                         {.6305521436606074416224090755688129, .3623231377435471446183267343597729},
                                         {.6265773298563063142335123137534265, .2907712058836674150248168174816732},
                                         {.9142099849296254122399670993850469, .0711657108777507625475924502924336}};
    static const double w111_14[4] = {.0170636442122334512900253993849472, .0096834664255066004075209630934194,
                                      .0363857559284850056220113277642717, .0069646633735184124253997225042413};
    if (order <= 8) {
        w3 = .1443156076777871682510911104890646;
        a21 = a21_8, w21 = w21_8, n21 = 3, a111 = a111_8, w111 = w111_8, n111 = 1;
    } else {
        w3 = .0585962852260285941278938063477560;
        a21 = a21_14, w21 = w21_14, n21 = 7, a111 = a111_14, w111 = w111_14, n111 = 4;
    }
    int q = 0;
    x[q][0] = x[q][1] = 1.0 / 3.0;
    w[q++] = w3;
    for (int j = 0; j < n21; j++) {       // orbit S21: three points
        const double a = a21[j], c = 1.0 - 2.0 * a;
        const double p[3][2] = {{a, a}, {a, c}, {c, a}};
        for (int k = 0; k < 3; k++, q++) {
            x[q][0] = p[k][0], x[q][1] = p[k][1];
            w[q] = w21[j];
        }
    }
    for (int j = 0; j < n111; j++) {      // orbit S111: six points
        const double a = a111[j][0], b = a111[j][1], c = 1.0 - a - b;
        const double p[6][2] = {{a, b}, {b, a}, {a, c}, {b, c}, {c, a}, {c, b}};
        for (int k = 0; k < 6; k++, q++) {
            x[q][0] = p[k][0], x[q][1] = p[k][1];
            w[q] = w111[j];
        }
    }
    return q;
}

int symmetric_tetrahedron(double (*x)[3], double *w) {   // order 8, 46 points
    static const double a31[4] = {.0396754230703899012650713295393895, .3144878006980963137841605626971483,
                                  .1019866930627033000000000000000000, .1842036969491915122759464173489092};
    static const double w31[4] = {.0063971477799023213214514203351730, .0401904480209661724881611584798178,
                                  .0243079755047703211748691087719226, .0548588924136974404669241239903914};
    static const double a22 = .0634362877545398924051412387018983, w22 = .0357196122340991824649509689966176;
    static const double a211[2][2] = {{.0216901620677280048026624826249302, .7199319220394659358894349533527348},
                                      {.2044800806367957142413355748727453, .5805771901288092241753981713906204}};
    static const double w211[2] = {.0071831906978525394094511052198038, .0163721819453191175409381397561191};
    int q = 0;
    for (int j = 0; j < 4; j++) {         // orbit S31: four points
        const double a = a31[j], c = 1.0 - 3.0 * a;
        const double p[4][3] = {{a, a, a}, {a, a, c}, {a, c, a}, {c, a, a}};
        for (int k = 0; k < 4; k++, q++) {
            for (int d = 0; d < 3; d++) x[q][d] = p[k][d];
            w[q] = w31[j];
        }
    }
    {                                     // orbit S22: six points
        const double a = a22, c = 0.5 - a;
        const double p[6][3] = {{a, a, c}, {a, c, a}, {c, a, a}, {c, a, c}, {c, c, a}, {a, c, c}};
        for (int k = 0; k < 6; k++, q++) {
            for (int d = 0; d < 3; d++) x[q][d] = p[k][d];
            w[q] = w22;
        }
    }
    for (int j = 0; j < 2; j++) {         // orbit S211: twelve points
        const double a = a211[j][0], b = a211[j][1], c = 1.0 - 2.0 * a - b;
        const double p[12][3] = {{a, a, b}, {a, b, a}, {b, a, a}, {a, a, c}, {a, c, a}, {c, a, a},
                                 {a, b, c}, {a, c, b}, {c, a, b}, {b, a, c}, {b, c, a}, {c, b, a}};
        for (int k = 0; k < 12; k++, q++) {
            for (int d = 0; d < 3; d++) x[q][d] = p[k][d];
            w[q] = w211[j];
        }
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
        case GRMP_FE_H1P2B: return dim == 2 ? 3 : -1;   // src/fedefs/h1_p2b.jl:24-26
        case GRMP_FE_HDIVRT1: return 2;
        case GRMP_FE_HDIVBDM2: return 2;
    }
    return -1;
}

int grmp_fe_nb(int fe, int dim) {
    switch (fe) {
        case GRMP_FE_H1P1: return dim + 1;
        case GRMP_FE_H1P2: return dim == 2 ? 6 : 10;
        case GRMP_FE_H1BR: return dim == 2 ? 6 : 8;
        case GRMP_FE_L2P0: return 1;
        case GRMP_FE_H1P2B: return dim == 2 ? 7 : 0;
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
        case GRMP_FE_H1P2B: return dim == 2 ? 7 * ncomp : 0;
    }
    return 0;
}

int grmp_quadrature(int dim, int order, double (*x)[3], double *w) {
    std::memset(x, 0, sizeof(double) * 3 * GRMP_MAXQ);
    if (order < 0) order = 0;
    if (dim == 1) {   // src/quadrature.jl:130-148: midpoint, Simpson, then Gauss-Legendre
        if (order <= 1) {
            x[0][0] = 0.5;
            w[0] = 1.0;
            return 1;
        }
        if (order == 2) {
            x[0][0] = 0.0, x[1][0] = 0.5, x[2][0] = 1.0;
            w[0] = 1.0 / 6.0, w[1] = 2.0 / 3.0, w[2] = 1.0 / 6.0;
            return 3;
        }
        const int n = order / 2 + 1;
        if (n > 16) return 0;
        double dg[16] = {0}, of[16], r[16], v1[16];
        for (int i = 1; i < n; i++) of[i - 1] = i / std::sqrt(4.0 * i * i - 1.0);
        tridiag_eig(n, dg, of, r, v1);
        for (int i = 0; i < n; i++) {
            x[i][0] = 0.5 * r[i] + 0.5;
            w[i] = 0.5 * (2.0 * v1[i] * v1[i]);
        }
        return n;
    }
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
        if (order == 8 || (order >= 12 && order <= 14)) return symmetric_triangle(order, x, w);
        if (order <= 20) return stroud(order, x, w);
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
        return symmetric_tetrahedron(x, w);   // orders above 8: the order-8 rule, as the reference
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
