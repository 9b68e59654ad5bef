/*
 * grmp_oracle.c -- CPU restatement of GradientRobustMultiPhysics.jl (v0.12.0)
 * global assembly for the finite-element hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library is
 * compared against; it is loaded by the tests, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg.  Nothing in the product links or calls it.
 *
 * Parity status: the reference is Julia and cannot run here (no julia binary,
 * and ExtendableGrids / ExtendableSparse / LinearSolve are not vendored).  This
 * restatement is pinned against the reference's own known-answer tests
 * (test/runtests.jl quadrature exactness, polynomial reproduction of the
 * elements, Stokes / pressure-robustness exactness) which the pytest suite
 * re-implements.  Mesh numbering, the affine-map inverse and face orientation
 * come from ExtendableGrids and are restated here as conventions shared
 * with the host mesh module; they are "parity unpinned".
 *
 * Every routine follows the operation order of the reference file it cites so
 * that the drop-exact-zero sparsity rule (src/fematrix.jl:54-65) sees the same
 * floating-point zeros.  Build with -ffp-contract=off (no fused multiply-add),
 * which is what Julia does for plain `a*b + c`.
 *
 * Threads: the global assembly loops are run by OpenMP threads that each own
 * a contiguous range of rows (DoFs).  Every thread walks all cells in
 * ascending order and applies only the updates whose row it owns, so each row
 * receives exactly the additions of the sequential loop, in the same order:
 * the result is bit-identical to the single-threaded reference loop for any
 * thread count (cells spanning several row ranges are evaluated by each of
 * their owners).
 */

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAXQ 128
#define OR_MAXD 32

/* Threads of the OpenMP regions that follow (assembly rows, CG): n > 0
 * threads, n <= 0 all processors.  Lets the CPU baseline be timed on one
 * core (the reference assembles in one Julia task) beside all cores. */
void oracle_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
    (void)n;
#endif
}

/* Row range [lo, hi) of the calling thread (the whole range outside a
 * parallel region). */
static void or_row_range(int n, int *lo, int *hi)
{
#ifdef _OPENMP
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
    const int t = 0, nt = 1;
#endif
    *lo = (int)((long long)n * t / nt);
    *hi = (int)((long long)n * (t + 1) / nt);
}

static int or_touches(const int *dofs, int nd, int lo, int hi)
{
    for (int i = 0; i < nd; i++)
        if (dofs[i] >= lo && dofs[i] < hi) return 1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Quadrature (src/quadrature.jl)                                            */
/* ------------------------------------------------------------------------- */

/* Symmetric tridiagonal eigen-decomposition by cyclic Jacobi rotations;
 * returns ascending eigenvalues and the first component of each normalised
 * eigenvector (all that Golub-Welsch needs).  The reference uses Julia's
 * `eigen` (LAPACK); results agree to rounding. */
static void sym_eig_first(int n, const double *diag, const double *off,
                          double *evals, double *v1)
{
    double a[16][16], v[16][16];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) { a[i][j] = 0.0; v[i][j] = (i == j) ? 1.0 : 0.0; }
    for (int i = 0; i < n; i++) a[i][i] = diag[i];
    for (int i = 0; i + 1 < n; i++) { a[i][i + 1] = off[i]; a[i + 1][i] = off[i]; }
    for (int sweep = 0; sweep < 100; sweep++) {
        double offn = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) offn += a[p][q] * a[p][q];
        if (offn < 1e-300) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                if (fabs(a[p][q]) < 1e-300) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int idx[16];
    for (int i = 0; i < n; i++) idx[i] = i;
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (a[idx[j]][idx[j]] < a[idx[i]][idx[i]]) { int t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
    for (int i = 0; i < n; i++) {
        evals[i] = a[idx[i]][idx[i]];
        double nrm = 0.0;
        for (int k = 0; k < n; k++) nrm += v[k][idx[i]] * v[k][idx[i]];
        v1[i] = v[0][idx[i]] / sqrt(nrm);
    }
}

/* Gauss-Legendre on [0,1] (src/quadrature.jl:506-525). */
static int gauss01(int order, double *x, double *w)
{
    int n = order / 2 + 1;
    double diag[16] = {0}, off[16], ev[16], v1[16];
    for (int i = 1; i <= n - 1; i++) off[i - 1] = i / sqrt(4.0 * i * i - 1.0);
    sym_eig_first(n, diag, off, ev, v1);
    for (int i = 0; i < n; i++) { x[i] = 0.5 * ev[i] + 0.5; w[i] = 0.5 * (2.0 * v1[i] * v1[i]); }
    return n;
}

/* Stroud conical product rule on the reference triangle
 * (src/quadrature.jl:528-562): points [s_j, r_i (1 - s_j)], weights a_i b_j,
 * point index (j-1)*n + i. */
static int stroud_tri(int order, double (*xref)[3], double *w)
{
    int n = order / 2 + 1;
    double diag[16] = {0}, off[16], r[16], a[16], s[16], b[16], v1[16];
    for (int i = 1; i <= n - 1; i++) off[i - 1] = i / sqrt(4.0 * i * i - 1.0);
    sym_eig_first(n, diag, off, r, v1);
    for (int i = 0; i < n; i++) a[i] = 2.0 * v1[i] * v1[i];
    for (int i = 1; i <= n; i++) diag[i - 1] = -1.0 / (4.0 * i * i - 1.0);
    for (int i = 1; i <= n - 1; i++) off[i - 1] = sqrt((double)(i + 1) * i) / (2.0 * (i + 1) - 1.0);
    sym_eig_first(n, diag, off, s, v1);
    for (int i = 0; i < n; i++) b[i] = 2.0 * v1[i] * v1[i];
    for (int i = 0; i < n; i++) {
        r[i] = 0.5 * r[i] + 0.5; s[i] = 0.5 * s[i] + 0.5;
        a[i] = 0.5 * a[i]; b[i] = 0.5 * b[i];
    }
    int q = 0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            xref[q][0] = s[j] * 1.0 - r[i] * (s[j] - 1.0) * 0.0;
            xref[q][1] = s[j] * 0.0 - r[i] * (s[j] - 1.0) * 1.0;
            xref[q][2] = 0.0;
            w[q] = a[i] * b[j];
            q++;
        }
    return q;
}

/* Symmetric rules of Zhang, Cui and Liu (J. Comput. Math. 27 (2009) 89-96)
 * as src/quadrature.jl:332-499 tabulates and expands them: orbit constants,
 * points in the reference's order.  Triangles: order 8 (16 points) and
 * orders 9-14 (46 points); tetrahedra: order 8 (46 points). */
static int sym_tri(int order, double xr[][3], double *w)
{
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
    const int big = order > 8;
    const double *a21 = big ? a21_14 : a21_8, *w21 = big ? w21_14 : w21_8, *w111 = big ? w111_14 : w111_8;
    const double (*a111)[2] = big ? a111_14 : a111_8;
    const int n21 = big ? 7 : 3, n111 = big ? 4 : 1;
    int q = 0;
    xr[q][0] = 1.0 / 3.0; xr[q][1] = 1.0 / 3.0; xr[q][2] = 0.0;
    w[q++] = big ? .0585962852260285941278938063477560 : .1443156076777871682510911104890646;
    for (int j = 0; j < n21; j++) {
        double a = a21[j], c = 1.0 - 2.0 * a;
        double p[3][2] = {{a, a}, {a, c}, {c, a}};
        for (int k = 0; k < 3; k++, q++) { xr[q][0] = p[k][0]; xr[q][1] = p[k][1]; xr[q][2] = 0.0; w[q] = w21[j]; }
    }
    for (int j = 0; j < n111; j++) {
        double a = a111[j][0], b = a111[j][1], c = 1.0 - a - b;
        double p[6][2] = {{a, b}, {b, a}, {a, c}, {b, c}, {c, a}, {c, b}};
        for (int k = 0; k < 6; k++, q++) { xr[q][0] = p[k][0]; xr[q][1] = p[k][1]; xr[q][2] = 0.0; w[q] = w111[j]; }
    }
    return q;
}

static int sym_tet8(double xr[][3], double *w)
{
    static const double a31[4] = {.0396754230703899012650713295393895, .3144878006980963137841605626971483,
                                  .1019866930627033000000000000000000, .1842036969491915122759464173489092};
    static const double w31[4] = {.0063971477799023213214514203351730, .0401904480209661724881611584798178,
                                  .0243079755047703211748691087719226, .0548588924136974404669241239903914};
    static const double a211[2][2] = {{.0216901620677280048026624826249302, .7199319220394659358894349533527348},
                                      {.2044800806367957142413355748727453, .5805771901288092241753981713906204}};
    static const double w211[2] = {.0071831906978525394094511052198038, .0163721819453191175409381397561191};
    const double a22 = .0634362877545398924051412387018983, w22 = .0357196122340991824649509689966176;
    int q = 0;
    for (int j = 0; j < 4; j++) {
        double a = a31[j], c = 1.0 - 3.0 * a;
        double p[4][3] = {{a, a, a}, {a, a, c}, {a, c, a}, {c, a, a}};
        for (int k = 0; k < 4; k++, q++) { for (int d = 0; d < 3; d++) xr[q][d] = p[k][d]; w[q] = w31[j]; }
    }
    {
        double a = a22, c = 0.5 - a;
        double p[6][3] = {{a, a, c}, {a, c, a}, {c, a, a}, {c, a, c}, {c, c, a}, {a, c, c}};
        for (int k = 0; k < 6; k++, q++) { for (int d = 0; d < 3; d++) xr[q][d] = p[k][d]; w[q] = w22; }
    }
    for (int j = 0; j < 2; j++) {
        double a = a211[j][0], b = a211[j][1], c = 1.0 - 2.0 * a - b;
        double p[12][3] = {{a, a, b}, {a, b, a}, {b, a, a}, {a, a, c}, {a, c, a}, {c, a, a},
                           {a, b, c}, {a, c, b}, {c, a, b}, {b, a, c}, {b, c, a}, {c, b, a}};
        for (int k = 0; k < 12; k++, q++) { for (int d = 0; d < 3; d++) xr[q][d] = p[k][d]; w[q] = w211[j]; }
    }
    return q;
}

/* Quadrature rule for a simplex of dimension dim (2 = Triangle2D,
 * 3 = Tetrahedron3D) and the given order; src/quadrature.jl:173-194 (tri),
 * :268-325 (tet).  Orders served: tri 0..20 (Stroud, the symmetric rules at
 * 8 and 12..14), tet any order (hard-coded rules 0..4, the symmetric order-8
 * rule above).  Returns npoints, or 0 if the order is not available. */
int oracle_qrule(int dim, int order, double *xref_out, double *w_out)
{
    double xr[OR_MAXQ][3];
    double w[OR_MAXQ];
    int n = 0, flag = 1;
    memset(xr, 0, sizeof(xr));
    if (dim == 1) {
        if (order <= 1) { xr[0][0] = 0.5; w[0] = 1.0; n = 1; }
        else if (order == 2) {
            xr[0][0] = 0.0; xr[1][0] = 0.5; xr[2][0] = 1.0;
            w[0] = 1.0 / 6.0; w[1] = 2.0 / 3.0; w[2] = 1.0 / 6.0; n = 3;
        } else {
            double x[16], ww[16];
            n = gauss01(order, x, ww);
            for (int i = 0; i < n; i++) { xr[i][0] = x[i]; w[i] = ww[i]; }
        }
    } else if (dim == 2) {
        if (order <= 1) { xr[0][0] = 1.0 / 3.0; xr[0][1] = 1.0 / 3.0; w[0] = 1.0; n = 1; }
        else if (order == 2) {
            xr[0][0] = 0.5; xr[0][1] = 0.5;
            xr[1][0] = 0.0; xr[1][1] = 0.5;
            xr[2][0] = 0.5; xr[2][1] = 0.0;
            w[0] = w[1] = w[2] = 1.0 / 3.0; n = 3;
        } else if (order == 8 || (order >= 12 && order <= 14)) {
            n = sym_tri(order, xr, w);
        } else if (order <= 20) {
            n = stroud_tri(order, xr, w);
        } else return 0;
    } else if (dim == 3) {
        if (order <= 1) { xr[0][0] = xr[0][1] = xr[0][2] = 0.25; w[0] = 1.0; n = 1; }
        else if (order == 2) {
            const double a = 0.1381966011250105, b = 0.5854101966249685;
            double p[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
            for (int i = 0; i < 4; i++) { for (int k = 0; k < 3; k++) xr[i][k] = p[i][k]; w[i] = 0.25; }
            n = 4;
        } else if (order == 3) {
            double p[5][3] = {{1.0 / 4, 1.0 / 4, 1.0 / 4}, {1.0 / 2, 1.0 / 6, 1.0 / 6}, {1.0 / 6, 1.0 / 6, 1.0 / 6},
                              {1.0 / 6, 1.0 / 6, 1.0 / 2}, {1.0 / 6, 1.0 / 2, 1.0 / 6}};
            double ww[5] = {-4.0 / 5, 9.0 / 20, 9.0 / 20, 9.0 / 20, 9.0 / 20};
            for (int i = 0; i < 5; i++) { for (int k = 0; k < 3; k++) xr[i][k] = p[i][k]; w[i] = ww[i]; }
            n = 5;
        } else if (order == 4) {
            const double c = 0.2500000000000000, d = 0.7857142857142857, e = 0.0714285714285714,
                         f = 0.1005964238332008, g = 0.3994035761667992;
            double p[11][3] = {{c, c, c}, {d, e, e}, {e, e, e}, {e, e, d}, {e, d, e},
                               {f, g, g}, {g, f, g}, {g, g, f}, {g, f, f}, {f, g, f}, {f, f, g}};
            double ww[11] = {-0.0789333333333333, 0.0457333333333333, 0.0457333333333333, 0.0457333333333333,
                             0.0457333333333333, 0.1493333333333333, 0.1493333333333333, 0.1493333333333333,
                             0.1493333333333333, 0.1493333333333333, 0.1493333333333333};
            for (int i = 0; i < 11; i++) { for (int k = 0; k < 3; k++) xr[i][k] = p[i][k]; w[i] = ww[i]; }
            n = 11;
        } else {
            n = sym_tet8(xr, w);   /* orders 5-8; above 8 the reference warns and takes order 8 */
        }
    } else return 0;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) xref_out[3 * i + k] = xr[i][k];
        w_out[i] = w[i];
    }
    return flag * n;
}

/* ------------------------------------------------------------------------- */
/* Reference bases with ForwardDiff-ordered derivatives                      */
/* ------------------------------------------------------------------------- */

/* Dual number with up to 3 partials; products follow ForwardDiff's
 * `vy*px + vx*py`, scalar*dual scales value and partials. */
typedef struct { double v, d[3]; } dual;

static dual dvar(double x, int j) { dual r = {x, {0, 0, 0}}; r.d[j] = 1.0; return r; }
static dual dconst(double c) { dual r = {c, {0, 0, 0}}; return r; }
static dual dmul(dual x, dual y)
{
    dual r; r.v = x.v * y.v;
    for (int i = 0; i < 3; i++) r.d[i] = y.v * x.d[i] + x.v * y.d[i];
    return r;
}
static dual dscale(double c, dual x)
{
    dual r; r.v = c * x.v;
    for (int i = 0; i < 3; i++) r.d[i] = c * x.d[i];
    return r;
}
static dual dsubc(dual x, double c) { dual r = x; r.v = x.v - c; return r; }
static dual dcsub(double c, dual x)
{
    dual r; r.v = c - x.v;
    for (int i = 0; i < 3; i++) r.d[i] = -x.d[i];
    return r;
}
static dual dsub(dual x, dual y)
{
    dual r; r.v = x.v - y.v;
    for (int i = 0; i < 3; i++) r.d[i] = x.d[i] - y.d[i];
    return r;
}

enum { OR_FE_P1 = 1, OR_FE_P2 = 2, OR_FE_BR = 3, OR_FE_RT0 = 4, OR_FE_BDM1 = 5, OR_FE_P0 = 6 };

/* Scalar reference basis (one component) of H1P1 / H1P2 on the simplex of
 * dimension dim, evaluated on duals.  src/fedefs/h1_p1.jl:64-75,
 * src/fedefs/h1_p2.jl:134-165.  Returns number of basis functions. */
static int h1_scalar_basis(int fe, int dim, const dual *x, dual *out)
{
    if (fe == OR_FE_P1) {
        dual r = dcsub(1.0, x[0]);
        for (int j = 1; j < dim; j++) r = dsub(r, x[j]);
        out[0] = r;
        for (int j = 0; j < dim; j++) out[1 + j] = x[j];
        return dim + 1;
    }
    if (fe == OR_FE_P2 && dim == 2) {
        dual r = dsub(dcsub(1.0, x[0]), x[1]);
        out[0] = dmul(dscale(2.0, r), dsubc(r, 0.5));
        out[1] = dmul(dscale(2.0, x[0]), dsubc(x[0], 0.5));
        out[2] = dmul(dscale(2.0, x[1]), dsubc(x[1], 0.5));
        out[3] = dmul(dscale(4.0, r), x[0]);
        out[4] = dmul(dscale(4.0, x[0]), x[1]);
        out[5] = dmul(dscale(4.0, x[1]), r);
        return 6;
    }
    if (fe == OR_FE_P2 && dim == 3) {
        dual r = dsub(dsub(dcsub(1.0, x[0]), x[1]), x[2]);
        out[0] = dmul(dscale(2.0, r), dsubc(r, 0.5));
        out[1] = dmul(dscale(2.0, x[0]), dsubc(x[0], 0.5));
        out[2] = dmul(dscale(2.0, x[1]), dsubc(x[1], 0.5));
        out[3] = dmul(dscale(2.0, x[2]), dsubc(x[2], 0.5));
        out[4] = dmul(dscale(4.0, r), x[0]);
        out[5] = dmul(dscale(4.0, r), x[1]);
        out[6] = dmul(dscale(4.0, r), x[2]);
        out[7] = dmul(dscale(4.0, x[0]), x[1]);
        out[8] = dmul(dscale(4.0, x[0]), x[2]);
        out[9] = dmul(dscale(4.0, x[1]), x[2]);
        return 10;
    }
    return 0;
}

/* Tabulate the scalar reference basis at the quadrature points:
 * vals[q*nb + a], derivs[(q*nb + a)*dim + j] = d/dxref_j. */
int oracle_basis_tables(int fe, int dim, int nq, const double *xref, double *vals, double *derivs)
{
    int nb = 0;
    for (int q = 0; q < nq; q++) {
        dual x[3], out[OR_MAXD];
        for (int j = 0; j < dim; j++) x[j] = dvar(xref[3 * q + j], j);
        nb = h1_scalar_basis(fe, dim, x, out);
        for (int a = 0; a < nb; a++) {
            vals[q * nb + a] = out[a].v;
            for (int j = 0; j < dim; j++) derivs[(q * nb + a) * dim + j] = out[a].d[j];
        }
    }
    return nb;
}

/* ------------------------------------------------------------------------- */
/* Geometry (ExtendableGrids L2GTransformer role; restated convention)      */
/* ------------------------------------------------------------------------- */

/* A = [x1-x0, x2-x0(, x3-x0)] (columns).  G = A^{-T} = cof(A)/det(A), the
 * matrix `L2GAinv` with cvals[k] = sum_j G[k][j] dref_j
 * (src/feevaluator_h1.jl:61-74).  vol = |det|/2 or |det|/6. */
void oracle_geometry(int dim, const double *X, double A[3][3], double G[3][3], double *det, double *vol)
{
    for (int k = 0; k < dim; k++)
        for (int j = 0; j < dim; j++) A[k][j] = X[(j + 1) * dim + k] - X[k];
    if (dim == 2) {
        double d = A[0][0] * A[1][1] - A[0][1] * A[1][0];
        G[0][0] = A[1][1] / d;  G[0][1] = -A[1][0] / d;
        G[1][0] = -A[0][1] / d; G[1][1] = A[0][0] / d;
        *det = d; *vol = fabs(d) / 2.0;
    } else {
        double c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
        double c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
        double c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
        double c10 = A[0][2] * A[2][1] - A[0][1] * A[2][2];
        double c11 = A[0][0] * A[2][2] - A[0][2] * A[2][0];
        double c12 = A[0][1] * A[2][0] - A[0][0] * A[2][1];
        double c20 = A[0][1] * A[1][2] - A[0][2] * A[1][1];
        double c21 = A[0][2] * A[1][0] - A[0][0] * A[1][2];
        double c22 = A[0][0] * A[1][1] - A[0][1] * A[1][0];
        double d = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
        G[0][0] = c00 / d; G[0][1] = c01 / d; G[0][2] = c02 / d;
        G[1][0] = c10 / d; G[1][1] = c11 / d; G[1][2] = c12 / d;
        G[2][0] = c20 / d; G[2][1] = c21 / d; G[2][2] = c22 / d;
        *det = d; *vol = fabs(d) / 6.0;
    }
}

/* ------------------------------------------------------------------------- */
/* Sparse accumulator with the reference's accumulation order                */
/* ------------------------------------------------------------------------- */

typedef struct { int n, cap; int *col; double *val; } orow;
typedef struct { int nrows; orow *rows; } omat;

static omat *omat_new(int n)
{
    omat *m = (omat *)calloc(1, sizeof(omat));
    m->nrows = n;
    m->rows = (orow *)calloc((size_t)n, sizeof(orow));
    return m;
}

/* _addnz (src/fematrix.jl:54-58): skip exact zeros, otherwise
 * rawupdateindex!(+): accumulate in call order. */
static void omat_addnz(omat *m, int i, int j, double v, double fac)
{
    if (v == 0.0) return;
    orow *r = &m->rows[i];
    for (int k = 0; k < r->n; k++)
        if (r->col[k] == j) { r->val[k] += v * fac; return; }
    if (r->n == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 8;
        r->col = (int *)realloc(r->col, sizeof(int) * (size_t)r->cap);
        r->val = (double *)realloc(r->val, sizeof(double) * (size_t)r->cap);
    }
    r->col[r->n] = j; r->val[r->n] = v * fac; r->n++;
}

static void omat_set(omat *m, int i, int j, double v)
{
    orow *r = &m->rows[i];
    for (int k = 0; k < r->n; k++)
        if (r->col[k] == j) { r->val[k] = v; return; }
    omat_addnz(m, i, j, v, 1.0);
    for (int k = 0; k < r->n; k++)
        if (r->col[k] == j) { r->val[k] = v; return; }
}

void *oracle_mat_new(int n) { return omat_new(n); }

void oracle_mat_free(void *h)
{
    omat *m = (omat *)h;
    if (!m) return;
    for (int i = 0; i < m->nrows; i++) { free(m->rows[i].col); free(m->rows[i].val); }
    free(m->rows); free(m);
}

long long oracle_mat_nnz(void *h)
{
    omat *m = (omat *)h;
    long long nnz = 0;
    for (int i = 0; i < m->nrows; i++) nnz += m->rows[i].n;
    return nnz;
}

static int cmp_colval(const void *a, const void *b)
{
    const int ca = *(const int *)a, cb = *(const int *)b;
    return (ca > cb) - (ca < cb);
}

/* Export as CSR with columns ascending (rows sorted independently, in
 * parallel). */
void oracle_mat_csr(void *h, long long *rowptr, int *cols, double *vals)
{
    omat *m = (omat *)h;
    typedef struct { int c; double v; } cv;
    long long p = 0;
    for (int i = 0; i < m->nrows; i++) {
        rowptr[i] = p;
        p += m->rows[i].n;
    }
    rowptr[m->nrows] = p;
#pragma omp parallel
    {
    cv *buf = NULL; int bcap = 0;
#pragma omp for schedule(static)
    for (int i = 0; i < m->nrows; i++) {
        orow *r = &m->rows[i];
        if (r->n > bcap) { bcap = r->n; buf = (cv *)realloc(buf, sizeof(cv) * (size_t)bcap); }
        for (int k = 0; k < r->n; k++) { buf[k].c = r->col[k]; buf[k].v = r->val[k]; }
        qsort(buf, (size_t)r->n, sizeof(cv), cmp_colval);
        long long q = rowptr[i];
        for (int k = 0; k < r->n; k++) { cols[q] = buf[k].c; vals[q] = buf[k].v; q++; }
    }
    free(buf);
    }
}

/* apply_penalties! (src/fematrix.jl:349-355): A[d,d] = penalty. */
void oracle_mat_penalize(void *h, int nfixed, const int *fixed, double penalty)
{
    omat *m = (omat *)h;
    for (int k = 0; k < nfixed; k++) omat_set(m, fixed[k], fixed[k], penalty);
}

/* ------------------------------------------------------------------------- */
/* Operator evaluation at quadrature points (cvals)                          */
/* ------------------------------------------------------------------------- */

enum {
    OR_OP_IDENTITY = 0,     /* Identity                          */
    OR_OP_GRADIENT = 1,     /* Gradient                          */
    OR_OP_SYMGRAD = 2,      /* SymmetricGradient{1} (Voigt)      */
    OR_OP_DIVERGENCE = 3    /* Divergence                        */
};

/* cvals[(q*nd + dof)*rdim + k] for H1P1/H1P2 with ncomp components,
 * local dof = c*nb + a.  Loop orders follow src/feevaluator_h1.jl:61-74
 * (Gradient), :97-116 (SymmetricGradient), :119-131 (Divergence); the
 * Identity values are the reference values (src/feevaluator.jl:107-115). */
static int h1_cvals(int op, int dim, int ncomp, int nb, int nq, const double *vals, const double *derivs,
                    double G[3][3], double *cv)
{
    int nd = nb * ncomp;
    int rdim;
    if (op == OR_OP_IDENTITY) rdim = ncomp;
    else if (op == OR_OP_GRADIENT) rdim = dim * ncomp;
    else if (op == OR_OP_SYMGRAD) rdim = (dim == 2) ? 3 : 6;
    else rdim = 1;
    memset(cv, 0, sizeof(double) * (size_t)nq * nd * rdim);
    static const int comp2[4] = {0, 2, 2, 1};
    static const int comp3[9] = {0, 5, 4, 5, 1, 3, 4, 3, 2};
    for (int q = 0; q < nq; q++) {
        if (op == OR_OP_IDENTITY) {
            for (int dof = 0; dof < nd; dof++)
                for (int k = 0; k < ncomp; k++) {
                    int c = dof / nb, a = dof % nb;
                    cv[(q * nd + dof) * rdim + k] = (c == k) ? vals[q * nb + a] : 0.0;
                }
        } else if (op == OR_OP_GRADIENT) {
            /* for i, c, j, k, dof: cvals[k+off_c, dof] += G[k,j]*dref[dof+off2_c, j] */
            for (int c = 0; c < ncomp; c++)
                for (int j = 0; j < dim; j++)
                    for (int k = 0; k < dim; k++)
                        for (int dof = 0; dof < nd; dof++) {
                            int cd = dof / nb, a = dof % nb;
                            double d = (cd == c) ? derivs[(q * nb + a) * dim + j] : 0.0;
                            cv[(q * nd + dof) * rdim + k + c * dim] += G[k][j] * d;
                        }
        } else if (op == OR_OP_SYMGRAD) {
            const int *comp = (dim == 2) ? comp2 : comp3;
            for (int dof = 0; dof < nd; dof++)
                for (int c = 0; c < ncomp; c++)
                    for (int k = 0; k < dim; k++)
                        for (int j = 0; j < dim; j++) {
                            int cd = dof / nb, a = dof % nb;
                            double d = (cd == c) ? derivs[(q * nb + a) * dim + j] : 0.0;
                            int t = comp[k + c * dim];
                            if (k != c) cv[(q * nd + dof) * rdim + t] += 1.0 * G[k][j] * d;
                            else cv[(q * nd + dof) * rdim + t] += G[k][j] * d;
                        }
        } else { /* divergence */
            for (int dof = 0; dof < nd; dof++)
                for (int k = 0; k < dim; k++)
                    for (int j = 0; j < dim; j++) {
                        int cd = dof / nb, a = dof % nb;
                        double d = (cd == k) ? derivs[(q * nb + a) * dim + j] : 0.0;
                        cv[(q * nd + dof) * rdim] += G[k][j] * d;
                    }
        }
    }
    return rdim;
}

/* ------------------------------------------------------------------------- */
/* BilinearForm assembly (src/assemblypatterns/bilinearform.jl:92-380)       */
/* ------------------------------------------------------------------------- */

enum {
    OR_ACT_NONE = 0,       /* NoAction: result = input                     */
    OR_ACT_CELLSCALE = 1,  /* result = coef[cell] * input ("I" dependency)  */
    OR_ACT_HOOKE2D = 2,    /* tensor_apply_2d, src/pdeoperators.jl:265-270 */
    OR_ACT_HOOKE3D = 3     /* tensor_apply_3d                               */
};

typedef struct {
    int dim;            /* 2 or 3                                  */
    int nverts;
    const double *coords;   /* [nverts][dim]                       */
    int ncells;
    const int *cellnodes;   /* [ncells][dim+1]                     */
    int fe;             /* OR_FE_P1 / OR_FE_P2                     */
    int ncomp;
    int ldofs;          /* local dofs per cell = nb*ncomp          */
    const int *celldofs;    /* [ncells][ldofs], 0-based            */
} or_space;

/* Assemble one BilinearForm with operator `op` on both arguments into the
 * accumulator `h` (which may already hold other operators).  `symmetric`
 * selects APT_SymmetricBilinearForm (upper triangle computed once and
 * scattered twice, :196-210, :329-346) versus APT_BilinearForm (full block,
 * :180-192, :347-367).  The local matrix is built qp-outer, dof_i, dof_j as in
 * basismul!; the scatter value is local[i,j] * (volume * factor) and exact
 * zeros are dropped by _addnz. */
int oracle_assemble_bilinear(void *h, int dim, int nverts, const double *coords, int ncells, const int *cellnodes,
                             int fe, int ncomp, const int *celldofs, int op, int symmetric, double factor,
                             int action, const double *cellcoef, double mu, double lambda, int bonus_quadorder)
{
    omat *m = (omat *)h;
    int nb = (fe == OR_FE_P1) ? dim + 1 : (dim == 2 ? 6 : 10);
    int nd = nb * ncomp;
    int polyorder = (fe == OR_FE_P1) ? 1 : 2;
    int derivorder = (op == OR_OP_IDENTITY) ? 0 : 1;
    int order = bonus_quadorder + 2 * (polyorder - derivorder);
    if (order < 0) order = 0;
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(dim, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    double *vals = (double *)malloc(sizeof(double) * (size_t)nq * nb);
    double *derivs = (double *)malloc(sizeof(double) * (size_t)nq * nb * dim);
    oracle_basis_tables(fe, dim, nq, xref, vals, derivs);
#pragma omp parallel
    {
    int lo, hi;
    or_row_range(m->nrows, &lo, &hi);
    double *cv = (double *)malloc(sizeof(double) * (size_t)nq * nd * 6 * 3);
    double *loc = (double *)malloc(sizeof(double) * (size_t)nd * nd);
    double X[4 * 3];
    for (int cell = 0; cell < ncells; cell++) {
        if (!or_touches(&celldofs[(size_t)cell * nd], nd, lo, hi)) continue;
        for (int v = 0; v <= dim; v++)
            for (int k = 0; k < dim; k++) X[v * dim + k] = coords[(size_t)cellnodes[(size_t)cell * (dim + 1) + v] * dim + k];
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(dim, X, A, G, &det, &vol);
        int rdim = h1_cvals(op, dim, ncomp, nb, nq, vals, derivs, G, cv);
        memset(loc, 0, sizeof(double) * (size_t)nd * nd);
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < nd; i++) {
                double res[6];
                const double *in = &cv[(q * nd + i) * rdim];
                if (action == OR_ACT_NONE) for (int k = 0; k < rdim; k++) res[k] = in[k];
                else if (action == OR_ACT_CELLSCALE) for (int k = 0; k < rdim; k++) res[k] = cellcoef[cell] * in[k];
                else if (action == OR_ACT_HOOKE2D) {
                    res[0] = (lambda + 2 * mu) * in[0] + lambda * in[1];
                    res[1] = (lambda + 2 * mu) * in[1] + lambda * in[0];
                    res[2] = mu * in[2];
                } else {
                    /* tensor_apply_3d, src/pdeoperators.jl:304-312 */
                    res[0] = (lambda + 2 * mu) * in[0] + lambda * (in[1] + in[2]);
                    res[1] = (lambda + 2 * mu) * in[1] + lambda * (in[0] + in[2]);
                    res[2] = (lambda + 2 * mu) * in[2] + lambda * (in[0] + in[1]);
                    res[3] = mu * in[3]; res[4] = mu * in[4]; res[5] = mu * in[5];
                }
                int j0 = symmetric ? i : 0;
                for (int j = j0; j < nd; j++) {
                    double t = 0;
                    for (int k = 0; k < rdim; k++) t += res[k] * cv[(q * nd + j) * rdim + k];
                    loc[i * nd + j] += w[q] * t;
                }
            }
        double itemfactor = vol * factor;
        const int *dofs = &celldofs[(size_t)cell * nd];
#define OR_MINE(r) ((r) >= lo && (r) < hi)
        if (symmetric) {
            for (int i = 0; i < nd; i++)
                for (int j = i + 1; j < nd; j++) {
                    if (OR_MINE(dofs[i])) omat_addnz(m, dofs[i], dofs[j], loc[i * nd + j] * itemfactor, 1.0);
                    if (OR_MINE(dofs[j])) omat_addnz(m, dofs[j], dofs[i], loc[i * nd + j] * itemfactor, 1.0);
                }
            for (int i = 0; i < nd; i++)
                if (OR_MINE(dofs[i])) omat_addnz(m, dofs[i], dofs[i], loc[i * nd + i] * itemfactor, 1.0);
        } else {
            for (int i = 0; i < nd; i++)
                if (OR_MINE(dofs[i]))
                    for (int j = 0; j < nd; j++) omat_addnz(m, dofs[i], dofs[j], loc[i * nd + j] * itemfactor, 1.0);
        }
#undef OR_MINE
    }
    free(cv); free(loc);
    }
    free(vals); free(derivs);
    return nq;
}

/* ------------------------------------------------------------------------- */
/* LinearForm assembly (src/assemblypatterns/linearform.jl:47-237)           */
/* ------------------------------------------------------------------------- */

enum {
    OR_RHS_CONST = 0,    /* f = const vector (ncomp values)                     */
    OR_RHS_CELL = 1,     /* f = per-cell vector [ncells][ncomp] ("I")            */
    OR_RHS_FOURIER = 2,  /* f = sum_m a_m sin(pi k_m . x) (scalar, "X")          */
    OR_RHS_POLY = 3      /* f_c = sum_t coef_t x^e1 y^e2 z^e3 (vector, "X")      */
};


/* x^e of polynomial data: integer e in [1, 8] by repeated multiplication
 * left to right (x*x*x: Julia's literal powers x^2, x^3 in the reference's
 * data functions), e = 0 gives 1, other exponents pow. */
static double or_pow(double x, double e)
{
    const int k = (int)e;
    if (e == 0) return 1.0;
    if ((double)k == e && k >= 1 && k <= 8) {
        double r = x;
        for (int i = 1; i < k; i++) r = r * x;
        return r;
    }
    return pow(x, e);
}

/* Evaluate f at a physical point: eval_trafo! gives x = x0 + A xref. */
static void rhs_eval(int kind, int dim, int ncomp, const double *par, int npar, int cell, const double *x, double *f)
{
    if (kind == OR_RHS_CONST) { for (int c = 0; c < ncomp; c++) f[c] = par[c]; return; }
    if (kind == OR_RHS_CELL) { for (int c = 0; c < ncomp; c++) f[c] = par[(size_t)cell * ncomp + c]; return; }
    if (kind == OR_RHS_FOURIER) {
        /* par = [a_m, k_m1, k_m2, (k_m3)] per mode */
        int stride = 1 + dim, nm = npar / stride;
        double s = 0;
        for (int mm = 0; mm < nm; mm++) {
            double arg = 0;
            for (int j = 0; j < dim; j++) arg += par[mm * stride + 1 + j] * x[j];
            s += par[mm * stride] * sin(M_PI * arg);
        }
        f[0] = s;
        for (int c = 1; c < ncomp; c++) f[c] = 0;
        return;
    }
    /* polynomial: par = [comp, coef, e1, e2, e3] per term */
    for (int c = 0; c < ncomp; c++) f[c] = 0;
    int nt = npar / 5;
    for (int t = 0; t < nt; t++) {
        int c = (int)par[5 * t];
        double v = par[5 * t + 1];
        for (int j = 0; j < dim; j++) v *= or_pow(x[j], par[5 * t + 2 + j]);
        f[c] += v;
    }
}

/* b[dof] += (factor*vol) * sum_q w_q sum_k f_k(x_q) cvals[k,dof,q] with the
 * Identity test operator; quadrature order polyorder + bonus. */
int oracle_assemble_linear(double *b, int dim, int nverts, const double *coords, int ncells, const int *cellnodes,
                           int fe, int ncomp, const int *celldofs, int rhs_kind, const double *par, int npar,
                           double factor, int bonus_quadorder)
{
    int nb = (fe == OR_FE_P1) ? dim + 1 : (dim == 2 ? 6 : 10);
    int nd = nb * ncomp;
    int polyorder = (fe == OR_FE_P1) ? 1 : 2;
    int order = polyorder + bonus_quadorder;
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(dim, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    double *vals = (double *)malloc(sizeof(double) * (size_t)nq * nb);
    double *derivs = (double *)malloc(sizeof(double) * (size_t)nq * nb * dim);
    oracle_basis_tables(fe, dim, nq, xref, vals, derivs);
    int ndofs = 0;   /* rows: one past the largest DoF */
    for (size_t k = 0; k < (size_t)ncells * nd; k++)
        if (celldofs[k] + 1 > ndofs) ndofs = celldofs[k] + 1;
#pragma omp parallel
    {
    int lo, hi;
    or_row_range(ndofs, &lo, &hi);
    double G[3][3];
    double *cv = (double *)malloc(sizeof(double) * (size_t)nq * nd * 6);
    double *locb = (double *)malloc(sizeof(double) * (size_t)nd);
    double X[12];
    for (int cell = 0; cell < ncells; cell++) {
        if (!or_touches(&celldofs[(size_t)cell * nd], nd, lo, hi)) continue;
        for (int v = 0; v <= dim; v++)
            for (int k = 0; k < dim; k++) X[v * dim + k] = coords[(size_t)cellnodes[(size_t)cell * (dim + 1) + v] * dim + k];
        double A[3][3], det, vol;
        oracle_geometry(dim, X, A, G, &det, &vol);
        h1_cvals(OR_OP_IDENTITY, dim, ncomp, nb, nq, vals, derivs, G, cv);
        memset(locb, 0, sizeof(double) * (size_t)nd);
        for (int q = 0; q < nq; q++) {
            double x[3] = {0, 0, 0}, f[3];
            for (int k = 0; k < dim; k++) {
                x[k] = X[k];
                for (int j = 0; j < dim; j++) x[k] += A[k][j] * xref[3 * q + j];
            }
            rhs_eval(rhs_kind, dim, ncomp, par, npar, cell, x, f);
            for (int i = 0; i < nd; i++) {
                double t = 0;
                for (int k = 0; k < ncomp; k++) t += f[k] * cv[(q * nd + i) * ncomp + k];
                locb[i] += t * w[q];
            }
        }
        double itemfactor = factor * vol;
        for (int i = 0; i < nd; i++) {
            const int r = celldofs[(size_t)cell * nd + i];
            if (r >= lo && r < hi) b[r] += locb[i] * itemfactor;
        }
    }
    free(cv); free(locb);
    }
    free(vals); free(derivs);
    return nq;
}

/* ------------------------------------------------------------------------- */
/* ItemIntegrator over cells (src/assemblypatterns/itemintegrator.jl)        */
/* ------------------------------------------------------------------------- */

/* L2ErrorIntegrator (:40-94), L2NormIntegrator (:96-130) and
 * L2DifferenceIntegrator (:132-158) evaluated by evaluate! (:173-300):
 * per cell in ascending order and per quadrature point,
 *   input_k = sum_dof u[dof] cvals[k,dof,q]            (eval_febe!, dof ascending)
 *   result  = sum_j (f_j(x_q) - factor*input_j)^2       (error; f = 0: norm)
 *           = sum_j (input_j - input2_j)^2              (difference, v given)
 *   cellv[cell] += result * w_q * vol,  total += result * w_q * vol
 * (the AccumulatingVector of evaluate, :314-330, sums in the same order).
 * Quadrature order: polyorder + shift(op) + quadorder
 * (src/assemblypatterns.jl:559-565; Gradient shifts by -1).
 * Returns the number of quadrature points, or -1. */
int oracle_item_l2error(double *cellv, double *total, int dim, int nverts, const double *coords, int ncells,
                        const int *cellnodes, int fe, int ncomp, const int *celldofs, const double *u,
                        const double *v, int op, int data_kind, const double *par, int npar, double factor,
                        int quadorder)
{
    (void)nverts;
    if (op != OR_OP_IDENTITY && op != OR_OP_GRADIENT) return -1;
    int nb = (fe == OR_FE_P1) ? dim + 1 : (dim == 2 ? 6 : 10);
    int nd = nb * ncomp;
    int polyorder = (fe == OR_FE_P1) ? 1 : 2;
    int order = polyorder + (op == OR_OP_GRADIENT ? -1 : 0) + quadorder;
    if (order < 0) order = 0;
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(dim, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    double *vals = (double *)malloc(sizeof(double) * (size_t)nq * nb);
    double *derivs = (double *)malloc(sizeof(double) * (size_t)nq * nb * dim);
    oracle_basis_tables(fe, dim, nq, xref, vals, derivs);
    double G[3][3];
    double *cv = (double *)malloc(sizeof(double) * (size_t)nq * nd * 9);
    double X[12];
    double acc = 0.0;
    for (int cell = 0; cell < ncells; cell++) {
        for (int vv = 0; vv <= dim; vv++)
            for (int k = 0; k < dim; k++) X[vv * dim + k] = coords[(size_t)cellnodes[(size_t)cell * (dim + 1) + vv] * dim + k];
        double A[3][3], det, vol;
        oracle_geometry(dim, X, A, G, &det, &vol);
        int rdim = h1_cvals(op, dim, ncomp, nb, nq, vals, derivs, G, cv);
        double cellacc = 0.0;
        for (int q = 0; q < nq; q++) {
            double in1[9] = {0}, in2[9] = {0}, f[9] = {0};
            for (int dof = 0; dof < nd; dof++) {
                double c1 = u[celldofs[(size_t)cell * nd + dof]];
                for (int k = 0; k < rdim; k++) in1[k] += c1 * cv[(q * nd + dof) * rdim + k];
            }
            if (v)
                for (int dof = 0; dof < nd; dof++) {
                    double c2 = v[celldofs[(size_t)cell * nd + dof]];
                    for (int k = 0; k < rdim; k++) in2[k] += c2 * cv[(q * nd + dof) * rdim + k];
                }
            double result = 0.0;
            if (v) {
                for (int j = 0; j < rdim; j++) result += (in1[j] - in2[j]) * (in1[j] - in2[j]);
            } else {
                if (data_kind >= 0) {
                    double x[3] = {0, 0, 0};
                    for (int k = 0; k < dim; k++) {
                        x[k] = X[k];
                        for (int j = 0; j < dim; j++) x[k] += A[k][j] * xref[3 * q + j];
                    }
                    rhs_eval(data_kind, dim, rdim, par, npar, cell, x, f);
                }
                for (int j = 0; j < rdim; j++) {
                    double e = f[j] - in1[j] * factor;
                    result += e * e;
                }
            }
            double contrib = result * w[q] * vol;
            cellacc += contrib;
            acc += contrib;
        }
        if (cellv) cellv[cell] = cellacc;
    }
    if (total) *total = acc;
    free(vals); free(derivs); free(cv);
    return nq;
}

/* ------------------------------------------------------------------------- */
/* FP64 CG (Jacobi) on CSR -- used for sizes where a sparse-direct           */
/* factorisation does not fit, and as the multi-threaded CPU baseline solve. */
/* ------------------------------------------------------------------------- */

static void csr_mv(int n, const long long *rp, const int *ci, const double *v, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double s = 0;
        for (long long p = rp[i]; p < rp[i + 1]; p++) s += v[p] * x[ci[p]];
        y[i] = s;
    }
}

static double dotp(int n, const double *a, const double *b)
{
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* Returns iterations; stops when ||r|| <= reltol*||b|| or maxit. */
int oracle_cg(int n, const long long *rp, const int *ci, const double *v, const double *b, double *x, double reltol,
              int maxit, double *final_relres)
{
    double *r = (double *)malloc(sizeof(double) * (size_t)n), *z = (double *)malloc(sizeof(double) * (size_t)n);
    double *p = (double *)malloc(sizeof(double) * (size_t)n), *q = (double *)malloc(sizeof(double) * (size_t)n);
    double *dinv = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) {
        double d = 1.0;
        for (long long k = rp[i]; k < rp[i + 1]; k++) if (ci[k] == i) d = v[k];
        dinv[i] = 1.0 / d;
    }
    csr_mv(n, rp, ci, v, x, q);
#pragma omp parallel for
    for (int i = 0; i < n; i++) { r[i] = b[i] - q[i]; z[i] = dinv[i] * r[i]; p[i] = z[i]; }
    double bn = sqrt(dotp(n, b, b));
    if (bn == 0) bn = 1;
    double rz = dotp(n, r, z);
    int it = 0;
    double rn = sqrt(dotp(n, r, r));
    while (it < maxit && rn > reltol * bn) {
        csr_mv(n, rp, ci, v, p, q);
        double alpha = rz / dotp(n, p, q);
#pragma omp parallel for
        for (int i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; z[i] = dinv[i] * r[i]; }
        double rz2 = dotp(n, r, z);
        double beta = rz2 / rz;
        rz = rz2;
#pragma omp parallel for
        for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        rn = sqrt(dotp(n, r, r));
        it++;
    }
    if (final_relres) *final_relres = rn / bn;
    free(r); free(z); free(p); free(q); free(dinv);
    return it;
}

/* r = b - A x with each row's sum carried in double-double and rounded once:
 * products split exactly by fma (Dekker's TwoProduct), sums by Knuth's TwoSum,
 * the low parts accumulated separately (the compensated dot product of Ogita,
 * Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26,
 * 2005).  The residual of iterative refinement in twice the working
 * precision. */
void oracle_resid_dd(int n, const long long *rp, const int *ci, const double *v, const double *x, const double *b,
                     double *r)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double hi = b[i], lo = 0.0;
        for (long long k = rp[i]; k < rp[i + 1]; k++) {
            const double p = -v[k] * x[ci[k]];
            const double pe = fma(-v[k], x[ci[k]], -p);
            const double s = hi + p;
            const double bv = s - hi;
            const double se = (hi - (s - bv)) + (p - bv);
            hi = s;
            lo += se + pe;
        }
        r[i] = hi + lo;
    }
}

/* ------------------------------------------------------------------------- */
/* Bernardi-Raugel (H1BR{2}) with the RT0 reconstruction, 2D triangles       */
/* ------------------------------------------------------------------------- */

/* Local DoFs of a cell: 0-2 P1 component 1 (nodes), 3-5 P1 component 2,
 * 6-8 face bubbles (src/fedefs/h1v_br.jl:33 "N1f1").  Scalar basis table:
 * 0-2 P1 functions, 3-5 bubbles (:117-130).  Coefficients (:150-162):
 * 1 for P1 DoFs, the global unit normal of face f for bubble f. */
static void br_component_derivs(int dof, int c, int q, int nb, const double *derivs, double *d)
{
    int s;
    if (dof < 3) s = (c == 0) ? dof : -1;
    else if (dof < 6) s = (c == 1) ? dof - 3 : -1;
    else s = 3 + (dof - 6);
    for (int j = 0; j < 2; j++) d[j] = (s >= 0) ? derivs[(q * nb + s) * 2 + j] : 0.0;
}

static double br_coef(int dof, int c, const double *nrm /* [3][2] of the cell's faces */)
{
    if (dof < 6) return 1.0;
    return nrm[(dof - 6) * 2 + c];
}

/* RT0 reconstruction coefficients R[9][3] of one cell
 * (src/reconstructions.jl:381-403): R[(k)*3+node][f] = (1/2 |F|) n_F[k] for
 * the two nodes of face f, R[6+f][f] = |F|. */
static void br_rt0_coeffs(const double *fvol, const double *nrm, double R[9][3])
{
    memset(R, 0, sizeof(double) * 27);
    for (int f = 0; f < 3; f++) {
        int nodes[2] = {f, (f + 1) % 3};
        for (int n = 0; n < 2; n++)
            for (int k = 0; k < 2; k++) R[3 * k + nodes[n]][f] = (0.5 * fvol[f]) * nrm[f * 2 + k];
        R[6 + f][f] = fvol[f];
    }
}

/* BDM1 reconstruction coefficients R[9][6] of one cell
 * (src/reconstructions.jl:351-379): columns 2f (RT0 function of face f) and
 * 2f+1 (linear-moment BDM1 function of face f); for the two nodes of face f,
 * R[3k+node][2f] = (1/2 |F|) n_F[k], R[3k+node][2f+1] = c_n |F| n_F[k] s_f
 * with c = (-1/12, 1/12) and s_f the cell-face sign; R[6+f][2f] = |F|. */
static void br_bdm1_coeffs(const double *fvol, const double *nrm, const double *sg, double R[9][6])
{
    const double c[2] = {-1.0 / 12.0, 1.0 / 12.0};
    memset(R, 0, sizeof(double) * 54);
    for (int f = 0; f < 3; f++) {
        int nodes[2] = {f, (f + 1) % 3};
        for (int n = 0; n < 2; n++)
            for (int k = 0; k < 2; k++) {
                R[3 * k + nodes[n]][2 * f] = (0.5 * fvol[f]) * nrm[f * 2 + k];
                R[3 * k + nodes[n]][2 * f + 1] = ((c[n] * fvol[f]) * nrm[f * 2 + k]) * sg[f];
            }
        R[6 + f][2 * f] = fvol[f];
    }
}

/* Reference HDIVBDM1{2} basis on the triangle (src/fedefs/hdiv_bdm1.jl:81-92),
 * rows in the reference order: RT0 of face 1, BDM1 of face 1, RT0 of face 2, ... */
static void bdm1_ref_basis(double xi, double eta, double out[6][2])
{
    out[0][0] = xi; out[0][1] = eta - 1;
    out[1][0] = 6 * xi; out[1][1] = 6 - 12 * xi - 6 * eta;
    out[2][0] = xi; out[2][1] = eta;
    out[3][0] = -6 * xi; out[3][1] = 6 * eta;
    out[4][0] = xi - 1; out[4][1] = eta;
    out[5][0] = 6 * (xi - 1) + 12 * eta; out[5][1] = -6 * eta;
}

typedef struct {
    const double *coords; const int *cells; const int *cell_faces; const double *fnormals;
    const double *fvolumes; const signed char *signs; const int *celldofs;
} br_mesh;

static void br_cell(const br_mesh *m, int cell, double X[6], double nrm[6], double fv[3], double sg[3])
{
    for (int v = 0; v < 3; v++)
        for (int k = 0; k < 2; k++) X[v * 2 + k] = m->coords[(size_t)m->cells[(size_t)cell * 3 + v] * 2 + k];
    for (int f = 0; f < 3; f++) {
        int F = m->cell_faces[(size_t)cell * 3 + f];
        nrm[f * 2] = m->fnormals[(size_t)F * 2];
        nrm[f * 2 + 1] = m->fnormals[(size_t)F * 2 + 1];
        fv[f] = m->fvolumes[F];
        sg[f] = (double)m->signs[(size_t)cell * 3 + f];
    }
}

/* nu (grad u, grad v) on H1BR{2} (LaplaceOperator, APT_SymmetricBilinearForm;
 * Gradient with coefficients, src/feevaluator_h1.jl:77-94) plus
 * lambda (div R u, div R v) (BilinearForm([ReconstructionDivergence{HDIVRT0{2}}]^2),
 * APT_BilinearForm; src/feevaluator_h1.jl:409-437).  cellnu (optional)
 * replaces nu by a per-cell action coefficient. */
int oracle_br_assemble(void *h, int ncells, const double *coords, const int *cells, const int *cell_faces,
                       const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                       double nu, const double *cellnu, double lambda)
{
    omat *M = (omat *)h;
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(2, 2, xref, w); /* order 2(2-1) = 2 for both terms */
    double vals[OR_MAXQ * 6], derivs[OR_MAXQ * 6 * 2];
    /* scalar basis: P1 then bubbles, with ForwardDiff-ordered derivatives */
    for (int q = 0; q < nq; q++) {
        dual x[2] = {dvar(xref[3 * q], 0), dvar(xref[3 * q + 1], 1)};
        dual r = dsub(dcsub(1.0, x[0]), x[1]);
        dual o[6] = {r, x[0], x[1], dmul(dscale(6.0, x[0]), r), dmul(dscale(6.0, x[1]), x[0]), dmul(dscale(6.0, r), x[1])};
        for (int a = 0; a < 6; a++) {
            vals[q * 6 + a] = o[a].v;
            derivs[(q * 6 + a) * 2] = o[a].d[0];
            derivs[(q * 6 + a) * 2 + 1] = o[a].d[1];
        }
    }
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], nrm[6], fv[3], sg[3];
        br_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(2, X, A, G, &det, &vol);
        const int *dofs = &celldofs[(size_t)cell * 9];
        /* Laplace with coefficients: cv[q][dof][k + 2c] */
        double cv[OR_MAXQ][9][4];
        for (int q = 0; q < nq; q++)
            for (int dof = 0; dof < 9; dof++)
                for (int c = 0; c < 2; c++)
                    for (int k = 0; k < 2; k++) {
                        double d[2], s = 0;
                        br_component_derivs(dof, c, q, 6, derivs, d);
                        for (int j = 0; j < 2; j++) s += G[k][j] * d[j];
                        s *= br_coef(dof, c, nrm);
                        cv[q][dof][k + 2 * c] = s;
                    }
        double loc[9][9];
        memset(loc, 0, sizeof(loc));
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < 9; i++) {
                double res[4];
                for (int k = 0; k < 4; k++) res[k] = cellnu ? cellnu[cell] * cv[q][i][k] : cv[q][i][k];
                for (int j = i; j < 9; j++) {
                    double t = 0;
                    for (int k = 0; k < 4; k++) t += res[k] * cv[q][j][k];
                    loc[i][j] += w[q] * t;
                }
            }
        double itemfactor = vol * (cellnu ? 1.0 : nu);
        for (int i = 0; i < 9; i++)
            for (int j = i + 1; j < 9; j++) {
                omat_addnz(M, dofs[i], dofs[j], loc[i][j] * itemfactor, 1.0);
                omat_addnz(M, dofs[j], dofs[i], loc[i][j] * itemfactor, 1.0);
            }
        for (int i = 0; i < 9; i++) omat_addnz(M, dofs[i], dofs[i], loc[i][i] * itemfactor, 1.0);
        if (lambda == 0.0) continue;
        /* reconstruction divergence, constant per cell but evaluated per qp */
        double R[9][3];
        br_rt0_coeffs(fv, nrm, R);
        double dv[OR_MAXQ][9];
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < 9; i++) {
                double s = 0;
                for (int j = 0; j < 3; j++)
                    if (R[i][j] != 0)
                        for (int jd = 0; jd < 2; jd++) s += R[i][j] * 1.0 * sg[j];
                s /= det;
                dv[q][i] = s;
            }
        double lp[9][9];
        memset(lp, 0, sizeof(lp));
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < 9; i++)
                for (int j = 0; j < 9; j++) {
                    double t = 0;
                    t += dv[q][i] * dv[q][j];
                    lp[i][j] += w[q] * t;
                }
        double pf = vol * lambda;
        for (int i = 0; i < 9; i++)
            for (int j = 0; j < 9; j++) omat_addnz(M, dofs[i], dofs[j], lp[i][j] * pf, 1.0);
    }
    return nq;
}

/* b += factor * (f, R v), f polynomial (RHS_POLY params, 2 components), with
 * the ReconstructionIdentity{HDIVRT0{2}} (recon 1) or
 * ReconstructionIdentity{HDIVBDM1{2}} (recon 2) test operator
 * (src/feevaluator_h1.jl:342-381, src/assemblypatterns/linearform.jl:181-220);
 * quadrature order polyorder(H1BR{2}) = 2 plus bonus. */
int oracle_br_rhs_recon(double *b, int ncells, const double *coords, const int *cells, const int *cell_faces,
                        const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                        const double *par, int npar, double factor, int bonus_quadorder, int recon)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(2, 2 + bonus_quadorder, xref, w);
    if (nq < 0) nq = -nq;
    const int nr = recon == 2 ? 6 : 3;
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], nrm[6], fv[3], sg[3];
        br_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(2, X, A, G, &det, &vol);
        double R[9][6];
        if (recon == 2) {
            br_bdm1_coeffs(fv, nrm, sg, R);
        } else {
            double R3[9][3];
            br_rt0_coeffs(fv, nrm, R3);
            for (int i = 0; i < 9; i++)
                for (int j = 0; j < 3; j++) R[i][j] = R3[i][j];
        }
        double locb[9] = {0};
        for (int q = 0; q < nq; q++) {
            double xi = xref[3 * q], eta = xref[3 * q + 1];
            double rt[6][2], coef[6];
            if (recon == 2) {
                bdm1_ref_basis(xi, eta, rt);
                for (int j = 0; j < 6; j++) coef[j] = (j % 2 == 0) ? sg[j / 2] : 1.0;   /* signs on RT0 only */
            } else {
                double r3[3][2] = {{xi, eta - 1}, {xi, eta}, {xi - 1, eta}};
                for (int j = 0; j < 3; j++) { rt[j][0] = r3[j][0]; rt[j][1] = r3[j][1]; coef[j] = sg[j]; }
            }
            double te[6][2];
            for (int j = 0; j < nr; j++)
                for (int k = 0; k < 2; k++) {
                    double s = 0;
                    for (int l = 0; l < 2; l++) s += A[k][l] * rt[j][l];
                    s *= coef[j] / det;
                    te[j][k] = s;
                }
            double x[2], f[2];
            for (int k = 0; k < 2; k++) {
                x[k] = X[k];
                for (int j = 0; j < 2; j++) x[k] += A[k][j] * xref[3 * q + j];
            }
            rhs_eval(OR_RHS_POLY, 2, 2, par, npar, cell, x, f);
            for (int i = 0; i < 9; i++) {
                double cv[2] = {0, 0};
                for (int j = 0; j < nr; j++)
                    if (R[i][j] != 0)
                        for (int k = 0; k < 2; k++) cv[k] += R[i][j] * te[j][k];
                double t = 0;
                for (int k = 0; k < 2; k++) t += f[k] * cv[k];
                locb[i] += t * w[q];
            }
        }
        double itemfactor = factor * vol;
        for (int i = 0; i < 9; i++) b[celldofs[(size_t)cell * 9 + i]] += locb[i] * itemfactor;
    }
    return nq;
}

int oracle_br_rhs(double *b, int ncells, const double *coords, const int *cells, const int *cell_faces,
                  const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                  const double *par, int npar, double factor, int bonus_quadorder)
{
    return oracle_br_rhs_recon(b, ncells, coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs, par, npar,
                               factor, bonus_quadorder, 1);
}

/* ------------------------------------------------------------------------- */
/* H1BR{3} on tetrahedra with the RT0 reconstruction                         */
/* ------------------------------------------------------------------------- */

/* Local faces of a tetrahedron (the reference's face_nodes of Tetrahedron3D):
 * [0,1,2], [0,1,3], [1,2,3], [0,2,3]. */
static const int BR3_FACES[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};

/* Scalar basis of H1BR{3} (src/fedefs/h1v_br.jl:221-233): the four P1
 * functions, then the face bubbles 60 x r y, 60 r x z, 60 x y z, 60 r y z
 * (r = 1 - x - y - z), products in the reference's left-to-right order. */
static void br3_basis(const double *xr, double vals[8], double derivs[8][3])
{
    dual x[3] = {dvar(xr[0], 0), dvar(xr[1], 1), dvar(xr[2], 2)};
    dual r = dsub(dsub(dcsub(1.0, x[0]), x[1]), x[2]);
    dual o[8] = {r, x[0], x[1], x[2],
                 dmul(dmul(dscale(60.0, x[0]), r), x[1]),
                 dmul(dmul(dscale(60.0, r), x[0]), x[2]),
                 dmul(dmul(dscale(60.0, x[0]), x[1]), x[2]),
                 dmul(dmul(dscale(60.0, r), x[1]), x[2])};
    for (int a = 0; a < 8; a++) {
        vals[a] = o[a].v;
        for (int j = 0; j < 3; j++) derivs[a][j] = o[a].d[j];
    }
}

/* local DoF layout (pattern "N1f1"): 0-11 P1, component-major (4 c + node),
 * 12-15 the face bubbles (all three components, times n_F[c]) */
static int br3_scalar(int dof, int c)
{
    if (dof < 12) return (dof / 4 == c) ? dof % 4 : -1;
    return 4 + (dof - 12);
}
static double br3_coef(int dof, int c, const double *nrm /* [4][3] */)
{
    if (dof < 12) return 1.0;
    return nrm[(dof - 12) * 3 + c];
}

/* RT0 reconstruction coefficients R[16][4] (src/reconstructions.jl:474-491):
 * R[4k + node][f] = (1/3 |F|) n_F[k] for the three nodes of face f,
 * R[12 + f][f] = |F|. */
static void br3_rt0_coeffs(const double *fvol, const double *nrm, double R[16][4])
{
    memset(R, 0, sizeof(double) * 64);
    for (int f = 0; f < 4; f++) {
        for (int n = 0; n < 3; n++)
            for (int k = 0; k < 3; k++) R[4 * k + BR3_FACES[f][n]][f] = ((1.0 / 3.0) * fvol[f]) * nrm[f * 3 + k];
        R[12 + f][f] = fvol[f];
    }
}

/* HDIVRT0{3} reference basis on the tetrahedron (src/fedefs/hdiv_rt0.jl:93-100) */
static void rt03_ref_basis(double x, double y, double z, double out[4][3])
{
    out[0][0] = 2 * x; out[0][1] = 2 * y; out[0][2] = 2 * (z - 1);
    out[1][0] = 2 * x; out[1][1] = 2 * (y - 1); out[1][2] = 2 * z;
    out[2][0] = 2 * x; out[2][1] = 2 * y; out[2][2] = 2 * z;
    out[3][0] = 2 * (x - 1); out[3][1] = 2 * y; out[3][2] = 2 * z;
}

static void br3_cell(const br_mesh *m, int cell, double X[12], double nrm[12], double fv[4], double sg[4])
{
    for (int v = 0; v < 4; v++)
        for (int k = 0; k < 3; k++) X[v * 3 + k] = m->coords[(size_t)m->cells[(size_t)cell * 4 + v] * 3 + k];
    for (int f = 0; f < 4; f++) {
        int F = m->cell_faces[(size_t)cell * 4 + f];
        for (int k = 0; k < 3; k++) nrm[f * 3 + k] = m->fnormals[(size_t)F * 3 + k];
        fv[f] = m->fvolumes[F];
        sg[f] = (double)m->signs[(size_t)cell * 4 + f];
    }
}

/* L2 error / norm / difference of an H1BR{dim} function: the ItemIntegrator
 * (src/assemblypatterns/itemintegrator.jl:173-300) on the Bernardi-Raugel
 * element with Identity or Gradient "with coefficients"
 * (src/feevaluator_h1.jl:77-94): cvals[k][dof] = coef(dof, c) * (value or
 * gradient of the scalar basis function s(dof, c)), the coefficient 1 for a
 * vertex DoF and n_F[c] for the bubble of face F; summed DoF by DoF.  Rule
 * order: polyorder(H1BR{dim}) = dim + shift(op) + quadorder. */
int oracle_item_l2error_br(double *cellv, double *total, int dim, int ncells, const double *coords, const int *cells,
                           const int *cell_faces, const double *fnormals, const int *celldofs, const double *u,
                           const double *v, int op, int data_kind, const double *par, int npar, double factor,
                           int quadorder)
{
    if (op != OR_OP_IDENTITY && op != OR_OP_GRADIENT) return -1;
    if (dim != 2 && dim != 3) return -1;
    const int nv = dim + 1, nb = 2 * nv, nd = dim * nv + nv;
    int order = dim + (op == OR_OP_GRADIENT ? -1 : 0) + quadorder;
    if (order < 0) order = 0;
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(dim, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    double vals[OR_MAXQ][8], derivs[OR_MAXQ][8][3];
    for (int q = 0; q < nq; q++) {
        if (dim == 3) {
            br3_basis(&xref[3 * q], vals[q], derivs[q]);
        } else {   /* P1 functions and the bubbles 6 x r, 6 y x, 6 r y (src/fedefs/h1v_br.jl:117-130) */
            dual x[2] = {dvar(xref[3 * q], 0), dvar(xref[3 * q + 1], 1)};
            dual r = dsub(dcsub(1.0, x[0]), x[1]);
            dual o[6] = {r, x[0], x[1], dmul(dscale(6.0, x[0]), r), dmul(dscale(6.0, x[1]), x[0]),
                         dmul(dscale(6.0, r), x[1])};
            for (int a = 0; a < 6; a++) {
                vals[q][a] = o[a].v;
                for (int j = 0; j < 2; j++) derivs[q][a][j] = o[a].d[j];
            }
        }
    }
    (void)nb;
    const int rdim = op == OR_OP_GRADIENT ? dim * dim : dim;
    double acc = 0.0;
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], nrm[12];
        for (int vv = 0; vv < nv; vv++)
            for (int k = 0; k < dim; k++) X[vv * dim + k] = coords[(size_t)cells[(size_t)cell * nv + vv] * dim + k];
        for (int f = 0; f < nv; f++)
            for (int k = 0; k < dim; k++) nrm[f * dim + k] = fnormals[(size_t)cell_faces[(size_t)cell * nv + f] * dim + k];
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(dim, X, A, G, &det, &vol);
        double cellacc = 0.0;
        for (int q = 0; q < nq; q++) {
            double in1[9] = {0}, in2[9] = {0}, f[9] = {0};
            for (int dof = 0; dof < nd; dof++) {
                double cv[9] = {0};
                for (int c = 0; c < dim; c++) {
                    const int sidx = dof < dim * nv ? (dof / nv == c ? dof % nv : -1) : nv + (dof - dim * nv);
                    if (sidx < 0) continue;
                    const double coef = dof < dim * nv ? 1.0 : nrm[(dof - dim * nv) * dim + c];
                    if (op == OR_OP_IDENTITY) {
                        cv[c] = vals[q][sidx] * coef;
                    } else {
                        for (int k = 0; k < dim; k++) {
                            double g = 0.0;
                            for (int j = 0; j < dim; j++) g += G[k][j] * derivs[q][sidx][j];
                            cv[c * dim + k] = g * coef;
                        }
                    }
                }
                const double c1 = u[celldofs[(size_t)cell * nd + dof]];
                const double c2 = v ? v[celldofs[(size_t)cell * nd + dof]] : 0.0;
                for (int k = 0; k < rdim; k++) {
                    in1[k] += c1 * cv[k];
                    in2[k] += c2 * cv[k];
                }
            }
            double result = 0.0;
            if (v) {
                for (int j = 0; j < rdim; j++) result += (in1[j] - in2[j]) * (in1[j] - in2[j]);
            } else {
                if (data_kind >= 0) {
                    double x[3] = {0, 0, 0};
                    for (int k = 0; k < dim; k++) {
                        x[k] = X[k];
                        for (int j = 0; j < dim; j++) x[k] += A[k][j] * xref[3 * q + j];
                    }
                    rhs_eval(data_kind, dim, rdim, par, npar, cell, x, f);
                }
                for (int j = 0; j < rdim; j++) {
                    const double e = f[j] - in1[j] * factor;
                    result += e * e;
                }
            }
            const double contrib = result * w[q] * vol;
            cellacc += contrib;
            acc += contrib;
        }
        if (cellv) cellv[cell] = cellacc;
    }
    if (total) *total = acc;
    return nq;
}

/* nu (grad u, grad v) on H1BR{3} (Gradient with coefficients) plus
 * lambda (div R u, div R v) with R the RT0 reconstruction; both on the rule of
 * order 2 (polyorder 3 - 1) = 4.  The reconstructed divergence follows
 * src/feevaluator_h1.jl:409-437: sum over faces and the three partial
 * derivatives (2 each) of R * dphi * sign, divided by det A. */
int oracle_br3_assemble(void *h, int ncells, const double *coords, const int *cells, const int *cell_faces,
                        const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                        double nu, const double *cellnu, double lambda)
{
    omat *M = (omat *)h;
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(3, 4, xref, w);
    if (nq < 0) nq = -nq;
    double vals[OR_MAXQ][8], derivs[OR_MAXQ][8][3];
    for (int q = 0; q < nq; q++) br3_basis(&xref[3 * q], vals[q], derivs[q]);
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], nrm[12], fv[4], sg[4];
        br3_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(3, X, A, G, &det, &vol);
        const int *dofs = &celldofs[(size_t)cell * 16];
        static double cv[OR_MAXQ][16][9];
        for (int q = 0; q < nq; q++)
            for (int dof = 0; dof < 16; dof++)
                for (int c = 0; c < 3; c++)
                    for (int k = 0; k < 3; k++) {
                        const int sidx = br3_scalar(dof, c);
                        double s = 0;
                        for (int j = 0; j < 3; j++) s += G[k][j] * (sidx >= 0 ? derivs[q][sidx][j] : 0.0);
                        s *= br3_coef(dof, c, nrm);
                        cv[q][dof][k + 3 * c] = s;
                    }
        double loc[16][16];
        memset(loc, 0, sizeof(loc));
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < 16; i++) {
                double res[9];
                for (int k = 0; k < 9; k++) res[k] = cellnu ? cellnu[cell] * cv[q][i][k] : cv[q][i][k];
                for (int j = i; j < 16; j++) {
                    double t = 0;
                    for (int k = 0; k < 9; k++) t += res[k] * cv[q][j][k];
                    loc[i][j] += w[q] * t;
                }
            }
        const double itemfactor = vol * (cellnu ? 1.0 : nu);
        for (int i = 0; i < 16; i++)
            for (int j = i + 1; j < 16; j++) {
                omat_addnz(M, dofs[i], dofs[j], loc[i][j] * itemfactor, 1.0);
                omat_addnz(M, dofs[j], dofs[i], loc[i][j] * itemfactor, 1.0);
            }
        for (int i = 0; i < 16; i++) omat_addnz(M, dofs[i], dofs[i], loc[i][i] * itemfactor, 1.0);
        if (lambda == 0.0) continue;
        double R[16][4];
        br3_rt0_coeffs(fv, nrm, R);
        double dv[16];
        for (int i = 0; i < 16; i++) {
            double s = 0;
            for (int j = 0; j < 4; j++)
                if (R[i][j] != 0)
                    for (int jd = 0; jd < 3; jd++) s += R[i][j] * 2.0 * sg[j];
            dv[i] = s / fabs(det);
        }
        double lp[16][16];
        memset(lp, 0, sizeof(lp));
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < 16; i++)
                for (int j = 0; j < 16; j++) {
                    double t = 0;
                    t += dv[i] * dv[j];
                    lp[i][j] += w[q] * t;
                }
        const double pf = vol * lambda;
        for (int i = 0; i < 16; i++)
            for (int j = 0; j < 16; j++) omat_addnz(M, dofs[i], dofs[j], lp[i][j] * pf, 1.0);
    }
    return nq;
}

/* b += factor * (f, R v) on H1BR{3}, f polynomial (3 components), with the
 * ReconstructionIdentity{HDIVRT0{3}} test operator (src/feevaluator_h1.jl:
 * 342-381): Piola A phi_hat * sign / det; quadrature order 3 + bonus. */
int oracle_br3_rhs(double *b, int ncells, const double *coords, const int *cells, const int *cell_faces,
                   const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                   const double *par, int npar, double factor, int bonus_quadorder)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(3, 3 + bonus_quadorder, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], nrm[12], fv[4], sg[4];
        br3_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(3, X, A, G, &det, &vol);
        double R[16][4];
        br3_rt0_coeffs(fv, nrm, R);
        double locb[16] = {0};
        for (int q = 0; q < nq; q++) {
            double rt[4][3];
            rt03_ref_basis(xref[3 * q], xref[3 * q + 1], xref[3 * q + 2], rt);
            double te[4][3];
            for (int j = 0; j < 4; j++)
                for (int k = 0; k < 3; k++) {
                    double s = 0;
                    for (int l = 0; l < 3; l++) s += A[k][l] * rt[j][l];
                    s *= sg[j] / fabs(det);
                    te[j][k] = s;
                }
            double x[3], f[3];
            for (int k = 0; k < 3; k++) {
                x[k] = X[k];
                for (int j = 0; j < 3; j++) x[k] += A[k][j] * xref[3 * q + j];
            }
            rhs_eval(OR_RHS_POLY, 3, 3, par, npar, cell, x, f);
            for (int i = 0; i < 16; i++) {
                double cvv[3] = {0, 0, 0};
                for (int j = 0; j < 4; j++)
                    if (R[i][j] != 0)
                        for (int k = 0; k < 3; k++) cvv[k] += R[i][j] * te[j][k];
                double t = 0;
                for (int k = 0; k < 3; k++) t += f[k] * cvv[k];
                locb[i] += t * w[q];
            }
        }
        const double itemfactor = factor * vol;
        for (int i = 0; i < 16; i++) b[celldofs[(size_t)cell * 16 + i]] += locb[i] * itemfactor;
    }
    return nq;
}

/* H1BR{3} -> HDIVBDM1{3} reconstruction (src/reconstructions.jl:493-535):
 * R phi is the BDM1 function (a linear vector field on the tetrahedron)
 * whose normal-flux moments against P1 on every face equal those of phi --
 * the functionals the reference's coefficients encode: for a P1 function
 * lambda_p e_k the constant moment |F| n_k / 3 (its RT0 coefficient) and the
 * linear moments int_F lambda_p (lambda_a - 1/3) n_k = |F| n_k (1/18 if
 * a = p, -1/36 otherwise) (_P1_INTO_BDM1_COEFFS_3D), for a face bubble its
 * flux |F| and vanishing linear moments.  The reference's choice of two of
 * the three linear moments per face by CellFaceOrientations only selects a
 * basis; R phi does not depend on it, so it is computed here from the
 * moments themselves.  On face f with vertices V and moments m_a = int_F
 * (phi . n_F) lambda_a (a in V), the normal components of the linear field
 * at the face's vertices are s_i = (12/|F|) (m_i - (m_0 + m_1 + m_2)/4)
 * (the inverse of the P1 mass matrix of the face); the field's value w_i at
 * vertex i solves n_F . w_i = s_i^F over the three faces at i.  Output
 * W[dof][vertex][component]. */
static void br3_bdm1_fields(const double *fvol, const double *nrm, double W[16][4][3])
{
    for (int dof = 0; dof < 16; dof++) {
        double s[4][3];   /* [face][position in BR3_FACES[face]] */
        for (int f = 0; f < 4; f++) {
            const double *nf = &nrm[f * 3];
            double m[3] = {0, 0, 0};
            for (int a = 0; a < 3; a++) {
                const int va = BR3_FACES[f][a];
                if (dof < 12) {
                    const int k = dof / 4, p = dof % 4;
                    int onface = 0;
                    for (int b = 0; b < 3; b++) onface |= BR3_FACES[f][b] == p;
                    if (onface) m[a] = nf[k] * fvol[f] * (va == p ? 2.0 : 1.0) / 12.0;
                } else if (dof - 12 == f) {
                    const double nn = nf[0] * nf[0] + nf[1] * nf[1] + nf[2] * nf[2];
                    m[a] = nn * fvol[f] / 3.0;   /* 60 int_F l_i l_j l_k l_a = |F| / 3 */
                }
            }
            const double mean = (m[0] + m[1] + m[2]) / 4.0;
            for (int a = 0; a < 3; a++) s[f][a] = (12.0 / fvol[f]) * (m[a] - mean);
        }
        for (int i = 0; i < 4; i++) {
            double N[3][3], r[3];
            int row = 0;
            for (int f = 0; f < 4; f++)
                for (int a = 0; a < 3; a++)
                    if (BR3_FACES[f][a] == i) {
                        for (int k = 0; k < 3; k++) N[row][k] = nrm[f * 3 + k];
                        r[row++] = s[f][a];
                    }
            /* Cramer's rule on the 3 x 3 system N w = r */
            const double det = N[0][0] * (N[1][1] * N[2][2] - N[1][2] * N[2][1]) -
                               N[0][1] * (N[1][0] * N[2][2] - N[1][2] * N[2][0]) +
                               N[0][2] * (N[1][0] * N[2][1] - N[1][1] * N[2][0]);
            for (int c = 0; c < 3; c++) {
                double M[3][3];
                for (int x = 0; x < 3; x++)
                    for (int y = 0; y < 3; y++) M[x][y] = (y == c) ? r[x] : N[x][y];
                const double dc = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                                  M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                                  M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
                W[dof][i][c] = dc / det;
            }
        }
    }
}

/* b += LinearForm(ReconstructionIdentity{HDIVRT0{3}} (recon 1) or
 * {HDIVBDM1{3}} (recon 2), f) on H1BR{3}: the RT0 case as oracle_br3_rhs,
 * the BDM1 case with R phi from br3_bdm1_fields (linear in the barycentric
 * coordinates: R phi(x_q) = sum_i lambda_i(x_q) w_i). */
int oracle_br3_rhs_recon(double *b, int ncells, const double *coords, const int *cells, const int *cell_faces,
                         const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                         const double *par, int npar, double factor, int bonus_quadorder, int recon)
{
    if (recon == 1)
        return oracle_br3_rhs(b, ncells, coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs, par, npar,
                              factor, bonus_quadorder);
    if (recon != 2) return -1;
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(3, 3 + bonus_quadorder, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], nrm[12], fv[4], sg[4];
        br3_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(3, X, A, G, &det, &vol);
        double W[16][4][3];
        br3_bdm1_fields(fv, nrm, W);
        double locb[16] = {0};
        for (int q = 0; q < nq; q++) {
            const double *xr = &xref[3 * q];
            const double lam[4] = {1.0 - xr[0] - xr[1] - xr[2], xr[0], xr[1], xr[2]};
            double x[3], f[3];
            for (int k = 0; k < 3; k++) {
                x[k] = X[k];
                for (int j = 0; j < 3; j++) x[k] += A[k][j] * xr[j];
            }
            rhs_eval(OR_RHS_POLY, 3, 3, par, npar, cell, x, f);
            for (int i = 0; i < 16; i++) {
                double t = 0;
                for (int k = 0; k < 3; k++) {
                    double rv = 0;
                    for (int v = 0; v < 4; v++) rv += lam[v] * W[i][v][k];
                    t += f[k] * rv;
                }
                locb[i] += t * w[q];
            }
        }
        const double itemfactor = factor * vol;
        for (int i = 0; i < 16; i++) b[celldofs[(size_t)cell * 16 + i]] += locb[i] * itemfactor;
    }
    return nq;
}

/* L2ErrorIntegrator(data, ReconstructionIdentity{HDIVRT0{3}} (recon 1) /
 * {HDIVBDM1{3}} (recon 2)) of an H1BR{3} function u (the velocity error of
 * the reference's p-robust tests, test/runtests.jl:627-638): sum over cells
 * of int_T |R u - f|^2 with f polynomial data (params as rhs_eval's POLY),
 * quadrature of order `order`.  Returns the sum (the squared error). */
double oracle_br3_recon_l2error(int ncells, const double *coords, const int *cells, const int *cell_faces,
                                const double *fnormals, const double *fvolumes, const signed char *signs,
                                const int *celldofs, const double *u, const double *par, int npar, int recon,
                                int order)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(3, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1.0;
    double total = 0;
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], nrm[12], fv[4], sg[4];
        br3_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(3, X, A, G, &det, &vol);
        double W[16][4][3], R[16][4];
        if (recon == 2) br3_bdm1_fields(fv, nrm, W);
        else br3_rt0_coeffs(fv, nrm, R);
        const int *dofs = &celldofs[(size_t)cell * 16];
        double e = 0;
        for (int q = 0; q < nq; q++) {
            const double *xr = &xref[3 * q];
            const double lam[4] = {1.0 - xr[0] - xr[1] - xr[2], xr[0], xr[1], xr[2]};
            double ru[3] = {0, 0, 0};
            if (recon == 2) {
                for (int j = 0; j < 16; j++)
                    for (int v = 0; v < 4; v++)
                        for (int k = 0; k < 3; k++) ru[k] += u[dofs[j]] * lam[v] * W[j][v][k];
            } else {
                double rt[4][3];
                rt03_ref_basis(xr[0], xr[1], xr[2], rt);
                for (int f = 0; f < 4; f++) {
                    double cf = 0;
                    for (int j = 0; j < 16; j++) cf += u[dofs[j]] * R[j][f];
                    for (int k = 0; k < 3; k++) {
                        double t = 0;
                        for (int l = 0; l < 3; l++) t += A[k][l] * rt[f][l];
                        ru[k] += cf * t * sg[f] / fabs(det);
                    }
                }
            }
            double x[3], f[3];
            for (int k = 0; k < 3; k++) {
                x[k] = X[k];
                for (int j = 0; j < 3; j++) x[k] += A[k][j] * xr[j];
            }
            rhs_eval(OR_RHS_POLY, 3, 3, par, npar, cell, x, f);
            double r2 = 0;
            for (int k = 0; k < 3; k++) r2 += (ru[k] - f[k]) * (ru[k] - f[k]);
            e += r2 * w[q];
        }
        total += e * vol;
    }
    return total;
}

/* Linear face moments of the BDM1 reconstruction of the P1 function
 * lambda_p e_k on face f, int_F (R phi . n_F)(lambda_a - 1/3) for the face's
 * three vertices a, divided by |F| n_F[k] (the entries of the reference's
 * _P1_INTO_BDM1_COEFFS_3D when p lies on the face); for checking the
 * reconstruction against that table. */
void oracle_br3_bdm1_moments(const double *fvol, const double *nrm, int p, int k, int f, double out[3])
{
    double W[16][4][3];
    br3_bdm1_fields(fvol, nrm, W);
    const double *nf = &nrm[f * 3];
    double sn[3];   /* normal component of R phi at the face's vertices */
    for (int a = 0; a < 3; a++) {
        const int v = BR3_FACES[f][a];
        sn[a] = W[4 * k + p][v][0] * nf[0] + W[4 * k + p][v][1] * nf[1] + W[4 * k + p][v][2] * nf[2];
    }
    /* int_F (sum_b sn_b l_b)(l_a - 1/3) = |F| (sum_b sn_b (1 + d_ab)/12 - (sum_b sn_b)/9) */
    const double tot = sn[0] + sn[1] + sn[2];
    for (int a = 0; a < 3; a++) {
        const double ma = (tot + sn[a]) / 12.0 - tot / 9.0;
        out[a] = ma / nf[k];
    }
}

/* Divergence of H1BR{3} functions with coefficients on the rule of order 2
 * (polyorder 3 - 1 + 0 for (div u, q_P0); exact for the quadratic divergence
 * of the bubbles): divu[cell] = (1/|T|) int_T div u and
 * b[dof] += int_T p_T div phi_dof (either output may be NULL). */
void oracle_br3_div(int ncells, const double *coords, const int *cells, const int *cell_faces, const double *fnormals,
                    const double *fvolumes, const signed char *signs, const int *celldofs, const double *u,
                    const double *p, double *divu, double *b)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(3, 2, xref, w);
    double vals[OR_MAXQ][8], derivs[OR_MAXQ][8][3];
    for (int q = 0; q < nq; q++) br3_basis(&xref[3 * q], vals[q], derivs[q]);
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], nrm[12], fv[4], sg[4];
        br3_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(3, X, A, G, &det, &vol);
        const int *dofs = &celldofs[(size_t)cell * 16];
        double dint = 0;
        double lb[16] = {0};
        for (int q = 0; q < nq; q++) {
            double dq = 0;
            for (int dof = 0; dof < 16; dof++) {
                double cv = 0;
                for (int k = 0; k < 3; k++)
                    for (int j = 0; j < 3; j++) {
                        const int sidx = br3_scalar(dof, k);
                        cv += G[k][j] * (sidx >= 0 ? derivs[q][sidx][j] : 0.0) * br3_coef(dof, k, nrm);
                    }
                if (u) dq += u[dofs[dof]] * cv;
                if (b && p) lb[dof] += (p[cell] * cv) * w[q];
            }
            dint += dq * w[q];
        }
        if (divu) divu[cell] = dint;
        if (b && p)
            for (int dof = 0; dof < 16; dof++) b[dofs[dof]] += lb[dof] * vol;
    }
}

/* Divergence of H1BR{2} functions with coefficients
 * (src/feevaluator_h1.jl:133-145) at the midpoint: per cell
 * divu[cell] = (1/|T|) int_T div u  (the rule of order 1 is exact), and
 * b[dof] += int_T p_T div phi_dof  (the (p, div v) term of the velocity
 * update, BilinearForm([Divergence, Identity]; factor = -1) moved to the
 * right-hand side).  Either output may be NULL. */
void oracle_br_div(int ncells, const double *coords, const int *cells, const int *cell_faces, const double *fnormals,
                   const double *fvolumes, const signed char *signs, const int *celldofs, const double *u,
                   const double *p, double *divu, double *b)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(2, 1, xref, w);
    double derivs[OR_MAXQ * 6 * 2];
    for (int q = 0; q < nq; q++) {
        dual x[2] = {dvar(xref[3 * q], 0), dvar(xref[3 * q + 1], 1)};
        dual r = dsub(dcsub(1.0, x[0]), x[1]);
        dual o[6] = {r, x[0], x[1], dmul(dscale(6.0, x[0]), r), dmul(dscale(6.0, x[1]), x[0]), dmul(dscale(6.0, r), x[1])};
        for (int a = 0; a < 6; a++) { derivs[(q * 6 + a) * 2] = o[a].d[0]; derivs[(q * 6 + a) * 2 + 1] = o[a].d[1]; }
    }
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], nrm[6], fv[3], sg[3];
        br_cell(&m, cell, X, nrm, fv, sg);
        double A[3][3], G[3][3], det, vol;
        oracle_geometry(2, X, A, G, &det, &vol);
        const int *dofs = &celldofs[(size_t)cell * 9];
        double dint = 0;
        double lb[9] = {0};
        for (int q = 0; q < nq; q++) {
            double dq = 0;
            for (int dof = 0; dof < 9; dof++) {
                double cv = 0;
                for (int k = 0; k < 2; k++)
                    for (int j = 0; j < 2; j++) {
                        double d[2];
                        br_component_derivs(dof, k, q, 6, derivs, d);
                        cv += G[k][j] * d[j] * br_coef(dof, k, nrm);
                    }
                if (u) dq += u[dofs[dof]] * cv;
                if (b && p) lb[dof] += (p[cell] * cv) * w[q];
            }
            dint += dq * w[q];
        }
        if (divu) divu[cell] = dint;
        if (b && p)
            for (int i = 0; i < 9; i++) b[dofs[i]] += lb[i] * vol;
    }
}

/* ------------------------------------------------------------------------- */
/* H1P2B{2,2} with the RT1 / BDM2 reconstructions, 2D triangles              */
/* ------------------------------------------------------------------------- */

/* Local DoFs (src/fedefs/h1_p2b.jl:33 "N1F1I1", components blocked): 7k + s,
 * s = 0-2 nodes, 3-5 faces (face f joins nodes f and f+1 mod 3), 6 the cell
 * bubble.  Scalar basis on duals: the P2 functions of src/fedefs/h1_p2.jl:
 * 134-144 and the bubble 60 (1-x-y) x y of src/fedefs/h1_p2b.jl:126-137. */
static void p2b_basis_dual(double xi, double eta, dual o[7])
{
    dual x = dvar(xi, 0), y = dvar(eta, 1);
    dual l = dsub(dcsub(1.0, x), y);
    o[0] = dmul(dscale(2.0, l), dsubc(l, 0.5));
    o[1] = dmul(dscale(2.0, x), dsubc(x, 0.5));
    o[2] = dmul(dscale(2.0, y), dsubc(y, 0.5));
    o[3] = dmul(dscale(4.0, l), x);
    o[4] = dmul(dscale(4.0, x), y);
    o[5] = dmul(dscale(4.0, y), l);
    o[6] = dmul(dmul(dscale(60.0, dsub(dcsub(1.0, x), y)), x), y);
}

/* HDIVRT1{2} reference basis (src/fedefs/hdiv_rt1.jl:106-121): RT0 of face
 * f at 2f, its linear-flux partner at 2f+1, interior functions 6, 7. */
static void rt1_ref_basis(double x, double y, double o[8][2])
{
    o[0][0] = x; o[0][1] = y - 1;
    o[2][0] = x; o[2][1] = y;
    o[4][0] = x - 1; o[4][1] = y;
    for (int k = 0; k < 2; k++) {
        o[1][k] = -12 * (0.5 - x - y) * o[0][k];
        o[3][k] = -(12 * (x - 0.5)) * o[2][k];
        o[5][k] = -(12 * (y - 0.5)) * o[4][k];
        o[6][k] = 12 * y * o[0][k];
        o[7][k] = 12 * x * o[4][k];
    }
}

/* HDIVBDM2{2} reference basis (src/fedefs/hdiv_bdm2.jl:171-194): per face f
 * the RT0 function (3f), the linear BDM1 function (3f+1) and the quadratic
 * one (3f+2); interior functions 9-11. */
static void bdm2_ref_basis(double x, double y, double o[12][2])
{
    const double l = 1 - x - y;
    o[0][0] = x; o[0][1] = y - 1;
    o[3][0] = x; o[3][1] = y;
    o[6][0] = x - 1; o[6][1] = y;
    o[1][0] = 6 * x; o[1][1] = 6 - 12 * x - 6 * y;
    o[4][0] = -6 * x; o[4][1] = 6 * y;
    o[7][0] = 6 * (x - 1) + 12 * y; o[7][1] = -6 * y;
    for (int k = 0; k < 2; k++) {
        o[2][k] = -15 * ((l - 0.5) * o[1][k] + o[0][k]);
        o[5][k] = -15 * ((x - 0.5) * o[4][k] + o[3][k]);
        o[8][k] = -15 * ((y - 0.5) * o[7][k] + o[6][k]);
        o[9][k] = y * o[1][k];
        o[10][k] = l * o[4][k];
        o[11][k] = x * o[7][k];
    }
}

/* Number of reconstruction functions and the element coefficients (face
 * signs): RT1 (hdiv_rt1.jl:124-135) signs the RT0 functions 2f, BDM2
 * (hdiv_bdm2.jl:197-210) the functions 3f and 3f+2. */
static int p2b_recon_target(int recon, const double sg[3], double coef[12])
{
    const int nr = recon == 4 ? 12 : 8;
    for (int j = 0; j < nr; j++) coef[j] = 1.0;
    for (int f = 0; f < 3; f++) {
        if (recon == 4) { coef[3 * f] = sg[f]; coef[3 * f + 2] = sg[f]; }
        else coef[2 * f] = sg[f];
    }
    return nr;
}

static void p2b_recon_basis(int recon, double x, double y, double o[12][2])
{
    if (recon == 4) bdm2_ref_basis(x, y, o);
    else {
        double t[8][2];
        rt1_ref_basis(x, y, t);
        for (int j = 0; j < 8; j++) { o[j][0] = t[j][0]; o[j][1] = t[j][1]; }
    }
}

/* Face part of the reconstruction coefficients R[14][nr]
 * (src/reconstructions.jl:405-469): for the two nodes n of face f and each
 * component k, RT0 column (1/6)|F| n_k, linear column c_n |F| n_k s_f with
 * c = (-1/12, 1/12), BDM2's quadratic column (1/90)|F| n_k; the face DoF
 * gets (2/3)|F| n_k in the RT0 column and BDM2's quadratic column -(1/45)|F| n_k. */
static void p2b_face_coeffs(int recon, const double fv[3], const double nrm[6], const double sg[3], double R[14][12])
{
    const double c[2] = {-1.0 / 12.0, 1.0 / 12.0};
    const int w = recon == 4 ? 3 : 2;
    memset(R, 0, sizeof(double) * 14 * 12);
    for (int f = 0; f < 3; f++) {
        const int nodes[2] = {f, (f + 1) % 3};
        for (int n = 0; n < 2; n++)
            for (int k = 0; k < 2; k++) {
                R[7 * k + nodes[n]][w * f] = (1.0 / 6.0) * fv[f] * nrm[f * 2 + k];
                R[7 * k + nodes[n]][w * f + 1] = c[n] * fv[f] * nrm[f * 2 + k] * sg[f];
                if (recon == 4) R[7 * k + nodes[n]][w * f + 2] = (1.0 / 90.0) * fv[f] * nrm[f * 2 + k];
            }
        for (int k = 0; k < 2; k++) {
            R[7 * k + 3 + f][w * f] = (2.0 / 3.0) * fv[f] * nrm[f * 2 + k];
            if (recon == 4) R[7 * k + 3 + f][w * f + 2] = (-1.0 / 45.0) * fv[f] * nrm[f * 2 + k];
        }
    }
}

/* Interior RT1 coefficients (columns 6, 7; src/reconstructions.jl:43-161):
 * the integrals of the face RT1 functions over the cell from closed forms in
 * the vertices C, edge midpoints E and centroid M, the inverse of the 2x2
 * integral matrix of the interior functions, and for every P2B function the
 * interior pair that restores its cell integral (node functions 0, face
 * functions |T|/3, bubble |T| in its own component). */
static void p2b_rt1_interior(const double X[6], const double sg[3], double vol, double R[14][12])
{
    double M[2] = {0, 0}, E[2][3] = {{0, 0, 0}, {0, 0, 0}}, A[2][8];
    for (int n = 0; n < 3; n++)
        for (int k = 0; k < 2; k++) M[k] += X[n * 2 + k] / 3;
    for (int f = 0; f < 3; f++)
        for (int n = 0; n < 2; n++)
            for (int k = 0; k < 2; k++) E[k][f] += X[((f + n) % 3) * 2 + k] / 2;
    for (int k = 0; k < 2; k++) {
        A[k][0] = (M[k] - X[2 * 2 + k]) / 2 * sg[0];
        A[k][1] = X[1 * 2 + k] - E[k][1];
        A[k][2] = (M[k] - X[0 * 2 + k]) / 2 * sg[1];
        A[k][3] = X[2 * 2 + k] - E[k][2];
        A[k][4] = (M[k] - X[1 * 2 + k]) / 2 * sg[2];
        A[k][5] = X[0 * 2 + k] - E[k][0];
    }
    A[1][7] = (E[0][0] - X[2 * 2 + 0]);
    A[1][6] = -(E[1][0] - X[2 * 2 + 1]);
    A[0][7] = -(E[0][2] - X[1 * 2 + 0]);
    A[0][6] = (E[1][2] - X[1 * 2 + 1]);
    const double det = A[0][6] * A[1][7] - A[1][6] * A[0][7];
    A[0][6] /= det; A[0][7] /= det; A[1][6] /= det; A[1][7] /= det;
    for (int k = 0; k < 2; k++) {
        for (int n = 0; n < 3; n++) {
            for (int pass = 0; pass < 2; pass++) {   /* node function, then face function */
                const int dof = 7 * k + n + 3 * pass;
                double b[2] = {0, 0};
                if (pass == 1) b[k] = vol / 3;
                for (int c = 0; c < 2; c++)
                    for (int j = 0; j < 6; j++) b[c] -= R[dof][j] * A[c][j];
                for (int kk = 0; kk < 2; kk++) R[dof][6 + kk] = A[kk][6] * b[0] + A[kk][7] * b[1];
            }
        }
        const int dof = 7 * k + 6;
        double b[2] = {0, 0};
        b[k] = vol;
        for (int kk = 0; kk < 2; kk++) R[dof][6 + kk] = A[kk][6] * b[0] + A[kk][7] * b[1];
    }
}

/* x = M^{-1} b for a 3x3 matrix: LU with partial pivoting (the factorisation
 * lu() computes for a small dense matrix), then the two triangular solves. */
static void p2b_lu3(double M[3][3], int piv[3])
{
    for (int j = 0; j < 3; j++) {
        int p = j;
        for (int i = j + 1; i < 3; i++)
            if (fabs(M[i][j]) > fabs(M[p][j])) p = i;
        piv[j] = p;
        if (p != j)
            for (int c = 0; c < 3; c++) { double t = M[j][c]; M[j][c] = M[p][c]; M[p][c] = t; }
        for (int i = j + 1; i < 3; i++) {
            M[i][j] /= M[j][j];
            for (int c = j + 1; c < 3; c++) M[i][c] -= M[i][j] * M[j][c];
        }
    }
}

static void p2b_lu3_solve(const double M[3][3], const int piv[3], const double b[3], double x[3])
{
    double y[3] = {b[0], b[1], b[2]};
    for (int j = 0; j < 3; j++)
        if (piv[j] != j) { double t = y[j]; y[j] = y[piv[j]]; y[piv[j]] = t; }
    for (int i = 1; i < 3; i++)
        for (int j = 0; j < i; j++) y[i] -= M[i][j] * y[j];
    for (int i = 2; i >= 0; i--) {
        for (int j = i + 1; j < 3; j++) y[i] -= M[i][j] * y[j];
        y[i] /= M[i][i];
    }
    x[0] = y[0]; x[1] = y[1]; x[2] = y[2];
}

/* Interior BDM2 coefficients (columns 9-11; src/reconstructions.jl:164-330):
 * on the order-4 rule, the moments of the interior BDM2 functions, of the
 * face BDM2 functions and of every P2B function against grad(P1 functions
 * 1, 2) and curl(cell bubble), then per P2B function the 3x3 solve that makes
 * the reconstruction keep those moments. */
static void p2b_bdm2_interior(const double A[3][3], const double G[3][3], double det, double vol, const double sg[3],
                              double R[14][12])
{
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(2, 4, xref, w);
    if (nq < 0) nq = -nq;
    double coef[12];
    p2b_recon_target(4, sg, coef);
    double IMM[3][3] = {{0}}, IMMf[3][9] = {{0}};
    double b1[OR_MAXQ][14][2], b2[OR_MAXQ][12][2], b3[2][2], b4[OR_MAXQ][2];
    /* grad of the P1 functions 1 - x - y and x (constant) */
    const double dp1[2][2] = {{-1, -1}, {1, 0}};
    for (int a = 0; a < 2; a++)
        for (int k = 0; k < 2; k++) {
            double s = 0;
            for (int j = 0; j < 2; j++) s += G[k][j] * dp1[a][j];
            b3[a][k] = s;
        }
    for (int q = 0; q < nq; q++) {
        const double xi = xref[3 * q], eta = xref[3 * q + 1];
        dual o[7];
        p2b_basis_dual(xi, eta, o);
        for (int dof = 0; dof < 14; dof++) {
            const int k = dof / 7, s = dof % 7;
            b1[q][dof][k] = o[s].v;
            b1[q][dof][1 - k] = 0.0;
        }
        double rb[12][2];
        bdm2_ref_basis(xi, eta, rb);
        for (int j = 0; j < 12; j++)
            for (int k = 0; k < 2; k++) {
                double s = 0;
                for (int l = 0; l < 2; l++) s += A[k][l] * rb[j][l];
                s *= coef[j] / det;
                b2[q][j][k] = s;
            }
        /* CurlScalar of the bubble (src/feevaluator_h1.jl:270-285): (-d/dy, d/dx) */
        double cu[2] = {0, 0};
        for (int j = 0; j < 2; j++) {
            cu[0] -= G[1][j] * o[6].d[j];
            cu[1] += G[0][j] * o[6].d[j];
        }
        b4[q][0] = cu[0];
        b4[q][1] = cu[1];
    }
    for (int q = 0; q < nq; q++)
        for (int dof = 0; dof < 3; dof++) {
            for (int d2 = 0; d2 < 2; d2++) {
                double t = 0;
                for (int k = 0; k < 2; k++) t += b2[q][9 + dof][k] * b3[d2][k];
                IMM[d2][dof] += t * vol * w[q];
            }
            double t = 0;
            for (int k = 0; k < 2; k++) t += b2[q][9 + dof][k] * b4[q][k];
            IMM[2][dof] += t * vol * w[q];
            for (int d2 = 0; d2 < 9; d2++) {
                double u = 0;
                for (int k = 0; k < 2; k++) u += (dof < 2 ? b3[dof][k] : b4[q][k]) * b2[q][d2][k];
                IMMf[dof][d2] += u * vol * w[q];
            }
        }
    int piv[3];
    p2b_lu3(IMM, piv);
    for (int d1 = 0; d1 < 14; d1++) {
        double lb[3] = {0, 0, 0};
        for (int q = 0; q < nq; q++) {
            for (int id = 0; id < 2; id++) {
                double t = 0;
                for (int k = 0; k < 2; k++) t += b1[q][d1][k] * b3[id][k];
                lb[id] += t * vol * w[q];
            }
            double t = 0;
            for (int k = 0; k < 2; k++) t += b1[q][d1][k] * b4[q][k];
            lb[2] += t * vol * w[q];
        }
        for (int id = 0; id < 3; id++)
            for (int d2 = 0; d2 < 9; d2++) lb[id] -= R[d1][d2] * IMMf[id][d2];
        double x[3];
        p2b_lu3_solve(IMM, piv, lb, x);
        for (int id = 0; id < 3; id++) R[d1][9 + id] = x[id];
    }
}

/* All reconstruction coefficients R[14][nr] of one cell (recon 3 = RT1,
 * 4 = BDM2; get_rcoefficients!, src/reconstructions.jl:34-40). */
static int p2b_coeffs(int recon, const double X[6], const double A[3][3], const double G[3][3], double det,
                      double vol, const double fv[3], const double nrm[6], const double sg[3], double R[14][12])
{
    p2b_face_coeffs(recon, fv, nrm, sg, R);
    if (recon == 4) p2b_bdm2_interior(A, G, det, vol, sg, R);
    else p2b_rt1_interior(X, sg, vol, R);
    return recon == 4 ? 12 : 8;
}

/* Coefficients of every cell: out[ncells][14][12] (columns past nr zero). */
void oracle_p2b_coeffs(int ncells, const double *coords, const int *cells, const int *cell_faces,
                       const double *fnormals, const double *fvolumes, const signed char *signs, int recon,
                       double *out)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, NULL};
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], nrm[6], fv[3], sg[3], A[3][3], G[3][3], det, vol, R[14][12];
        br_cell(&m, cell, X, nrm, fv, sg);
        oracle_geometry(2, X, A, G, &det, &vol);
        p2b_coeffs(recon, X, A, G, det, vol, fv, nrm, sg, R);
        memcpy(out + (size_t)cell * 168, R, sizeof(R));
    }
}

/* b += factor * (f, R v) over H1P2B{2,2}, R = ReconstructionIdentity{HDIVRT1{2}}
 * (recon 3) or {HDIVBDM2{2}} (recon 4), f polynomial with 2 components
 * (src/feevaluator_h1.jl:342-381, src/assemblypatterns/linearform.jl:181-220);
 * quadrature order polyorder(H1P2B) = 3 plus bonus. */
int oracle_p2b_rhs_recon(double *b, int ncells, const double *coords, const int *cells, const int *cell_faces,
                         const double *fnormals, const double *fvolumes, const signed char *signs, const int *celldofs,
                         const double *par, int npar, double factor, int bonus_quadorder, int recon)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(2, 3 + bonus_quadorder, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], nrm[6], fv[3], sg[3], A[3][3], G[3][3], det, vol, R[14][12];
        br_cell(&m, cell, X, nrm, fv, sg);
        oracle_geometry(2, X, A, G, &det, &vol);
        const int nr = p2b_coeffs(recon, X, A, G, det, vol, fv, nrm, sg, R);
        double coef[12];
        p2b_recon_target(recon, sg, coef);
        double locb[14] = {0};
        for (int q = 0; q < nq; q++) {
            double rb[12][2], te[12][2];
            p2b_recon_basis(recon, xref[3 * q], xref[3 * q + 1], rb);
            for (int j = 0; j < nr; j++)
                for (int k = 0; k < 2; k++) {
                    double s = 0;
                    for (int l = 0; l < 2; l++) s += A[k][l] * rb[j][l];
                    s *= coef[j] / det;
                    te[j][k] = s;
                }
            double x[2], f[2];
            for (int k = 0; k < 2; k++) {
                x[k] = X[k];
                for (int j = 0; j < 2; j++) x[k] += A[k][j] * xref[3 * q + j];
            }
            rhs_eval(OR_RHS_POLY, 2, 2, par, npar, cell, x, f);
            for (int i = 0; i < 14; i++) {
                double cv[2] = {0, 0};
                for (int j = 0; j < nr; j++)
                    if (R[i][j] != 0)
                        for (int k = 0; k < 2; k++) cv[k] += R[i][j] * te[j][k];
                double t = 0;
                for (int k = 0; k < 2; k++) t += f[k] * cv[k];
                locb[i] += t * w[q];
            }
        }
        const double itemfactor = factor * vol;
        for (int i = 0; i < 14; i++) b[celldofs[(size_t)cell * 14 + i]] += locb[i] * itemfactor;
    }
    return nq;
}

/* Velocity-pressure blocks of the P2B / P1-broken Stokes system:
 * nu (grad u, grad v) into the sparse accumulator (order 4), and
 * Bloc[cell][l][i] = int_T lambda_l div phi_i for the three barycentric
 * pressure functions (order 3). */
int oracle_p2b_stokes(void *h, int ncells, const double *coords, const int *cells, const int *celldofs, double nu,
                      double *Bloc)
{
    omat *M = (omat *)h;
    double xa[3 * OR_MAXQ], wa[OR_MAXQ], xb[3 * OR_MAXQ], wb[OR_MAXQ];
    int na = oracle_qrule(2, 4, xa, wa), nb = oracle_qrule(2, 3, xb, wb);
    if (na < 0) na = -na;
    if (nb < 0) nb = -nb;
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], A[3][3], G[3][3], det, vol;
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 2; k++) X[v * 2 + k] = coords[(size_t)cells[(size_t)cell * 3 + v] * 2 + k];
        oracle_geometry(2, X, A, G, &det, &vol);
        const int *dofs = &celldofs[(size_t)cell * 14];
        double K[7][7] = {{0}};
        for (int q = 0; q < na; q++) {
            dual o[7];
            p2b_basis_dual(xa[3 * q], xa[3 * q + 1], o);
            double g[7][2];
            for (int s = 0; s < 7; s++)
                for (int k = 0; k < 2; k++) {
                    double t = 0;
                    for (int j = 0; j < 2; j++) t += G[k][j] * o[s].d[j];
                    g[s][k] = t;
                }
            for (int a = 0; a < 7; a++)
                for (int bb = 0; bb < 7; bb++) K[a][bb] += (g[a][0] * g[bb][0] + g[a][1] * g[bb][1]) * wa[q];
        }
        for (int c = 0; c < 2; c++)
            for (int a = 0; a < 7; a++)
                for (int bb = 0; bb < 7; bb++) omat_addnz(M, dofs[7 * c + a], dofs[7 * c + bb], K[a][bb] * vol * nu, 1.0);
        double *Bl = Bloc + (size_t)cell * 42;
        for (int i = 0; i < 42; i++) Bl[i] = 0.0;
        for (int q = 0; q < nb; q++) {
            const double xi = xb[3 * q], eta = xb[3 * q + 1];
            const double lam[3] = {1 - xi - eta, xi, eta};
            dual o[7];
            p2b_basis_dual(xi, eta, o);
            for (int i = 0; i < 14; i++) {
                const int c = i / 7, s = i % 7;
                double dv = 0;
                for (int j = 0; j < 2; j++) dv += G[c][j] * o[s].d[j];
                for (int l = 0; l < 3; l++) Bl[l * 14 + i] += lam[l] * dv * wb[q] * vol;
            }
        }
    }
    return na;
}

/* sum over cells of int_T |R u - f|^2 (quadrature order `order`), u an
 * H1P2B{2,2} vector, f polynomial data (2 components). */
double oracle_p2b_recon_l2error(int ncells, const double *coords, const int *cells, const int *cell_faces,
                                const double *fnormals, const double *fvolumes, const signed char *signs,
                                const int *celldofs, const double *u, const double *par, int npar, int recon,
                                int order)
{
    br_mesh m = {coords, cells, cell_faces, fnormals, fvolumes, signs, celldofs};
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(2, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1.0;
    double total = 0.0;
    for (int cell = 0; cell < ncells; cell++) {
        double X[6], nrm[6], fv[3], sg[3], A[3][3], G[3][3], det, vol, R[14][12], coef[12];
        br_cell(&m, cell, X, nrm, fv, sg);
        oracle_geometry(2, X, A, G, &det, &vol);
        const int nr = p2b_coeffs(recon, X, A, G, det, vol, fv, nrm, sg, R);
        p2b_recon_target(recon, sg, coef);
        double acc = 0.0;
        for (int q = 0; q < nq; q++) {
            double rb[12][2], v[2] = {0, 0};
            p2b_recon_basis(recon, xref[3 * q], xref[3 * q + 1], rb);
            for (int i = 0; i < 14; i++) {
                const double ui = u[celldofs[(size_t)cell * 14 + i]];
                for (int j = 0; j < nr; j++)
                    for (int k = 0; k < 2; k++) {
                        double s = 0;
                        for (int l = 0; l < 2; l++) s += A[k][l] * rb[j][l];
                        v[k] += ui * R[i][j] * (s * (coef[j] / det));
                    }
            }
            double x[2], f[2];
            for (int k = 0; k < 2; k++) {
                x[k] = X[k];
                for (int j = 0; j < 2; j++) x[k] += A[k][j] * xref[3 * q + j];
            }
            rhs_eval(OR_RHS_POLY, 2, 2, par, npar, cell, x, f);
            acc += ((v[0] - f[0]) * (v[0] - f[0]) + (v[1] - f[1]) * (v[1] - f[1])) * w[q];
        }
        total += acc * vol;
    }
    return total;
}

/* ------------------------------------------------------------------------- */
/* NonlinearForm: Newton terms (src/assemblypatterns/nonlinearform.jl:44-240) */
/* ------------------------------------------------------------------------- */

enum { OR_NL_DIFFUSION = 1, OR_NL_GRAD_DIFFUSION = 2, OR_NL_CONVECTION = 3 };

/* Kernel value K and Jacobian J (row-major, nin columns) of the closed set of
 * nonlinear kernels:  DIFFUSION ((kappa + beta u^2) grad u, input [u, grad u]),
 * GRAD_DIFFUSION ((kappa + |grad u|^2) grad u, input [grad u]), CONVECTION
 * ((u . grad) u, input [u, grad u] with grad u component-major). */
static void nl_kernel(int kind, int dim, double kappa, double beta, const double *in, double *K, double *J, int nin)
{
    for (int i = 0; i < dim * nin; i++) J[i] = 0.0;
    if (kind == OR_NL_DIFFUSION) {
        const double u = in[0], c = kappa + beta * (u * u);
        for (int k = 0; k < dim; k++) {
            K[k] = c * in[1 + k];
            J[k * nin + 0] = (beta * (2.0 * u)) * in[1 + k];
            J[k * nin + 1 + k] = c;
        }
    } else if (kind == OR_NL_GRAD_DIFFUSION) {
        double g2 = 0.0;
        for (int k = 0; k < dim; k++) g2 += in[k] * in[k];
        const double c = kappa + g2;
        for (int k = 0; k < dim; k++) {
            K[k] = c * in[k];
            for (int l = 0; l < dim; l++) J[k * nin + l] = (2.0 * in[l]) * in[k];
            J[k * nin + k] += c;
        }
    } else {
        for (int c = 0; c < dim; c++) {
            double s = 0.0;
            for (int l = 0; l < dim; l++) s += in[l] * in[dim + c * dim + l];
            K[c] = s;
            for (int m = 0; m < dim; m++) J[c * nin + m] = in[dim + c * dim + m];
            for (int l = 0; l < dim; l++) J[c * nin + dim + c * dim + l] = in[l];
        }
    }
}

/* Adds the Newton terms of one NonlinearForm at the iterate u: DG(u) into M
 * (row = test DoF, column = ansatz DoF: transposed_assembly, skipping exact
 * zeros as _addnz does) and DG(u) u - G(u) into b.  Quadrature order: bonus
 * plus, per operator, polyorder + shift (src/assemblypatterns.jl:558-565). */
int oracle_nl_assemble(void *h, double *b, int dim, const double *coords, int ncells, const int *cellnodes, int fe,
                       int ncomp, const int *celldofs, const double *u, int kind, double factor, double kappa,
                       double beta, int bonus_quadorder)
{
    omat *M = (omat *)h;
    const int nb = (fe == OR_FE_P1) ? dim + 1 : (dim == 2 ? 6 : 10);
    const int ld = nb * ncomp, p = (fe == OR_FE_P1) ? 1 : 2;
    int order = bonus_quadorder;
    if (kind == OR_NL_DIFFUSION) order += p + 2 * (p - 1);
    else if (kind == OR_NL_GRAD_DIFFUSION) order += 2 * (p - 1);
    else order += 2 * p + (p - 1);
    if (order < 0) order = 0;
    double xref[3 * OR_MAXQ], w[OR_MAXQ];
    int nq = oracle_qrule(dim, order, xref, w);
    if (nq < 0) nq = -nq;
    if (nq == 0) return -1;
    double *vals = (double *)malloc(sizeof(double) * (size_t)nq * nb);
    double *derivs = (double *)malloc(sizeof(double) * (size_t)nq * nb * dim);
    oracle_basis_tables(fe, dim, nq, xref, vals, derivs);
    const int nin = (kind == OR_NL_CONVECTION) ? dim + dim * dim : (kind == OR_NL_GRAD_DIFFUSION ? dim : 1 + dim);
    double *in = (double *)malloc(sizeof(double) * (size_t)nq * nin);
    double *cvid = (double *)malloc(sizeof(double) * (size_t)nq * ld * nin);   /* input(phi_i) per q */
    double *cvt = (double *)malloc(sizeof(double) * (size_t)nq * ld * dim);    /* test(phi_j) per q */
    double *lm = (double *)malloc(sizeof(double) * (size_t)ld * ld);
    double *lb = (double *)malloc(sizeof(double) * (size_t)ld);
    double K[3], J[3 * 12], ar[3];
    for (int cell = 0; cell < ncells; cell++) {
        double X[12], A[3][3], G[3][3], det, vol;
        for (int v = 0; v <= dim; v++)
            for (int k = 0; k < dim; k++) X[v * dim + k] = coords[(size_t)cellnodes[(size_t)cell * (dim + 1) + v] * dim + k];
        oracle_geometry(dim, X, A, G, &det, &vol);
        const int *dofs = &celldofs[(size_t)cell * ld];
        /* operator evaluations of every local basis function */
        for (int q = 0; q < nq; q++)
            for (int i = 0; i < ld; i++) {
                const int c = i / nb, a = i % nb;
                double gr[3];
                for (int k = 0; k < dim; k++) {
                    double s = 0;
                    for (int j = 0; j < dim; j++) s += G[k][j] * derivs[(q * nb + a) * dim + j];
                    gr[k] = s;
                }
                double *ci = cvid + ((size_t)q * ld + i) * nin;
                double *ct = cvt + ((size_t)q * ld + i) * dim;
                for (int m = 0; m < nin; m++) ci[m] = 0.0;
                if (kind == OR_NL_CONVECTION) {
                    ci[c] = vals[q * nb + a];
                    for (int k = 0; k < dim; k++) ci[dim + c * dim + k] = gr[k];
                    for (int k = 0; k < dim; k++) ct[k] = (k == c) ? vals[q * nb + a] : 0.0;
                } else {
                    if (kind == OR_NL_DIFFUSION) {
                        ci[0] = vals[q * nb + a];
                        for (int k = 0; k < dim; k++) ci[1 + k] = gr[k];
                    } else {
                        for (int k = 0; k < dim; k++) ci[k] = gr[k];
                    }
                    for (int k = 0; k < dim; k++) ct[k] = gr[k];
                }
            }
        /* current iterate: eval_febe! over the DoFs in order */
        for (int q = 0; q < nq; q++) {
            double *iq = in + (size_t)q * nin;
            for (int m = 0; m < nin; m++) iq[m] = 0.0;
            for (int i = 0; i < ld; i++) {
                const double ui = u[dofs[i]];
                const double *ci = cvid + ((size_t)q * ld + i) * nin;
                for (int m = 0; m < nin; m++) iq[m] += ui * ci[m];
            }
        }
        for (int i = 0; i < ld * ld; i++) lm[i] = 0.0;
        for (int j = 0; j < ld; j++) lb[j] = 0.0;
        for (int q = 0; q < nq; q++) {
            const double *iq = in + (size_t)q * nin;
            nl_kernel(kind, dim, kappa, beta, iq, K, J, nin);
            for (int i = 0; i < ld; i++) {
                const double *ci = cvid + ((size_t)q * ld + i) * nin;
                for (int k = 0; k < dim; k++) {
                    double s = 0;
                    for (int m = 0; m < nin; m++) s += J[k * nin + m] * ci[m];
                    ar[k] = s;
                }
                for (int j = 0; j < ld; j++) {
                    const double *ct = cvt + ((size_t)q * ld + j) * dim;
                    double t = 0;
                    for (int k = 0; k < dim; k++) t += ar[k] * ct[k];
                    lm[i * ld + j] += t * w[q];
                }
            }
            for (int k = 0; k < dim; k++) {
                double s = 0;
                for (int m = 0; m < nin; m++) s += J[k * nin + m] * iq[m];
                ar[k] = s;
            }
            for (int j = 0; j < ld; j++) {
                const double *ct = cvt + ((size_t)q * ld + j) * dim;
                double t = 0;
                for (int k = 0; k < dim; k++) t += (ar[k] - K[k]) * ct[k];
                lb[j] += t * w[q];
            }
        }
        const double itemfactor = vol * factor;
        for (int i = 0; i < ld; i++)
            for (int j = 0; j < ld; j++) omat_addnz(M, dofs[j], dofs[i], lm[i * ld + j], itemfactor);
        for (int j = 0; j < ld; j++) b[dofs[j]] += lb[j] * itemfactor;
    }
    free(vals); free(derivs); free(in); free(cvid); free(cvt); free(lm); free(lb);
    return nq;
}

/* ------------------------------------------------------------------------- */
/* Interior-face terms with Jump(Gradient) (src/assemblypatterns.jl:103-153)  */
/* ------------------------------------------------------------------------- */

/* Local vertices of face f of a simplex (the mesh module's numbering). */
static int or_face_vertex(int dim, int f, int k)
{
    static const int t3[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
    return dim == 2 ? (f + k) % 3 : t3[f][k];
}

/* Face quadrature points as reference coordinates of `cell`: barycentric
 * weights over the face's vertices in ascending global vertex order. */
static void or_face_points(int dim, const int *cells, int cell, int f, int nq, const double *lam, double *xh)
{
    int loc[3], gid[3];
    for (int k = 0; k < dim; k++) { loc[k] = or_face_vertex(dim, f, k); gid[k] = cells[(size_t)cell * (dim + 1) + loc[k]]; }
    for (int i = 1; i < dim; i++)
        for (int j = i; j > 0 && gid[j] < gid[j - 1]; j--) {
            int t = gid[j]; gid[j] = gid[j - 1]; gid[j - 1] = t;
            t = loc[j]; loc[j] = loc[j - 1]; loc[j - 1] = t;
        }
    for (int q = 0; q < nq; q++)
        for (int j = 0; j < dim; j++) {
            double s = 0.0;
            for (int k = 0; k < dim; k++) s += loc[k] == j + 1 ? lam[q * 3 + k] : 0.0;
            xh[q * 3 + j] = s;
        }
}

static int or_face_rule(int dim, int order, double *lam, double *w)
{
    double xr[3 * OR_MAXQ];
    int nq = oracle_qrule(dim - 1, order, xr, w);
    if (nq < 0) nq = -nq;
    for (int q = 0; q < nq; q++) {
        if (dim == 2) { lam[q * 3] = 1.0 - xr[3 * q]; lam[q * 3 + 1] = xr[3 * q]; lam[q * 3 + 2] = 0.0; }
        else {
            lam[q * 3] = 1.0 - xr[3 * q] - xr[3 * q + 1];
            lam[q * 3 + 1] = xr[3 * q];
            lam[q * 3 + 2] = xr[3 * q + 1];
        }
    }
    return nq;
}

/* physical gradients g[a*3 + k] of the scalar basis at reference point xh */
static int or_grads(int fe, int dim, const double *xh, double G[3][3], double *g)
{
    dual x[3], o[10];
    for (int j = 0; j < 3; j++) x[j] = dvar(j < dim ? xh[j] : 0.0, j);
    const int nb = h1_scalar_basis(fe, dim, x, o);
    for (int a = 0; a < nb; a++)
        for (int k = 0; k < dim; k++) {
            double s = 0;
            for (int j = 0; j < dim; j++) s += G[k][j] * o[a].d[j];
            g[a * 3 + k] = s;
        }
    return nb;
}

/* face -> (lower cell, higher cell or -1), registered in ascending cell order */
static void or_face_cells(int dim, int ncells, const int *cell_faces, int nfaces, int *fc)
{
    for (int F = 0; F < 2 * nfaces; F++) fc[F] = -1;
    for (int c = 0; c < ncells; c++)
        for (int f = 0; f <= dim; f++) {
            const int F = cell_faces[(size_t)c * (dim + 1) + f];
            if (fc[2 * F] < 0) fc[2 * F] = c; else fc[2 * F + 1] = c;
        }
}

/* factor |F| |F|^power sum_q w_q [grad phi_a].[grad phi_b] over the 2 x ld
 * functions of the two cells of every interior face (jump coefficient +1 on
 * the lower cell, -1 on the other; ascending faces; exact zeros skipped). */
int oracle_face_jumpgrad(void *h, int dim, const double *coords, int ncells, const int *cells, const int *cell_faces,
                         int nfaces, int fe, const int *celldofs, double factor, double power, int bonus_quadorder)
{
    omat *M = (omat *)h;
    const int p = (fe == OR_FE_P1) ? 1 : 2;
    const int nb = (fe == OR_FE_P1) ? dim + 1 : (dim == 2 ? 6 : 10);
    int order = 2 * (p - 1) + bonus_quadorder;
    double lam[3 * OR_MAXQ], w[OR_MAXQ];
    const int nq = or_face_rule(dim, order < 0 ? 0 : order, lam, w);
    if (nq <= 0) return -1;
    int *fc = (int *)malloc(sizeof(int) * 2 * (size_t)nfaces);
    or_face_cells(dim, ncells, cell_faces, nfaces, fc);
    double *xh = (double *)malloc(sizeof(double) * 3 * (size_t)nq);
    double *g = (double *)malloc(sizeof(double) * (size_t)nq * 2 * nb * 3);
    for (int F = 0; F < nfaces; F++) {
        const int c[2] = {fc[2 * F], fc[2 * F + 1]};
        if (c[1] < 0) continue;
        double fvol = 0;
        for (int side = 0; side < 2; side++) {
            int f = 0;
            for (int k = 0; k <= dim; k++) if (cell_faces[(size_t)c[side] * (dim + 1) + k] == F) f = k;
            double X[12], A[3][3], G[3][3], det, vol;
            for (int v = 0; v <= dim; v++)
                for (int k = 0; k < dim; k++) X[v * dim + k] = coords[(size_t)cells[(size_t)c[side] * (dim + 1) + v] * dim + k];
            oracle_geometry(dim, X, A, G, &det, &vol);
            or_face_points(dim, cells, c[side], f, nq, lam, xh);
            const double sgn = side == 0 ? 1.0 : -1.0;
            for (int q = 0; q < nq; q++) {
                double gq[30];
                or_grads(fe, dim, xh + 3 * q, G, gq);
                for (int a = 0; a < nb; a++)
                    for (int k = 0; k < 3; k++) g[((size_t)q * 2 * nb + side * nb + a) * 3 + k] = k < dim ? sgn * gq[a * 3 + k] : 0.0;
            }
            if (side == 0) {
                /* face measure from the face's vertices */
                double P[3][3];
                for (int k = 0; k < dim; k++)
                    for (int j = 0; j < dim; j++) P[k][j] = coords[(size_t)cells[(size_t)c[0] * (dim + 1) + or_face_vertex(dim, f, k)] * dim + j];
                if (dim == 2) fvol = sqrt((P[1][0] - P[0][0]) * (P[1][0] - P[0][0]) + (P[1][1] - P[0][1]) * (P[1][1] - P[0][1]));
                else {
                    double u[3], v[3];
                    for (int j = 0; j < 3; j++) { u[j] = P[1][j] - P[0][j]; v[j] = P[2][j] - P[0][j]; }
                    double cx = u[1] * v[2] - u[2] * v[1], cy = u[2] * v[0] - u[0] * v[2], cz = u[0] * v[1] - u[1] * v[0];
                    fvol = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
                }
            }
        }
        double act = 1.0;
        for (int i = 0; i < (int)power; i++) act *= fvol;
        if ((double)(int)power != power) act = pow(fvol, power);
        const double itemfactor = fvol * factor;
        for (int a = 0; a < 2 * nb; a++)
            for (int b = 0; b < 2 * nb; b++) {
                double lm = 0;
                for (int q = 0; q < nq; q++) {
                    double t = 0;
                    for (int k = 0; k < dim; k++) t += (act * g[((size_t)q * 2 * nb + a) * 3 + k]) * g[((size_t)q * 2 * nb + b) * 3 + k];
                    lm += t * w[q];
                }
                const int ra = celldofs[(size_t)c[a / nb] * nb + a % nb], rb = celldofs[(size_t)c[b / nb] * nb + b % nb];
                omat_addnz(M, ra, rb, lm, itemfactor);
            }
    }
    free(fc); free(xh); free(g);
    return nq;
}

/* per interior face: factor |F| |F|^power sum_q w_q g(q), g = |[grad u]|^2
 * (kind 0) or ([grad u].n)^2 (kind 1); boundary faces 0.  fnormals /
 * fvolumes: the mesh's face data. */
int oracle_face_jumps(int dim, const double *coords, int ncells, const int *cells, const int *cell_faces, int nfaces,
                      const double *fnormals, const double *fvolumes, int fe, const int *celldofs, const double *u,
                      int kind, double power, double factor, int bonus_quadorder, double *out)
{
    const int p = (fe == OR_FE_P1) ? 1 : 2;
    const int nb = (fe == OR_FE_P1) ? dim + 1 : (dim == 2 ? 6 : 10);
    int order = 2 * (p - 1) + bonus_quadorder;
    double lam[3 * OR_MAXQ], w[OR_MAXQ];
    const int nq = or_face_rule(dim, order < 0 ? 0 : order, lam, w);
    if (nq <= 0) return -1;
    int *fc = (int *)malloc(sizeof(int) * 2 * (size_t)nfaces);
    or_face_cells(dim, ncells, cell_faces, nfaces, fc);
    double *xh = (double *)malloc(sizeof(double) * 3 * (size_t)nq);
    double *J = (double *)malloc(sizeof(double) * 3 * (size_t)nq);
    for (int F = 0; F < nfaces; F++) {
        out[F] = 0.0;
        const int c[2] = {fc[2 * F], fc[2 * F + 1]};
        if (c[1] < 0) continue;
        for (int i = 0; i < 3 * nq; i++) J[i] = 0.0;
        for (int side = 0; side < 2; side++) {
            int f = 0;
            for (int k = 0; k <= dim; k++) if (cell_faces[(size_t)c[side] * (dim + 1) + k] == F) f = k;
            double X[12], A[3][3], G[3][3], det, vol;
            for (int v = 0; v <= dim; v++)
                for (int k = 0; k < dim; k++) X[v * dim + k] = coords[(size_t)cells[(size_t)c[side] * (dim + 1) + v] * dim + k];
            oracle_geometry(dim, X, A, G, &det, &vol);
            or_face_points(dim, cells, c[side], f, nq, lam, xh);
            for (int q = 0; q < nq; q++) {
                double gq[30];
                or_grads(fe, dim, xh + 3 * q, G, gq);
                for (int a = 0; a < nb; a++) {
                    const double ua = u[celldofs[(size_t)c[side] * nb + a]];
                    for (int k = 0; k < dim; k++) J[3 * q + k] += (side == 0 ? ua : -ua) * gq[a * 3 + k];
                }
            }
        }
        double acc = 0.0;
        for (int q = 0; q < nq; q++) {
            double val = 0.0;
            if (kind == 1) {
                double jn = 0.0;
                for (int k = 0; k < dim; k++) jn += J[3 * q + k] * fnormals[(size_t)F * dim + k];
                val = jn * jn;
            } else
                for (int k = 0; k < dim; k++) val += J[3 * q + k] * J[3 * q + k];
            acc += w[q] * val;
        }
        const double fv = fvolumes[F];
        double act = 1.0;
        for (int i = 0; i < (int)power; i++) act *= fv;
        if ((double)(int)power != power) act = pow(fv, power);
        out[F] = acc * act * fv * factor;
    }
    free(fc); free(xh); free(J);
    return nq;
}
