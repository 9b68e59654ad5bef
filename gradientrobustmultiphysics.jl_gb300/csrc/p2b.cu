// Right-hand sides of H1P2B{2,2} (P2 + cell bubble, vector, triangles) with
// the reconstruction test operators ReconstructionIdentity{HDIVRT1{2}} and
// ReconstructionIdentity{HDIVBDM2{2}}: b_I += factor (f, R phi_I)
// (src/feevaluator_h1.jl:342-381, src/assemblypatterns/linearform.jl:181-220,
// coefficients src/reconstructions.jl:43-330, :405-469).
//
// One thread per cell builds the cell's reconstruction coefficients R[14][NR]
// in FP64 -- face part from the face measures, normals and signs, interior
// part from closed-form cell integrals (RT1) or from a 3x3 moment system on
// the order-4 rule (BDM2) -- integrates f against the Piola-mapped target
// basis and writes the 14 local values; a row kernel then adds each DoF's
// cell values in ascending cell order (deterministic, no atomics).
#include "grmp_internal.h"

#include <cstring>

namespace {

constexpr int TPB = 256;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

struct P2bMesh {
    const double *coords;
    const int32_t *cells, *cell_faces;
    const double *fnormals, *fvolumes;
    const int8_t *signs;
};

struct P2bRhs {
    const double *par;     // [ngroups][nt][5] polynomial terms (component, coef, e1, e2, e3)
    int nt;
    const int32_t *group;  // [ncells] group of each cell (nullptr: one group)
    double factor;
    int nq;                // rule of order polyorder(H1P2B) = 3 plus the data's bonus
    double xref[64][2];
    double w[64];
    int nq4;               // order-4 rule of the BDM2 moment system
    double x4[16][2];
    double w4[16];
};

__device__ __forceinline__ double p2b_pow(double x, double e) {
    const int k = (int)e;
    if ((double)k == e && k >= 0 && k <= 8) {
        double r = 1.0;
        for (int i = 0; i < k; i++) r *= x;
        return r;
    }
    return pow(x, e);
}

// RT1 / BDM2 reference basis (src/fedefs/hdiv_rt1.jl:106-121,
// src/fedefs/hdiv_bdm2.jl:171-194)
template <int NR>
__device__ __forceinline__ void recon_basis(double x, double y, double o[NR][2]) {
    if constexpr (NR == 8) {
        o[0][0] = x, o[0][1] = y - 1;
        o[2][0] = x, o[2][1] = y;
        o[4][0] = x - 1, o[4][1] = y;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            o[1][k] = -12 * (0.5 - x - y) * o[0][k];
            o[3][k] = -(12 * (x - 0.5)) * o[2][k];
            o[5][k] = -(12 * (y - 0.5)) * o[4][k];
            o[6][k] = 12 * y * o[0][k];
            o[7][k] = 12 * x * o[4][k];
        }
    } else {
        const double l = 1 - x - y;
        o[0][0] = x, o[0][1] = y - 1;
        o[3][0] = x, o[3][1] = y;
        o[6][0] = x - 1, o[6][1] = y;
        o[1][0] = 6 * x, o[1][1] = 6 - 12 * x - 6 * y;
        o[4][0] = -6 * x, o[4][1] = 6 * y;
        o[7][0] = 6 * (x - 1) + 12 * y, o[7][1] = -6 * y;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            o[2][k] = -15 * ((l - 0.5) * o[1][k] + o[0][k]);
            o[5][k] = -15 * ((x - 0.5) * o[4][k] + o[3][k]);
            o[8][k] = -15 * ((y - 0.5) * o[7][k] + o[6][k]);
            o[9][k] = y * o[1][k];
            o[10][k] = l * o[4][k];
            o[11][k] = x * o[7][k];
        }
    }
}

// element coefficients of the target: the face sign on RT1's functions 2f,
// on BDM2's functions 3f and 3f+2 (hdiv_rt1.jl:124-135, hdiv_bdm2.jl:197-210)
template <int NR>
__device__ __forceinline__ void recon_signs(const double sg[3], double coef[NR]) {
#pragma unroll
    for (int j = 0; j < NR; j++) coef[j] = 1.0;
#pragma unroll
    for (int f = 0; f < 3; f++) {
        if constexpr (NR == 12) {
            coef[3 * f] = sg[f];
            coef[3 * f + 2] = sg[f];
        } else {
            coef[2 * f] = sg[f];
        }
    }
}

// P2B scalar basis value and reference gradient (h1_p2.jl:134-144,
// h1_p2b.jl:126-137); the gradient of the bubble only
__device__ __forceinline__ void p2b_values(double x, double y, double v[7]) {
    const double l = 1 - x - y;
    v[0] = 2 * l * (l - 0.5);
    v[1] = 2 * x * (x - 0.5);
    v[2] = 2 * y * (y - 0.5);
    v[3] = 4 * l * x;
    v[4] = 4 * x * y;
    v[5] = 4 * y * l;
    v[6] = 60 * (1 - x - y) * x * y;
}

// d/dx, d/dy of 60 (1 - x - y) x y in the product order of a forward-mode
// evaluation of ((60 (1 - x - y)) x) y
__device__ __forceinline__ void bubble_grad(double x, double y, double d[2]) {
    const double a = 60 * (1 - x - y);
    // a' = (-60, -60); (a x)' = (x a'_x + a, x a'_y); ((a x) y)' = (y (a x)'_x, y (a x)'_y + a x)
    const double ax = a * x;
    const double ax_dx = x * -60.0 + a * 1.0, ax_dy = x * -60.0 + a * 0.0;
    d[0] = y * ax_dx + ax * 0.0;
    d[1] = y * ax_dy + ax * 1.0;
}

__device__ void lu3(double M[3][3], int piv[3]) {
    for (int j = 0; j < 3; j++) {
        int p = j;
        for (int i = j + 1; i < 3; i++)
            if (fabs(M[i][j]) > fabs(M[p][j])) p = i;
        piv[j] = p;
        if (p != j)
            for (int c = 0; c < 3; c++) {
                const double t = M[j][c];
                M[j][c] = M[p][c];
                M[p][c] = t;
            }
        for (int i = j + 1; i < 3; i++) {
            M[i][j] /= M[j][j];
            for (int c = j + 1; c < 3; c++) M[i][c] -= M[i][j] * M[j][c];
        }
    }
}

__device__ void lu3_solve(const double M[3][3], const int piv[3], double y[3]) {
    for (int j = 0; j < 3; j++)
        if (piv[j] != j) {
            const double t = y[j];
            y[j] = y[piv[j]];
            y[piv[j]] = t;
        }
    for (int i = 1; i < 3; i++)
        for (int j = 0; j < i; j++) y[i] -= M[i][j] * y[j];
    for (int i = 2; i >= 0; i--) {
        for (int j = i + 1; j < 3; j++) y[i] -= M[i][j] * y[j];
        y[i] /= M[i][i];
    }
}

template <int NR>
__global__ void __launch_bounds__(128) k_p2b_rhs_cells(int ncells, P2bMesh m, P2bRhs r, double *loc) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[6], nrm[3][2], fv[3], sg[3];
    for (int v = 0; v < 3; v++)
        for (int k = 0; k < 2; k++) X[v * 2 + k] = m.coords[(size_t)m.cells[(size_t)cell * 3 + v] * 2 + k];
    for (int f = 0; f < 3; f++) {
        const int F = m.cell_faces[(size_t)cell * 3 + f];
        nrm[f][0] = m.fnormals[(size_t)F * 2];
        nrm[f][1] = m.fnormals[(size_t)F * 2 + 1];
        fv[f] = m.fvolumes[F];
        sg[f] = (double)m.signs[(size_t)cell * 3 + f];
    }
    double A[2][2];
    for (int k = 0; k < 2; k++)
        for (int j = 0; j < 2; j++) A[k][j] = X[(j + 1) * 2 + k] - X[k];
    const double det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    const double vol = fabs(det) / 2.0;
    // face part (src/reconstructions.jl:405-469)
    constexpr int W = NR == 12 ? 3 : 2;
    double R[14][NR];
    for (int i = 0; i < 14; i++)
        for (int j = 0; j < NR; j++) R[i][j] = 0.0;
    {
        const double c[2] = {-1.0 / 12.0, 1.0 / 12.0};
        for (int f = 0; f < 3; f++) {
            const int nodes[2] = {f, (f + 1) % 3};
            for (int n = 0; n < 2; n++)
                for (int k = 0; k < 2; k++) {
                    R[7 * k + nodes[n]][W * f] = (1.0 / 6.0) * fv[f] * nrm[f][k];
                    R[7 * k + nodes[n]][W * f + 1] = c[n] * fv[f] * nrm[f][k] * sg[f];
                    if constexpr (NR == 12) R[7 * k + nodes[n]][W * f + 2] = (1.0 / 90.0) * fv[f] * nrm[f][k];
                }
            for (int k = 0; k < 2; k++) {
                R[7 * k + 3 + f][W * f] = (2.0 / 3.0) * fv[f] * nrm[f][k];
                if constexpr (NR == 12) R[7 * k + 3 + f][W * f + 2] = (-1.0 / 45.0) * fv[f] * nrm[f][k];
            }
        }
    }
    double coef[NR];
    recon_signs<NR>(sg, coef);
    if constexpr (NR == 8) {
        // interior RT1 pair (src/reconstructions.jl:43-161): closed-form cell
        // integrals of the face functions, inverse 2x2 of the interior ones
        double M[2] = {0, 0}, E[2][3] = {{0, 0, 0}, {0, 0, 0}}, B[2][8];
        for (int n = 0; n < 3; n++)
            for (int k = 0; k < 2; k++) M[k] += X[n * 2 + k] / 3;
        for (int f = 0; f < 3; f++)
            for (int n = 0; n < 2; n++)
                for (int k = 0; k < 2; k++) E[k][f] += X[((f + n) % 3) * 2 + k] / 2;
        for (int k = 0; k < 2; k++) {
            B[k][0] = (M[k] - X[2 * 2 + k]) / 2 * sg[0];
            B[k][1] = X[1 * 2 + k] - E[k][1];
            B[k][2] = (M[k] - X[0 * 2 + k]) / 2 * sg[1];
            B[k][3] = X[2 * 2 + k] - E[k][2];
            B[k][4] = (M[k] - X[1 * 2 + k]) / 2 * sg[2];
            B[k][5] = X[0 * 2 + k] - E[k][0];
        }
        B[1][7] = (E[0][0] - X[2 * 2 + 0]);
        B[1][6] = -(E[1][0] - X[2 * 2 + 1]);
        B[0][7] = -(E[0][2] - X[1 * 2 + 0]);
        B[0][6] = (E[1][2] - X[1 * 2 + 1]);
        const double dB = B[0][6] * B[1][7] - B[1][6] * B[0][7];
        B[0][6] /= dB, B[0][7] /= dB, B[1][6] /= dB, B[1][7] /= dB;
        for (int k = 0; k < 2; k++) {
            for (int n = 0; n < 3; n++)
                for (int pass = 0; pass < 2; pass++) {   // node function, then face function
                    const int dof = 7 * k + n + 3 * pass;
                    double b[2] = {0, 0};
                    if (pass == 1) b[k] = vol / 3;
                    for (int c = 0; c < 2; c++)
                        for (int j = 0; j < 6; j++) b[c] -= R[dof][j] * B[c][j];
                    for (int kk = 0; kk < 2; kk++) R[dof][6 + kk] = B[kk][6] * b[0] + B[kk][7] * b[1];
                }
            const int dof = 7 * k + 6;   // the bubble: cell integral |T| in its component
            double b[2] = {0, 0};
            b[k] = vol;
            for (int kk = 0; kk < 2; kk++) R[dof][6 + kk] = B[kk][6] * b[0] + B[kk][7] * b[1];
        }
    } else {
        // interior BDM2 triple (src/reconstructions.jl:164-330): keep the
        // moments against grad(P1 functions 1, 2) and curl(cell bubble)
        double G[2][2];
        G[0][0] = A[1][1] / det, G[0][1] = -A[1][0] / det;
        G[1][0] = -A[0][1] / det, G[1][1] = A[0][0] / det;
        const double dp1[2][2] = {{-1, -1}, {1, 0}};
        double b3[2][2];
        for (int a = 0; a < 2; a++)
            for (int k = 0; k < 2; k++) {
                double s = 0;
                for (int j = 0; j < 2; j++) s += G[k][j] * dp1[a][j];
                b3[a][k] = s;
            }
        double IMM[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, IMMf[3][9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 9; j++) IMMf[i][j] = 0.0;
        double lb[14][3];
        for (int i = 0; i < 14; i++) lb[i][0] = lb[i][1] = lb[i][2] = 0.0;
        for (int q = 0; q < r.nq4; q++) {
            const double xi = r.x4[q][0], eta = r.x4[q][1];
            double rb[12][2], b2[12][2];
            recon_basis<12>(xi, eta, rb);
            for (int j = 0; j < 12; j++)
                for (int k = 0; k < 2; k++) {
                    double s = 0;
                    for (int l = 0; l < 2; l++) s += A[k][l] * rb[j][l];
                    s *= coef[j] / det;
                    b2[j][k] = s;
                }
            double d[2], b4[2] = {0, 0};
            bubble_grad(xi, eta, d);
            for (int j = 0; j < 2; j++) {
                b4[0] -= G[1][j] * d[j];
                b4[1] += G[0][j] * d[j];
            }
            for (int dof = 0; dof < 3; dof++) {
                for (int d2 = 0; d2 < 2; d2++) {
                    double t = 0;
                    for (int k = 0; k < 2; k++) t += b2[9 + dof][k] * b3[d2][k];
                    IMM[d2][dof] += t * vol * r.w4[q];
                }
                double t = 0;
                for (int k = 0; k < 2; k++) t += b2[9 + dof][k] * b4[k];
                IMM[2][dof] += t * vol * r.w4[q];
                for (int d2 = 0; d2 < 9; d2++) {
                    double u = 0;
                    for (int k = 0; k < 2; k++) u += (dof < 2 ? b3[dof][k] : b4[k]) * b2[d2][k];
                    IMMf[dof][d2] += u * vol * r.w4[q];
                }
            }
            // moments of the P2B functions (one nonzero component each)
            double v[7];
            p2b_values(xi, eta, v);
            for (int d1 = 0; d1 < 14; d1++) {
                const int c = d1 / 7, s = d1 % 7;
                for (int id = 0; id < 2; id++) {
                    double t = 0;
                    for (int k = 0; k < 2; k++) t += (k == c ? v[s] : 0.0) * b3[id][k];
                    lb[d1][id] += t * vol * r.w4[q];
                }
                double t = 0;
                for (int k = 0; k < 2; k++) t += (k == c ? v[s] : 0.0) * b4[k];
                lb[d1][2] += t * vol * r.w4[q];
            }
        }
        int piv[3];
        lu3(IMM, piv);
        for (int d1 = 0; d1 < 14; d1++) {
            double y[3] = {lb[d1][0], lb[d1][1], lb[d1][2]};
            for (int id = 0; id < 3; id++)
                for (int d2 = 0; d2 < 9; d2++) y[id] -= R[d1][d2] * IMMf[id][d2];
            lu3_solve(IMM, piv, y);
            for (int id = 0; id < 3; id++) R[d1][9 + id] = y[id];
        }
    }
    // (f, R phi_I) on the rhs rule
    const double *par = r.par + (size_t)(r.group ? r.group[cell] : 0) * r.nt * 5;
    double lbv[14];
    for (int i = 0; i < 14; i++) lbv[i] = 0.0;
    for (int q = 0; q < r.nq; q++) {
        const double xi = r.xref[q][0], eta = r.xref[q][1];
        double rb[NR][2], te[NR][2];
        recon_basis<NR>(xi, eta, rb);
        for (int j = 0; j < NR; j++)
            for (int k = 0; k < 2; k++) {
                double s = 0;
                for (int l = 0; l < 2; l++) s += A[k][l] * rb[j][l];
                s *= coef[j] / det;
                te[j][k] = s;
            }
        double x[2], f[2] = {0, 0};
        for (int k = 0; k < 2; k++) {
            x[k] = X[k];
            for (int j = 0; j < 2; j++) x[k] += A[k][j] * (j == 0 ? xi : eta);
        }
        for (int t = 0; t < r.nt; t++) {
            const int c = (int)par[5 * t];
            double v = par[5 * t + 1];
            for (int j = 0; j < 2; j++) v *= p2b_pow(x[j], par[5 * t + 2 + j]);
            f[c] += v;
        }
        for (int i = 0; i < 14; i++) {
            double cv[2] = {0, 0};
            for (int j = 0; j < NR; j++)
                if (R[i][j] != 0)
                    for (int k = 0; k < 2; k++) cv[k] += R[i][j] * te[j][k];
            double t = 0;
            for (int k = 0; k < 2; k++) t += f[k] * cv[k];
            lbv[i] += t * r.w[q];
        }
    }
    const double itemfactor = r.factor * vol;
    for (int i = 0; i < 14; i++) loc[(size_t)cell * 14 + i] = lbv[i] * itemfactor;
}

// b[row] += sum over the row's (cell, local) incidences, ascending cells
__global__ void k_gather_rows14(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell,
                                const uint8_t *inc_loc, const double *loc, double *b) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    double acc = b[row];
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) acc += loc[(size_t)inc_cell[p] * 14 + inc_loc[p]];
    b[row] = acc;
}

}  // namespace

int grmp_p2b_rhs(grmp_space s, const grmp_rhs *rhs, grmp_vector b) {
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    if (rhs->test_operator != 3 && rhs->test_operator != 4)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED,
                         "H1P2B right-hand sides use a reconstruction test operator (3 = RT1, 4 = BDM2)");
    if (rhs->kind != GRMP_RHS_POLY || rhs->ncomponents != 2)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1P2B reconstructed rhs: 2-component polynomial data only");
    const long long ng = rhs->cell_group ? rhs->ngroups : 1;
    if (ng <= 0 || rhs->nparams % (5 * ng)) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: parameter layout");
    const int nt = (int)(rhs->nparams / (5 * ng));
    for (long long t = 0; t < ng * nt; t++)
        if (rhs->params[5 * t] < 0 || rhs->params[5 * t] > 1)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: polynomial component out of range");
    if (rhs->cell_group)
        for (int c = 0; c < m->ncells; c++)
            if (rhs->cell_group[c] < 0 || rhs->cell_group[c] >= ng)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: cell group out of range");
    P2bRhs r;
    std::memset(&r, 0, sizeof(r));
    {
        double (*x)[3] = new double[GRMP_MAXQ][3];
        double *w = new double[GRMP_MAXQ];
        const int order = 3 + rhs->bonus_quadorder;   // get_polynomialorder(H1P2B, Triangle2D) = 3
        int nq = grmp_quadrature(2, order, x, w);
        bool ok = nq > 0 && nq <= 64;
        if (ok) {
            r.nq = nq;
            for (int q = 0; q < nq; q++) r.xref[q][0] = x[q][0], r.xref[q][1] = x[q][1], r.w[q] = w[q];
            nq = grmp_quadrature(2, 4, x, w);
            ok = nq > 0 && nq <= 16;
            r.nq4 = nq;
            for (int q = 0; ok && q < nq; q++) r.x4[q][0] = x[q][0], r.x4[q][1] = x[q][1], r.w4[q] = w[q];
        }
        delete[] x;
        delete[] w;
        if (!ok) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no triangle rule of order %d", order);
    }
    r.nt = nt;
    r.factor = rhs->factor;
    double *dpar = nullptr;
    int32_t *dgrp = nullptr;
    int rc = grmp_upload(ctx, &dpar, rhs->params, (size_t)rhs->nparams);
    if (!rc && rhs->cell_group) rc = grmp_upload(ctx, &dgrp, rhs->cell_group, (size_t)m->ncells);
    if (!rc && !s->d_locbuf) rc = grmp_alloc(ctx, (void **)&s->d_locbuf, (size_t)m->ncells * 14 * 8);
    if (!rc) {
        r.par = dpar;
        r.group = dgrp;
        const P2bMesh pm{m->d_coords, m->d_cells, m->d_cell_faces, m->d_face_normals, m->d_face_volumes,
                         m->d_cell_face_signs};
        if (rhs->test_operator == 4)
            k_p2b_rhs_cells<12><<<nblk(m->ncells, 128), 128, 0, ctx->stream>>>(m->ncells, pm, r, s->d_locbuf);
        else
            k_p2b_rhs_cells<8><<<nblk(m->ncells, 128), 128, 0, ctx->stream>>>(m->ncells, pm, r, s->d_locbuf);
        GRMP_LAUNCHED(ctx);
        k_gather_rows14<<<nblk(s->ndofs), TPB, 0, ctx->stream>>>(s->ndofs, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc,
                                                                 s->d_locbuf, b->d);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "H1P2B rhs");
    }
    grmp_free(ctx, dpar, (size_t)rhs->nparams * 8);
    grmp_free(ctx, dgrp, (size_t)m->ncells * 4);
    return rc;
}
