// Newton linearisation of NonlinearForms on H1P1 / H1P2 spaces
// (full_assemble!, src/assemblypatterns/nonlinearform.jl:44-240).
//
// For an operator G(u) = (K(input(u)), test(v)) with input = the current
// iterate's operator evaluations at a quadrature point, the Newton step adds
// the Jacobian DG(u) to the matrix and DG(u) u - G(u) to the right-hand side:
//   A[j][i] += vol factor sum_q w_q (J(q) input(phi_i)(q)) . test(phi_j)(q)
//   b[j]    += vol factor sum_q w_q (J(q) input(u)(q) - K(q)) . test(phi_j)(q)
// with J = dK/dinput.  The reference differentiates user kernels by
// ForwardDiff; the device has a closed set of kernels with their Jacobians
// written out (grmp_nl_kind).
//
// Layout: one thread per (cell, test DoF j) evaluates row j of the cell's
// local matrix (all ansatz DoFs i) and the local right-hand side entry, into
// LT[cell][j][i] and LB[cell][j]; a row kernel then adds each DoF's cell
// contributions in ascending cell order through the pattern's slot map
// (deterministic, no atomics).
#include "element.cuh"
#include "grmp_internal.h"

#include <cstring>
#include <vector>

namespace {

constexpr int TPB = 256;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

struct NlDev {
    int kind;
    double factor, kappa, beta;
    TablesDev tab;
};

// input / result sizes of a kernel: DIFFUSION [u, grad u] -> grad-test (dim);
// GRAD_DIFFUSION [grad u] -> dim; CONVECTION [u (dim), grad u (dim x dim,
// component-major)] -> identity-test (dim)
template <int DIM, int NC>
struct NlShape {
    static constexpr int ID = NC == 1 ? 1 + DIM : DIM + DIM * DIM;   // input of DIFFUSION / CONVECTION
    static constexpr int RD = DIM;
};

// value K and Jacobian J[k][m] = dK_k / dinput_m at one quadrature point
template <int DIM, int NC>
__device__ __forceinline__ void nl_kernel(const NlDev &t, const double *in, double *K, double (*J)[NlShape<DIM, NC>::ID]) {
    constexpr int ID = NlShape<DIM, NC>::ID;
    for (int k = 0; k < DIM; k++)
        for (int m = 0; m < ID; m++) J[k][m] = 0.0;
    if (t.kind == GRMP_NL_DIFFUSION) {          // (kappa + beta u^2) grad u
        const double u = in[0];
        const double c = t.kappa + t.beta * (u * u);
        for (int k = 0; k < DIM; k++) {
            K[k] = c * in[1 + k];
            J[k][0] = (t.beta * (2.0 * u)) * in[1 + k];
            J[k][1 + k] = c;
        }
    } else if (t.kind == GRMP_NL_GRAD_DIFFUSION) {   // (kappa + |grad u|^2) grad u; input[0] unused
        double g2 = 0.0;
        for (int k = 0; k < DIM; k++) g2 += in[1 + k] * in[1 + k];
        const double c = t.kappa + g2;
        for (int k = 0; k < DIM; k++) {
            K[k] = c * in[1 + k];
            for (int l = 0; l < DIM; l++) J[k][1 + l] = (2.0 * in[1 + l]) * in[1 + k];
            J[k][1 + k] += c;
        }
    } else {                                         // (u . grad) u
        for (int c = 0; c < DIM; c++) {
            double s = 0.0;
            for (int l = 0; l < DIM; l++) s += in[l] * in[DIM + c * DIM + l];
            K[c] = s;
            for (int m = 0; m < DIM; m++) J[c][m] = in[DIM + c * DIM + m];
            for (int l = 0; l < DIM; l++) J[c][DIM + c * DIM + l] = in[l];
        }
    }
}

template <int DIM, int NB, int NC>
__global__ void __launch_bounds__(128) k_nl_cells(int ncells, const double *coords, const int32_t *cells,
                                                  const int32_t *celldofs, const double *u, NlDev t, double *LT,
                                                  double *LB) {
    constexpr int LD = NB * NC;
    constexpr int ID = NlShape<DIM, NC>::ID;
    const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (gid >= (long long)ncells * LD) return;
    const int cell = (int)(gid / LD), j = (int)(gid % LD);
    double X[(DIM + 1) * DIM];
    for (int v = 0; v <= DIM; v++)
        for (int k = 0; k < DIM; k++) X[v * DIM + k] = coords[(size_t)cells[(size_t)cell * (DIM + 1) + v] * DIM + k];
    double A[3][3], G[3][3], vol;
    simplex_geometry_rn<DIM>(X, A, G, vol);
    double uc[LD];
    for (int b = 0; b < LD; b++) uc[b] = u[celldofs[(size_t)cell * LD + b]];
    const int cj = j / NB, aj = j - cj * NB;
    double lm[LD];
    for (int i = 0; i < LD; i++) lm[i] = 0.0;
    double lb = 0.0;
    for (int q = 0; q < t.tab.nq; q++) {
        const double *vq = t.tab.vals + (size_t)q * NB;
        double gr[NB][DIM];
        for (int a = 0; a < NB; a++)
            for (int k = 0; k < DIM; k++) {
                double s = 0.0;
                for (int l = 0; l < DIM; l++) s += G[k][l] * t.tab.derivs[((size_t)q * NB + a) * DIM + l];
                gr[a][k] = s;
            }
        // current iterate's operator evaluations (in the DoF order of eval_febe!)
        double in[ID];
        for (int m = 0; m < ID; m++) in[m] = 0.0;
        for (int b = 0; b < LD; b++) {
            const int c = b / NB, a = b - c * NB;
            if (NC == 1) {
                in[0] += uc[b] * vq[a];
                for (int k = 0; k < DIM; k++) in[1 + k] += uc[b] * gr[a][k];
            } else {
                in[c] += uc[b] * vq[a];
                for (int k = 0; k < DIM; k++) in[DIM + c * DIM + k] += uc[b] * gr[a][k];
            }
        }
        double K[DIM], J[DIM][ID];
        nl_kernel<DIM, NC>(t, in, K, J);
        // test operator of phi_j: gradient (scalar kernels) or identity (convection)
        double tv[DIM];
        for (int k = 0; k < DIM; k++) tv[k] = NC == 1 ? gr[aj][k] : (k == cj ? vq[aj] : 0.0);
        const double w = t.tab.w[q];
        for (int i = 0; i < LD; i++) {
            const int ci = i / NB, ai = i - ci * NB;
            double in2[ID];
            for (int m = 0; m < ID; m++) in2[m] = 0.0;
            if (NC == 1) {
                in2[0] = vq[ai];
                for (int k = 0; k < DIM; k++) in2[1 + k] = gr[ai][k];
            } else {
                in2[ci] = vq[ai];
                for (int k = 0; k < DIM; k++) in2[DIM + ci * DIM + k] = gr[ai][k];
            }
            double temp = 0.0;
            for (int k = 0; k < DIM; k++) {
                double ar = 0.0;
                for (int m = 0; m < ID; m++) ar += J[k][m] * in2[m];
                temp += ar * tv[k];
            }
            lm[i] += temp * w;
        }
        double temp = 0.0;
        for (int k = 0; k < DIM; k++) {
            double ar = 0.0;
            for (int m = 0; m < ID; m++) ar += J[k][m] * in[m];
            temp += (ar - K[k]) * tv[k];
        }
        lb += temp * w;
    }
    const double itemfactor = vol * t.factor;
    double *row = LT + ((size_t)cell * LD + j) * LD;
    for (int i = 0; i < LD; i++) row[i] = lm[i] * itemfactor;
    LB[(size_t)cell * LD + j] = lb * itemfactor;
}

// A[row][.] (+)= sum over the row's incidences (ascending cells) of the cell
// rows LT[cell][local][.] through the slot map; b[row] (+)= LB.  A nonzero
// contribution that the pattern dropped raises *missing.
template <typename S>
__global__ void k_nl_gather(int32_t nrows, int ld, const int32_t *inc_ptr, const int32_t *inc_cell,
                            const uint8_t *inc_loc, const S *slot, const int32_t *rowptr, const double *LT,
                            const double *LB, double *v64, float *v32, double *b, int add, int *missing) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    const S DROP = (S)~(S)0;
    const int r0 = rowptr[row], r1 = rowptr[row + 1];
    if (!add)
        for (int k = r0; k < r1; k++) {
            v64[k] = 0.0;
            if (v32) v32[k] = 0.0f;
        }
    double bb = add ? b[row] : 0.0;
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) {
        const int cell = inc_cell[p], a = inc_loc[p];
        const double *lt = LT + ((size_t)cell * ld + a) * ld;
        const S *sl = slot + (size_t)p * ld;
        for (int B = 0; B < ld; B++) {
            const double v = lt[B];
            const S s = sl[B];
            if (s == DROP) {
                if (v != 0.0) atomicExch(missing, 1);
                continue;
            }
            v64[r0 + s] += v;
            if (v32) v32[r0 + s] += (float)v;
        }
        bb += LB[(size_t)cell * ld + a];
    }
    b[row] = bb;
}

template <int DIM, int NB, int NC>
void launch_nl_cells(grmp_space s, const double *u, const NlDev &t, double *LT, double *LB) {
    grmp_mesh m = s->mesh;
    const long long n = (long long)m->ncells * NB * NC;
    k_nl_cells<DIM, NB, NC><<<nblk(n, 128), 128, 0, m->ctx->stream>>>(m->ncells, m->d_coords, m->d_cells,
                                                                      s->d_celldofs, u, t, LT, LB);
}

}  // namespace

int grmp_assemble_nonlinear_impl(grmp_matrix A, grmp_vector b, grmp_vector u, const grmp_nonlinear_term *term,
                                 int precision, int add) {
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    const int dim = m->dim;
    if (A->imported) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "nonlinear form: the matrix was imported from CSC");
    if (s->fe != GRMP_FE_H1P1 && s->fe != GRMP_FE_H1P2)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "nonlinear forms are built on H1P1 / H1P2 spaces");
    const bool scalar_kind = term->kind == GRMP_NL_DIFFUSION || term->kind == GRMP_NL_GRAD_DIFFUSION;
    if (!scalar_kind && term->kind != GRMP_NL_CONVECTION)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "nonlinear form: kind %d", term->kind);
    if (scalar_kind && s->ncomp != 1)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "nonlinear diffusion needs a scalar space");
    if (!scalar_kind && s->ncomp != dim)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "convection needs ncomponents == dim");
    if (precision != GRMP_FP64 && precision != GRMP_FP64_FP32)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "nonlinear form: precision FP64 or FP64_FP32");
    // quadrature order (src/assemblypatterns.jl:558-565): bonus + sum over the
    // operators of polyorder + shift (Identity 0, Gradient -1)
    const int p = grmp_fe_polyorder(s->fe, dim);
    int order = term->bonus_quadorder;
    if (term->kind == GRMP_NL_DIFFUSION) order += p + (p - 1) + (p - 1);          // [Identity, Gradient] x Gradient
    else if (term->kind == GRMP_NL_GRAD_DIFFUSION) order += (p - 1) + (p - 1);    // [Gradient] x Gradient
    else order += p + (p - 1) + p;                                                // [Identity, Gradient] x Identity
    if (order < 0) order = 0;
    RefTables *rt = new RefTables;
    int rc = grmp_tables(dim, s->fe, order, rt);
    if (rc || rt->nq <= 0) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no quadrature rule of order %d in %dD", order, dim);
    }
    const int nq = rt->nq, nb = rt->nb;
    std::vector<double> buf((size_t)nq + (size_t)nq * nb + (size_t)nq * nb * dim);
    double *w = buf.data(), *v = w + nq, *dv = v + (size_t)nq * nb;
    for (int q = 0; q < nq; q++) {
        w[q] = rt->w[q];
        for (int a = 0; a < nb; a++) {
            v[q * nb + a] = rt->vals[q][a];
            for (int j = 0; j < dim; j++) dv[((size_t)q * nb + a) * dim + j] = rt->derivs[q][a][j];
        }
    }
    delete rt;
    const int ld = s->ldofs;
    double *dtab = nullptr, *LT = nullptr, *LB = nullptr;
    int *dmiss = nullptr;
    const size_t ltn = (size_t)m->ncells * ld * ld, lbn = (size_t)m->ncells * ld;
    rc = grmp_upload(ctx, &dtab, buf.data(), buf.size());
    if (!rc) rc = grmp_alloc(ctx, (void **)&LT, ltn * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&LB, lbn * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&dmiss, 4);
    if (!rc && !A->d_vals64) rc = grmp_alloc(ctx, (void **)&A->d_vals64, (size_t)A->nnz * 8);
    if (!rc && precision == GRMP_FP64_FP32 && !A->d_vals32) rc = grmp_alloc(ctx, (void **)&A->d_vals32, (size_t)A->nnz * 4);
    if (!rc) {
        NlDev t;
        std::memset(&t, 0, sizeof(t));
        t.kind = term->kind;
        t.factor = term->factor;
        t.kappa = term->param[0];
        t.beta = term->param[1];
        t.tab.nq = nq;
        t.tab.nb = nb;
        t.tab.dim = dim;
        t.tab.w = dtab;
        t.tab.vals = dtab + nq;
        t.tab.derivs = dtab + nq + (size_t)nq * nb;
        if (dim == 2 && nb == 3 && s->ncomp == 1) launch_nl_cells<2, 3, 1>(s, u->d, t, LT, LB);
        else if (dim == 2 && nb == 6 && s->ncomp == 1) launch_nl_cells<2, 6, 1>(s, u->d, t, LT, LB);
        else if (dim == 3 && nb == 4 && s->ncomp == 1) launch_nl_cells<3, 4, 1>(s, u->d, t, LT, LB);
        else if (dim == 3 && nb == 10 && s->ncomp == 1) launch_nl_cells<3, 10, 1>(s, u->d, t, LT, LB);
        else if (dim == 2 && nb == 3 && s->ncomp == 2) launch_nl_cells<2, 3, 2>(s, u->d, t, LT, LB);
        else if (dim == 2 && nb == 6 && s->ncomp == 2) launch_nl_cells<2, 6, 2>(s, u->d, t, LT, LB);
        else if (dim == 3 && nb == 4 && s->ncomp == 3) launch_nl_cells<3, 4, 3>(s, u->d, t, LT, LB);
        else if (dim == 3 && nb == 10 && s->ncomp == 3) launch_nl_cells<3, 10, 3>(s, u->d, t, LT, LB);
        else rc = grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "nonlinear form: element layout dim=%d nb=%d nc=%d", dim, nb,
                            s->ncomp);
        if (!rc) {
            GRMP_LAUNCHED(ctx);
            cudaMemsetAsync(dmiss, 0, 4, ctx->stream);
            float *v32 = precision == GRMP_FP64_FP32 ? A->d_vals32 : nullptr;
            if (A->slot_bytes == 1)
                k_nl_gather<uint8_t><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(
                    A->nrows, ld, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc, (const uint8_t *)A->d_slot, A->d_rowptr,
                    LT, LB, A->d_vals64, v32, b->d, add, dmiss);
            else
                k_nl_gather<uint16_t><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(
                    A->nrows, ld, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc, (const uint16_t *)A->d_slot, A->d_rowptr,
                    LT, LB, A->d_vals64, v32, b->d, add, dmiss);
            GRMP_LAUNCHED(ctx);
            int hmiss = 0;
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(&hmiss, dmiss, 4, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "nonlinear form kernels");
            else if (hmiss)
                rc = grmp_fail(ctx, GRMP_ERR_INVALID_ARG,
                               "nonlinear form: the pattern lacks local couplings of the Jacobian "
                               "(build it with a GRMP_OP_STRUCTURAL term)");
            if (!rc) {
                A->has64 = true;
                if (v32) A->has32 = true;
                A->eliminated = false;
            }
        }
    }
    grmp_free(ctx, dtab, buf.size() * 8);
    grmp_free(ctx, LT, ltn * 8);
    grmp_free(ctx, LB, lbn * 8);
    grmp_free(ctx, dmiss, 4);
    return rc;
}
