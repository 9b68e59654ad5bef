// ItemIntegrator over cells: L2 errors, norms and differences of a discrete
// function (src/assemblypatterns/itemintegrator.jl: L2ErrorIntegrator :40-94,
// L2NormIntegrator :96-130, L2DifferenceIntegrator :132-158, evaluate!
// :173-300, evaluate :314-330).
//
// One thread per cell.  At each quadrature point the operator evaluation of
// the cell's coefficients (eval_febe!: sum over the cell's DoFs in local
// order) is compared with the data function at the physical point, and
//   cell[c] = sum_q  result_q * w_q * |T|
// is written per cell.  The total is the sum over cells in a fixed tree
// order (per-block partial sums, then the partials in block order on the
// host), so it is reproducible run to run; the reference's single running sum
// differs from it by rounding only.
#include <cmath>

#include <vector>

#include "element.cuh"
#include "grmp_internal.h"

namespace {

constexpr int kTB = 128;
constexpr int kMaxIn = 9;   // operator evaluation length: dim * ncomp <= 9

template <int DIM>
__global__ void __launch_bounds__(kTB) k_item_l2(int ncells, const double *coords, const int32_t *cells,
                                                 const int32_t *celldofs, int nb, int ncomp, int op, const double *u,
                                                 const double *v, RhsDev data, double factor, const double *tw,
                                                 const double *txref, const double *tvals, const double *tderivs,
                                                 int nq, double *cellv) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[4 * 3];
    for (int k = 0; k <= DIM; k++)
        for (int j = 0; j < DIM; j++) X[k * DIM + j] = coords[(size_t)cells[(size_t)cell * (DIM + 1) + k] * DIM + j];
    double G[3][3], A[3][3], vol;
    simplex_geometry<DIM, double>(X, G, vol, A);
    const int ld = nb * ncomp;
    const int rdim = op == GRMP_ITEM_GRADIENT ? DIM * ncomp : ncomp;
    double cu[GRMP_MAX_LDOFS], cv[GRMP_MAX_LDOFS];
    for (int i = 0; i < ld; i++) {
        const int d = celldofs[(size_t)cell * ld + i];
        cu[i] = u[d];
        cv[i] = v ? v[d] : 0.0;
    }
    double acc = 0.0;
    for (int q = 0; q < nq; q++) {
        double in1[kMaxIn], in2[kMaxIn];
        for (int k = 0; k < rdim; k++) in1[k] = in2[k] = 0.0;
        // eval_febe!: input_k = sum_dof coeff[dof] * cvals[k, dof, q]
        for (int c = 0; c < ncomp; c++)
            for (int a = 0; a < nb; a++) {
                const int dof = c * nb + a;
                if (op == GRMP_ITEM_GRADIENT) {
                    for (int k = 0; k < DIM; k++) {
                        double g = 0.0;
                        for (int j = 0; j < DIM; j++) g += G[k][j] * tderivs[(q * nb + a) * DIM + j];
                        in1[c * DIM + k] += cu[dof] * g;
                        if (v) in2[c * DIM + k] += cv[dof] * g;
                    }
                } else {
                    const double phi = tvals[q * nb + a];
                    in1[c] += cu[dof] * phi;
                    if (v) in2[c] += cv[dof] * phi;
                }
            }
        double result = 0.0;
        if (v) {
            for (int j = 0; j < rdim; j++) result += (in1[j] - in2[j]) * (in1[j] - in2[j]);
        } else {
            double f[kMaxIn];
            for (int j = 0; j < rdim; j++) f[j] = 0.0;
            if (data.kind >= 0) {
                double x[3] = {0, 0, 0};
                for (int k = 0; k < DIM; k++) {
                    x[k] = X[k];
                    for (int j = 0; j < DIM; j++) x[k] += A[k][j] * txref[3 * q + j];
                }
                rhs_eval(data, DIM, cell, x, f);
            }
            for (int j = 0; j < rdim; j++) {
                const double e = f[j] - in1[j] * factor;
                result += e * e;
            }
        }
        acc += result * tw[q] * vol;
    }
    cellv[cell] = acc;
}

// The same on an H1BR{DIM} function (Identity / Gradient "with
// coefficients", src/feevaluator_h1.jl:77-94): local DoF I < DIM*(DIM+1) is
// the P1 function I % (DIM+1) in component I / (DIM+1); the others are the
// face bubbles (scalar function DIM+1+f) times the global unit normal n_F.
template <int DIM>
__global__ void __launch_bounds__(kTB) k_item_l2_br(int ncells, const double *coords, const int32_t *cells,
                                                    const int32_t *cell_faces, const double *fnormals,
                                                    const int32_t *celldofs, int nb, int op, const double *u,
                                                    const double *v, RhsDev data, double factor, const double *tw,
                                                    const double *txref, const double *tvals, const double *tderivs,
                                                    int nq, double *cellv) {
    constexpr int NV = DIM + 1, ND = DIM * NV + NV;
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[4 * 3], nrm[4][3];
    for (int k = 0; k < NV; k++)
        for (int j = 0; j < DIM; j++) X[k * DIM + j] = coords[(size_t)cells[(size_t)cell * NV + k] * DIM + j];
    for (int f = 0; f < NV; f++)
        for (int j = 0; j < DIM; j++) nrm[f][j] = fnormals[(size_t)cell_faces[(size_t)cell * NV + f] * DIM + j];
    double G[3][3], A[3][3], vol;
    simplex_geometry<DIM, double>(X, G, vol, A);
    const int rdim = op == GRMP_ITEM_GRADIENT ? DIM * DIM : DIM;
    double cu[ND], cvv[ND];
    for (int i = 0; i < ND; i++) {
        const int d = celldofs[(size_t)cell * ND + i];
        cu[i] = u[d];
        cvv[i] = v ? v[d] : 0.0;
    }
    double acc = 0.0;
    for (int q = 0; q < nq; q++) {
        double in1[kMaxIn], in2[kMaxIn];
        for (int k = 0; k < rdim; k++) in1[k] = in2[k] = 0.0;
        for (int dof = 0; dof < ND; dof++) {
            double cv[kMaxIn];
            for (int k = 0; k < rdim; k++) cv[k] = 0.0;
            for (int c = 0; c < DIM; c++) {
                const int si = dof < DIM * NV ? (dof / NV == c ? dof % NV : -1) : NV + (dof - DIM * NV);
                if (si < 0) continue;
                const double coef = dof < DIM * NV ? 1.0 : nrm[dof - DIM * NV][c];
                if (op == GRMP_ITEM_GRADIENT) {
                    for (int k = 0; k < DIM; k++) {
                        double g = 0.0;
                        for (int j = 0; j < DIM; j++) g += G[k][j] * tderivs[(q * nb + si) * DIM + j];
                        cv[c * DIM + k] = g * coef;
                    }
                } else {
                    cv[c] = tvals[q * nb + si] * coef;
                }
            }
            for (int k = 0; k < rdim; k++) {
                in1[k] += cu[dof] * cv[k];
                in2[k] += cvv[dof] * cv[k];
            }
        }
        double result = 0.0;
        if (v) {
            for (int j = 0; j < rdim; j++) result += (in1[j] - in2[j]) * (in1[j] - in2[j]);
        } else {
            double f[kMaxIn];
            for (int j = 0; j < rdim; j++) f[j] = 0.0;
            if (data.kind >= 0) {
                double x[3] = {0, 0, 0};
                for (int k = 0; k < DIM; k++) {
                    x[k] = X[k];
                    for (int j = 0; j < DIM; j++) x[k] += A[k][j] * txref[3 * q + j];
                }
                rhs_eval(data, DIM, cell, x, f);
            }
            for (int j = 0; j < rdim; j++) {
                const double e = f[j] - in1[j] * factor;
                result += e * e;
            }
        }
        acc += result * tw[q] * vol;
    }
    cellv[cell] = acc;
}

// per-block sums of cellv in a fixed tree order
__global__ void __launch_bounds__(256) k_block_sum(int n, const double *x, double *part) {
    __shared__ double sh[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    sh[threadIdx.x] = i < n ? x[i] : 0.0;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

}  // namespace

int grmp_item_l2error_impl(grmp_space s, grmp_vector u, grmp_vector v, int op, const grmp_rhs *data, double factor,
                           int quadorder, double *cell_values, double *total) {
    grmp_context ctx = s->mesh->ctx;
    grmp_mesh m = s->mesh;
    const int dim = m->dim;
    const bool br = s->fe == GRMP_FE_H1BR;
    if (s->fe != GRMP_FE_H1P1 && s->fe != GRMP_FE_H1P2 && !br)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "item integrator: element %d (H1P1, H1P2 and H1BR are supported)",
                         s->fe);
    if (br && (m->nfaces == 0 || s->ncomp != dim))
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: H1BR needs the mesh's face data");
    if (op != GRMP_ITEM_IDENTITY && op != GRMP_ITEM_GRADIENT)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: operator %d", op);
    if (u->n != s->ndofs || (v && v->n != s->ndofs))
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: vector length != space DoFs");
    if (v && data) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: data and a second vector given");
    const int rdim = op == GRMP_ITEM_GRADIENT ? dim * s->ncomp : s->ncomp;
    if (rdim > kMaxIn) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "item integrator: %d operator components", rdim);
    long long need = 0;
    if (data) {
        if (data->ncomponents != rdim)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: data has %d components, the operator %d",
                             data->ncomponents, rdim);
        switch (data->kind) {
            case GRMP_RHS_CONST: need = rdim; break;
            case GRMP_RHS_CELL: need = (long long)m->ncells * rdim; break;
            case GRMP_RHS_FOURIER: need = 1 + dim; break;
            case GRMP_RHS_POLY: need = 5; break;
            default: return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: data kind %d", data->kind);
        }
        if (data->nparams < need || !data->params)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: too few data parameters");
        if ((data->kind == GRMP_RHS_FOURIER && data->nparams % (1 + dim)) ||
            (data->kind == GRMP_RHS_POLY && data->nparams % 5))
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: parameter count not a multiple of the record");
        if (data->kind == GRMP_RHS_POLY)
            for (long long t = 0; t < data->nparams / 5; t++)
                if (data->params[5 * t] < 0 || data->params[5 * t] >= rdim)
                    return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "item integrator: polynomial component out of range");
    }
    // quadrature order: polyorder + shift(op) + bonus (src/assemblypatterns.jl:559-565); "auto" bonus:
    // twice the data's bonus order (L2ErrorIntegrator), 2 without data (L2Norm/L2Difference defaults)
    const int bonus = quadorder >= 0 ? quadorder : (data ? 2 * data->bonus_quadorder : 2);
    int order = grmp_fe_polyorder(s->fe, dim) + (op == GRMP_ITEM_GRADIENT ? -1 : 0) + bonus;
    if (order < 0) order = 0;
    RefTables *rt = new RefTables;
    int rc = grmp_tables(dim, s->fe, order, rt);
    if (rc) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "item integrator: no quadrature rule of order %d in %dD", order, dim);
    }
    const int nq = rt->nq, nb = rt->nb;
    std::vector<double> buf((size_t)nq * (1 + 3 + nb + nb * dim));
    double *bw = buf.data(), *bx = bw + nq, *bv = bx + 3 * nq, *bd = bv + (size_t)nq * nb;
    for (int q = 0; q < nq; q++) {
        bw[q] = rt->w[q];
        for (int k = 0; k < 3; k++) bx[3 * q + k] = rt->xref[q][k];
        for (int a = 0; a < nb; a++) {
            bv[q * nb + a] = rt->vals[q][a];
            for (int j = 0; j < dim; j++) bd[(q * nb + a) * dim + j] = rt->derivs[q][a][j];
        }
    }
    delete rt;
    const int ncells = m->ncells;
    const int nblocks = std::max(1, (ncells + 255) / 256);
    double *dtab = nullptr, *dpar = nullptr, *dcell = nullptr, *dpart = nullptr;
    rc = grmp_upload(ctx, &dtab, buf.data(), buf.size());
    if (!rc && data) rc = grmp_upload(ctx, &dpar, data->params, (size_t)data->nparams);
    if (!rc) rc = grmp_alloc(ctx, (void **)&dcell, (size_t)std::max(1, ncells) * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&dpart, (size_t)nblocks * 8);
    std::vector<double> part(nblocks);
    if (!rc && ncells > 0) {
        const double *dw = dtab, *dx = dtab + nq, *dv = dx + 3 * nq, *dd = dv + (size_t)nq * nb;
        RhsDev r{data ? data->kind : -1, rdim, dpar, data ? data->nparams : 0, 1.0, nq, nb, dw, dx, dv};
        const double *vd = v ? v->d : nullptr;
        if (br && dim == 2)
            k_item_l2_br<2><<<(ncells + kTB - 1) / kTB, kTB, 0, ctx->stream>>>(
                ncells, m->d_coords, m->d_cells, m->d_cell_faces, m->d_face_normals, s->d_celldofs, nb, op, u->d, vd, r,
                factor, dw, dx, dv, dd, nq, dcell);
        else if (br)
            k_item_l2_br<3><<<(ncells + kTB - 1) / kTB, kTB, 0, ctx->stream>>>(
                ncells, m->d_coords, m->d_cells, m->d_cell_faces, m->d_face_normals, s->d_celldofs, nb, op, u->d, vd, r,
                factor, dw, dx, dv, dd, nq, dcell);
        else if (dim == 2)
            k_item_l2<2><<<(ncells + kTB - 1) / kTB, kTB, 0, ctx->stream>>>(
                ncells, m->d_coords, m->d_cells, s->d_celldofs, nb, s->ncomp, op, u->d, vd, r, factor, dw, dx, dv, dd,
                nq, dcell);
        else
            k_item_l2<3><<<(ncells + kTB - 1) / kTB, kTB, 0, ctx->stream>>>(
                ncells, m->d_coords, m->d_cells, s->d_celldofs, nb, s->ncomp, op, u->d, vd, r, factor, dw, dx, dv, dd,
                nq, dcell);
        GRMP_LAUNCHED(ctx);
        k_block_sum<<<nblocks, 256, 0, ctx->stream>>>(ncells, dcell, dpart);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(part.data(), dpart, (size_t)nblocks * 8, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess && cell_values)
            e = cudaMemcpyAsync(cell_values, dcell, (size_t)ncells * 8, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "item integrator kernels");
    }
    if (!rc && total) {
        double t = 0.0;
        for (int b = 0; b < (ncells > 0 ? nblocks : 0); b++) t += part[b];
        *total = t;
    }
    grmp_free(ctx, dtab, buf.size() * 8);
    if (data) grmp_free(ctx, dpar, (size_t)data->nparams * 8);
    grmp_free(ctx, dcell, (size_t)std::max(1, ncells) * 8);
    grmp_free(ctx, dpart, (size_t)nblocks * 8);
    return rc;
}
