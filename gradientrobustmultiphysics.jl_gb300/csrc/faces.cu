// Interior-face (ON_IFACES) terms with discontinuous operators: the gradient
// jump [grad u] = grad u|T1 - grad u|T2 across each interior face
// (Jump(Gradient), update_dii4op!, src/assemblypatterns.jl:103-153).
//
//   * BilinearForm([Jump(Gradient), Jump(Gradient)], Action(input |F|^p);
//     AT = ON_IFACES, factor tau): tau |F| |F|^p sum_q w_q [grad phi_i].[grad phi_j],
//     the interior-penalty stabilisation of
//     examples/Example203_ReactionConvectionDiffusion2D.jl:89-92;
//   * ItemIntegrator([Jump(Gradient)], ...; AT = ON_IFACES): per-face
//     integrals of |[grad u]|^2 or ([grad u].n_F)^2 times |F|^p, the jump part
//     of the error estimator of examples/Example210_PoissonLshapeAdaptive2D.jl:58-75.
//
// A face couples the DoFs of its two cells, so a matrix with face terms holds
// the DoFs of the face neighbours of each row's cells (pattern.cu).  Values
// are added row by row: each row walks its cells in ascending order and their
// interior faces (a face shared by two of the row's cells is taken once, from
// the lower cell), evaluates the jumps of its own basis function and of every
// function of the two cells at the face's quadrature points and adds the
// products into its CSR entries (deterministic, no atomics).  Quadrature points
// of a face are placed by barycentric weights over the face's vertices in
// ascending global vertex order, so both cells see the same points.
#include "element.cuh"
#include "grmp_internal.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int TPB = 256;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// ------------------------------------------------------------------ adjacency
__global__ void k_face_count(long long n, int nf, const int32_t *cell_faces, int32_t *cnt, int32_t *fc) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int F = cell_faces[i];
    const int slot = atomicAdd(&cnt[F], 1);
    if (slot < 2) fc[2 * (size_t)F + slot] = (int32_t)(i / nf);
}

// lower cell id first, -1 for the missing neighbour of a boundary face
__global__ void k_face_order(int32_t nfaces, const int32_t *cnt, int32_t *fc, int *bad) {
    const int F = blockIdx.x * blockDim.x + threadIdx.x;
    if (F >= nfaces) return;
    const int n = cnt[F];
    if (n < 1 || n > 2) {
        atomicExch(bad, 1);
        fc[2 * (size_t)F] = fc[2 * (size_t)F + 1] = -1;
        return;
    }
    if (n == 1) {
        fc[2 * (size_t)F + 1] = -1;
        return;
    }
    const int a = fc[2 * (size_t)F], b = fc[2 * (size_t)F + 1];
    fc[2 * (size_t)F] = min(a, b);
    fc[2 * (size_t)F + 1] = max(a, b);
}

__global__ void k_cell_nbr(long long n, int nf, const int32_t *cell_faces, const int32_t *fc, int32_t *nbr) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int F = cell_faces[i], c = (int)(i / nf);
    const int a = fc[2 * (size_t)F], b = fc[2 * (size_t)F + 1];
    nbr[i] = b < 0 ? -1 : (a == c ? b : a);
}

// ------------------------------------------------------------------ element evaluation
// local vertices of the faces of a simplex (the mesh module's local face
// numbering: triangles [0,1], [1,2], [2,0]; tetrahedra [0,1,2], [0,1,3],
// [1,2,3], [0,2,3])
__device__ __forceinline__ int face_vertex(int dim, int f, int k) {
    if (dim == 2) return (f + k) % 3;
    const int t[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
    return t[f][k];
}

// the face's vertices in ascending global vertex order, as local vertices of the cell
template <int DIM>
__device__ __forceinline__ void face_canon(const int32_t *cells, int cell, int f, int loc[DIM]) {
    int gid[DIM];
    for (int k = 0; k < DIM; k++) {
        loc[k] = face_vertex(DIM, f, k);
        gid[k] = cells[(size_t)cell * (DIM + 1) + loc[k]];
    }
    for (int i = 1; i < DIM; i++)
        for (int j = i; j > 0 && gid[j] < gid[j - 1]; j--) {
            int t = gid[j]; gid[j] = gid[j - 1]; gid[j - 1] = t;
            t = loc[j]; loc[j] = loc[j - 1]; loc[j - 1] = t;
        }
}

// reference coordinates of the point with barycentric weights lam over the
// face's canonical vertices: reference vertex 0 is the origin, vertex v >= 1
// the unit vector e_{v-1}
template <int DIM>
__device__ __forceinline__ void face_point(const double *lam, const int loc[DIM], double xh[DIM]) {
    for (int j = 0; j < DIM; j++) {
        double s = 0.0;
        for (int k = 0; k < DIM; k++) s += loc[k] == j + 1 ? lam[k] : 0.0;
        xh[j] = s;
    }
}

struct Dd {
    double v, d[3];
};
__device__ __forceinline__ Dd dmul(Dd x, Dd y) {
    Dd r;
    r.v = x.v * y.v;
    for (int i = 0; i < 3; i++) r.d[i] = y.v * x.d[i] + x.v * y.d[i];
    return r;
}
__device__ __forceinline__ Dd dscal(double c, Dd x) {
    Dd r;
    r.v = c * x.v;
    for (int i = 0; i < 3; i++) r.d[i] = c * x.d[i];
    return r;
}
__device__ __forceinline__ Dd dsubc(Dd x, double c) {
    x.v -= c;
    return x;
}
__device__ __forceinline__ Dd dcsub(double c, Dd x) {
    Dd r;
    r.v = c - x.v;
    for (int i = 0; i < 3; i++) r.d[i] = -x.d[i];
    return r;
}
__device__ __forceinline__ Dd dsub(Dd x, Dd y) {
    Dd r;
    r.v = x.v - y.v;
    for (int i = 0; i < 3; i++) r.d[i] = x.d[i] - y.d[i];
    return r;
}

// physical gradients of the scalar P1 / P2 basis (h1_p1.jl:64-75,
// h1_p2.jl:134-165; forward-mode derivative order) at reference point xh
template <int DIM, int NB>
__device__ void basis_grads(const double *xh, const double G[3][3], double g[NB][DIM]) {
    Dd x[3];
    for (int j = 0; j < 3; j++) {
        x[j].v = j < DIM ? xh[j] : 0.0;
        for (int i = 0; i < 3; i++) x[j].d[i] = i == j ? 1.0 : 0.0;
    }
    Dd o[NB];
    Dd r = dcsub(1.0, x[0]);
    for (int j = 1; j < DIM; j++) r = dsub(r, x[j]);
    if constexpr (NB == DIM + 1) {
        o[0] = r;
        for (int j = 0; j < DIM; j++) o[1 + j] = x[j];
    } else if constexpr (DIM == 2) {
        o[0] = dmul(dscal(2.0, r), dsubc(r, 0.5));
        o[1] = dmul(dscal(2.0, x[0]), dsubc(x[0], 0.5));
        o[2] = dmul(dscal(2.0, x[1]), dsubc(x[1], 0.5));
        o[3] = dmul(dscal(4.0, r), x[0]);
        o[4] = dmul(dscal(4.0, x[0]), x[1]);
        o[5] = dmul(dscal(4.0, x[1]), r);
    } else {
        o[0] = dmul(dscal(2.0, r), dsubc(r, 0.5));
        o[1] = dmul(dscal(2.0, x[0]), dsubc(x[0], 0.5));
        o[2] = dmul(dscal(2.0, x[1]), dsubc(x[1], 0.5));
        o[3] = dmul(dscal(2.0, x[2]), dsubc(x[2], 0.5));
        o[4] = dmul(dscal(4.0, r), x[0]);
        o[5] = dmul(dscal(4.0, r), x[1]);
        o[6] = dmul(dscal(4.0, r), x[2]);
        o[7] = dmul(dscal(4.0, x[0]), x[1]);
        o[8] = dmul(dscal(4.0, x[0]), x[2]);
        o[9] = dmul(dscal(4.0, x[1]), x[2]);
    }
    for (int a = 0; a < NB; a++)
        for (int k = 0; k < DIM; k++) {
            double s = 0.0;
            for (int j = 0; j < DIM; j++) s += G[k][j] * o[a].d[j];
            g[a][k] = s;
        }
}

template <int DIM>
__device__ __forceinline__ void cell_geometry(const double *coords, const int32_t *cells, int c, double G[3][3]) {
    double X[(DIM + 1) * DIM], A[3][3], vol;
    for (int v = 0; v <= DIM; v++)
        for (int k = 0; k < DIM; k++) X[v * DIM + k] = coords[(size_t)cells[(size_t)c * (DIM + 1) + v] * DIM + k];
    simplex_geometry_rn<DIM>(X, A, G, vol);
}

__device__ __forceinline__ double power_of(double x, double p) {
    const int k = (int)p;
    if ((double)k == p && k >= 0 && k <= 8) {
        double r = 1.0;
        for (int i = 0; i < k; i++) r *= x;
        return r;
    }
    return pow(x, p);
}

struct FaceRule {
    int nq;
    double lam[32][3];   // barycentric weights over the face's canonical vertices
    double w[32];        // weights (sum 1 over the face)
};

struct FaceTermDev {
    double factor, power;
};

// ------------------------------------------------------------------ face bilinear terms
template <int DIM, int NB>
__global__ void __launch_bounds__(128) k_face_rows(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell,
                                                   const uint8_t *inc_loc, const int32_t *celldofs,
                                                   const int32_t *cells, const double *coords,
                                                   const int32_t *cell_faces, const double *fvol, const int32_t *nbr,
                                                   const int32_t *rowptr, const int32_t *cols, FaceTermDev t,
                                                   FaceRule r, double *v64, float *v32, int *missing) {
    constexpr int NF = DIM + 1, LD = NB;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    const int r0 = rowptr[row], r1 = rowptr[row + 1];
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) {
        const int c = inc_cell[p], a = inc_loc[p];
        for (int f = 0; f < NF; f++) {
            const int c2 = nbr[(size_t)c * NF + f];
            if (c2 < 0) continue;
            int a2 = -1;
            for (int b = 0; b < LD; b++)
                if (celldofs[(size_t)c2 * LD + b] == row) a2 = b;
            if (a2 >= 0 && c2 < c) continue;   // taken from the lower of the row's two cells
            const int F = cell_faces[(size_t)c * NF + f];
            int f2 = 0;
            for (int g = 0; g < NF; g++)
                if (cell_faces[(size_t)c2 * NF + g] == F) f2 = g;
            int loc1[DIM], loc2[DIM];
            face_canon<DIM>(cells, c, f, loc1);
            face_canon<DIM>(cells, c2, f2, loc2);
            double G1[3][3], G2[3][3];
            cell_geometry<DIM>(coords, cells, c, G1);
            cell_geometry<DIM>(coords, cells, c2, G2);
            const double s1 = c < c2 ? 1.0 : -1.0, s2 = -s1;
            // columns: the DoFs of c, then those of c2 that c lacks
            int32_t colid[2 * LD];
            int l1[2 * LD], l2[2 * LD], ncol = 0;
            for (int b = 0; b < LD; b++) {
                const int32_t col = celldofs[(size_t)c * LD + b];
                int b2 = -1;
                for (int e = 0; e < LD; e++)
                    if (celldofs[(size_t)c2 * LD + e] == col) b2 = e;
                colid[ncol] = col, l1[ncol] = b, l2[ncol] = b2, ncol++;
            }
            for (int b2 = 0; b2 < LD; b2++) {
                const int32_t col = celldofs[(size_t)c2 * LD + b2];
                bool inc1 = false;
                for (int e = 0; e < LD; e++) inc1 = inc1 || celldofs[(size_t)c * LD + e] == col;
                if (inc1) continue;
                colid[ncol] = col, l1[ncol] = -1, l2[ncol] = b2, ncol++;
            }
            double acc[2 * LD];
            for (int k = 0; k < ncol; k++) acc[k] = 0.0;
            for (int q = 0; q < r.nq; q++) {
                double xh1[DIM], xh2[DIM], g1[NB][DIM], g2[NB][DIM];
                face_point<DIM>(r.lam[q], loc1, xh1);
                face_point<DIM>(r.lam[q], loc2, xh2);
                basis_grads<DIM, NB>(xh1, G1, g1);
                basis_grads<DIM, NB>(xh2, G2, g2);
                double Ji[DIM];
                for (int k = 0; k < DIM; k++) Ji[k] = s1 * g1[a][k] + (a2 >= 0 ? s2 * g2[a2][k] : 0.0);
                for (int m = 0; m < ncol; m++) {
                    double d = 0.0;
                    for (int k = 0; k < DIM; k++) {
                        const double Jj = (l1[m] >= 0 ? s1 * g1[l1[m]][k] : 0.0) + (l2[m] >= 0 ? s2 * g2[l2[m]][k] : 0.0);
                        d += Ji[k] * Jj;
                    }
                    acc[m] += r.w[q] * d;
                }
            }
            const double fv = fvol[F];
            const double scale = t.factor * fv * power_of(fv, t.power);
            for (int m = 0; m < ncol; m++) {
                int lo = r0, hi = r1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (cols[mid] < colid[m]) lo = mid + 1;
                    else hi = mid;
                }
                if (lo >= r1 || cols[lo] != colid[m]) {
                    atomicExch(missing, 1);
                    continue;
                }
                const double v = acc[m] * scale;
                v64[lo] += v;
                if (v32) v32[lo] += (float)v;
            }
        }
    }
}

// ------------------------------------------------------------------ jump integrator
template <int DIM, int NB>
__global__ void k_face_jumps(int32_t nfaces, const int32_t *face_cells, const int32_t *cell_faces,
                             const int32_t *cells, const double *coords, const int32_t *celldofs, const double *u,
                             const double *fnormals, const double *fvol, int kind, double power, double factor,
                             FaceRule r, double *out) {
    constexpr int NF = DIM + 1, LD = NB;
    const int F = blockIdx.x * blockDim.x + threadIdx.x;
    if (F >= nfaces) return;
    const int c1 = face_cells[2 * (size_t)F], c2 = face_cells[2 * (size_t)F + 1];
    if (c1 < 0 || c2 < 0) {
        out[F] = 0.0;
        return;
    }
    int f1 = 0, f2 = 0;
    for (int g = 0; g < NF; g++) {
        if (cell_faces[(size_t)c1 * NF + g] == F) f1 = g;
        if (cell_faces[(size_t)c2 * NF + g] == F) f2 = g;
    }
    int loc1[DIM], loc2[DIM];
    face_canon<DIM>(cells, c1, f1, loc1);
    face_canon<DIM>(cells, c2, f2, loc2);
    double G1[3][3], G2[3][3];
    cell_geometry<DIM>(coords, cells, c1, G1);
    cell_geometry<DIM>(coords, cells, c2, G2);
    double acc = 0.0;
    for (int q = 0; q < r.nq; q++) {
        double xh1[DIM], xh2[DIM], g1[NB][DIM], g2[NB][DIM];
        face_point<DIM>(r.lam[q], loc1, xh1);
        face_point<DIM>(r.lam[q], loc2, xh2);
        basis_grads<DIM, NB>(xh1, G1, g1);
        basis_grads<DIM, NB>(xh2, G2, g2);
        double J[DIM];
        for (int k = 0; k < DIM; k++) J[k] = 0.0;
        for (int b = 0; b < LD; b++) {
            const double u1 = u[celldofs[(size_t)c1 * LD + b]], u2 = u[celldofs[(size_t)c2 * LD + b]];
            for (int k = 0; k < DIM; k++) J[k] += u1 * g1[b][k] - u2 * g2[b][k];
        }
        double val;
        if (kind == 1) {
            double jn = 0.0;
            for (int k = 0; k < DIM; k++) jn += J[k] * fnormals[(size_t)F * DIM + k];
            val = jn * jn;
        } else {
            val = 0.0;
            for (int k = 0; k < DIM; k++) val += J[k] * J[k];
        }
        acc += r.w[q] * val;
    }
    const double fv = fvol[F];
    out[F] = acc * power_of(fv, power) * fv * factor;
}

// rule on the face's reference element (edge or triangle) as barycentric weights
int face_rule(grmp_context ctx, int dim, int order, FaceRule *r) {
    double (*x)[3] = new double[GRMP_MAXQ][3];
    double *w = new double[GRMP_MAXQ];
    const int nq = grmp_quadrature(dim - 1, order, x, w);
    const bool ok = nq > 0 && nq <= 32;
    if (ok) {
        r->nq = nq;
        for (int q = 0; q < nq; q++) {
            if (dim == 2) {
                r->lam[q][0] = 1.0 - x[q][0];
                r->lam[q][1] = x[q][0];
                r->lam[q][2] = 0.0;
            } else {
                r->lam[q][0] = 1.0 - x[q][0] - x[q][1];
                r->lam[q][1] = x[q][0];
                r->lam[q][2] = x[q][1];
            }
            r->w[q] = w[q];
        }
    }
    delete[] x;
    delete[] w;
    return ok ? GRMP_OK : grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no face rule of order %d", order);
}

}  // namespace

int grmp_mesh_neighbors(grmp_mesh m) {
    grmp_context ctx = m->ctx;
    if (m->d_cell_nbr && m->d_face_cells) return GRMP_OK;
    if (m->nfaces <= 0) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "face terms need the mesh's faces (set or build them)");
    const int nf = m->dim + 1;
    const long long n = (long long)m->ncells * nf;
    int32_t *cnt = nullptr, *fc = nullptr, *nbr = nullptr;
    int *bad = nullptr;
    int rc = grmp_alloc(ctx, (void **)&cnt, (size_t)m->nfaces * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&fc, (size_t)m->nfaces * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&nbr, (size_t)n * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&bad, 4);
    int hbad = 0;
    if (!rc) {
        cudaMemsetAsync(cnt, 0, (size_t)m->nfaces * 4, ctx->stream);
        cudaMemsetAsync(bad, 0, 4, ctx->stream);
        k_face_count<<<nblk(n), TPB, 0, ctx->stream>>>(n, nf, m->d_cell_faces, cnt, fc);
        GRMP_LAUNCHED(ctx);
        k_face_order<<<nblk(m->nfaces), TPB, 0, ctx->stream>>>(m->nfaces, cnt, fc, bad);
        GRMP_LAUNCHED(ctx);
        k_cell_nbr<<<nblk(n), TPB, 0, ctx->stream>>>(n, nf, m->d_cell_faces, fc, nbr);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "face adjacency");
        else if (hbad) rc = grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "face adjacency: a face has no cell or more than two");
    }
    grmp_free(ctx, cnt, (size_t)m->nfaces * 4);
    grmp_free(ctx, bad, 4);
    if (rc) {
        grmp_free(ctx, fc, (size_t)m->nfaces * 8);
        grmp_free(ctx, nbr, (size_t)n * 4);
        return rc;
    }
    m->d_face_cells = fc;
    m->d_cell_nbr = nbr;
    return GRMP_OK;
}

int grmp_face_assemble(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision) {
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    const int dim = m->dim;
    if (s->ncomp != 1 || (s->fe != GRMP_FE_H1P1 && s->fe != GRMP_FE_H1P2))
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "face terms: scalar H1P1 / H1P2 spaces");
    int rc = grmp_mesh_neighbors(m);
    if (rc) return rc;
    int *dmiss = nullptr;
    rc = grmp_alloc(ctx, (void **)&dmiss, 4);
    if (rc) return rc;
    cudaMemsetAsync(dmiss, 0, 4, ctx->stream);
    double *v64 = precision != GRMP_FP32 ? A->d_vals64 : nullptr;
    float *v32 = precision != GRMP_FP64 ? A->d_vals32 : nullptr;
    const int p = grmp_fe_polyorder(s->fe, dim);
    for (int i = 0; i < nterms && !rc; i++) {
        FaceRule r;
        std::memset(&r, 0, sizeof(r));
        // Jump(Gradient) x Jump(Gradient) on the face geometry: 2 (p - 1) + bonus
        int order = 2 * (p - 1) + terms[i].bonus_quadorder;
        rc = face_rule(ctx, dim, order < 0 ? 0 : order, &r);
        if (rc) break;
        FaceTermDev t{terms[i].factor, terms[i].param[0]};
        // the FP32 values get the FP64 contributions rounded; v64 is always
        // present here (the cell assembly that precedes this allocates it)
        double *w64 = v64;
        float *w32 = v32;
        if (!w64) {
            rc = grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "face terms: FP64 values are required (use FP64 or FP64_FP32)");
            break;
        }
        auto go = [&](auto kern) {
            kern<<<nblk(A->nrows, 128), 128, 0, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc,
                                                               s->d_celldofs, m->d_cells, m->d_coords, m->d_cell_faces,
                                                               m->d_face_volumes, m->d_cell_nbr, A->d_rowptr,
                                                               A->d_cols, t, r, w64, w32, dmiss);
        };
        if (dim == 2 && s->nb == 3) go(k_face_rows<2, 3>);
        else if (dim == 2 && s->nb == 6) go(k_face_rows<2, 6>);
        else if (dim == 3 && s->nb == 4) go(k_face_rows<3, 4>);
        else go(k_face_rows<3, 10>);
        GRMP_LAUNCHED(ctx);
    }
    int hmiss = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hmiss, dmiss, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, dmiss, 4);
    if (!rc && e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "face terms");
    if (!rc && hmiss)
        rc = grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "face terms: the pattern lacks face couplings (build it with the face terms)");
    return rc;
}

extern "C" int grmp_item_face_jumps(grmp_space s, grmp_vector u, int kind, double power, double factor,
                                    int bonus_quadorder, double *face_values, double *total) {
    if (!s || !u || (kind != 0 && kind != 1)) return GRMP_ERR_INVALID_ARG;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    if (u->ctx != ctx || u->n != s->ndofs) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "face jumps: vector mismatch");
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (s->ncomp != 1 || (s->fe != GRMP_FE_H1P1 && s->fe != GRMP_FE_H1P2))
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "face jumps: scalar H1P1 / H1P2 spaces");
    int rc = grmp_mesh_neighbors(m);
    if (rc) return rc;
    const int dim = m->dim, p = grmp_fe_polyorder(s->fe, dim);
    FaceRule r;
    std::memset(&r, 0, sizeof(r));
    int order = 2 * (p - 1) + bonus_quadorder;
    rc = face_rule(ctx, dim, order < 0 ? 0 : order, &r);
    if (rc) return rc;
    double *dout = nullptr;
    rc = grmp_alloc(ctx, (void **)&dout, (size_t)m->nfaces * 8);
    if (rc) return rc;
    auto go = [&](auto kern) {
        kern<<<nblk(m->nfaces), TPB, 0, ctx->stream>>>(m->nfaces, m->d_face_cells, m->d_cell_faces, m->d_cells,
                                                       m->d_coords, s->d_celldofs, u->d, m->d_face_normals,
                                                       m->d_face_volumes, kind, power, factor, r, dout);
    };
    if (dim == 2 && s->nb == 3) go(k_face_jumps<2, 3>);
    else if (dim == 2 && s->nb == 6) go(k_face_jumps<2, 6>);
    else if (dim == 3 && s->nb == 4) go(k_face_jumps<3, 4>);
    else go(k_face_jumps<3, 10>);
    GRMP_LAUNCHED(ctx);
    std::vector<double> h((size_t)m->nfaces);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), dout, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, dout, (size_t)m->nfaces * 8);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "face jumps");
    double sum = 0.0;   // ascending face order (evaluate!, itemintegrator.jl:314-330)
    for (double v : h) sum += v;
    if (face_values) std::memcpy(face_values, h.data(), h.size() * 8);
    if (total) *total = sum;
    return GRMP_OK;
}
