// Sparsity pattern construction: DoF->cell incidence, the drop-exact-zero
// mask and CSR rows with a cell-to-slot map.
//
// Reference behaviour being reproduced: FEMatrix entries are created by
// _addnz (src/fematrix.jl:54-65), which skips any local contribution that is
// exactly 0.0.  Whether a contribution is exactly zero depends on the
// operation order, so the mask kernel evaluates the local matrices in the
// order of src/feevaluator_h1.jl:61-131 (operator values) and
// src/assemblypatterns/bilinearform.jl:180-210, :281-346 (quadrature loop,
// action, scatter) with explicitly rounded FP64 operations (no FMA).
#include <algorithm>

#include "element.cuh"
#include "grmp_internal.h"

namespace {

constexpr int TPB = 256;

inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// ------------------------------------------------------------------ scan
__global__ void k_block_sums(const int32_t *in, int32_t n, int32_t *bsum) {
    __shared__ int32_t sh[1024];
    int32_t v = 0;
    for (int k = 0; k < 4; k++) {
        int idx = blockIdx.x * 4096 + k * 1024 + threadIdx.x;
        if (idx < n) v += in[idx];
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = sh[0];
}

// exclusive scan of the block sums by one block (any count, sequential chunks)
__global__ void k_scan_small(int32_t *a, int32_t n, int32_t *total) {
    __shared__ int32_t sh[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        int idx = base + threadIdx.x;
        int32_t v = idx < n ? a[idx] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            int32_t t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (idx < n) a[idx] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_blocks(const int32_t *in, int32_t *out, int32_t n, const int32_t *boff) {
    __shared__ int32_t sh[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = boff[blockIdx.x];
    __syncthreads();
    for (int k = 0; k < 4; k++) {
        int idx = blockIdx.x * 4096 + k * 1024 + threadIdx.x;
        int32_t v = idx < n ? in[idx] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            int32_t t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (idx < n) out[idx] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
}

// ------------------------------------------------------------------ incidence
__global__ void k_inc_count(const int32_t *celldofs, long long n, int32_t *cnt) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&cnt[celldofs[i]], 1);
}

__global__ void k_inc_fill(const int32_t *celldofs, long long n, int ldofs, const int32_t *ptr, int32_t *cursor,
                           int32_t *inc_cell, uint8_t *inc_loc) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t d = celldofs[i];
    int32_t pos = ptr[d] + atomicAdd(&cursor[d], 1);
    inc_cell[pos] = (int32_t)(i / ldofs);
    inc_loc[pos] = (uint8_t)(i % ldofs);
}

// sort each DoF's incidence list by (cell, local) -- fixed order, run to run
__global__ void k_inc_sort(int32_t ndofs, const int32_t *ptr, int32_t *inc_cell, uint8_t *inc_loc) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndofs) return;
    int b = ptr[d], e = ptr[d + 1];
    for (int i = b + 1; i < e; i++) {
        int32_t c = inc_cell[i];
        uint8_t l = inc_loc[i];
        int j = i - 1;
        while (j >= b && (inc_cell[j] > c || (inc_cell[j] == c && inc_loc[j] > l))) {
            inc_cell[j + 1] = inc_cell[j];
            inc_loc[j + 1] = inc_loc[j];
            j--;
        }
        inc_cell[j + 1] = c;
        inc_loc[j + 1] = l;
    }
}

// ------------------------------------------------------------------ reference-order local matrices
enum { OPV_IDENTITY = 0, OPV_GRADIENT = 1, OPV_SYMGRAD = 2 };

// cv[q][dof][k] for H1 elements (scalar basis nb, nc components), explicitly
// rounded: src/feevaluator_h1.jl:61-116.
template <int DIM, int NB, int NC>
__device__ void ref_cvals(int opv, const TablesDev &tb, const double G[3][3], double cv[][NB * NC][DIM * NC]) {
    constexpr int LD = NB * NC;
    constexpr int RD = DIM * NC;
    for (int q = 0; q < tb.nq; q++)
        for (int dof = 0; dof < LD; dof++) {
            for (int k = 0; k < RD; k++) cv[q][dof][k] = 0.0;
            int c = dof / NB, a = dof % NB;
            if (opv == OPV_IDENTITY) {
                cv[q][dof][c] = tb.vals[q * tb.nb + a];
            } else if (opv == OPV_GRADIENT) {
                for (int k = 0; k < DIM; k++) {
                    double s = 0.0;
                    for (int j = 0; j < DIM; j++)
                        s = __dadd_rn(s, __dmul_rn(G[k][j], tb.derivs[(q * tb.nb + a) * DIM + j]));
                    cv[q][dof][k + c * DIM] = s;
                }
            } else {  // symmetric gradient (Voigt), off-diagonal weight 1
                for (int k = 0; k < DIM; k++) {
                    int t = voigt_slot(DIM, c, k);
                    double s = cv[q][dof][t];
                    for (int j = 0; j < DIM; j++)
                        s = __dadd_rn(s, __dmul_rn(G[k][j], tb.derivs[(q * tb.nb + a) * DIM + j]));
                    cv[q][dof][t] = s;
                }
            }
        }
}

template <int DIM, int NB, int NC>
__device__ void ref_action(const TermDev &t, int cell, const double *in, double *res, int rdim) {
    if (t.op == GRMP_OP_HOOKE) {
        double l = t.lambda, m = t.mu;
        double l2m = __dadd_rn(l, __dmul_rn(2.0, m));
        if (DIM == 2) {
            res[0] = __dadd_rn(__dmul_rn(l2m, in[0]), __dmul_rn(l, in[1]));
            res[1] = __dadd_rn(__dmul_rn(l2m, in[1]), __dmul_rn(l, in[0]));
            res[2] = __dmul_rn(m, in[2]);
        } else {
            res[0] = __dadd_rn(__dmul_rn(l2m, in[0]), __dmul_rn(l, __dadd_rn(in[1], in[2])));
            res[1] = __dadd_rn(__dmul_rn(l2m, in[1]), __dmul_rn(l, __dadd_rn(in[0], in[2])));
            res[2] = __dadd_rn(__dmul_rn(l2m, in[2]), __dmul_rn(l, __dadd_rn(in[0], in[1])));
            res[3] = __dmul_rn(m, in[3]);
            res[4] = __dmul_rn(m, in[4]);
            res[5] = __dmul_rn(m, in[5]);
        }
        return;
    }
    if (t.cell_coef) {
        double c = t.cell_coef[cell];
        for (int k = 0; k < rdim; k++) res[k] = __dmul_rn(c, in[k]);
    } else {
        for (int k = 0; k < rdim; k++) res[k] = in[k];
    }
}

// Nonzero mask of the summed local matrices: mask[cell*LD + i] bit j set when
// some term's local contribution (i, j) is not exactly zero.
template <int DIM, int NB, int NC>
__global__ void k_nzmask(int ncells, const double *coords, const int32_t *cells, TermsDev terms, uint32_t *mask) {
    constexpr int LD = NB * NC;
    constexpr int RD = DIM * NC;
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[4 * 3];
    for (int v = 0; v <= DIM; v++)
        for (int k = 0; k < DIM; k++) X[v * DIM + k] = coords[(size_t)cells[(size_t)cell * (DIM + 1) + v] * DIM + k];
    double A[3][3], G[3][3], vol;
    simplex_geometry_rn<DIM>(X, A, G, vol);
    uint32_t m[LD];
    for (int i = 0; i < LD; i++) m[i] = 0;
    double cv[16][LD][RD];
    for (int ti = 0; ti < terms.n; ti++) {
        const TermDev &t = terms.t[ti];
        if (t.op == GRMP_OP_STRUCTURAL || t.op == GRMP_OP_JUMPGRAD) {   // every local pair
            for (int i = 0; i < LD; i++) m[i] = LD >= 32 ? ~0u : ((1u << LD) - 1u);
            continue;
        }
        int opv = t.op == GRMP_OP_MASS ? OPV_IDENTITY : (t.op == GRMP_OP_LAPLACE ? OPV_GRADIENT : OPV_SYMGRAD);
        int rdim = opv == OPV_IDENTITY ? NC : (opv == OPV_GRADIENT ? DIM * NC : (DIM == 2 ? 3 : 6));
        ref_cvals<DIM, NB, NC>(opv, t.tab, G, cv);
        double itemfactor = __dmul_rn(vol, t.factor);
        for (int i = 0; i < LD; i++) {
            for (int j = (t.symmetric ? i : 0); j < LD; j++) {
                double loc = 0.0;
                for (int q = 0; q < t.tab.nq; q++) {
                    double res[9];
                    ref_action<DIM, NB, NC>(t, cell, cv[q][i], res, rdim);
                    double tt = 0.0;
                    for (int k = 0; k < rdim; k++) tt = __dadd_rn(tt, __dmul_rn(res[k], cv[q][j][k]));
                    loc = __dadd_rn(loc, __dmul_rn(t.tab.w[q], tt));
                }
                if (__dmul_rn(loc, itemfactor) != 0.0) {
                    m[i] |= 1u << j;
                    if (t.symmetric) m[j] |= 1u << i;
                }
            }
        }
    }
    for (int i = 0; i < LD; i++) mask[(size_t)cell * LD + i] = m[i];
}

// ------------------------------------------------------------------ rows
// Sorted unique column list of one row from its incidences and the mask.
// With face terms (nbr != nullptr) the row also holds every DoF of the cells
// across the faces of its cells.
__device__ __forceinline__ bool list_insert(int32_t *list, int &n, int32_t col, int *overflow) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (list[mid] < col) lo = mid + 1; else hi = mid;
    }
    if (lo < n && list[lo] == col) return true;
    if (n >= GRMP_MAX_ROW_NNZ) {
        *overflow = 1;
        return false;
    }
    for (int k = n; k > lo; k--) list[k] = list[k - 1];
    list[lo] = col;
    n++;
    return true;
}

__device__ int row_columns(int row, const int32_t *inc_ptr, const int32_t *inc_cell, const uint8_t *inc_loc,
                           const uint32_t *mask, const int32_t *celldofs, int ld, const int32_t *nbr, int nf,
                           int32_t *list, int *overflow) {
    int n = 0;
    if (nbr)
        for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++)
            for (int f = 0; f < nf; f++) {
                const int c2 = nbr[(size_t)inc_cell[p] * nf + f];
                if (c2 < 0) continue;
                for (int b = 0; b < ld; b++)
                    if (!list_insert(list, n, celldofs[(size_t)c2 * ld + b], overflow)) return n;
            }
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) {
        int cell = inc_cell[p], a = inc_loc[p];
        uint32_t bits = mask[(size_t)cell * ld + a];
        while (bits) {
            int b = __ffs(bits) - 1;
            bits &= bits - 1;
            int32_t col = celldofs[(size_t)cell * ld + b];
            // insertion into the sorted list
            int lo = 0, hi = n;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (list[mid] < col) lo = mid + 1; else hi = mid;
            }
            if (lo < n && list[lo] == col) continue;
            if (n >= GRMP_MAX_ROW_NNZ) {
                *overflow = 1;
                return n;
            }
            for (int k = n; k > lo; k--) list[k] = list[k - 1];
            list[lo] = col;
            n++;
        }
    }
    return n;
}

__global__ void k_row_count(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell, const uint8_t *inc_loc,
                            const uint32_t *mask, const int32_t *celldofs, int ld, const int32_t *nbr, int nf,
                            int32_t *cnt, int32_t *maxcnt, int *overflow) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    int32_t list[GRMP_MAX_ROW_NNZ];
    int n = row_columns(row, inc_ptr, inc_cell, inc_loc, mask, celldofs, ld, nbr, nf, list, overflow);
    cnt[row] = n;
    atomicMax(maxcnt, n);
}

template <typename S>
__global__ void k_row_fill(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell, const uint8_t *inc_loc,
                           const uint32_t *mask, const int32_t *celldofs, int ld, const int32_t *nbr, int nf,
                           const int32_t *rowptr, int32_t *cols, S *slot, int *overflow) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    int32_t list[GRMP_MAX_ROW_NNZ];
    int n = row_columns(row, inc_ptr, inc_cell, inc_loc, mask, celldofs, ld, nbr, nf, list, overflow);
    int32_t base = rowptr[row];
    for (int k = 0; k < n; k++) cols[base + k] = list[k];
    const S DROP = (S)~(S)0;
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) {
        int cell = inc_cell[p], a = inc_loc[p];
        uint32_t bits = mask[(size_t)cell * ld + a];
        for (int b = 0; b < ld; b++) {
            S s = DROP;
            if (bits & (1u << b)) {
                int32_t col = celldofs[(size_t)cell * ld + b];
                int lo = 0, hi = n;
                while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (list[mid] < col) lo = mid + 1; else hi = mid;
                }
                s = (S)lo;
            }
            slot[(size_t)p * ld + b] = s;
        }
    }
}

__global__ void k_fill_f64(double *v, long long n, double val) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) v[i] = val;
}

template <int DIM, int NB, int NC>
void launch_mask(grmp_space s, const TermsDev &td, uint32_t *mask) {
    grmp_mesh m = s->mesh;
    k_nzmask<DIM, NB, NC><<<nblk(m->ncells, 128), 128, 0, m->ctx->stream>>>(m->ncells, m->d_coords, m->d_cells, td, mask);
    GRMP_LAUNCHED(m->ctx);
}

}  // namespace

// ---------------------------------------------------------------------- scan
int grmp_scan_i32(grmp_context ctx, const int32_t *d_in, int32_t *d_out, int32_t n, int32_t *total) {
    int nb = (n + 4095) / 4096;
    if (nb < 1) nb = 1;
    int32_t *bsum = nullptr, *dtot = nullptr;
    int rc = grmp_alloc(ctx, (void **)&bsum, (size_t)nb * 4);
    if (rc) return rc;
    rc = grmp_alloc(ctx, (void **)&dtot, 4);
    if (rc) {
        grmp_free(ctx, bsum, (size_t)nb * 4);
        return rc;
    }
    k_block_sums<<<nb, 1024, 0, ctx->stream>>>(d_in, n, bsum); GRMP_LAUNCHED(ctx);
    k_scan_small<<<1, 1024, 0, ctx->stream>>>(bsum, nb, dtot); GRMP_LAUNCHED(ctx);
    k_scan_blocks<<<nb, 1024, 0, ctx->stream>>>(d_in, d_out, n, bsum); GRMP_LAUNCHED(ctx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && total) e = cudaMemcpyAsync(total, dtot, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, bsum, (size_t)nb * 4);
    grmp_free(ctx, dtot, 4);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "scan");
    return GRMP_OK;
}

// ---------------------------------------------------------------------- incidence
int grmp_build_incidence(grmp_space s) {
    grmp_context ctx = s->mesh->ctx;
    long long n = (long long)s->mesh->ncells * s->ldofs;
    int32_t *cnt = nullptr;
    int rc = grmp_alloc(ctx, (void **)&cnt, ((size_t)s->ndofs + 1) * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&s->d_inc_ptr, ((size_t)s->ndofs + 1) * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&s->d_inc_cell, (size_t)n * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&s->d_inc_loc, (size_t)n);
    if (rc) {
        grmp_free(ctx, cnt, ((size_t)s->ndofs + 1) * 4);
        return rc;
    }
    cudaMemsetAsync(cnt, 0, ((size_t)s->ndofs + 1) * 4, ctx->stream);
    k_inc_count<<<nblk(n), TPB, 0, ctx->stream>>>(s->d_celldofs, n, cnt); GRMP_LAUNCHED(ctx);
    int32_t total = 0;
    rc = grmp_scan_i32(ctx, cnt, s->d_inc_ptr, s->ndofs + 1, &total);
    if (!rc && total != n) rc = grmp_fail(ctx, GRMP_ERR_DEVICE, "incidence: count %d != %lld", total, n);
    if (!rc) {
        cudaMemsetAsync(cnt, 0, ((size_t)s->ndofs + 1) * 4, ctx->stream);
        k_inc_fill<<<nblk(n), TPB, 0, ctx->stream>>>(s->d_celldofs, n, s->ldofs, s->d_inc_ptr, cnt, s->d_inc_cell,
                                                      s->d_inc_loc); GRMP_LAUNCHED(ctx);
        k_inc_sort<<<nblk(s->ndofs), TPB, 0, ctx->stream>>>(s->ndofs, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc); GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "incidence kernels");
    }
    grmp_free(ctx, cnt, ((size_t)s->ndofs + 1) * 4);
    return rc;
}

// ---------------------------------------------------------------------- terms
int grmp_br_mask(grmp_space s, int nterms, const grmp_bilinear_term *terms, uint32_t *mask);

// Host helper shared with assemble.cu: validate terms and upload the tables
// they need.  Returns device tables in `keep` (freed by the caller).
int grmp_prepare_terms(grmp_space s, int nterms, const grmp_bilinear_term *terms, TermsDev *td,
                       std::vector<std::pair<void *, size_t>> &keep) {
    grmp_context ctx = s->mesh->ctx;
    int dim = s->mesh->dim;
    if (s->fe != GRMP_FE_H1P1 && s->fe != GRMP_FE_H1P2)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED,
                         "bilinear terms on element %d are not built here (H1BR has its own path)", s->fe);
    td->n = nterms;
    for (int i = 0; i < nterms; i++) {
        const grmp_bilinear_term &t = terms[i];
        TermDev &d = td->t[i];
        d.op = t.op_kind;
        d.symmetric = t.symmetric ? 1 : 0;
        d.factor = t.factor;
        d.mu = t.param[0];
        d.lambda = t.param[1];
        d.cell_coef = nullptr;
        int deriv;
        if (t.op_kind == GRMP_OP_LAPLACE || t.op_kind == GRMP_OP_JUMPGRAD) deriv = 1;
        else if (t.op_kind == GRMP_OP_MASS || t.op_kind == GRMP_OP_STRUCTURAL) deriv = 0;
        else if (t.op_kind == GRMP_OP_HOOKE) {
            deriv = 1;
            if (s->ncomp != dim)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "Hooke operator needs ncomponents == dim");
            if (t.cell_coef) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "Hooke operator takes no per-cell coefficient");
        } else
            return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "operator %d not available on H1 elements", t.op_kind);
        int order = t.bonus_quadorder + 2 * (grmp_fe_polyorder(s->fe, dim) - deriv);
        if (order < 0) order = 0;
        RefTables *rt = new RefTables;
        int rc = grmp_tables(dim, s->fe, order, rt);
        if (rc || rt->nq > 16) {
            delete rt;
            return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no quadrature rule of order %d in %dD", order, dim);
        }
        int nq = rt->nq, nb = rt->nb;
        std::vector<double> buf(nq + 3 * nq + nq * nb + nq * nb * dim);
        double *w = buf.data(), *x = w + nq, *v = x + 3 * nq, *dv = v + nq * nb;
        for (int q = 0; q < nq; q++) {
            w[q] = rt->w[q];
            for (int k = 0; k < 3; k++) x[3 * q + k] = rt->xref[q][k];
            for (int a = 0; a < nb; a++) {
                v[q * nb + a] = rt->vals[q][a];
                for (int j = 0; j < dim; j++) dv[(q * nb + a) * dim + j] = rt->derivs[q][a][j];
            }
        }
        delete rt;
        double *dbuf = nullptr;
        rc = grmp_upload(ctx, &dbuf, buf.data(), buf.size());
        if (rc) return rc;
        keep.push_back({dbuf, buf.size() * 8});
        d.tab.nq = nq;
        d.tab.nb = nb;
        d.tab.dim = dim;
        d.tab.w = dbuf;
        d.tab.xref = dbuf + nq;
        d.tab.vals = dbuf + 4 * nq;
        d.tab.derivs = dbuf + 4 * nq + nq * nb;
        if (t.cell_coef && t.coef_on_device) {
            cudaPointerAttributes pa;
            if (cudaPointerGetAttributes(&pa, t.cell_coef) != cudaSuccess || pa.type != cudaMemoryTypeDevice ||
                pa.device != ctx->device) {
                cudaGetLastError();
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "cell_coef is not device memory of this context's GPU");
            }
            d.cell_coef = t.cell_coef;
        } else if (t.cell_coef) {
            double *dc = nullptr;
            rc = grmp_upload(ctx, &dc, t.cell_coef, (size_t)s->mesh->ncells);
            if (rc) return rc;
            keep.push_back({dc, (size_t)s->mesh->ncells * 8});
            d.cell_coef = dc;
        }
    }
    return GRMP_OK;
}

void grmp_release(grmp_context ctx, std::vector<std::pair<void *, size_t>> &keep) {
    for (auto &p : keep) grmp_free(ctx, p.first, p.second);
    keep.clear();
}

int grmp_pattern_build_impl(grmp_space s, int nterms, const grmp_bilinear_term *terms, grmp_matrix *out) {
    grmp_context ctx = s->mesh->ctx;
    int dim = s->mesh->dim, nb = s->nb, nc = s->ncomp, ld = s->ldofs;
    *out = nullptr;
    TermsDev td;
    std::vector<std::pair<void *, size_t>> keep;
    size_t ncl = (size_t)s->mesh->ncells * ld;
    uint32_t *mask = nullptr;
    int rc = grmp_alloc(ctx, (void **)&mask, ncl * 4);
    if (rc) return rc;
    bool launched = true;
    if (s->fe == GRMP_FE_H1BR) {
        rc = grmp_br_mask(s, nterms, terms, mask);
        if (rc) {
            grmp_free(ctx, mask, ncl * 4);
            return rc;
        }
    } else {
        rc = grmp_prepare_terms(s, nterms, terms, &td, keep);
        if (rc) {
            grmp_free(ctx, mask, ncl * 4);
            grmp_release(ctx, keep);
            return rc;
        }
    }
    if (s->fe == GRMP_FE_H1BR) launched = true;
    else if (dim == 2 && nb == 3 && nc == 1) launch_mask<2, 3, 1>(s, td, mask);
    else if (dim == 2 && nb == 3 && nc == 2) launch_mask<2, 3, 2>(s, td, mask);
    else if (dim == 2 && nb == 6 && nc == 1) launch_mask<2, 6, 1>(s, td, mask);
    else if (dim == 2 && nb == 6 && nc == 2) launch_mask<2, 6, 2>(s, td, mask);
    else if (dim == 3 && nb == 4 && nc == 1) launch_mask<3, 4, 1>(s, td, mask);
    else if (dim == 3 && nb == 4 && nc == 3) launch_mask<3, 4, 3>(s, td, mask);
    else if (dim == 3 && nb == 10 && nc == 1) launch_mask<3, 10, 1>(s, td, mask);
    else if (dim == 3 && nb == 10 && nc == 3) launch_mask<3, 10, 3>(s, td, mask);
    else launched = false;
    if (!launched) {
        grmp_free(ctx, mask, ncl * 4);
        grmp_release(ctx, keep);
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "pattern: element layout dim=%d nb=%d nc=%d", dim, nb, nc);
    }
    // face terms couple the DoFs of face neighbours
    const int32_t *nbr = nullptr;
    bool faces = false;
    for (int i = 0; i < nterms; i++) faces = faces || terms[i].op_kind == GRMP_OP_JUMPGRAD;
    if (faces) {
        if (s->fe == GRMP_FE_H1BR || s->ncomp != 1) rc = grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "face terms: scalar H1P1 / H1P2");
        if (!rc) rc = grmp_mesh_neighbors(s->mesh);
        if (rc) {
            grmp_free(ctx, mask, ncl * 4);
            grmp_release(ctx, keep);
            return rc;
        }
        nbr = s->mesh->d_cell_nbr;
    }
    grmp_matrix A = new grmp_matrix_s();
    A->space = s;
    A->nrows = s->ndofs;
    int32_t *cnt = nullptr, *dmax = nullptr;
    int *dovf = nullptr;
    rc = grmp_alloc(ctx, (void **)&cnt, ((size_t)A->nrows + 1) * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&dmax, 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&dovf, 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_rowptr, ((size_t)A->nrows + 1) * 4);
    int32_t total = 0, hmax = 0;
    int hovf = 0;
    if (!rc) {
        cudaMemsetAsync(cnt, 0, ((size_t)A->nrows + 1) * 4, ctx->stream);
        cudaMemsetAsync(dmax, 0, 4, ctx->stream);
        cudaMemsetAsync(dovf, 0, 4, ctx->stream);
        k_row_count<<<nblk(A->nrows, 128), 128, 0, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc,
                                                                 mask, s->d_celldofs, ld, nbr, dim + 1, cnt, dmax,
                                                                 dovf);
        GRMP_LAUNCHED(ctx);
        rc = grmp_scan_i32(ctx, cnt, A->d_rowptr, A->nrows + 1, &total);
    }
    if (!rc) {
        cudaMemcpyAsync(&hmax, dmax, 4, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(&hovf, dovf, 4, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "pattern count");
        else if (hovf) rc = grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "pattern: a row has more than %d nonzeros", GRMP_MAX_ROW_NNZ);
    }
    if (!rc) {
        A->nnz = total;
        A->max_row_nnz = hmax;
        A->slot_bytes = hmax < 255 ? 1 : 2;
        rc = grmp_alloc(ctx, (void **)&A->d_cols, (size_t)total * 4);
        if (!rc) rc = grmp_alloc(ctx, &A->d_slot, ncl * ld * A->slot_bytes);   // ld slots per incidence
    }
    if (!rc) {
        if (A->slot_bytes == 1)
            k_row_fill<uint8_t><<<nblk(A->nrows, 128), 128, 0, ctx->stream>>>(
                A->nrows, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc, mask, s->d_celldofs, ld, nbr, dim + 1,
                A->d_rowptr, A->d_cols, (uint8_t *)A->d_slot, dovf);
        else
            k_row_fill<uint16_t><<<nblk(A->nrows, 128), 128, 0, ctx->stream>>>(
                A->nrows, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc, mask, s->d_celldofs, ld, nbr, dim + 1,
                A->d_rowptr, A->d_cols, (uint16_t *)A->d_slot, dovf);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "pattern fill");
    }
    grmp_free(ctx, cnt, ((size_t)A->nrows + 1) * 4);
    grmp_free(ctx, dmax, 4);
    grmp_free(ctx, dovf, 4);
    grmp_free(ctx, mask, ncl * 4);
    grmp_release(ctx, keep);
    if (rc) {
        grmp_matrix_destroy(A);
        return rc;
    }
    *out = A;
    return GRMP_OK;
}

extern "C" int grmp_matrix_destroy(grmp_matrix A) {
    if (!A) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    cudaSetDevice(ctx->device);
    size_t ncl = (size_t)A->space->mesh->ncells * A->space->ldofs;
    grmp_free(ctx, A->d_rowptr, ((size_t)A->nrows + 1) * 4);
    grmp_free(ctx, A->d_cols, (size_t)A->nnz * 4);
    grmp_free(ctx, A->d_slot, ncl * A->space->ldofs * A->slot_bytes);
    grmp_free(ctx, A->d_vals64, (size_t)A->nnz * 8);
    grmp_free(ctx, A->d_vals32, (size_t)A->nnz * 4);
    grmp_free(ctx, A->d_pack32, (size_t)A->nnz * 8);
    grmp_free(ctx, A->d_stg_row0, ((size_t)A->stg_nwin + 1) * 4);
    grmp_free(ctx, A->d_stg_rec, A->stg_rec_bytes);
    grmp_duo_free(A);
    grmp_free(ctx, A->d_fixed, (size_t)A->nrows);
    grmp_free(ctx, A->d_work, A->work_bytes);
    grmp_free(ctx, A->d_cellfac, A->cellfac_bytes);
    grmp_direct_cache_free(A);
    grmp_mf_cache_free(A);
    grmp_import_free(A);
    cudaStreamSynchronize(ctx->stream);
    if (A->imported) {   // the placeholder mesh / space of a CSC import belong to the matrix
        delete A->space->mesh;
        delete A->space;
    }
    delete A;
    return GRMP_OK;
}

__global__ void k_rowptr64(const int32_t *rp, int64_t *out, int32_t n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) out[i] = rp[i];
}

__global__ void k_f32_to_f64(const float *a, double *b, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

extern "C" int grmp_matrix_download(grmp_matrix A, int precision, int64_t *rowptr, int32_t *cols, double *vals) {
    if (!A) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (rowptr) {
        int64_t *d = nullptr;
        int rc = grmp_alloc(ctx, (void **)&d, ((size_t)A->nrows + 1) * 8);
        if (rc) return rc;
        k_rowptr64<<<nblk(A->nrows + 1), TPB, 0, ctx->stream>>>(A->d_rowptr, d, A->nrows); GRMP_LAUNCHED(ctx);
        cudaMemcpyAsync(rowptr, d, ((size_t)A->nrows + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        grmp_free(ctx, d, ((size_t)A->nrows + 1) * 8);
    }
    if (cols) GRMP_CUDA(ctx, cudaMemcpyAsync(cols, A->d_cols, (size_t)A->nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (vals) {
        if (precision == GRMP_FP64) {
            if (!A->has64) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "no FP64 values assembled");
            GRMP_CUDA(ctx, cudaMemcpyAsync(vals, A->d_vals64, (size_t)A->nnz * 8, cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            if (!A->has32) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "no FP32 values assembled");
            double *d = nullptr;
            int rc = grmp_alloc(ctx, (void **)&d, (size_t)A->nnz * 8);
            if (rc) return rc;
            k_f32_to_f64<<<nblk(A->nnz), TPB, 0, ctx->stream>>>(A->d_vals32, d, A->nnz); GRMP_LAUNCHED(ctx);
            cudaMemcpyAsync(vals, d, (size_t)A->nnz * 8, cudaMemcpyDeviceToHost, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
            grmp_free(ctx, d, (size_t)A->nnz * 8);
        }
    }
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GRMP_OK;
}

extern "C" int grmp_vector_fill(grmp_vector v, double value) {
    if (!v) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(v->ctx->device);
    k_fill_f64<<<nblk(v->n), TPB, 0, v->ctx->stream>>>(v->d, v->n, value); GRMP_LAUNCHED(v->ctx);
    GRMP_CUDA(v->ctx, cudaGetLastError());
    GRMP_CUDA(v->ctx, cudaStreamSynchronize(v->ctx->stream));
    return GRMP_OK;
}
