// Matrices imported from a host CSC: the solve seam of the reference, where
// solve_direct! hands LinearSolve a SparseMatrixCSC{Float64,Int64} with the
// Dirichlet rows penalised (src/solvers.jl:89-101, :640-661) and fixpoint
// loops replace its values while keeping the pattern (:906-911, :1160-1165).
//
// The CSC arrays become the handle's CSR arrays: for a symmetric matrix the
// CSC of A is the CSR of A^T = A (the arrays are used as they are, the index
// base removed); otherwise the host transposes them once (counting sort by
// row) and keeps the position map, so value updates are a device gather.
//
// Penalty rows (a diagonal >= penalty_threshold, the reference's 1e60 rows)
// are taken out of the system the solvers see: the handle holds the
// eliminated matrix (penalty rows and columns zeroed, diagonal 1) in FP64 and
// rounded to FP32, and every solve maps the caller's right-hand side b to
//     b'_d = b_d / a_dd                      (penalty row d)
//     b'_i = b_i - sum_d a_id b'_d           (other rows, ascending entries)
// which gives the penalised system's solution up to O(1 / a_dd) relative
// (x_d = b_d / a_dd - sum_j a_dj x_j / a_dd).  The FP32 copy then never sees
// 1e60 (which overflows FP32), so the mixed and FP32-factor solvers apply.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "grmp_internal.h"

namespace {

constexpr int TPB = 256;
inline int nblk(long long n) { return (int)((n + TPB - 1) / TPB); }

__global__ void k_gather_f64(long long nnz, const int64_t *src, const double *in, double *out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) out[k] = in[src[k]];
}

// penalty flags and diagonal; counts the penalty rows
__global__ void k_pen_detect(int n, const int32_t *rowptr, const int32_t *cols, const double *orig, double thr,
                             uint8_t *flag, double *diag, int *count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (cols[k] == i) d = orig[k];
    diag[i] = d;
    const bool p = thr > 0.0 && d >= thr;
    flag[i] = p ? 1 : 0;
    if (p) atomicAdd(count, 1);
}

// eliminated FP64 values and their FP32 rounding
__global__ void k_pen_elim(int n, const int32_t *rowptr, const int32_t *cols, const double *orig, const uint8_t *flag,
                           double *v64, float *v32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool fi = flag[i] != 0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
        const int c = cols[k];
        double v = orig[k];
        if (fi || flag[c]) v = (c == i) ? 1.0 : 0.0;
        v64[k] = v;
        v32[k] = (float)v;
    }
}

__global__ void k_pen_rhs(int n, const int32_t *rowptr, const int32_t *cols, const double *orig, const uint8_t *flag,
                          const double *diag, const double *b, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flag[i]) {
        out[i] = b[i] / diag[i];
        return;
    }
    double s = b[i];
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
        const int c = cols[k];
        if (flag[c]) s -= orig[k] * (b[c] / diag[c]);
    }
    out[i] = s;
}

void free_import(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    const size_t n = (size_t)A->nrows, nz = (size_t)A->nnz;
    grmp_free(ctx, A->d_imp_orig, nz * 8);
    grmp_free(ctx, A->d_imp_src, A->d_imp_src ? nz * 8 : 0);
    grmp_free(ctx, A->d_imp_flag, n);
    grmp_free(ctx, A->d_imp_diag, n * 8);
    grmp_free(ctx, A->d_imp_b, n * 8);
    grmp_free(ctx, A->d_imp_count, 4);
    A->d_imp_orig = A->d_imp_diag = A->d_imp_b = nullptr;
    A->d_imp_src = nullptr;
    A->d_imp_flag = nullptr;
    A->d_imp_count = nullptr;
}

// values (in the handle's CSR order, on the device in d_imp_orig) -> penalty
// detection, eliminated FP64 / FP32 values
int refresh_values(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    cudaMemsetAsync(A->d_imp_count, 0, 4, ctx->stream);
    k_pen_detect<<<nblk(n), TPB, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_imp_orig, A->imp_threshold,
                                                   A->d_imp_flag, A->d_imp_diag, A->d_imp_count);
    GRMP_LAUNCHED(ctx);
    k_pen_elim<<<nblk(n), TPB, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_imp_orig, A->d_imp_flag,
                                                 A->d_vals64, A->d_vals32);
    GRMP_LAUNCHED(ctx);
    int cnt = 0;
    cudaError_t e = cudaMemcpyAsync(&cnt, A->d_imp_count, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "CSC import: value refresh");
    A->imp_npen = cnt;
    A->has64 = A->has32 = true;
    A->pack_fresh = A->duo_fresh = A->duo_sfresh = false;
    return GRMP_OK;
}

// upload caller values (CSC order) and bring them into CSR order
int load_values(grmp_matrix A, const double *nzval) {
    grmp_context ctx = A->space->mesh->ctx;
    const size_t nz = (size_t)A->nnz;
    if (!A->d_imp_src) {
        if (nz) GRMP_CUDA(ctx, cudaMemcpyAsync(A->d_imp_orig, nzval, nz * 8, cudaMemcpyHostToDevice, ctx->stream));
        GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the caller may free nzval on return
        return GRMP_OK;
    }
    double *tmp = nullptr;
    int rc = grmp_alloc(ctx, (void **)&tmp, nz * 8);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(tmp, nzval, nz * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        k_gather_f64<<<nblk((long long)nz), TPB, 0, ctx->stream>>>((long long)nz, A->d_imp_src, tmp, A->d_imp_orig);
        GRMP_LAUNCHED(ctx);
        e = cudaStreamSynchronize(ctx->stream);
    }
    grmp_free(ctx, tmp, nz * 8);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "CSC import: value upload");
    return GRMP_OK;
}

}  // namespace

// Right-hand side of the eliminated system for a solve (see the file header);
// returns the caller's vector itself when the matrix has no penalty rows.
int grmp_import_rhs(grmp_matrix A, grmp_vector b, grmp_vector_s *tmp, grmp_vector *out) {
    *out = b;
    if (!A->imported || A->imp_npen == 0) return GRMP_OK;
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    k_pen_rhs<<<nblk(n), TPB, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_imp_orig, A->d_imp_flag,
                                                A->d_imp_diag, b->d, A->d_imp_b);
    GRMP_LAUNCHED(ctx);
    GRMP_CUDA(ctx, cudaGetLastError());
    tmp->ctx = ctx;
    tmp->n = n;
    tmp->d = A->d_imp_b;
    *out = tmp;
    return GRMP_OK;
}

void grmp_import_free(grmp_matrix A) {
    if (A->imported) free_import(A);
}

extern "C" int grmp_matrix_from_csc(grmp_context ctx, int32_t n, const int64_t *colptr, const int64_t *rowval,
                                    const double *nzval, int index_base, int symmetric, double penalty_threshold,
                                    grmp_matrix *out) {
    if (!ctx || !ctx->stream || !out || n <= 0 || !colptr || (index_base != 0 && index_base != 1) ||
        !(penalty_threshold >= 0.0))
        return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    const int64_t nnz = colptr[n] - colptr[0];
    if (colptr[0] != index_base || nnz < 0 || nnz > (int64_t)INT32_MAX || (nnz > 0 && (!rowval || !nzval)))
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "CSC import: colptr[0] must be %d and the entry count fit 32 bits",
                         index_base);
    // validate: monotone column pointers, row indices in range and strictly increasing per column
    for (int j = 0; j < n; j++) {
        const int64_t b = colptr[j] - index_base, e = colptr[j + 1] - index_base;
        if (e < b || e > nnz) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "CSC import: colptr not monotone at %d", j);
        for (int64_t k = b; k < e; k++) {
            const int64_t r = rowval[k] - index_base;
            if (r < 0 || r >= n)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "CSC import: row index %lld out of range in column %d",
                                 (long long)rowval[k], j);
            if (k > b && r <= rowval[k - 1] - index_base)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG,
                                 "CSC import: row indices of column %d not strictly increasing", j);
        }
    }
    // CSR arrays (and the CSR -> CSC position map when transposing)
    std::vector<int32_t> rp((size_t)n + 1, 0), ci((size_t)nnz);
    std::vector<int64_t> src;
    if (symmetric) {
        for (int j = 0; j <= n; j++) rp[j] = (int32_t)(colptr[j] - index_base);
        for (int64_t k = 0; k < nnz; k++) ci[k] = (int32_t)(rowval[k] - index_base);
    } else {
        src.resize((size_t)nnz);
        for (int64_t k = 0; k < nnz; k++) rp[rowval[k] - index_base + 1]++;
        for (int i = 0; i < n; i++) rp[i + 1] += rp[i];
        std::vector<int32_t> fill(rp.begin(), rp.end() - 1);
        for (int j = 0; j < n; j++)   // columns ascending: each row receives its columns in order
            for (int64_t k = colptr[j] - index_base; k < colptr[j + 1] - index_base; k++) {
                const int32_t p = fill[rowval[k] - index_base]++;
                ci[p] = j;
                src[p] = k;
            }
    }
    cudaError_t se = cudaSetDevice(ctx->device);
    if (se != cudaSuccess) return grmp_cuda_fail(ctx, se, "CSC import: cudaSetDevice");
    std::lock_guard<std::mutex> lk(ctx->mu);
    // a matrix without an assembly space: a placeholder mesh / space carry the context
    grmp_mesh m = new (std::nothrow) grmp_mesh_s();
    grmp_space s = new (std::nothrow) grmp_space_s();
    grmp_matrix A = new (std::nothrow) grmp_matrix_s();
    if (!m || !s || !A) {
        delete m;
        delete s;
        delete A;
        return GRMP_ERR_OUT_OF_MEMORY;
    }
    m->ctx = ctx;
    s->mesh = m;
    s->ndofs = n;
    A->space = s;
    A->imported = true;
    A->nrows = n;
    A->nnz = nnz;
    A->imp_threshold = penalty_threshold;
    int mx = 0;
    for (int i = 0; i < n; i++) mx = std::max(mx, rp[i + 1] - rp[i]);
    A->max_row_nnz = mx;
    int rc = grmp_upload(ctx, &A->d_rowptr, rp.data(), rp.size());
    if (!rc) rc = grmp_upload(ctx, &A->d_cols, ci.data(), ci.size());
    if (!rc && !symmetric) rc = grmp_upload(ctx, &A->d_imp_src, src.data(), src.size());
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_vals64, (size_t)nnz * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_vals32, (size_t)nnz * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_imp_orig, (size_t)nnz * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_imp_flag, (size_t)n);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_imp_diag, (size_t)n * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_imp_b, (size_t)n * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_imp_count, 4);
    if (!rc) rc = load_values(A, nzval);
    if (!rc) rc = refresh_values(A);
    if (rc) {
        grmp_matrix_destroy(A);
        return rc;
    }
    *out = A;
    return GRMP_OK;
}

extern "C" int grmp_matrix_update_values(grmp_matrix A, const double *nzval) {
    if (!A || (!nzval && A->nnz > 0)) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    if (!A->imported) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "update values: the matrix was not imported from a CSC");
    cudaError_t se = cudaSetDevice(ctx->device);
    if (se != cudaSuccess) return grmp_cuda_fail(ctx, se, "update values: cudaSetDevice");
    std::lock_guard<std::mutex> lk(ctx->mu);
    int rc = load_values(A, nzval);
    if (!rc) rc = refresh_values(A);
    return rc;
}

extern "C" int grmp_matrix_penalty_rows(grmp_matrix A, int32_t *count) {
    if (!A || !count) return GRMP_ERR_INVALID_ARG;
    *count = A->imported ? A->imp_npen : 0;
    return GRMP_OK;
}
