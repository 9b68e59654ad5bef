// C-ABI entry points: contexts, meshes, spaces, vectors and the thin
// wrappers around the pattern / assembly / solve implementations.
#include <cstdarg>
#include <new>

#include "grmp_internal.h"

namespace {
bool valid_ctx(grmp_context c) { return c != nullptr && c->stream != nullptr; }
}  // namespace

int grmp_fail(grmp_context ctx, int code, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

int grmp_cuda_fail(grmp_context ctx, cudaError_t e, const char *what) {
    int code = (e == cudaErrorMemoryAllocation) ? GRMP_ERR_OUT_OF_MEMORY : GRMP_ERR_DEVICE;
    return grmp_fail(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

int grmp_alloc(grmp_context ctx, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return GRMP_OK;
    if (ctx->budget && ctx->in_use + bytes > ctx->budget)
        return grmp_fail(ctx, GRMP_ERR_BUDGET, "allocation of %zu bytes exceeds the HBM budget (%zu of %zu in use)",
                         bytes, ctx->in_use, ctx->budget);
    cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        return grmp_cuda_fail(ctx, e, "cudaMallocAsync");
    }
    ctx->in_use += bytes;
    return GRMP_OK;
}

void grmp_free(grmp_context ctx, void *p, size_t bytes) {
    if (!p) return;
    cudaFreeAsync(p, ctx->stream);
    ctx->in_use -= bytes;
}

extern "C" {

int grmp_version(void) { return 10000; }

int grmp_create_context(int device, size_t hbm_budget_bytes, grmp_context *out) {
    if (!out) return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GRMP_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) return GRMP_ERR_INVALID_ARG;
    grmp_context c = new (std::nothrow) grmp_context_s();
    if (!c) return GRMP_ERR_OUT_OF_MEMORY;
    c->device = device;
    c->budget = hbm_budget_bytes;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return GRMP_ERR_DEVICE;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    // keep freed blocks in the stream-ordered pool instead of returning them to the driver
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = c;
    return GRMP_OK;
}

int grmp_destroy_context(grmp_context ctx) {
    if (!valid_ctx(ctx)) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GRMP_OK;
}

const char *grmp_last_error(grmp_context ctx) {
    if (!ctx) return "invalid context";
    return ctx->last_error.c_str();
}

int grmp_context_stream(grmp_context ctx, void **stream) {
    if (!valid_ctx(ctx) || !stream) return GRMP_ERR_INVALID_ARG;
    *stream = (void *)ctx->stream;
    return GRMP_OK;
}

int grmp_synchronize(grmp_context ctx) {
    if (!valid_ctx(ctx)) return GRMP_ERR_INVALID_ARG;
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GRMP_OK;
}

int grmp_context_memory(grmp_context ctx, size_t *bytes) {
    if (!valid_ctx(ctx) || !bytes) return GRMP_ERR_INVALID_ARG;
    *bytes = ctx->in_use;
    return GRMP_OK;
}

int grmp_context_launches(grmp_context ctx, uint64_t *launches) {
    if (!valid_ctx(ctx) || !launches) return GRMP_ERR_INVALID_ARG;
    *launches = ctx->launches.load();
    return GRMP_OK;
}

int grmp_context_set_wait_limit(grmp_context ctx, int64_t polls) {
    if (!valid_ctx(ctx) || polls < 0) return GRMP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->wait_limit = polls > 0 ? (long long)polls : GRMP_SPIN_LIMIT;
    return GRMP_OK;
}

int grmp_vector_device_ptr(grmp_vector v, void **dptr) {
    if (!v || !dptr) return GRMP_ERR_INVALID_ARG;
    *dptr = (void *)v->d;
    return GRMP_OK;
}

// ---------------------------------------------------------------- mesh
int grmp_mesh_upload(grmp_context ctx, int dim, int32_t nverts, const double *coords, int32_t ncells,
                     const int32_t *cell_verts, grmp_mesh *out) {
    if (!valid_ctx(ctx) || !out || !coords || !cell_verts) return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    if ((dim != 2 && dim != 3) || nverts <= 0 || ncells <= 0)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "mesh: dim=%d nverts=%d ncells=%d", dim, nverts, ncells);
    for (int64_t i = 0; i < (int64_t)ncells * (dim + 1); i++)
        if (cell_verts[i] < 0 || cell_verts[i] >= nverts)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "mesh: cell vertex index %d out of range", cell_verts[i]);
    cudaSetDevice(ctx->device);
    grmp_mesh m = new (std::nothrow) grmp_mesh_s();
    if (!m) return GRMP_ERR_OUT_OF_MEMORY;
    m->ctx = ctx;
    m->dim = dim;
    m->nverts = nverts;
    m->ncells = ncells;
    int rc = grmp_upload(ctx, &m->d_coords, coords, (size_t)nverts * dim);
    if (!rc) rc = grmp_upload(ctx, &m->d_cells, cell_verts, (size_t)ncells * (dim + 1));
    if (!rc) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GRMP_OK : GRMP_ERR_DEVICE;
    if (rc) {
        grmp_mesh_destroy(m);
        return rc;
    }
    *out = m;
    return GRMP_OK;
}

int grmp_mesh_set_faces(grmp_mesh m, int32_t nfaces, const int32_t *cell_faces, const double *face_normals,
                        const double *face_volumes, const int8_t *cell_face_signs) {
    if (!m || !cell_faces || !face_normals || !face_volumes || !cell_face_signs || nfaces <= 0)
        return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = m->ctx;
    size_t nl = (size_t)m->ncells * (m->dim + 1);
    for (size_t i = 0; i < nl; i++)
        if (cell_faces[i] < 0 || cell_faces[i] >= nfaces)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "mesh faces: index %d out of range", cell_faces[i]);
    cudaSetDevice(ctx->device);
    grmp_free(ctx, m->d_cell_faces, nl * 4);
    grmp_free(ctx, m->d_face_normals, (size_t)m->nfaces * m->dim * 8);
    grmp_free(ctx, m->d_face_volumes, (size_t)m->nfaces * 8);
    grmp_free(ctx, m->d_cell_face_signs, nl);
    grmp_free(ctx, m->d_cell_nbr, nl * 4);
    grmp_free(ctx, m->d_face_cells, (size_t)m->nfaces * 8);
    m->d_cell_nbr = m->d_face_cells = nullptr;
    m->nfaces = nfaces;
    int rc = grmp_upload(ctx, &m->d_cell_faces, cell_faces, nl);
    if (!rc) rc = grmp_upload(ctx, &m->d_face_normals, face_normals, (size_t)nfaces * m->dim);
    if (!rc) rc = grmp_upload(ctx, &m->d_face_volumes, face_volumes, (size_t)nfaces);
    if (!rc) rc = grmp_upload(ctx, &m->d_cell_face_signs, cell_face_signs, nl);
    if (!rc) GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return rc;
}

int grmp_mesh_destroy(grmp_mesh m) {
    if (!m) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = m->ctx;
    cudaSetDevice(ctx->device);
    size_t nl = (size_t)m->ncells * (m->dim + 1);
    grmp_free(ctx, m->d_coords, (size_t)m->nverts * m->dim * 8);
    grmp_free(ctx, m->d_cells, nl * 4);
    grmp_free(ctx, m->d_cell_faces, nl * 4);
    grmp_free(ctx, m->d_face_normals, (size_t)m->nfaces * m->dim * 8);
    grmp_free(ctx, m->d_face_volumes, (size_t)m->nfaces * 8);
    grmp_free(ctx, m->d_cell_face_signs, nl);
    grmp_free(ctx, m->d_cell_nbr, nl * 4);
    grmp_free(ctx, m->d_face_cells, (size_t)m->nfaces * 8);
    cudaStreamSynchronize(ctx->stream);
    delete m;
    return GRMP_OK;
}

// ---------------------------------------------------------------- space
int grmp_space_create(grmp_mesh mesh, int fe_kind, int ncomponents, const int32_t *celldofs, int32_t ndofs,
                      grmp_space *out) {
    if (!mesh || !out || !celldofs || ndofs <= 0) return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    grmp_context ctx = mesh->ctx;
    int dim = mesh->dim;
    bool ok = (fe_kind == GRMP_FE_H1P1 && ncomponents >= 1 && ncomponents <= 3) ||
              (fe_kind == GRMP_FE_H1P2 && ncomponents >= 1 && ncomponents <= 3) ||
              (fe_kind == GRMP_FE_H1BR && ncomponents == dim) ||
              (fe_kind == GRMP_FE_H1P2B && ncomponents == 2 && dim == 2) ||
              (fe_kind == GRMP_FE_L2P0 && ncomponents >= 1 && ncomponents <= 3);
    if (!ok)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "space: element %d with %d components in %dD is not built", fe_kind,
                         ncomponents, dim);
    if ((fe_kind == GRMP_FE_H1BR || fe_kind == GRMP_FE_H1P2B) && mesh->nfaces == 0)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "space: H1BR / H1P2B need grmp_mesh_set_faces first");
    int ldofs = grmp_fe_ldofs(fe_kind, dim, ncomponents);
    if (ldofs <= 0 || ldofs > GRMP_MAX_LDOFS) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "space: %d local dofs", ldofs);
    size_t n = (size_t)mesh->ncells * ldofs;
    for (size_t i = 0; i < n; i++)
        if (celldofs[i] < 0 || celldofs[i] >= ndofs)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "space: cell dof %d out of range [0,%d)", celldofs[i], ndofs);
    cudaSetDevice(ctx->device);
    grmp_space s = new (std::nothrow) grmp_space_s();
    if (!s) return GRMP_ERR_OUT_OF_MEMORY;
    s->mesh = mesh;
    s->fe = fe_kind;
    s->ncomp = ncomponents;
    s->ldofs = ldofs;
    s->nb = grmp_fe_nb(fe_kind, dim);
    s->ndofs = ndofs;
    int rc = grmp_upload(ctx, &s->d_celldofs, celldofs, n);
    if (!rc) rc = grmp_build_incidence(s);
    if (!rc) GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (rc) {
        grmp_space_destroy(s);
        return rc;
    }
    *out = s;
    return GRMP_OK;
}

int grmp_space_destroy(grmp_space s) {
    if (!s) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = s->mesh->ctx;
    cudaSetDevice(ctx->device);
    size_t n = (size_t)s->mesh->ncells * s->ldofs;
    grmp_free(ctx, s->d_celldofs, n * 4);
    grmp_free(ctx, s->d_inc_ptr, ((size_t)s->ndofs + 1) * 4);
    grmp_free(ctx, s->d_inc_cell, n * 4);
    grmp_free(ctx, s->d_inc_loc, n);
    grmp_free(ctx, s->d_locbuf, n * 8);
    cudaStreamSynchronize(ctx->stream);
    delete s;
    return GRMP_OK;
}

int grmp_space_ndofs4cell(grmp_space s, int *out) {
    if (!s || !out) return GRMP_ERR_INVALID_ARG;
    *out = s->ldofs;
    return GRMP_OK;
}

// ---------------------------------------------------------------- vectors
int grmp_vector_create(grmp_context ctx, int32_t n, grmp_vector *out) {
    if (!valid_ctx(ctx) || !out || n <= 0) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    grmp_vector v = new (std::nothrow) grmp_vector_s();
    if (!v) return GRMP_ERR_OUT_OF_MEMORY;
    v->ctx = ctx;
    v->n = n;
    int rc = grmp_alloc(ctx, (void **)&v->d, (size_t)n * 8);
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(v->d, 0, (size_t)n * 8, ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "cudaMemsetAsync");
    }
    if (rc) {
        delete v;
        return rc;
    }
    *out = v;
    return GRMP_OK;
}

int grmp_vector_destroy(grmp_vector v) {
    if (!v) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(v->ctx->device);
    grmp_free(v->ctx, v->d, (size_t)v->n * 8);
    delete v;
    return GRMP_OK;
}

int grmp_vector_upload(grmp_vector v, const double *host) {
    if (!v || !host) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(v->ctx->device);
    GRMP_CUDA(v->ctx, cudaMemcpyAsync(v->d, host, (size_t)v->n * 8, cudaMemcpyHostToDevice, v->ctx->stream));
    GRMP_CUDA(v->ctx, cudaStreamSynchronize(v->ctx->stream));
    return GRMP_OK;
}

int grmp_vector_download(grmp_vector v, double *host) {
    if (!v || !host) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(v->ctx->device);
    GRMP_CUDA(v->ctx, cudaMemcpyAsync(host, v->d, (size_t)v->n * 8, cudaMemcpyDeviceToHost, v->ctx->stream));
    GRMP_CUDA(v->ctx, cudaStreamSynchronize(v->ctx->stream));
    return GRMP_OK;
}

// ---------------------------------------------------------------- thin wrappers
int grmp_pattern_build(grmp_space space, int nterms, const grmp_bilinear_term *terms, grmp_matrix *out) {
    if (!space || !out || nterms <= 0 || nterms > GRMP_MAX_TERMS || !terms) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(space->mesh->ctx->device);
    std::lock_guard<std::mutex> lk(space->mesh->ctx->mu);
    return grmp_pattern_build_impl(space, nterms, terms, out);
}

int grmp_assemble_bilinear(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision) {
    if (!A || nterms <= 0 || nterms > GRMP_MAX_TERMS || !terms) return GRMP_ERR_INVALID_ARG;
    if (A->imported)
        return grmp_fail(A->space->mesh->ctx, GRMP_ERR_INVALID_ARG,
                         "assemble: the matrix was imported from a CSC (no assembly space); use grmp_matrix_update_values");
    if (precision != GRMP_FP64 && precision != GRMP_FP32 && precision != GRMP_FP64_FP32) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(A->space->mesh->ctx->device);
    std::lock_guard<std::mutex> lk(A->space->mesh->ctx->mu);
    return grmp_assemble_bilinear_impl(A, nterms, terms, precision);
}

int grmp_assemble_nonlinear(grmp_matrix A, grmp_vector b, grmp_vector u, const grmp_nonlinear_term *term,
                            int precision, int add) {
    if (!A || !b || !u || !term || (add != 0 && add != 1)) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    if (b->n != A->nrows || u->n != A->nrows || b->ctx != ctx || u->ctx != ctx)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "nonlinear form: vector length or context mismatch");
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    return grmp_assemble_nonlinear_impl(A, b, u, term, precision, add);
}

int grmp_assemble_linear(grmp_space space, const grmp_rhs *rhs, grmp_vector b) {
    if (!space || !rhs || !b) return GRMP_ERR_INVALID_ARG;
    if (b->n != space->ndofs)
        return grmp_fail(space->mesh->ctx, GRMP_ERR_INVALID_ARG, "linear form: vector length %d != ndofs %d", b->n,
                         space->ndofs);
    cudaSetDevice(space->mesh->ctx->device);
    std::lock_guard<std::mutex> lk(space->mesh->ctx->mu);
    return grmp_assemble_linear_impl(space, rhs, b);
}

int grmp_item_l2error(grmp_space space, grmp_vector u, grmp_vector v, int op, const grmp_rhs *data, double factor,
                      int quadorder, double *cell_values, double *total) {
    if (!space || !u) return GRMP_ERR_INVALID_ARG;
    if (u->ctx != space->mesh->ctx || (v && v->ctx != space->mesh->ctx)) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(space->mesh->ctx->device);
    std::lock_guard<std::mutex> lk(space->mesh->ctx->mu);
    return grmp_item_l2error_impl(space, u, v, op, data, factor, quadorder, cell_values, total);
}

int grmp_apply_dirichlet(grmp_matrix A, grmp_vector b, int32_t nfixed, const int32_t *fixed, const double *values,
                         int mode, double penalty) {
    if (!A || nfixed < 0 || (nfixed > 0 && !fixed)) return GRMP_ERR_INVALID_ARG;
    if (mode != GRMP_DIRICHLET_PENALTY && mode != GRMP_DIRICHLET_ELIMINATE) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    if (b && b->n != A->nrows) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "dirichlet: rhs length mismatch");
    for (int32_t i = 0; i < nfixed; i++)
        if (fixed[i] < 0 || fixed[i] >= A->nrows)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "dirichlet: fixed dof %d out of range", fixed[i]);
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    return grmp_apply_dirichlet_impl(A, b, nfixed, fixed, values, mode, penalty);
}

int grmp_solve_params_default(grmp_solve_params *p) {
    if (!p) return GRMP_ERR_INVALID_ARG;
    std::memset(p, 0, sizeof(*p));
    p->abstol = 1e-12;
    p->reltol = 1e-12;
    p->maxiter = 100000;
    p->mode = GRMP_SOLVE_FP64;
    p->inner_reltol = 0.1;
    p->max_outer = 100;
    return GRMP_OK;
}

int grmp_solve(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *p, grmp_solve_stats *st) {
    if (!A || !b || !x || !p) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    if (b->n != A->nrows || x->n != A->nrows) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: size mismatch");
    if (p->mode < GRMP_SOLVE_FP64 || p->mode > GRMP_SOLVE_BICGSTAB) return GRMP_ERR_INVALID_ARG;
    if (!(p->reltol >= 0) || !(p->abstol >= 0) || p->maxiter <= 0) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    grmp_solve_stats local;
    if (!st) st = &local;
    std::memset(st, 0, sizeof(*st));
    // an imported matrix with penalty rows solves its eliminated system
    grmp_vector_s bt;
    grmp_vector bb = b;
    int rc = grmp_import_rhs(A, b, &bt, &bb);
    if (rc) return rc;
    if (p->mode == GRMP_SOLVE_DIRECT || p->mode == GRMP_SOLVE_MIXED_DIRECT) return grmp_mf_solve(A, bb, x, p, st);
    return grmp_solve_impl(A, bb, x, p, st);
}

int grmp_spmv(grmp_matrix A, int precision, grmp_vector x, grmp_vector y) {
    if (!A || !x || !y || x->n != A->nrows || y->n != A->nrows) return GRMP_ERR_INVALID_ARG;
    cudaSetDevice(A->space->mesh->ctx->device);
    std::lock_guard<std::mutex> lk(A->space->mesh->ctx->mu);
    return grmp_spmv_impl(A, precision, x, y);
}

int grmp_matrix_info(grmp_matrix A, int32_t *nrows, int64_t *nnz, int32_t *max_row_nnz) {
    if (!A) return GRMP_ERR_INVALID_ARG;
    if (nrows) *nrows = A->nrows;
    if (nnz) *nnz = A->nnz;
    if (max_row_nnz) *max_row_nnz = A->max_row_nnz;
    return GRMP_OK;
}

}  // extern "C"
