// Internal declarations of libgrmp_gpu.so (not part of the C-ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/grmp.h"

// ---------------------------------------------------------------- limits
constexpr int GRMP_MAX_LDOFS = 32;      // local DoFs per cell (mask width)
constexpr int GRMP_MAX_ROW_NNZ = 512;   // pattern build: per-row column list
constexpr int GRMP_MAXQ = 128;          // quadrature points
constexpr int GRMP_MAX_TERMS = 4;       // operator terms per assembly call
constexpr long long GRMP_SPIN_LIMIT = 1LL << 24;   // bounded device waits (default polls per wait)

// ---------------------------------------------------------------- handles
struct grmp_context_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t budget = 0;       // 0 = unlimited
    size_t in_use = 0;
    int num_sms = 0;
    long long wait_limit = GRMP_SPIN_LIMIT;   // polls of a bounded device wait in this context's solves
    std::atomic<unsigned long long> launches{0};
    std::string last_error;
    std::mutex mu;
};

struct grmp_mesh_s {
    grmp_context ctx = nullptr;
    int dim = 0;
    int32_t nverts = 0, ncells = 0;
    double *d_coords = nullptr;     // [nverts][dim]
    int32_t *d_cells = nullptr;     // [ncells][dim+1]
    // optional face data (H1BR / reconstruction)
    int32_t nfaces = 0;
    int32_t *d_cell_faces = nullptr;
    double *d_face_normals = nullptr;
    double *d_face_volumes = nullptr;
    int8_t *d_cell_face_signs = nullptr;
    // cell adjacency across faces (built on first use by face terms)
    int32_t *d_cell_nbr = nullptr;    // [ncells][dim+1] cell across local face f, -1 on the boundary
    int32_t *d_face_cells = nullptr;  // [nfaces][2] adjacent cells (lower id first), -1 if none
};

struct grmp_space_s {
    grmp_mesh mesh = nullptr;
    int fe = 0;
    int ncomp = 1;
    int ldofs = 0;          // local dofs per cell
    int nb = 0;             // scalar basis size of the H1 part
    int32_t ndofs = 0;
    int32_t *d_celldofs = nullptr;  // [ncells][ldofs]
    // DoF -> (cell, local) incidence, ascending cell per DoF
    int32_t *d_inc_ptr = nullptr;   // [ndofs+1]
    int32_t *d_inc_cell = nullptr;  // [ncells*ldofs]
    uint8_t *d_inc_loc = nullptr;   // [ncells*ldofs]
    double *d_locbuf = nullptr;     // [ncells][ldofs] linear-form cell vectors
};

struct grmp_matrix_s {
    grmp_space space = nullptr;
    int32_t nrows = 0;
    int64_t nnz = 0;
    int32_t max_row_nnz = 0;
    int32_t *d_rowptr = nullptr;    // [nrows+1]
    int32_t *d_cols = nullptr;      // [nnz]
    void *d_slot = nullptr;         // [ninc][ldofs] uint8 or uint16 (row-relative slot, all-ones = dropped)
    int slot_bytes = 1;
    double *d_vals64 = nullptr;     // [nnz]
    float *d_vals32 = nullptr;      // [nnz]
    void *d_pack32 = nullptr;       // [nnz] int2 (column, FP32 value bits), built by mixed solves
    bool has64 = false, has32 = false;
    uint8_t *d_fixed = nullptr;     // [nrows] Dirichlet flags (eliminated rows)
    bool eliminated = false;
    // cached workspace for solves
    void *d_work = nullptr;
    size_t work_bytes = 0;
    int tuned_cfg = 0;              // autotuned SpMV configuration, FP64 solves (0 = not tuned)
    int tuned_cfg32 = 0;            // autotuned SpMV configuration (100*lanes + loads), mixed solves
    int tuned_grid = 0;             // autotuned persistent grid (blocks; 0 = as many as fit), FP64 solves
    int tuned_grid32 = 0;           // the same, mixed solves
    // staged SpMV of mixed solves: the FP32 pairs re-laid out in fixed-size row
    // windows (state 0 = not built, 1 = built, -1 = a row does not fit a window)
    int stg_state = 0;
    int stg_nwin = 0;
    int32_t *d_stg_row0 = nullptr;  // [nwin+1] first row of each window
    char *d_stg_rec = nullptr;      // [nwin] window records
    size_t stg_rec_bytes = 0;
    // two-run 16-bit column copy of the FP32 values for mixed solves (duo
    // records; state 0 = not built, 1 = built, -1 = a run spans more than
    // 65535 columns)
    int duo_state = 0;
    int duo_span = 0;
    int64_t duo_nduo = 0;
    void *d_duo_meta = nullptr;     // [nrows+1] int4 {first duo, base1, base2, split | duos << 16}
    uint32_t *d_duo_off = nullptr;  // [nduo] two 16-bit column offsets
    int32_t *d_duo_src = nullptr;   // [nduo] CSR position of the first entry (-1 - pos: second is padding)
    void *d_duo_val = nullptr;      // [nduo] float2 values
    // Jacobi-scaled duo values a32_ij / sqrt(a32_ii a32_jj) of the FP32-assembled
    // values (formed in FP64, rounded once) and the FP64 scale
    // 1 / sqrt(a32_ii) of each row, for the scaled solver
    void *d_duo_sval = nullptr;     // [nduo] float2
    double *d_duo_sc = nullptr;     // [nrows]
    // the FP32 copies (packed pairs / staged windows, duo values, scaled duo
    // values) hold the values of the current solve
    bool pack_fresh = false, duo_fresh = false, duo_sfresh = false;
    // imported from a host CSC (grmp_matrix_from_csc): no assembly space; the
    // caller's values in CSR order, penalty rows (diagonal >= threshold)
    // eliminated from the FP64 / FP32 values the solvers use
    bool imported = false;
    double imp_threshold = 0.0;
    int imp_npen = 0;                  // penalty rows of the current values
    double *d_imp_orig = nullptr;      // [nnz] the caller's values, CSR order
    int64_t *d_imp_src = nullptr;      // [nnz] CSC position of each CSR entry (transposed imports)
    uint8_t *d_imp_flag = nullptr;     // [nrows] 1 = penalty row
    double *d_imp_diag = nullptr;      // [nrows] the caller's diagonal
    double *d_imp_b = nullptr;         // [nrows] right-hand side of the eliminated system
    int *d_imp_count = nullptr;
    // largest value count of a block of 32 / 64 / 128 consecutive rows (the
    // row-assembly kernels' shared-memory accumulator; -1 = not counted yet)
    int blk_nnz[3] = {-1, -1, -1};
    // rows per block of the row-assembly kernels, autotuned at the first
    // assembly: [0] FP64, [1] FP32, [2] both precisions in one walk (0 = not yet)
    int asm_tpb[3] = {0, 0, 0};
    // per-cell geometric factors (scratch for assembly)
    void *d_cellfac = nullptr;
    size_t cellfac_bytes = 0;
    // batched direct solver: symbolic analysis per distinct problem pattern
    struct DirectCache *direct = nullptr;
    // single-problem direct solvers: symbolic analysis + factor storage
    struct MfCache *mf = nullptr;
};

void grmp_duo_free(grmp_matrix A);   // duo copy of mixed solves (solve.cu)
void grmp_import_free(grmp_matrix A);   // arrays of a CSC import (import.cu)
// right-hand side of the eliminated system of an imported matrix with penalty
// rows (into A's scratch, described by *tmp); *out = b otherwise
int grmp_import_rhs(grmp_matrix A, grmp_vector b, struct grmp_vector_s *tmp, grmp_vector *out);
void grmp_direct_cache_free(grmp_matrix A);
void grmp_mf_cache_free(grmp_matrix A);
int grmp_mf_solve(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *p, grmp_solve_stats *st);

struct grmp_vector_s {
    grmp_context ctx = nullptr;
    int32_t n = 0;
    double *d = nullptr;
};

// ---------------------------------------------------------------- errors
int grmp_fail(grmp_context ctx, int code, const char *fmt, ...);
int grmp_cuda_fail(grmp_context ctx, cudaError_t e, const char *what);

#define GRMP_CUDA(ctx, call)                                  \
    do {                                                      \
        cudaError_t e__ = (call);                             \
        if (e__ != cudaSuccess) return grmp_cuda_fail((ctx), e__, #call); \
    } while (0)

// count one kernel launch of a context
#define GRMP_LAUNCHED(ctx) ((ctx)->launches.fetch_add(1, std::memory_order_relaxed))

// device memory accounted against the context budget
int grmp_alloc(grmp_context ctx, void **p, size_t bytes);
void grmp_free(grmp_context ctx, void *p, size_t bytes);

// ---------------------------------------------------------------- tables
// Reference tables for one element and quadrature order (host).
struct RefTables {
    int dim = 0, nq = 0, nb = 0;
    double xref[GRMP_MAXQ][3];
    double w[GRMP_MAXQ];
    double vals[GRMP_MAXQ][GRMP_MAX_LDOFS];            // scalar basis values
    double derivs[GRMP_MAXQ][GRMP_MAX_LDOFS][3];       // d/dxref_j
};
int grmp_quadrature(int dim, int order, double (*xref)[3], double *w);   // returns nq (0 = unavailable)
int grmp_tables(int dim, int fe, int order, RefTables *t);              // returns 0 on success
int grmp_fe_polyorder(int fe, int dim);
int grmp_fe_nb(int fe, int dim);          // scalar H1 basis size per component
int grmp_fe_ldofs(int fe, int dim, int ncomp);

// ---------------------------------------------------------------- internal entry points
int grmp_build_incidence(grmp_space s);
int grmp_scan_i32(grmp_context ctx, const int32_t *d_in, int32_t *d_out_excl, int32_t n, int32_t *total);

// pattern / assembly / solve implementations (pattern.cu, assemble.cu, solve.cu)
int grmp_pattern_build_impl(grmp_space space, int nterms, const grmp_bilinear_term *terms, grmp_matrix *out);
int grmp_assemble_bilinear_impl(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision);
int grmp_assemble_nonlinear_impl(grmp_matrix A, grmp_vector b, grmp_vector u, const grmp_nonlinear_term *term,
                                 int precision, int add);
int grmp_mesh_neighbors(grmp_mesh m);   // d_cell_nbr / d_face_cells (needs face data)
int grmp_face_assemble(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision);
int grmp_assemble_linear_impl(grmp_space space, const grmp_rhs *rhs, grmp_vector b);
int grmp_item_l2error_impl(grmp_space s, grmp_vector u, grmp_vector v, int op, const grmp_rhs *data, double factor,
                           int quadorder, double *cell_values, double *total);
int grmp_apply_dirichlet_impl(grmp_matrix A, grmp_vector b, int32_t nfixed, const int32_t *fixed,
                              const double *values, int mode, double penalty);
int grmp_solve_impl(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *p, grmp_solve_stats *st);
int grmp_spmv_impl(grmp_matrix A, int precision, grmp_vector x, grmp_vector y);

// upload a host array into a freshly allocated device array
template <typename T>
int grmp_upload(grmp_context ctx, T **dst, const T *src, size_t count) {
    int rc = grmp_alloc(ctx, (void **)dst, count * sizeof(T));
    if (rc) return rc;
    if (count) GRMP_CUDA(ctx, cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return GRMP_OK;
}

// ---------------------------------------------------------------- device helpers
#ifdef __CUDACC__
// Grid-wide barrier for a cooperative (co-resident) launch.  Every wait is
// bounded: after `limit` polls (one L2 round trip plus 32 ns each) the
// waiting block records GRMP_ERR_TIMEOUT in *status and leaves; callers
// check the return value and exit their loops.
//
// One 64-bit arrival counter that only grows (zeroed before the launch):
// block b's arrival at the k-th barrier returns a value in [k N, (k+1) N)
// -- no block reaches barrier k+1 before all N have arrived at barrier k --
// so the barrier is passed once the counter reaches (old / N + 1) N.  One
// atomic per block and a poll of the same word: the last arrival releases
// the waiters directly, with no reset or generation flip in between.
struct alignas(8) GridBarrier {
    unsigned long long arrived;
};

__device__ __forceinline__ bool grid_barrier(GridBarrier *gb, unsigned int nblocks, int *status,
                                             long long limit = GRMP_SPIN_LIMIT) {
    __shared__ int ok;   // one answer for the whole block, so its threads leave together
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned long long old = atomicAdd(&gb->arrived, 1ull);
        const unsigned long long target = (old / nblocks + 1ull) * nblocks;
        volatile unsigned long long *va = &gb->arrived;
        long long spins = 0;
        while (*va < target) {
            if (++spins > limit) {
                atomicCAS(status, 0, (int)GRMP_ERR_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        ok = *(volatile int *)status == 0;
    }
    __syncthreads();
    return ok != 0;
}
#endif
