// Global assembly: BilinearForm into the CSR values, LinearForm into a
// vector, Dirichlet treatment.
//
// Bilinear forms (src/assemblypatterns/bilinearform.jl:92-380).  For affine
// simplices and cell-wise constant coefficients every supported term is a
// contraction of per-cell geometric factors with reference tensors:
//   Laplace  local[(c,a),(c,b)] = vol*f*coef * sum_{p<=s} (G^T G)_{ps} S^{ps}_{ab}
//            S^{ps} = K^{ps} + K^{sp} (p<s), K^{pp} (p=s),
//            K^{ps}_{ab} = sum_q w_q dphi_a/dxi_p(q) dphi_b/dxi_s(q)
//   Mass     local[(c,a),(c,b)] = vol*f*coef * sum_q w_q phi_a(q) phi_b(q)
//   Hooke    local[(c1,a),(c2,b)] = vol*f * sum_{p,s} P^{c1c2}_{ps} K^{ps}_{ab},
//            P^{c1c2}_{ps} = sum_{k1,k2} V(c1,k1)^T C V(c2,k2) G_{k1 p} G_{k2 s}
// which is the reference's quadrature sum  sum_q w_q action(cvals_i).cvals_j
// (cvals_k = sum_p G_{kp} dphi/dxi_p, src/feevaluator_h1.jl:61-116)
// regrouped; it differs from the reference only by rounding.
//
// Deterministic scatter: one thread owns one CSR row and walks the row's
// incident cells in ascending cell order (the reference's item loop order),
// adding each cell's contribution into its slot -- no atomics, each nonzero
// written by one thread, bit-identical run to run.
#include <cmath>

#include "element.cuh"
#include "grmp_internal.h"

int grmp_prepare_terms(grmp_space s, int nterms, const grmp_bilinear_term *terms, TermsDev *td,
                       std::vector<std::pair<void *, size_t>> &keep);
void grmp_release(grmp_context ctx, std::vector<std::pair<void *, size_t>> &keep);

namespace {

constexpr int TPB = 256;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

// ------------------------------------------------------------------ term layout
struct FastTerm {
    int op;          // grmp_op_kind
    int nf;          // factors per cell
    int foff;        // offset of this term's factors in a cell's factor record
    int toff;        // offset of this term's reference tensors (elements)
    int ntens;       // number of NB x NB tensors
};

struct FastTerms {
    int n;
    int nf_total;    // factors per cell
    int tens_total;  // tensor elements
    FastTerm t[GRMP_MAX_TERMS];
    // per-term device data for the factor kernel
    double factor[GRMP_MAX_TERMS];
    double mu[GRMP_MAX_TERMS], lambda[GRMP_MAX_TERMS];
    const double *coef[GRMP_MAX_TERMS];
};

// Per-cell factors: fac[cell*nf_total + foff + f].  The factors are formed in
// FP64 (a few dozen operations per cell) and rounded once to the storage
// precision T, so FP32 element matrices carry no FP32 geometry error.
template <int DIM, int NC, typename T>
__global__ void k_cell_factors(int ncells, const double *coords, const int32_t *cells, FastTerms ft, T *fac) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[4 * 3];
    for (int v = 0; v <= DIM; v++)
        for (int k = 0; k < DIM; k++) X[v * DIM + k] = coords[(size_t)cells[(size_t)cell * (DIM + 1) + v] * DIM + k];
    double G[3][3], A[3][3], vol;
    simplex_geometry<DIM, double>(X, G, vol, A);
    T *out = fac + (size_t)cell * ft.nf_total;
    for (int ti = 0; ti < ft.n; ti++) {
        const FastTerm &t = ft.t[ti];
        double scale = vol * ft.factor[ti];
        if (ft.coef[ti]) scale *= ft.coef[ti][cell];
        if (t.op == GRMP_OP_LAPLACE) {
            int f = 0;
            for (int p = 0; p < DIM; p++)
                for (int s = p; s < DIM; s++) {
                    double m = 0;
                    for (int k = 0; k < DIM; k++) m += G[k][p] * G[k][s];
                    out[t.foff + f++] = (T)(scale * m);
                }
        } else if (t.op == GRMP_OP_MASS) {
            out[t.foff] = (T)scale;
        } else {  // Hooke: C in Voigt form, V(c,k) = unit vector of the Voigt slot
            const double l = ft.lambda[ti], mu = ft.mu[ti];
            constexpr int NV = DIM == 2 ? 3 : 6;
            double C[NV][NV];
            for (int i = 0; i < NV; i++)
                for (int j = 0; j < NV; j++) C[i][j] = 0;
            for (int i = 0; i < DIM; i++)
                for (int j = 0; j < DIM; j++) C[i][j] = (i == j) ? l + 2 * mu : l;
            for (int i = DIM; i < NV; i++) C[i][i] = mu;
            for (int c1 = 0; c1 < NC; c1++)
                for (int c2 = 0; c2 < NC; c2++)
                    for (int p = 0; p < DIM; p++)
                        for (int s = 0; s < DIM; s++) {
                            double acc = 0;
                            for (int k1 = 0; k1 < DIM; k1++)
                                for (int k2 = 0; k2 < DIM; k2++)
                                    acc += C[voigt_slot(DIM, c1, k1)][voigt_slot(DIM, c2, k2)] * G[k1][p] * G[k2][s];
                            out[t.foff + ((c1 * NC + c2) * DIM + p) * DIM + s] = (T)(scale * acc);
                        }
        }
    }
}

// Row-centric assembly.  S = slot index type (uint8_t / uint16_t).  A block
// owns blockDim.x consecutive rows; their values (contiguous in the CSR) are
// accumulated in shared memory, each thread adding its row's contributions in
// incidence order, and written out once with coalesced stores.
template <int DIM, int NB, int NC, typename T, typename S, bool LAP1 = false>
__global__ void __launch_bounds__(128) k_assemble_rows(int32_t nrows, const int32_t *__restrict__ inc_ptr,
                                                       const int32_t *__restrict__ inc_cell,
                                                       const uint8_t *__restrict__ inc_loc,
                                                       const S *__restrict__ slot, const int32_t *__restrict__ rowptr,
                                                       const T *__restrict__ fac, const T *__restrict__ gtens,
                                                       FastTerms ft, T *__restrict__ vals) {
    constexpr int LD = NB * NC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tens = reinterpret_cast<T *>(smem_raw);
    T *acc = tens + ((ft.tens_total + 1) & ~1);
    const int row0 = blockIdx.x * blockDim.x;
    const int row1 = min(row0 + (int)blockDim.x, nrows);
    const int v0 = rowptr[row0], nv = rowptr[row1] - v0;
    for (int i = threadIdx.x; i < ft.tens_total; i += blockDim.x) tens[i] = gtens[i];
    for (int i = threadIdx.x; i < nv; i += blockDim.x) acc[i] = T(0);
    __syncthreads();
    const int row = row0 + threadIdx.x;
    if (row < row1) {
        T *rv = acc + (rowptr[row] - v0);
        const S DROP = (S)~(S)0;
        const int pe = inc_ptr[row + 1];
        for (int p = inc_ptr[row]; p < pe; p++) {
            const int cell = inc_cell[p];
            const int A = inc_loc[p];
            const int c1 = A / NB, a = A - c1 * NB;
            const T *cf = fac + (size_t)cell * ft.nf_total;
            const S *sl = slot + (size_t)p * LD;
            if (LAP1) {   // one Laplace term: its DIM(DIM+1)/2 factors in registers
                constexpr int NT = DIM * (DIM + 1) / 2;
                T fl[NT];
#pragma unroll
                for (int q = 0; q < NT; q++) fl[q] = cf[q];
#pragma unroll
                for (int B = 0; B < LD; B++) {
                    const S s = sl[B];
                    if (s == DROP) continue;
                    const int c2 = B / NB, b = B - c2 * NB;
                    if (c1 != c2) continue;
                    const T *tt = tens + a * NB + b;
                    T v = 0;
#pragma unroll
                    for (int q = 0; q < NT; q++) v += fl[q] * tt[q * NB * NB];
                    rv[s] += v;
                }
                continue;
            }
            T f[GRMP_MAX_TERMS * 16];
            for (int i = 0; i < ft.nf_total && i < GRMP_MAX_TERMS * 16; i++) f[i] = cf[i];
#pragma unroll
            for (int B = 0; B < LD; B++) {
                const S s = sl[B];
                if (s == DROP) continue;
                const int c2 = B / NB, b = B - c2 * NB;
                T v = 0;
                for (int ti = 0; ti < ft.n; ti++) {
                    const FastTerm &t = ft.t[ti];
                    const T *tt = tens + t.toff + a * NB + b;
                    if (t.op == GRMP_OP_HOOKE) {
                        const T *ff = f + t.foff + (c1 * NC + c2) * DIM * DIM;
#pragma unroll
                        for (int q = 0; q < DIM * DIM; q++) v += ff[q] * tt[q * NB * NB];
                    } else if (c1 == c2) {
                        const T *ff = f + t.foff;
                        for (int q = 0; q < t.ntens; q++) v += ff[q] * tt[q * NB * NB];
                    }
                }
                rv[s] += v;
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nv; i += blockDim.x) vals[v0 + i] = acc[i];
}

// Both precisions in one walk: the FP64 and the FP32 contribution of every
// (row, cell, DoF) triple, each from its own factors and reference tensors in
// its own arithmetic, accumulated into two shared-memory row blocks.
template <int DIM, int NB, int NC, typename S, bool LAP1 = false>
__global__ void __launch_bounds__(128) k_assemble_rows2(int32_t nrows, const int32_t *__restrict__ inc_ptr,
                                                        const int32_t *__restrict__ inc_cell,
                                                        const uint8_t *__restrict__ inc_loc,
                                                        const S *__restrict__ slot, const int32_t *__restrict__ rowptr,
                                                        const double *__restrict__ fac64, const float *__restrict__ fac32,
                                                        const double *__restrict__ gtens64,
                                                        const float *__restrict__ gtens32, FastTerms ft,
                                                        double *__restrict__ vals64, float *__restrict__ vals32,
                                                        int block_nnz) {
    constexpr int LD = NB * NC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *tens64 = reinterpret_cast<double *>(smem_raw);
    double *acc64 = tens64 + ft.tens_total;
    float *tens32 = reinterpret_cast<float *>(acc64 + block_nnz);
    float *acc32 = tens32 + ((ft.tens_total + 1) & ~1);
    const int row0 = blockIdx.x * blockDim.x;
    const int row1 = min(row0 + (int)blockDim.x, nrows);
    const int v0 = rowptr[row0], nv = rowptr[row1] - v0;
    for (int i = threadIdx.x; i < ft.tens_total; i += blockDim.x) {
        tens64[i] = gtens64[i];
        tens32[i] = gtens32[i];
    }
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        acc64[i] = 0.0;
        acc32[i] = 0.f;
    }
    __syncthreads();
    const int row = row0 + threadIdx.x;
    if (row < row1) {
        double *rv64 = acc64 + (rowptr[row] - v0);
        float *rv32 = acc32 + (rowptr[row] - v0);
        const S DROP = (S)~(S)0;
        const int pe = inc_ptr[row + 1];
        for (int p = inc_ptr[row]; p < pe; p++) {
            const int cell = inc_cell[p];
            const int A = inc_loc[p];
            const int c1 = A / NB, a = A - c1 * NB;
            const double *cf64 = fac64 + (size_t)cell * ft.nf_total;
            const float *cf32 = fac32 + (size_t)cell * ft.nf_total;
            const S *sl = slot + (size_t)p * LD;
            if (LAP1) {   // one Laplace term: both precisions' factors in registers
                constexpr int NT = DIM * (DIM + 1) / 2;
                double g64[NT];
                float g32[NT];
#pragma unroll
                for (int q = 0; q < NT; q++) {
                    g64[q] = cf64[q];
                    g32[q] = cf32[q];
                }
#pragma unroll
                for (int B = 0; B < LD; B++) {
                    const S s = sl[B];
                    if (s == DROP) continue;
                    const int c2 = B / NB, b = B - c2 * NB;
                    if (c1 != c2) continue;
                    const int to = a * NB + b;
                    double v = 0;
                    float w = 0;
#pragma unroll
                    for (int q = 0; q < NT; q++) {
                        v += g64[q] * tens64[to + q * NB * NB];
                        w += g32[q] * tens32[to + q * NB * NB];
                    }
                    rv64[s] += v;
                    rv32[s] += w;
                }
                continue;
            }
            double f64[GRMP_MAX_TERMS * 16];
            float f32[GRMP_MAX_TERMS * 16];
            for (int i = 0; i < ft.nf_total && i < GRMP_MAX_TERMS * 16; i++) {
                f64[i] = cf64[i];
                f32[i] = cf32[i];
            }
#pragma unroll
            for (int B = 0; B < LD; B++) {
                const S s = sl[B];
                if (s == DROP) continue;
                const int c2 = B / NB, b = B - c2 * NB;
                double v = 0;
                float w = 0;
                for (int ti = 0; ti < ft.n; ti++) {
                    const FastTerm &t = ft.t[ti];
                    const int to = t.toff + a * NB + b;
                    if (t.op == GRMP_OP_HOOKE) {
                        const int fo = t.foff + (c1 * NC + c2) * DIM * DIM;
#pragma unroll
                        for (int q = 0; q < DIM * DIM; q++) {
                            v += f64[fo + q] * tens64[to + q * NB * NB];
                            w += f32[fo + q] * tens32[to + q * NB * NB];
                        }
                    } else if (c1 == c2) {
                        for (int q = 0; q < t.ntens; q++) {
                            v += f64[t.foff + q] * tens64[to + q * NB * NB];
                            w += f32[t.foff + q] * tens32[to + q * NB * NB];
                        }
                    }
                }
                rv64[s] += v;
                rv32[s] += w;
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        vals64[v0 + i] = acc64[i];
        vals32[v0 + i] = acc32[i];
    }
}

// Largest number of values a block of `tpb` consecutive rows holds (the
// shared-memory accumulator is sized by it, not by tpb x the longest row).
int block_nnz_max(grmp_matrix A, int tpb, int *out) {
    grmp_context ctx = A->space->mesh->ctx;
    const int k = tpb >= 128 ? 2 : (tpb >= 64 ? 1 : 0);
    if (A->blk_nnz[k] < 0) {   // all three block sizes from one download of the row pointers
        std::vector<int32_t> rp((size_t)A->nrows + 1);
        cudaError_t e = cudaMemcpyAsync(rp.data(), A->d_rowptr, rp.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "assembly: row pointer download");
        for (int q = 0; q < 3; q++) {
            const int b = 32 << q;
            int mx = 0;
            for (int r0 = 0; r0 < A->nrows; r0 += b) mx = std::max(mx, rp[std::min(A->nrows, r0 + b)] - rp[r0]);
            A->blk_nnz[q] = mx;
        }
    }
    *out = A->blk_nnz[k];
    return GRMP_OK;
}

// Rows per block of a row-assembly kernel (128, 64 or 32: the kernels are
// built for at most 128 threads) and its shared memory: the reference tensors
// (tens_b bytes) and the block's values (per_nnz bytes each, the largest
// block's count).  The first assembly of a matrix of at least kAsmTuneRows
// rows times every candidate that fits once with CUDA events and keeps the
// fastest in *cached; smaller matrices, and matrices whose *cached is
// negative (served requests), take the largest block within 100 KB (two
// blocks per SM).  The assembled values do not depend on the choice:
// every row is summed by one thread in incidence order.  go(tpb, shm)
// enqueues the kernel; on return it has run with the chosen shape.
constexpr int kAsmTuneRows = 20000;

template <typename L>
int assemble_rows_tuned(grmp_matrix A, size_t tens_b, size_t per_nnz, int *cached, L go) {
    grmp_context ctx = A->space->mesh->ctx;
    auto shm_of = [&](int tpb, size_t *shm) {
        int bnz = 0;
        const int rc = block_nnz_max(A, tpb, &bnz);
        *shm = tens_b + (size_t)bnz * per_nnz + 16;
        return rc;
    };
    if (*cached > 0) {
        size_t shm = 0;
        int rc = shm_of(*cached, &shm);
        if (rc) return rc;
        go(*cached, shm);
        return GRMP_OK;
    }
    if (*cached < 0 || A->nrows < kAsmTuneRows) {   // negative: the caller asked for the rule, not timing
        int tpb = 128;
        size_t shm = 0;
        int rc = shm_of(tpb, &shm);
        while (!rc && tpb > 32 && shm > 100 * 1024) {
            tpb /= 2;
            rc = shm_of(tpb, &shm);
        }
        if (rc) return rc;
        if (shm > 220 * 1024) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "assembly: rows too long for shared memory");
        if (*cached == 0) *cached = tpb;
        go(tpb, shm);
        return GRMP_OK;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = 0;
    float best_ms = 0.f;
    for (int tpb : {128, 64, 32}) {
        size_t shm = 0;
        int rc = shm_of(tpb, &shm);
        if (rc) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc;
        }
        if (shm > 220 * 1024) continue;
        cudaEventRecord(e0, ctx->stream);
        go(tpb, shm);
        cudaEventRecord(e1, ctx->stream);
        float ms = 0.f;
        if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
            (best == 0 || ms < best_ms)) {
            best = tpb;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best == 0) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "assembly: rows too long for shared memory");
    *cached = best;
    if (best != 32) {   // the values in place are the last candidate's (identical); keep the chosen launch last
        size_t shm = 0;
        int rc = shm_of(best, &shm);
        if (rc) return rc;
        go(best, shm);
    }
    return GRMP_OK;
}

// a single Laplace term: the register-resident kernel variants
inline bool single_laplace(const FastTerms &ft) { return ft.n == 1 && ft.t[0].op == GRMP_OP_LAPLACE; }

template <int DIM, int NB, int NC>
int run_assembly_dual(grmp_matrix A, const FastTerms &ft, const std::vector<double> &tens64) {
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    std::vector<float> tens32(tens64.begin(), tens64.end());
    double *dt64 = nullptr;
    float *dt32 = nullptr;
    int rc = grmp_upload(ctx, &dt64, tens64.data(), tens64.size());
    if (!rc) rc = grmp_upload(ctx, &dt32, tens32.data(), tens32.size());
    auto release = [&]() {
        grmp_free(ctx, dt64, tens64.size() * 8);
        grmp_free(ctx, dt32, tens32.size() * 4);
    };
    if (rc) {
        release();
        return rc;
    }
    const size_t f64b = (size_t)m->ncells * ft.nf_total * 8, f32b = (size_t)m->ncells * ft.nf_total * 4;
    const size_t fbytes = f64b + ((f32b + 255) & ~(size_t)255);
    if (A->cellfac_bytes < fbytes) {
        grmp_free(ctx, A->d_cellfac, A->cellfac_bytes);
        A->cellfac_bytes = 0;
        rc = grmp_alloc(ctx, &A->d_cellfac, fbytes);
        if (rc) {
            release();
            return rc;
        }
        A->cellfac_bytes = fbytes;
    }
    double *fac64 = (double *)A->d_cellfac;
    float *fac32 = (float *)((char *)A->d_cellfac + ((f64b + 255) & ~(size_t)255));
    k_cell_factors<DIM, NC, double><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, m->d_coords, m->d_cells, ft,
                                                                              fac64);
    GRMP_LAUNCHED(ctx);
    k_cell_factors<DIM, NC, float><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, m->d_coords, m->d_cells, ft,
                                                                             fac32);
    GRMP_LAUNCHED(ctx);
    if (!A->d_vals64) rc = grmp_alloc(ctx, (void **)&A->d_vals64, (size_t)A->nnz * 8);
    if (!rc && !A->d_vals32) rc = grmp_alloc(ctx, (void **)&A->d_vals32, (size_t)A->nnz * 4);
    if (rc) {
        release();
        return rc;
    }
    const size_t tens_b = tens64.size() * 8 + ((tens32.size() + 1) & ~(size_t)1) * 4;
    const bool lap1 = single_laplace(ft);
    auto go = [&](int tpb, size_t shm) {
        int bnz = 0;
        block_nnz_max(A, tpb, &bnz);   // counted by the caller already: no download here
        auto launch = [&](auto kern, const auto *slot) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
            kern<<<nblk(A->nrows, tpb), tpb, shm, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc,
                                                                slot, A->d_rowptr, fac64, fac32, dt64, dt32, ft,
                                                                A->d_vals64, A->d_vals32, bnz);
            GRMP_LAUNCHED(ctx);
        };
        if (A->slot_bytes == 1) {
            if (lap1) launch(k_assemble_rows2<DIM, NB, NC, uint8_t, true>, (const uint8_t *)A->d_slot);
            else launch(k_assemble_rows2<DIM, NB, NC, uint8_t, false>, (const uint8_t *)A->d_slot);
        } else {
            if (lap1) launch(k_assemble_rows2<DIM, NB, NC, uint16_t, true>, (const uint16_t *)A->d_slot);
            else launch(k_assemble_rows2<DIM, NB, NC, uint16_t, false>, (const uint16_t *)A->d_slot);
        }
    };
    rc = assemble_rows_tuned(A, tens_b, 12, &A->asm_tpb[2], go);
    if (rc) {
        release();
        return rc;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);   // the tensor uploads are released next
    release();
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "assembly kernels");
    A->has64 = A->has32 = true;
    return GRMP_OK;
}

template <int DIM, int NB, int NC, typename T>
int run_assembly(grmp_matrix A, const FastTerms &ft, const std::vector<double> &tens64) {
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    // reference tensors in precision T
    std::vector<T> tens(tens64.begin(), tens64.end());
    T *dtens = nullptr;
    int rc = grmp_upload(ctx, &dtens, tens.data(), tens.size());
    if (rc) return rc;
    size_t fbytes = (size_t)m->ncells * ft.nf_total * sizeof(T);
    if (A->cellfac_bytes < fbytes) {
        grmp_free(ctx, A->d_cellfac, A->cellfac_bytes);
        A->cellfac_bytes = 0;
        rc = grmp_alloc(ctx, &A->d_cellfac, fbytes);
        if (rc) {
            grmp_free(ctx, dtens, tens.size() * sizeof(T));
            return rc;
        }
        A->cellfac_bytes = fbytes;
    }
    T *fac = (T *)A->d_cellfac;
    k_cell_factors<DIM, NC, T><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, m->d_coords, m->d_cells, ft, fac); GRMP_LAUNCHED(ctx);
    T *vals;
    if (sizeof(T) == 8) {
        if (!A->d_vals64) {
            rc = grmp_alloc(ctx, (void **)&A->d_vals64, (size_t)A->nnz * 8);
            if (rc) return rc;
        }
        vals = (T *)A->d_vals64;
    } else {
        if (!A->d_vals32) {
            rc = grmp_alloc(ctx, (void **)&A->d_vals32, (size_t)A->nnz * 4);
            if (rc) return rc;
        }
        vals = (T *)A->d_vals32;
    }
    // rows per block (autotuned per matrix and precision): their values (the
    // largest block's count) and the reference tensors in shared memory
    const size_t tens_b = ((tens.size() + 1) & ~(size_t)1) * sizeof(T);
    const bool lap1 = single_laplace(ft);
    auto go = [&](int tpb, size_t shm) {
        auto launch = [&](auto kern, const auto *slot) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
            kern<<<nblk(A->nrows, tpb), tpb, shm, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc,
                                                                slot, A->d_rowptr, fac, dtens, ft, vals);
            GRMP_LAUNCHED(ctx);
        };
        if (A->slot_bytes == 1) {
            if (lap1) launch(k_assemble_rows<DIM, NB, NC, T, uint8_t, true>, (const uint8_t *)A->d_slot);
            else launch(k_assemble_rows<DIM, NB, NC, T, uint8_t, false>, (const uint8_t *)A->d_slot);
        } else {
            if (lap1) launch(k_assemble_rows<DIM, NB, NC, T, uint16_t, true>, (const uint16_t *)A->d_slot);
            else launch(k_assemble_rows<DIM, NB, NC, T, uint16_t, false>, (const uint16_t *)A->d_slot);
        }
    };
    rc = assemble_rows_tuned(A, tens_b, sizeof(T), &A->asm_tpb[sizeof(T) == 8 ? 0 : 1], go);
    if (rc) {
        grmp_free(ctx, dtens, tens.size() * sizeof(T));
        return rc;
    }
    cudaError_t e = cudaGetLastError();
    grmp_free(ctx, dtens, tens.size() * sizeof(T));
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "assembly kernels");
    if (sizeof(T) == 8) A->has64 = true; else A->has32 = true;
    return GRMP_OK;
}

template <int DIM, int NB, int NC>
int dispatch_precision(grmp_matrix A, const FastTerms &ft, const std::vector<double> &tens, int precision) {
    if (precision == GRMP_FP64) return run_assembly<DIM, NB, NC, double>(A, ft, tens);
    if (precision == GRMP_FP64_FP32) return run_assembly_dual<DIM, NB, NC>(A, ft, tens);
    return run_assembly<DIM, NB, NC, float>(A, ft, tens);
}

// ------------------------------------------------------------------ linear forms
// Cell-local vectors  loc[cell][(c,a)] = (factor*vol) * sum_q (f_c(x_q) phi_a(q)) w_q
// (src/assemblypatterns/linearform.jl:181-220; x_q = x0 + A xref_q).
template <int DIM>
__global__ void k_linear_cells(int ncells, const double *coords, const int32_t *cells, int nb, int ncomp, RhsDev r,
                               double *loc) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[4 * 3];
    for (int v = 0; v <= DIM; v++)
        for (int k = 0; k < DIM; k++) X[v * DIM + k] = coords[(size_t)cells[(size_t)cell * (DIM + 1) + v] * DIM + k];
    double A[3][3];
    for (int k = 0; k < DIM; k++)
        for (int j = 0; j < DIM; j++) A[k][j] = X[(j + 1) * DIM + k] - X[k];
    double det = DIM == 2 ? A[0][0] * A[1][1] - A[0][1] * A[1][0]
                          : A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) +
                                A[0][1] * (A[1][2] * A[2][0] - A[1][0] * A[2][2]) +
                                A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    double vol = fabs(det) / (DIM == 2 ? 2.0 : 6.0);
    double lb[GRMP_MAX_LDOFS];
    int ld = nb * ncomp;
    for (int i = 0; i < ld; i++) lb[i] = 0;
    for (int q = 0; q < r.nq; q++) {
        double x[3] = {0, 0, 0}, f[3];
        for (int k = 0; k < DIM; k++) {
            x[k] = X[k];
            for (int j = 0; j < DIM; j++) x[k] += A[k][j] * r.xref[3 * q + j];
        }
        rhs_eval(r, DIM, cell, x, f);
        for (int c = 0; c < ncomp; c++)
            for (int a = 0; a < nb; a++) lb[c * nb + a] += (f[c] * r.vals[q * nb + a]) * r.w[q];
    }
    double itemfactor = r.factor * vol;
    for (int i = 0; i < ld; i++) loc[(size_t)cell * ld + i] = lb[i] * itemfactor;
}

// b[row] += sum over incident cells (ascending) of loc[cell][local]
__global__ void k_gather_rows(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell, const uint8_t *inc_loc,
                              int ld, const double *loc, double *b) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    double acc = b[row];
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) acc += loc[(size_t)inc_cell[p] * ld + inc_loc[p]];
    b[row] = acc;
}

// ------------------------------------------------------------------ Dirichlet
__global__ void k_mark(const int32_t *fixed, int n, uint8_t *flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[fixed[i]] = 1;
}

__global__ void k_set_values(const int32_t *fixed, const double *vals, int n, double *u) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[fixed[i]] = vals ? vals[i] : 0.0;
}

// ELIMINATE: b -= A[:,fixed] u_D (rows not fixed), zero fixed columns and
// rows, unit diagonal, b[d] = u_D.  PENALTY: A[d,d] = penalty,
// b[d] = penalty*u_D (src/solvers.jl:640-652).
template <typename T>
__global__ void k_dirichlet_rows(int32_t nrows, const int32_t *rowptr, const int32_t *cols, T *vals,
                                 const uint8_t *flag, const double *ud, double *b, int mode, double penalty,
                                 int update_b) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    bool fr = flag[row] != 0;
    double bacc = update_b ? b[row] : 0.0;
    for (int k = rowptr[row]; k < rowptr[row + 1]; k++) {
        int c = cols[k];
        if (mode == GRMP_DIRICHLET_PENALTY) {
            if (fr && c == row) vals[k] = (T)penalty;
        } else {
            if (fr) {
                vals[k] = (c == row) ? T(1) : T(0);
            } else if (flag[c]) {
                if (ud) bacc -= (double)vals[k] * ud[c];
                vals[k] = T(0);
            }
        }
    }
    if (update_b) {
        if (fr) b[row] = (mode == GRMP_DIRICHLET_PENALTY) ? penalty * (ud ? ud[row] : 0.0) : (ud ? ud[row] : 0.0);
        else b[row] = bacc;
    }
}

}  // namespace

// ---------------------------------------------------------------------- bilinear
int grmp_br_assemble(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision);
int grmp_br_rhs(grmp_space s, const grmp_rhs *rhs, grmp_vector b);
int grmp_p2b_rhs(grmp_space s, const grmp_rhs *rhs, grmp_vector b);

int grmp_assemble_bilinear_impl(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision) {
    grmp_space s = A->space;
    grmp_context ctx = s->mesh->ctx;
    if (s->fe == GRMP_FE_H1BR) {
        int rc = precision == GRMP_FP64_FP32 ? grmp_br_assemble(A, nterms, terms, GRMP_FP64)
                                             : grmp_br_assemble(A, nterms, terms, precision);
        if (!rc && precision == GRMP_FP64_FP32) rc = grmp_br_assemble(A, nterms, terms, GRMP_FP32);
        if (!rc) A->eliminated = false;
        return rc;
    }
    int dim = s->mesh->dim, nb = s->nb, nc = s->ncomp;
    // pattern-only terms contribute nothing to the values
    // (and face terms are added after the cell terms)
    std::vector<grmp_bilinear_term> kept, faceterms;
    for (int i = 0; i < nterms; i++) {
        if (terms[i].op_kind == GRMP_OP_JUMPGRAD) faceterms.push_back(terms[i]);
        else if (terms[i].op_kind != GRMP_OP_STRUCTURAL) kept.push_back(terms[i]);
    }
    if (!faceterms.empty()) {
        const int rc0 = grmp_assemble_bilinear_impl(A, (int)kept.size(), kept.data(), precision);
        if (rc0) return rc0;
        return grmp_face_assemble(A, (int)faceterms.size(), faceterms.data(), precision);
    }
    nterms = (int)kept.size();
    terms = kept.data();
    if (nterms == 0) {   // only pattern terms: every value is zero
        int rz = GRMP_OK;
        const bool want64 = precision != GRMP_FP32, want32 = precision != GRMP_FP64;
        if (want64 && !A->d_vals64) rz = grmp_alloc(ctx, (void **)&A->d_vals64, (size_t)A->nnz * 8);
        if (!rz && want32 && !A->d_vals32) rz = grmp_alloc(ctx, (void **)&A->d_vals32, (size_t)A->nnz * 4);
        if (rz) return rz;
        if (want64) cudaMemsetAsync(A->d_vals64, 0, (size_t)A->nnz * 8, ctx->stream);
        if (want32) cudaMemsetAsync(A->d_vals32, 0, (size_t)A->nnz * 4, ctx->stream);
        GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (want64) A->has64 = true;
        if (want32) A->has32 = true;
        A->eliminated = false;
        return GRMP_OK;
    }
    TermsDev td;
    std::vector<std::pair<void *, size_t>> keep;
    int rc = grmp_prepare_terms(s, nterms, terms, &td, keep);
    if (rc) {
        grmp_release(ctx, keep);
        return rc;
    }
    // reference tensors (host, FP64) and the factor layout
    FastTerms ft;
    std::memset(&ft, 0, sizeof(ft));
    ft.n = nterms;
    std::vector<double> tens;
    int foff = 0;
    for (int i = 0; i < nterms; i++) {
        const grmp_bilinear_term &t = terms[i];
        int deriv = t.op_kind == GRMP_OP_MASS ? 0 : 1;
        int order = t.bonus_quadorder + 2 * (grmp_fe_polyorder(s->fe, dim) - deriv);
        RefTables *rt = new RefTables;
        grmp_tables(dim, s->fe, order < 0 ? 0 : order, rt);
        FastTerm &f = ft.t[i];
        f.op = t.op_kind;
        f.foff = foff;
        f.toff = (int)tens.size();
        ft.factor[i] = t.factor;
        ft.mu[i] = t.param[0];
        ft.lambda[i] = t.param[1];
        ft.coef[i] = td.t[i].cell_coef;
        auto K = [&](int p, int q2, int a, int b) {
            double acc = 0;
            for (int q = 0; q < rt->nq; q++) acc += rt->w[q] * rt->derivs[q][a][p] * rt->derivs[q][b][q2];
            return acc;
        };
        if (t.op_kind == GRMP_OP_LAPLACE) {
            f.ntens = f.nf = dim * (dim + 1) / 2;
            for (int p = 0; p < dim; p++)
                for (int q2 = p; q2 < dim; q2++)
                    for (int a = 0; a < nb; a++)
                        for (int b = 0; b < nb; b++) tens.push_back(p == q2 ? K(p, p, a, b) : K(p, q2, a, b) + K(q2, p, a, b));
        } else if (t.op_kind == GRMP_OP_MASS) {
            f.ntens = f.nf = 1;
            for (int a = 0; a < nb; a++)
                for (int b = 0; b < nb; b++) {
                    double acc = 0;
                    for (int q = 0; q < rt->nq; q++) acc += rt->w[q] * rt->vals[q][a] * rt->vals[q][b];
                    tens.push_back(acc);
                }
        } else {
            f.ntens = dim * dim;
            f.nf = nc * nc * dim * dim;
            for (int p = 0; p < dim; p++)
                for (int q2 = 0; q2 < dim; q2++)
                    for (int a = 0; a < nb; a++)
                        for (int b = 0; b < nb; b++) tens.push_back(K(p, q2, a, b));
        }
        delete rt;
        foff += f.nf;
    }
    ft.nf_total = foff;
    ft.tens_total = (int)tens.size();
    if (foff > GRMP_MAX_TERMS * 16) {
        grmp_release(ctx, keep);
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "too many per-cell factors (%d)", foff);
    }
    if (dim == 2 && nb == 3 && nc == 1) rc = dispatch_precision<2, 3, 1>(A, ft, tens, precision);
    else if (dim == 2 && nb == 3 && nc == 2) rc = dispatch_precision<2, 3, 2>(A, ft, tens, precision);
    else if (dim == 2 && nb == 6 && nc == 1) rc = dispatch_precision<2, 6, 1>(A, ft, tens, precision);
    else if (dim == 2 && nb == 6 && nc == 2) rc = dispatch_precision<2, 6, 2>(A, ft, tens, precision);
    else if (dim == 3 && nb == 4 && nc == 1) rc = dispatch_precision<3, 4, 1>(A, ft, tens, precision);
    else if (dim == 3 && nb == 10 && nc == 1) rc = dispatch_precision<3, 10, 1>(A, ft, tens, precision);
    else rc = grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "assembly: element layout dim=%d nb=%d nc=%d", dim, nb, nc);
    // the per-term uploads (tables, coefficients) must outlive the kernels
    cudaStreamSynchronize(ctx->stream);
    grmp_release(ctx, keep);
    if (!rc && A->eliminated) {
        // a fresh assembly overwrites eliminated rows: the caller re-applies Dirichlet data
        A->eliminated = false;
    }
    return rc;
}

// ---------------------------------------------------------------------- linear
int grmp_assemble_linear_impl(grmp_space s, const grmp_rhs *rhs, grmp_vector b) {
    grmp_context ctx = s->mesh->ctx;
    grmp_mesh m = s->mesh;
    int dim = m->dim;
    if (s->fe == GRMP_FE_H1BR) {
        if (rhs->test_operator != 1 && rhs->test_operator != 2)
            return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED,
                             "H1BR right-hand sides use a reconstruction test operator (1 = RT0, 2 = BDM1)");
        return grmp_br_rhs(s, rhs, b);
    }
    if (s->fe == GRMP_FE_H1P2B) return grmp_p2b_rhs(s, rhs, b);
    if (rhs->test_operator != 0) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "reconstruction test operator needs H1BR");
    if (s->fe != GRMP_FE_H1P1 && s->fe != GRMP_FE_H1P2)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "linear form on element %d", s->fe);
    if (rhs->ncomponents != s->ncomp) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs components != space components");
    long long need = 0;
    switch (rhs->kind) {
        case GRMP_RHS_CONST: need = rhs->ncomponents; break;
        case GRMP_RHS_CELL: need = (long long)m->ncells * rhs->ncomponents; break;
        case GRMP_RHS_FOURIER: need = 1 + dim; break;
        case GRMP_RHS_POLY: need = 5; break;
        default: return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs kind %d", rhs->kind);
    }
    if (rhs->nparams < need || !rhs->params) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: too few parameters");
    if ((rhs->kind == GRMP_RHS_FOURIER && rhs->nparams % (1 + dim)) || (rhs->kind == GRMP_RHS_POLY && rhs->nparams % 5))
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: parameter count not a multiple of the record size");
    if (rhs->kind == GRMP_RHS_POLY)
        for (long long t = 0; t < rhs->nparams / 5; t++)
            if (rhs->params[5 * t] < 0 || rhs->params[5 * t] >= rhs->ncomponents)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: polynomial component out of range");
    int order = grmp_fe_polyorder(s->fe, dim) + rhs->bonus_quadorder;
    RefTables *rt = new RefTables;
    int rc = grmp_tables(dim, s->fe, order, rt);
    if (rc) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no quadrature rule of order %d", order);
    }
    int nq = rt->nq, nb = rt->nb;
    std::vector<double> buf(nq + 3 * nq + nq * nb);
    for (int q = 0; q < nq; q++) {
        buf[q] = rt->w[q];
        for (int k = 0; k < 3; k++) buf[nq + 3 * q + k] = rt->xref[q][k];
        for (int a = 0; a < nb; a++) buf[4 * nq + q * nb + a] = rt->vals[q][a];
    }
    delete rt;
    double *dtab = nullptr, *dpar = nullptr;
    rc = grmp_upload(ctx, &dtab, buf.data(), buf.size());
    if (!rc) rc = grmp_upload(ctx, &dpar, rhs->params, (size_t)rhs->nparams);
    size_t ncl = (size_t)m->ncells * s->ldofs;
    if (!rc && !s->d_locbuf) rc = grmp_alloc(ctx, (void **)&s->d_locbuf, ncl * 8);
    if (!rc) {
        RhsDev r{rhs->kind, rhs->ncomponents, dpar, rhs->nparams, rhs->factor, nq, nb, dtab, dtab + nq, dtab + 4 * nq};
        if (dim == 2) k_linear_cells<2><<<nblk(m->ncells, 128), 128, 0, ctx->stream>>>(m->ncells, m->d_coords, m->d_cells,
                                                                                    nb, s->ncomp, r, s->d_locbuf);
        else k_linear_cells<3><<<nblk(m->ncells, 128), 128, 0, ctx->stream>>>(m->ncells, m->d_coords, m->d_cells, nb,
                                                                           s->ncomp, r, s->d_locbuf);
        GRMP_LAUNCHED(ctx);
        k_gather_rows<<<nblk(s->ndofs), TPB, 0, ctx->stream>>>(s->ndofs, s->d_inc_ptr, s->d_inc_cell, s->d_inc_loc,
                                                               s->ldofs, s->d_locbuf, b->d); GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "linear form kernels");
    }
    grmp_free(ctx, dtab, buf.size() * 8);
    grmp_free(ctx, dpar, (size_t)rhs->nparams * 8);
    return rc;
}

// ---------------------------------------------------------------------- Dirichlet
int grmp_apply_dirichlet_impl(grmp_matrix A, grmp_vector b, int32_t nfixed, const int32_t *fixed, const double *values,
                              int mode, double penalty) {
    grmp_context ctx = A->space->mesh->ctx;
    if (!A->has64 && !A->has32) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "dirichlet: matrix not assembled");
    if (mode == GRMP_DIRICHLET_PENALTY && A->has32)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "dirichlet: the penalty form overflows FP32 values; use ELIMINATE");
    int rc = GRMP_OK;
    if (!A->d_fixed) rc = grmp_alloc(ctx, (void **)&A->d_fixed, (size_t)A->nrows);
    if (rc) return rc;
    cudaMemsetAsync(A->d_fixed, 0, (size_t)A->nrows, ctx->stream);
    int32_t *dfix = nullptr;
    double *dval = nullptr, *ud = nullptr;
    if (nfixed > 0) {
        rc = grmp_upload(ctx, &dfix, fixed, (size_t)nfixed);
        if (!rc && values) rc = grmp_upload(ctx, &dval, values, (size_t)nfixed);
        if (!rc && values) rc = grmp_alloc(ctx, (void **)&ud, (size_t)A->nrows * 8);
        if (rc) {
            grmp_free(ctx, dfix, (size_t)nfixed * 4);
            grmp_free(ctx, dval, (size_t)nfixed * 8);
            return rc;
        }
        k_mark<<<nblk(nfixed), TPB, 0, ctx->stream>>>(dfix, nfixed, A->d_fixed); GRMP_LAUNCHED(ctx);
        if (ud) {
            cudaMemsetAsync(ud, 0, (size_t)A->nrows * 8, ctx->stream);
            k_set_values<<<nblk(nfixed), TPB, 0, ctx->stream>>>(dfix, dval, nfixed, ud); GRMP_LAUNCHED(ctx);
        }
    }
    int ub = b ? 1 : 0;
    double *bd = b ? b->d : nullptr;
    // the right-hand side is updated with the FP64 values only (b is FP64)
    if (A->has64) {
        k_dirichlet_rows<double><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(A->nrows, A->d_rowptr, A->d_cols, A->d_vals64,
                                                                         A->d_fixed, ud, bd, mode, penalty, ub);
        GRMP_LAUNCHED(ctx);
    }
    if (A->has32) {
        k_dirichlet_rows<float><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(A->nrows, A->d_rowptr, A->d_cols, A->d_vals32,
                                                                        A->d_fixed, ud, bd, mode, penalty,
                                                                        A->has64 ? 0 : ub);
        GRMP_LAUNCHED(ctx);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, dfix, (size_t)nfixed * 4);
    grmp_free(ctx, dval, (size_t)nfixed * 8);
    grmp_free(ctx, ud, (size_t)A->nrows * 8);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "dirichlet kernels");
    A->eliminated = (mode == GRMP_DIRICHLET_ELIMINATE);
    return GRMP_OK;
}
