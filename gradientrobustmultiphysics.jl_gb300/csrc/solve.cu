// Sparse solve: CSR SpMV and a persistent Jacobi-preconditioned CG.
//
// Stands in for the LinearSolve.jl call of solve_direct! (src/solvers.jl:
// 89-101, :658-668).  Two modes:
//  * FP64: plain Jacobi-PCG in FP64.
//  * MIXED: Jacobi-PCG in FP32 (FP32 matrix values, FP32 vectors, FP32
//    accumulation) inside an FP64 refinement loop.  The correction is
//    accumulated in FP32 and folded into the FP64 solution whenever the FP32
//    recurrence residual has dropped by `inner_reltol` since the last
//    refinement; then the true residual b - A x is recomputed with the FP64
//    matrix and replaces the FP32 residual ("reliable updates"), keeping the
//    FP32 search direction.  Convergence is decided on the FP64 residual only.
//
// The whole iteration runs in one cooperative launch: three grid barriers per
// iteration (bounded waits, see grid_barrier), dot products reduced through
// per-block partials summed in a fixed order by every block, so all blocks
// take identical decisions and results are reproducible run to run.
#include <cooperative_groups.h>

#include <chrono>
#include <cstring>
#include <mutex>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "grmp_internal.h"

namespace {

constexpr int PTPB = 256;   // threads per block of the persistent kernel
inline int nblk(long long n, int tpb = 256) { return (int)((n + tpb - 1) / tpb); }

struct WorkLayout {
    size_t vec, off_r64, off_part;
};

struct SolveState {
    GridBarrier bar;
    int status;
    int iters;
    int outer;
    int pad;
    double relres;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum NV values over the block; result valid in all threads.
template <int NV>
__device__ __forceinline__ void block_sum(double *v, double *sh /* [32*NV] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < NV; k++) sh[wid * NV + k] = v[k];
    __syncthreads();
    for (int k = 0; k < NV; k++) {
        double s = 0;
        for (int w = 0; w < nw; w++) s += sh[w * NV + k];   // fixed order
        v[k] = s;
    }
    __syncthreads();
}

// Write this block's partial sums, pass a grid barrier, then every block sums
// all partials in the same fixed order.  Returns false on a barrier timeout.
// The partial-sum area holds two buffers used alternately by successive
// reductions (`round` counts them): a block may start writing the next
// reduction's partials while a slower block still reads the previous ones,
// but it cannot reach the reduction after that before every block has left
// this one.
constexpr int kPartStride = 4 * 4096;   // doubles per buffer (4 values x up to 4096 blocks)

template <int NV>
__device__ __forceinline__ bool grid_sum(double *v, double *partial_area, double *sh, SolveState *st, int &round) {
    double *partial = partial_area + (round++ & 1) * kPartStride;
    block_sum<NV>(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) partial[blockIdx.x * 4 + k] = v[k];
    if (!grid_barrier(&st->bar, gridDim.x, &st->status)) return false;
    double acc[NV];
    for (int k = 0; k < NV; k++) acc[k] = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        for (int k = 0; k < NV; k++) acc[k] += __ldcg(&partial[b * 4 + k]);
    block_sum<NV>(acc, sh);
    for (int k = 0; k < NV; k++) v[k] = acc[k];
    return true;
}

// FP32 versions for the inner iteration of the mixed solver: on GB300 the
// FP64 pipe issues about 2 operations per clock per SM, so double-precision
// shuffles and sums in every reduction of every iteration are not free.  The
// summation order is fixed as in the FP64 versions.
template <int NV>
__device__ __forceinline__ void block_sum_f(float *v, float *sh /* [32*NV] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < NV; k++) sh[wid * NV + k] = v[k];
    __syncthreads();
    for (int k = 0; k < NV; k++) {
        float s = 0.f;
        for (int w = 0; w < nw; w++) s += sh[w * NV + k];
        v[k] = s;
    }
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ bool grid_sum_f(float *v, double *partial_area, float *sh, SolveState *st, int &round) {
    float *partial = reinterpret_cast<float *>(partial_area + (round++ & 1) * kPartStride);
    block_sum_f<NV>(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) partial[blockIdx.x * 4 + k] = v[k];
    if (!grid_barrier(&st->bar, gridDim.x, &st->status)) return false;
    float acc[NV];
    for (int k = 0; k < NV; k++) acc[k] = 0.f;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        for (int k = 0; k < NV; k++) acc[k] += __ldcg(&partial[b * 4 + k]);
    block_sum_f<NV>(acc, sh);
    for (int k = 0; k < NV; k++) v[k] = acc[k];
    return true;
}

// Row loop shared by the SpMV variants: groups of TPR lanes per row, each
// lane with U independent (column, value) loads per chunk.  With PIPE the
// loop is software pipelined over the grid-strided rows: while the gathers `x[col]` of the
// current row are in flight, the first chunk of the next row and the bounds
// of the row after it are already being loaded, so a warp keeps the matrix
// stream busy across the dependent gather.  Per-row summation order (chunk
// by chunk, u = 0..U-1 within a chunk, then the lane reduction) does not
// depend on the pipelining.  gather(c) returns x[c]; epi(r, s) consumes the
// row sum (lane 0 of the group).
// Matrix entry sources: CSR arrays (column indices and values apart), or
// the FP32 copy packed as (column, value bits) pairs, one 8-byte load each.
template <typename V>
struct CsrSource {
    const int32_t *__restrict__ cols;
    const V *__restrict__ vals;
    template <typename A>
    __device__ __forceinline__ void get(int idx, int &c, A &v) const {
        c = __ldg(cols + idx);
        v = (A)__ldg(vals + idx);
    }
};

struct PackedSource {
    const int2 *__restrict__ pack;
    __device__ __forceinline__ void get(int idx, int &c, float &v) const {
        const int2 p = __ldg(pack + idx);
        c = p.x;
        v = __int_as_float(p.y);
    }
};

template <int U, int TPR, typename A, typename S>
__device__ __forceinline__ void load_chunk(const S &src, int k, int e, int *c, A *v) {
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int idx = k + u * TPR;
        if (idx < e) {
            src.get(idx, c[u], v[u]);
        } else {
            c[u] = 0;
            v[u] = A(0);
        }
    }
}

template <int TPR, int U, bool PIPE, typename A, typename S, typename G, typename E>
__device__ __forceinline__ void spmv_rows(int n, const int32_t *__restrict__ rowptr, const S src, G gather, E epi) {
    constexpr int RPW = 32 / TPR;   // rows per warp per step
    constexpr int CH = TPR * U;
    const int lane = threadIdx.x & (TPR - 1);
    const int gin = (threadIdx.x & 31) / TPR;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int stride = ((gridDim.x * blockDim.x) >> 5) * RPW;
    if (!PIPE) {
        // plain: bounds, chunk loads and gathers of one row after another
        for (int base = warp * RPW; base < n; base += stride) {
            const int r = base + gin;
            A s = 0;
            if (r < n) {
                const int kb = __ldg(rowptr + r), e = __ldg(rowptr + r + 1);
                for (int k = kb + lane; k < e; k += CH) {
                    int c[U];
                    A v[U];
                    load_chunk<U, TPR>(src, k, e, c, v);
#pragma unroll
                    for (int u = 0; u < U; u++) s += v[u] * gather(c[u]);
                }
            }
#pragma unroll
            for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (r < n && lane == 0) epi(r, s);
        }
        return;
    }
    int r = warp * RPW + gin;
    int kb = 0, e = 0, kbn = 0, en = 0;
    if (r < n) {
        kb = __ldg(rowptr + r);
        e = __ldg(rowptr + r + 1);
    }
    if (r + stride < n) {
        kbn = __ldg(rowptr + r + stride);
        en = __ldg(rowptr + r + stride + 1);
    }
    int c[U];
    A v[U];
    load_chunk<U, TPR>(src, kb + lane, e, c, v);
    for (int base = warp * RPW; base < n; base += stride) {
        // next row: first chunk; the row after: bounds
        int cn[U];
        A vn[U];
        load_chunk<U, TPR>(src, kbn + lane, en, cn, vn);
        const int r2 = r + 2 * stride;
        int kb2 = 0, e2 = 0;
        if (r2 < n) {
            kb2 = __ldg(rowptr + r2);
            e2 = __ldg(rowptr + r2 + 1);
        }
        A s = 0;
#pragma unroll
        for (int u = 0; u < U; u++) s += v[u] * gather(c[u]);
        for (int k = kb + lane + CH; k < e; k += CH) {   // rows longer than one chunk
            int c2[U];
            A v2[U];
            load_chunk<U, TPR>(src, k, e, c2, v2);
#pragma unroll
            for (int u = 0; u < U; u++) s += v2[u] * gather(c2[u]);
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (r < n && lane == 0) epi(r, s);
        r += stride;
        kb = kbn;
        e = en;
        kbn = kb2;
        en = e2;
#pragma unroll
        for (int u = 0; u < U; u++) {
            c[u] = cn[u];
            v[u] = vn[u];
        }
    }
}

// y = A x over the rows of this grid.  If DOT, returns this thread's share
// of sum_r w[r]*y[r].  If RESID, y = b - A x (and DOT gives sum y^2).  The
// matrix is read-only for the whole solve (non-coherent path); x is written
// by other blocks between barriers (coherent loads).
template <int TPR, int U, bool PIPE, typename V, typename X, typename Y, bool DOT, bool RESID>
__device__ __forceinline__ double spmv_grid(int n, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                            const V *__restrict__ vals, const X *x, Y *y, const Y *w,
                                            const double *b) {
    using A = typename std::conditional<sizeof(V) == 8, double, float>::type;
    double dot = 0;
    A dacc = 0;
    spmv_rows<TPR, U, PIPE, A>(
        n, rowptr, CsrSource<V>{cols, vals}, [&](int c) { return (A)x[c]; },
        [&](int r, A s) {
            if (RESID) {
                double v = b[r] - (double)s;
                y[r] = (Y)v;
                if (DOT) dot += v * v;
            } else {
                y[r] = (Y)s;
                if (DOT) dacc += (A)w[r] * s;   // FP32 partial in the FP32 path
            }
        });
    return dot + (double)dacc;
}

// ------------------------------------------------------------------ FP64 PCG
template <int TPR, int U, bool PIPE>
__global__ void __launch_bounds__(PTPB, PIPE && U >= 8 ? 2 : 4) k_pcg64(int n, const int32_t *rowptr, const int32_t *cols,
                                                const double *vals, const double *b, double *x, const double *dinv,
                                                double *r, double *z, double *p, double *q, double *partial,
                                                SolveState *st, double abstol, double reltol, int maxit, int guess) {
    __shared__ double sh[32 * 4];
    int round = 0;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsz = gridDim.x * blockDim.x;
    // r = b - A x  (or b)
    if (guess) spmv_grid<TPR, U, PIPE, double, double, double, false, true>(n, rowptr, cols, vals, x, r, nullptr, b);
    if (!grid_barrier(&st->bar, gridDim.x, &st->status)) return;
    double v[3] = {0, 0, 0};
    for (int i = gtid; i < n; i += gsz) {
        double ri = guess ? r[i] : b[i];
        if (!guess) { r[i] = ri; x[i] = 0.0; }
        double zi = dinv[i] * ri;
        z[i] = zi;
        p[i] = zi;
        v[0] += ri * zi;
        v[1] += ri * ri;
        v[2] += b[i] * b[i];
    }
    if (!grid_sum<3>(v, partial, sh, st, round)) return;
    double rz = v[0], rr = v[1];
    const double bn = sqrt(v[2]);
    const double tol = fmax(abstol, reltol * bn);
    int it = 0;
    bool conv = sqrt(rr) <= tol;
    while (!conv && it < maxit) {
        double d[1];
        d[0] = spmv_grid<TPR, U, PIPE, double, double, double, true, false>(n, rowptr, cols, vals, p, q, p, nullptr);
        if (!grid_sum<1>(d, partial, sh, st, round)) return;
        const double pq = d[0];
        if (!(pq > 0) || !isfinite(pq)) {
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        const double alpha = rz / pq;
        double w[2] = {0, 0};
        for (int i = gtid; i < n; i += gsz) {
            x[i] += alpha * p[i];
            double ri = r[i] - alpha * q[i];
            r[i] = ri;
            double zi = dinv[i] * ri;
            z[i] = zi;
            w[0] += ri * zi;
            w[1] += ri * ri;
        }
        if (!grid_sum<2>(w, partial, sh, st, round)) return;
        it++;
        rr = w[1];
        conv = sqrt(rr) <= tol;
        if (conv) break;
        const double beta = w[0] / rz;
        rz = w[0];
        for (int i = gtid; i < n; i += gsz) p[i] = z[i] + beta * p[i];
        if (!grid_barrier(&st->bar, gridDim.x, &st->status)) return;
    }
    // true residual in FP64
    if (!grid_barrier(&st->bar, gridDim.x, &st->status)) return;
    double t[1];
    t[0] = spmv_grid<TPR, U, PIPE, double, double, double, true, true>(n, rowptr, cols, vals, x, r, nullptr, b);
    if (!grid_sum<1>(t, partial, sh, st, round)) return;
    if (gtid == 0) {
        st->iters = it;
        st->outer = 0;
        st->relres = sqrt(t[0]) / (bn > 0 ? bn : 1.0);
        if (st->status == 0 && !(sqrt(t[0]) <= fmax(tol, 0.0) || conv)) st->status = GRMP_ERR_NOT_CONVERGED;
    }
}

// ------------------------------------------------------------------ mixed PCG
// FP32 SpMV fused with the search-direction update.  The preconditioned
// residual z and the search direction p are stored interleaved (float2) and
// double-buffered: `cur` holds (z_k, p_{k-1}), the SpMV gathers
// p_k = z_k + beta p_{k-1} on the fly (one 8-byte load per nonzero, the same
// fmaf everywhere so all readers see identical values), the owner of row r
// stores p_k(r) into nxt[r].y, and phase B stores z_{k+1} into nxt[r].x.
// This removes the separate p-update pass and one grid barrier per iteration.
template <int TPR, int U, bool PIPE>
__device__ __forceinline__ float spmv_fused_zp(int n, const int32_t *__restrict__ rowptr, const int2 *__restrict__ pack,
                                               const float2 *cur, float *nxt_f, float *q, float beta) {
    float dacc = 0.f;
    spmv_rows<TPR, U, PIPE, float>(
        n, rowptr, PackedSource{pack},
        [&](int c) {
            const float2 g = cur[c];
            return __fmaf_rn(beta, g.y, g.x);
        },
        [&](int r, float s) {
            const float2 me = cur[r];
            const float pn = __fmaf_rn(beta, me.y, me.x);
            nxt_f[2 * r + 1] = pn;
            q[r] = s;
            dacc += pn * s;
        });
    return dacc;
}

template <int TPR, int U, bool PIPE>
__global__ void __launch_bounds__(PTPB, PIPE ? (U >= 8 ? 3 : (U >= 4 ? 4 : 6)) : (U >= 8 ? 4 : 5)) k_pcg_mixed(int n, const int32_t *rowptr, const int32_t *cols,
                                                    const double *vals64, const int2 *pack32, const double *b,
                                                    double *x, const float *dinv, float *r, float *q, float *xc,
                                                    float2 *zp0, float2 *zp1, double *r64, double *partial,
                                                    SolveState *st, double abstol, double reltol, double delta,
                                                    int maxit, int maxouter, int guess) {
    __shared__ double sh[32 * 4];
    __shared__ float shf[32 * 4];
    int round = 0;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsz = gridDim.x * blockDim.x;
    // FP64 residual of the initial guess
    double v[2] = {0, 0};
    if (guess) {
        v[0] = spmv_grid<TPR, U, PIPE, double, double, double, true, true>(n, rowptr, cols, vals64, x, r64, nullptr, b);
    } else {
        for (int i = gtid; i < n; i += gsz) {
            x[i] = 0.0;
            r64[i] = b[i];
            v[0] += b[i] * b[i];
        }
    }
    for (int i = gtid; i < n; i += gsz) v[1] += b[i] * b[i];
    if (!grid_sum<2>(v, partial, sh, st, round)) return;
    const double bn = sqrt(v[1]);
    const double tol = fmax(abstol, reltol * bn);
    double rn64 = sqrt(v[0]);
    int it = 0, outer = 0;
    bool conv = rn64 <= tol;
    // FP32 state from the FP64 residual; p_{-1} = 0
    float wf0 = 0.f, wf1 = 0.f;
    for (int i = gtid; i < n; i += gsz) {
        float ri = (float)r64[i];
        float zi = dinv[i] * ri;
        r[i] = ri;
        zp0[i] = make_float2(zi, 0.f);
        xc[i] = 0.0f;
        wf0 += ri * zi;
        wf1 += ri * ri;
    }
    double w[2] = {(double)wf0, (double)wf1};
    if (!grid_sum<2>(w, partial, sh, st, round)) return;
    // inner-iteration scalars in FP32 (every thread computes them; the FP64
    // pipe is scarce): rz, the FP32 residual norms, alpha, beta
    float rz = (float)w[0];
    float rmax = sqrtf((float)w[1]);
    const float tolf = (float)tol, deltaf = (float)delta;
    double prev_rn64 = rn64;
    int stall = 0;
    float beta = 0.f;
    float2 *cur = zp0, *nxt = zp1;
    while (!conv && it < maxit && outer < maxouter) {
        float *nxt_f = reinterpret_cast<float *>(nxt);
        float d[1] = {spmv_fused_zp<TPR, U, PIPE>(n, rowptr, pack32, cur, nxt_f, q, beta)};
        if (!grid_sum_f<1>(d, partial, shf, st, round)) return;   // barrier 1
        const float pq = d[0];
        if (!(pq > 0.f) || !isfinite(pq)) {
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        const float alpha = rz / pq;
        float uf0 = 0.f, uf1 = 0.f;
        for (int i = gtid; i < n; i += gsz) {
            const float pi = nxt_f[2 * i + 1];
            xc[i] += alpha * pi;
            float ri = r[i] - alpha * q[i];
            r[i] = ri;
            float zi = dinv[i] * ri;
            nxt_f[2 * i] = zi;
            uf0 += ri * zi;
            uf1 += ri * ri;
        }
        float u[2] = {uf0, uf1};
        if (!grid_sum_f<2>(u, partial, shf, st, round)) return;   // barrier 2
        it++;
        float rz_new = u[0];
        const float rn32 = sqrtf(u[1]);
        bool restart = false;
        if (rn32 <= deltaf * rmax || rn32 <= tolf || it >= maxit) {
            // refinement: fold the FP32 correction into x, recompute b - A x in FP64
            for (int i = gtid; i < n; i += gsz) {
                x[i] += (double)xc[i];
                xc[i] = 0.0f;
            }
            if (!grid_barrier(&st->bar, gridDim.x, &st->status)) return;
            double t[1];
            t[0] = spmv_grid<TPR, U, PIPE, double, double, double, true, true>(n, rowptr, cols, vals64, x, r64, nullptr, b);
            if (!grid_sum<1>(t, partial, sh, st, round)) return;
            outer++;
            rn64 = sqrt(t[0]);
            conv = rn64 <= tol;
            if (conv || it >= maxit) break;
            // Keeping the FP32 search direction across a refinement is exact only
            // while the FP32 matrix is a uniform rounding of the FP64 one; when the
            // true residual stops falling (FP32 element matrices of nearly
            // incompressible elasticity lose the soft modes to cancellation),
            // restart the inner CG: classical iterative refinement.
            restart = rn64 > 0.5 * prev_rn64;
            stall = (rn64 > 0.9 * prev_rn64) ? stall + 1 : 0;
            prev_rn64 = rn64;
            if (stall >= 16) break;   // no progress: report NOT_CONVERGED
            float yf0 = 0.f, yf1 = 0.f;
            for (int i = gtid; i < n; i += gsz) {
                float ri = (float)r64[i];
                float zi = dinv[i] * ri;
                r[i] = ri;
                nxt_f[2 * i] = zi;
                yf0 += ri * zi;
                yf1 += ri * ri;
            }
            float y[2] = {yf0, yf1};
            if (!grid_sum_f<2>(y, partial, shf, st, round)) return;
            rz_new = y[0];
            rmax = sqrtf(y[1]);
        }
        beta = restart ? 0.0f : rz_new / rz;
        rz = rz_new;
        float2 *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    if (gtid == 0) {
        st->iters = it;
        st->outer = outer;
        st->relres = rn64 / (bn > 0 ? bn : 1.0);
        if (st->status == 0 && !conv) st->status = GRMP_ERR_NOT_CONVERGED;
    }
}

// ------------------------------------------------------------------ helpers
// FP32 copy of the matrix packed as (column, value bits) pairs for the mixed
// solver's SpMV (one 8-byte load per nonzero instead of two 4-byte loads).
__global__ void k_pack32(long long nnz, const int32_t *cols, const float *vals, int2 *pack) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) pack[k] = make_int2(cols[k], __float_as_int(vals[k]));
}

template <typename V>
__global__ void k_dinv(int n, const int32_t *rowptr, const int32_t *cols, const V *vals, V *dinv, int *bad) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V d = 0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (cols[k] == i) d = vals[k];
    if (!(d > 0) || !isfinite((double)d)) {
        atomicExch(bad, 1);
        dinv[i] = V(1);
    } else {
        dinv[i] = V(1) / d;
    }
}

template <int TPR, typename V, typename X>
__global__ void __launch_bounds__(256) k_spmv(int n, const int32_t *rowptr, const int32_t *cols, const V *vals,
                                              const X *x, X *y) {
    spmv_grid<TPR, TPR >= 16 ? 2 : 4, false, V, X, X, false, false>(n, rowptr, cols, vals, x, y, nullptr, nullptr);
}

__global__ void k_f64_to_f32(const double *a, float *b, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}
__global__ void k_f32_to_f64v(const float *a, double *b, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (double)a[i];
}

template <typename V, typename X>
void launch_spmv(int tpr, int grid, cudaStream_t s, int n, const int32_t *rp, const int32_t *ci, const V *v, const X *x,
                 X *y) {
    switch (tpr) {
        case 1: k_spmv<1, V, X><<<grid, 256, 0, s>>>(n, rp, ci, v, x, y); break;
        case 2: k_spmv<2, V, X><<<grid, 256, 0, s>>>(n, rp, ci, v, x, y); break;
        case 4: k_spmv<4, V, X><<<grid, 256, 0, s>>>(n, rp, ci, v, x, y); break;
        case 8: k_spmv<8, V, X><<<grid, 256, 0, s>>>(n, rp, ci, v, x, y); break;
        case 16: k_spmv<16, V, X><<<grid, 256, 0, s>>>(n, rp, ci, v, x, y); break;
        default: k_spmv<32, V, X><<<grid, 256, 0, s>>>(n, rp, ci, v, x, y); break;
    }
}

// SpMV configurations of the persistent solvers: (lanes per row, loads in
// flight per lane), encoded 100*TPR + U.
constexpr int kConfigs[] = {208, 404, 408, 804, 1602, 10204, 10404, 10408, 10804, 10402, 10802};

int heuristic_tpr(grmp_matrix A) {
    double avg = (double)A->nnz / (double)std::max(1, A->nrows);
    if (avg <= 3) return 2;
    if (avg <= 6) return 4;
    if (avg <= 14) return 8;
    if (avg <= 40) return 16;
    return 32;
}

int heuristic_config(grmp_matrix A) {
    double avg = (double)A->nnz / (double)std::max(1, A->nrows);
    if (avg <= 8) return 208;
    if (avg <= 20) return 404;
    return 408;
}

template <typename K>
int coop_grid(grmp_context ctx, K kern, int n, int want) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PTPB, 0);
    int maxg = std::max(1, per_sm) * ctx->num_sms;
    int need = std::max(1, nblk(n, PTPB));
    int g = want > 0 ? std::min(want, maxg) : std::min(maxg, need);
    return std::max(1, g);
}

template <int TPR, int U, bool PIPE>
int launch_pcg(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p, grmp_solve_stats *out,
               char *work, SolveState *dst, WorkLayout lay) {
    grmp_context ctx = A->space->mesh->ctx;
    int n = A->nrows;
    bool mixed = p->mode == GRMP_SOLVE_MIXED;
    int guess = p->use_initial_guess ? 1 : 0;
    int grid;
    cudaError_t e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(dst, 0, sizeof(SolveState), ctx->stream);
    if (!mixed) {
        auto kern = k_pcg64<TPR, U, PIPE>;
        grid = coop_grid(ctx, kern, n, p->grid_blocks);
        double *dinv = (double *)work, *r = (double *)(work + lay.vec), *z = (double *)(work + 2 * lay.vec);
        double *pp = (double *)(work + 3 * lay.vec), *q = (double *)(work + 4 * lay.vec);
        double *part = (double *)(work + lay.off_part);
        int nn = n, mi = p->maxiter;
        double at = p->abstol, rt = p->reltol;
        const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
        const double *vv = A->d_vals64, *bb = bvec;
        double *xx = xvec;
        void *args[] = {&nn, &rp, &ci, &vv, &bb, &xx, &dinv, &r, &z, &pp, &q, &part, &dst, &at, &rt, &mi, &guess};
        cudaEventRecord(e0, ctx->stream);
        e = cudaLaunchCooperativeKernel((void *)kern, grid, PTPB, args, 0, ctx->stream);
        GRMP_LAUNCHED(ctx);
        cudaEventRecord(e1, ctx->stream);
    } else {
        auto kern = k_pcg_mixed<TPR, U, PIPE>;
        grid = coop_grid(ctx, kern, n, p->grid_blocks);
        float *dinv = (float *)work, *r = (float *)(work + lay.vec), *q = (float *)(work + 2 * lay.vec);
        float *xc = (float *)(work + 3 * lay.vec);
        float2 *zp0 = (float2 *)(work + 4 * lay.vec), *zp1 = (float2 *)(work + 6 * lay.vec);
        double *r64 = (double *)(work + lay.off_r64);
        double *part = (double *)(work + lay.off_part);
        int nn = n, mi = p->maxiter, mo = p->max_outer > 0 ? p->max_outer : 1000;
        double at = p->abstol, rt = p->reltol, dl = p->inner_reltol > 0 && p->inner_reltol < 1 ? p->inner_reltol : 0.1;
        const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
        const double *v64 = A->d_vals64, *bb = bvec;
        const int2 *v32 = (const int2 *)A->d_pack32;
        double *xx = xvec;
        void *args[] = {&nn, &rp, &ci, &v64, &v32, &bb, &xx, &dinv, &r, &q, &xc, &zp0, &zp1, &r64, &part, &dst,
                        &at, &rt, &dl, &mi, &mo, &guess};
        cudaEventRecord(e0, ctx->stream);
        e = cudaLaunchCooperativeKernel((void *)kern, grid, PTPB, args, 0, ctx->stream);
        GRMP_LAUNCHED(ctx);
        cudaEventRecord(e1, ctx->stream);
    }
    SolveState hs;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "persistent PCG launch");
    out->status = hs.status;
    out->iterations = hs.iters;
    out->outer_iterations = hs.outer;
    out->final_relres = hs.relres;
    out->spmv_config = 100 * TPR + U + (PIPE ? 10000 : 0);
    out->grid_blocks = grid;
    out->solve_ms = ms;
    if (hs.status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, GRMP_ERR_NOT_CONVERGED, "PCG: %d iterations, relative residual %.3e", hs.iters, hs.relres);
    if (hs.status == GRMP_ERR_TIMEOUT) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "PCG: a grid barrier wait timed out");
    if (hs.status == GRMP_ERR_NAN) return grmp_fail(ctx, GRMP_ERR_NAN, "PCG: breakdown (non-positive or non-finite p.Ap)");
    return hs.status;
}

int dispatch_pcg(int cfg, grmp_matrix A, const double *b, double *x, const grmp_solve_params *p, grmp_solve_stats *st,
                 char *work, SolveState *dst, WorkLayout lay) {
    switch (cfg) {
        case 208: return launch_pcg<2, 8, false>(A, b, x, p, st, work, dst, lay);
        case 404: return launch_pcg<4, 4, false>(A, b, x, p, st, work, dst, lay);
        case 408: return launch_pcg<4, 8, false>(A, b, x, p, st, work, dst, lay);
        case 804: return launch_pcg<8, 4, false>(A, b, x, p, st, work, dst, lay);
        case 1602: return launch_pcg<16, 2, false>(A, b, x, p, st, work, dst, lay);
        case 10204: return launch_pcg<2, 4, true>(A, b, x, p, st, work, dst, lay);
        case 10404: return launch_pcg<4, 4, true>(A, b, x, p, st, work, dst, lay);
        case 10408: return launch_pcg<4, 8, true>(A, b, x, p, st, work, dst, lay);
        case 10804: return launch_pcg<8, 4, true>(A, b, x, p, st, work, dst, lay);
        case 10402: return launch_pcg<4, 2, true>(A, b, x, p, st, work, dst, lay);
        case 10802: return launch_pcg<8, 2, true>(A, b, x, p, st, work, dst, lay);
    }
    return grmp_fail(A->space->mesh->ctx, GRMP_ERR_INVALID_ARG, "spmv_config: unknown configuration %d", cfg);
}

// Autotuner: run each configuration for a few iterations of the real solve
// on this matrix and right-hand side (into a scratch solution vector) and keep
// the one with the lowest time per iteration.  The persistent kernel's
// occupancy, barriers and vector phases are part of what is measured.
int autotune_config(grmp_matrix A, const grmp_vector_s *b, const grmp_solve_params *p, char *work, SolveState *dst,
                    WorkLayout lay) {
    grmp_context ctx = A->space->mesh->ctx;
    if (A->nrows < 20000) return heuristic_config(A);
    double *xs = nullptr;
    if (grmp_alloc(ctx, (void **)&xs, (size_t)A->nrows * 8)) return heuristic_config(A);
    grmp_solve_params q = *p;
    q.maxiter = 24;
    q.use_initial_guess = 0;
    q.reltol = 0.0;
    q.abstol = 0.0;
    int best = heuristic_config(A);
    double bt = 1e30;
    for (int cfg : kConfigs) {
        grmp_solve_stats s{};
        dispatch_pcg(cfg, A, b->d, xs, &q, &s, work, dst, lay);   // warm-up: first launch of this instantiation
        s = grmp_solve_stats{};
        dispatch_pcg(cfg, A, b->d, xs, &q, &s, work, dst, lay);
        if (s.iterations > 0) {
            double per = s.solve_ms / s.iterations;
            if (per < bt) {
                bt = per;
                best = cfg;
            }
        }
    }
    grmp_free(ctx, xs, (size_t)A->nrows * 8);
    ctx->last_error.clear();
    return best;
}

}  // namespace

int grmp_solve_impl(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *p, grmp_solve_stats *st) {
    grmp_context ctx = A->space->mesh->ctx;
    std::memset(st, 0, sizeof(*st));
    bool mixed = p->mode == GRMP_SOLVE_MIXED;
    if (!A->has64) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: FP64 values not assembled");
    if (mixed && !A->has32) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: MIXED needs FP32 values too");
    int n = A->nrows;
    // workspace, each array 256-byte aligned:
    //   FP64 : dinv r z p q (double)                  | partials | state
    //   MIXED: dinv r z p q xc (float) | r64 (double)  | partials | state
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t pbytes = (size_t)2 * kPartStride * 8;   // two alternating partial-sum buffers
    size_t vec = mixed ? al((size_t)n * 4) : al((size_t)n * 8);
    size_t nvec = mixed ? 8 : 5;   // MIXED: dinv r q xc (float) + two interleaved (z, p) float2 buffers
    size_t off_r64 = nvec * vec;
    size_t off_part = off_r64 + (mixed ? al((size_t)n * 8) : 0);
    size_t off_state = off_part + al(pbytes);
    size_t need = off_state + al(sizeof(SolveState));
    if (A->work_bytes < need) {
        grmp_free(ctx, A->d_work, A->work_bytes);
        A->work_bytes = 0;
        int rc = grmp_alloc(ctx, &A->d_work, need);
        if (rc) return rc;
        A->work_bytes = need;
    }
    char *work = (char *)A->d_work;
    SolveState *dst = (SolveState *)(work + off_state);
    WorkLayout lay{vec, off_r64, off_part};
    cudaMemsetAsync(dst, 0, sizeof(SolveState), ctx->stream);
    // Jacobi preconditioner
    int *bad = nullptr;
    int rc = grmp_alloc(ctx, (void **)&bad, 4);
    if (rc) return rc;
    cudaMemsetAsync(bad, 0, 4, ctx->stream);
    if (mixed)
        k_dinv<float><<<nblk(n), 256, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals32, (float *)work, bad);
    else
        k_dinv<double><<<nblk(n), 256, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, (double *)work, bad);
    GRMP_LAUNCHED(ctx);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, bad, 4);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "jacobi diagonal");
    if (hbad) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: non-positive or non-finite diagonal entry");
    if (mixed) {   // refresh the packed FP32 copy (values may have been reassembled)
        const size_t pb = (size_t)A->nnz * 8;
        if (!A->d_pack32) {
            int prc = grmp_alloc(ctx, &A->d_pack32, pb);
            if (prc) return prc;
        }
        k_pack32<<<(unsigned)((A->nnz + 255) / 256), 256, 0, ctx->stream>>>(A->nnz, A->d_cols, A->d_vals32,
                                                                           (int2 *)A->d_pack32);
        GRMP_LAUNCHED(ctx);
    }
    int cfg = p->spmv_config;
    if (cfg == 0) {   // autotuned once per matrix and solver mode
        int &slot = mixed ? A->tuned_cfg32 : A->tuned_cfg;
        if (!slot) slot = autotune_config(A, b, p, work, dst, lay);
        cfg = slot;
    } else if (cfg < 0) {   // heuristic from the row length: no timing, independent of other work on the GPU
        cfg = heuristic_config(A);
    }
    return dispatch_pcg(cfg, A, b->d, x->d, p, st, work, dst, lay);
}

int grmp_spmv_impl(grmp_matrix A, int precision, grmp_vector x, grmp_vector y) {
    grmp_context ctx = A->space->mesh->ctx;
    int n = A->nrows;
    int tpr = A->tuned_cfg ? A->tuned_cfg / 100 : heuristic_tpr(A);
    int grid = std::min(nblk(n, 256 / tpr), ctx->num_sms * 16);
    if (precision == GRMP_FP64) {
        if (!A->has64) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "spmv: no FP64 values");
        launch_spmv<double, double>(tpr, grid, ctx->stream, n, A->d_rowptr, A->d_cols, A->d_vals64, x->d, y->d);
        GRMP_LAUNCHED(ctx);
    } else {
        if (!A->has32) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "spmv: no FP32 values");
        float *xf = nullptr, *yf = nullptr;
        int rc = grmp_alloc(ctx, (void **)&xf, (size_t)n * 4);
        if (!rc) rc = grmp_alloc(ctx, (void **)&yf, (size_t)n * 4);
        if (rc) {
            grmp_free(ctx, xf, (size_t)n * 4);
            return rc;
        }
        k_f64_to_f32<<<nblk(n), 256, 0, ctx->stream>>>(x->d, xf, n); GRMP_LAUNCHED(ctx);
        launch_spmv<float, float>(tpr, grid, ctx->stream, n, A->d_rowptr, A->d_cols, A->d_vals32, xf, yf);
        GRMP_LAUNCHED(ctx);
        k_f32_to_f64v<<<nblk(n), 256, 0, ctx->stream>>>(yf, y->d, n); GRMP_LAUNCHED(ctx);
        grmp_free(ctx, xf, (size_t)n * 4);
        grmp_free(ctx, yf, (size_t)n * 4);
    }
    GRMP_CUDA(ctx, cudaGetLastError());
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GRMP_OK;
}

// ---------------------------------------------------------------------------
// FP64 PCG without device allocation (grmp_solve_fp64_noalloc).
//
// The work arrays are a file-scope device array sized for
// GRMP_NOALLOC_MAX_ROWS rows, laid out like the FP64 workspace of
// grmp_solve_impl:
//   [0, 5V)           dinv r z p q   (V = GRMP_NOALLOC_MAX_ROWS doubles each)
//   [5V, 5V+P)        per-block reduction partials (two buffers of 4 x 4096 doubles)
//   [5V+P, +256)      SolveState: grid-barrier counters + status  (zeroed per call)
//   [5V+P+256, +256)  diagonal check flag                          (zeroed per call)
// The array's address is looked up once per device; the first call makes
// that lookup with the context's device current.
namespace {

constexpr size_t kNaVec = (size_t)GRMP_NOALLOC_MAX_ROWS * 8;
constexpr size_t kNaPart = (size_t)2 * kPartStride * 8;
constexpr size_t kNaState = 5 * kNaVec + kNaPart;
constexpr size_t kNaFlag = kNaState + 256;
constexpr size_t kNaBytes = kNaFlag + 256;
static_assert(kNaVec % 256 == 0 && sizeof(SolveState) <= 256, "scratch layout");

__device__ __align__(256) char g_noalloc_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
char *g_na_ptr[kNaMaxDevices] = {};

int noalloc_scratch(grmp_context ctx, char **out) {
    if (ctx->device < 0 || ctx->device >= kNaMaxDevices)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "noalloc solve: device ordinal %d out of range", ctx->device);
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[ctx->device]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return grmp_cuda_fail(ctx, e, "noalloc solve: scratch address lookup");
        g_na_ptr[ctx->device] = (char *)ptr;
    }
    *out = g_na_ptr[ctx->device];
    return GRMP_OK;
}

template <int TPR, int U, bool PIPE>
cudaError_t launch_pcg64_static(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p,
                                char *work, int *grid_out) {
    grmp_context ctx = A->space->mesh->ctx;
    auto kern = k_pcg64<TPR, U, PIPE>;
    int grid = coop_grid(ctx, kern, A->nrows, p->grid_blocks);
    double *dinv = (double *)work, *r = (double *)(work + kNaVec), *z = (double *)(work + 2 * kNaVec);
    double *pp = (double *)(work + 3 * kNaVec), *q = (double *)(work + 4 * kNaVec);
    double *part = (double *)(work + 5 * kNaVec);
    SolveState *dst = (SolveState *)(work + kNaState);
    int nn = A->nrows, mi = p->maxiter, guess = p->use_initial_guess ? 1 : 0;
    double at = p->abstol, rt = p->reltol;
    const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
    const double *vv = A->d_vals64, *bb = bvec;
    double *xx = xvec;
    void *args[] = {&nn, &rp, &ci, &vv, &bb, &xx, &dinv, &r, &z, &pp, &q, &part, &dst, &at, &rt, &mi, &guess};
    *grid_out = grid;
    cudaError_t e = cudaLaunchCooperativeKernel((void *)kern, grid, PTPB, args, 0, ctx->stream);
    GRMP_LAUNCHED(ctx);
    return e;
}

}  // namespace

extern "C" int grmp_solve_fp64_noalloc(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *p,
                                       grmp_solve_stats *st) {
    if (!A || !b || !x || !p) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = A->space->mesh->ctx;
    grmp_solve_stats local;
    if (!st) st = &local;
    std::memset(st, 0, sizeof(*st));
    if (b->n != A->nrows || x->n != A->nrows) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: size mismatch");
    if (p->mode != GRMP_SOLVE_FP64)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "noalloc solve: only mode GRMP_SOLVE_FP64");
    if (!(p->reltol >= 0) || !(p->abstol >= 0) || p->maxiter <= 0) return GRMP_ERR_INVALID_ARG;
    if (A->nrows > GRMP_NOALLOC_MAX_ROWS)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: %d rows exceed the fixed scratch limit of %d rows",
                         A->nrows, GRMP_NOALLOC_MAX_ROWS);
    if (!A->has64) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: FP64 values not assembled");
    const auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    char *work = nullptr;
    int rc = noalloc_scratch(ctx, &work);
    if (rc) return rc;
    const int n = A->nrows;
    SolveState *dst = (SolveState *)(work + kNaState);
    int *bad = (int *)(work + kNaFlag);
    cudaError_t e = cudaMemsetAsync(work + kNaState, 0, 512, ctx->stream);   // state + flag start at zero
    if (e == cudaSuccess) {
        k_dinv<double><<<nblk(n), 256, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, (double *)work, bad);
        GRMP_LAUNCHED(ctx);
        e = cudaGetLastError();
    }
    int hbad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "noalloc solve: jacobi diagonal");
    if (hbad) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: non-positive or non-finite diagonal entry");
    int cfg = p->spmv_config > 0 ? p->spmv_config : (A->tuned_cfg ? A->tuned_cfg : heuristic_config(A));
    int grid = 0;
    switch (cfg) {
        case 208: e = launch_pcg64_static<2, 8, false>(A, b->d, x->d, p, work, &grid); break;
        case 404: e = launch_pcg64_static<4, 4, false>(A, b->d, x->d, p, work, &grid); break;
        case 408: e = launch_pcg64_static<4, 8, false>(A, b->d, x->d, p, work, &grid); break;
        case 804: e = launch_pcg64_static<8, 4, false>(A, b->d, x->d, p, work, &grid); break;
        case 1602: e = launch_pcg64_static<16, 2, false>(A, b->d, x->d, p, work, &grid); break;
        case 10204: e = launch_pcg64_static<2, 4, true>(A, b->d, x->d, p, work, &grid); break;
        case 10404: e = launch_pcg64_static<4, 4, true>(A, b->d, x->d, p, work, &grid); break;
        case 10408: e = launch_pcg64_static<4, 8, true>(A, b->d, x->d, p, work, &grid); break;
        case 10804: e = launch_pcg64_static<8, 4, true>(A, b->d, x->d, p, work, &grid); break;
        case 10402: e = launch_pcg64_static<4, 2, true>(A, b->d, x->d, p, work, &grid); break;
        case 10802: e = launch_pcg64_static<8, 2, true>(A, b->d, x->d, p, work, &grid); break;
        default: return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "spmv_config: unknown configuration %d", cfg);
    }
    SolveState hs;
    std::memset(&hs, 0, sizeof(hs));
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "noalloc solve: persistent PCG launch");
    st->status = hs.status;
    st->iterations = hs.iters;
    st->outer_iterations = 0;
    st->final_relres = hs.relres;
    st->spmv_config = cfg;
    st->grid_blocks = grid;
    st->solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (hs.status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, GRMP_ERR_NOT_CONVERGED, "PCG: %d iterations, relative residual %.3e", hs.iters, hs.relres);
    if (hs.status == GRMP_ERR_TIMEOUT) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "PCG: a grid barrier wait timed out");
    if (hs.status == GRMP_ERR_NAN) return grmp_fail(ctx, GRMP_ERR_NAN, "PCG: breakdown (non-positive or non-finite p.Ap)");
    return hs.status;
}
