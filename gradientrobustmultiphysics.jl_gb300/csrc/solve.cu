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
// The whole iteration runs in one persistent launch: a cooperative grid over
// the GPU (three grid barriers per FP64 iteration, two per mixed one; bounded
// waits, see grid_barrier) or, for the smallest systems, one thread-block
// cluster (hardware cluster barriers, see ClusterSync).  Dot products are
// reduced through per-block partials summed in a fixed order by every block,
// so all blocks take identical decisions and results are reproducible run to
// run.
#include <cooperative_groups.h>

#include <chrono>
#include <cstring>
#include <mutex>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "duo.h"
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

// Sum NV values over the block; result valid in all threads.  Warp sums,
// then warp 0 sums the per-warp values with the same fixed shuffle tree and
// publishes the totals: one thread's worth of additions per value instead of
// every thread re-adding all warps' values (on GB300 that redundant work lands
// on the narrow FP64 pipe).
template <int NV, typename T>
__device__ __forceinline__ void block_sum_t(T *v, T *sh /* [32*NV] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < NV; k++) sh[wid * NV + k] = v[k];
    __syncthreads();
    if (wid == 0) {
        T a[NV];
        for (int k = 0; k < NV; k++) a[k] = lane < nw ? sh[lane * NV + k] : T(0);
        for (int k = 0; k < NV; k++) a[k] = warp_sum(a[k]);
        if (lane == 0)
            for (int k = 0; k < NV; k++) sh[k] = a[k];
    }
    __syncthreads();
    for (int k = 0; k < NV; k++) v[k] = sh[k];
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_sum(double *v, double *sh /* [32*NV] */) {
    block_sum_t<NV, double>(v, sh);
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
__device__ __forceinline__ bool grid_sum(double *v, double *partial_area, double *sh, SolveState *st, int &round,
                                         long long spin) {
    double *partial = partial_area + (round++ & 1) * kPartStride;
    block_sum<NV>(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) partial[blockIdx.x * 4 + k] = v[k];
    if (!grid_barrier(&st->bar, gridDim.x, &st->status, spin)) return false;
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
    block_sum_t<NV, float>(v, sh);
}

template <int NV>
__device__ __forceinline__ bool grid_sum_f(float *v, double *partial_area, float *sh, SolveState *st, int &round,
                                           long long spin) {
    float *partial = reinterpret_cast<float *>(partial_area + (round++ & 1) * kPartStride);
    block_sum_f<NV>(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) partial[blockIdx.x * 4 + k] = v[k];
    if (!grid_barrier(&st->bar, gridDim.x, &st->status, spin)) return false;
    float acc[NV];
    for (int k = 0; k < NV; k++) acc[k] = 0.f;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        for (int k = 0; k < NV; k++) acc[k] += __ldcg(&partial[b * 4 + k]);
    block_sum_f<NV>(acc, sh);
    for (int k = 0; k < NV; k++) v[k] = acc[k];
    return true;
}

// Synchronisation policies of the persistent solvers.
//
// GridSync: a cooperative grid over the whole GPU; barriers and reductions
// through global memory (grid_barrier, grid_sum), every wait bounded.
//
// ClusterSync: the whole solve in ONE thread-block cluster (8 or 16 CTAs on
// one GPC) for problems whose matrix and vectors sit in L2: the barrier is
// the hardware cluster barrier (barrier.cluster.arrive.release / wait.acquire,
// the cluster's analogue of __syncthreads: it orders global and shared
// memory at cluster scope), and reductions read each CTA's partial sums out
// of that CTA's shared memory (distributed shared memory) instead of global
// memory.  Every CTA executes the same sequence of barriers -- all decisions
// come from sums that every CTA forms in the same fixed order -- so the
// barrier cannot wait on a CTA that took another path; finish() is a last
// barrier that keeps every CTA's shared memory alive until no CTA reads it.
struct GridSync {
    SolveState *st;
    double *part;
    long long spin;
    int round;
    __device__ __forceinline__ bool barrier() { return grid_barrier(&st->bar, gridDim.x, &st->status, spin); }
    template <int NV>
    __device__ __forceinline__ bool sum(double *v, double *sh) {
        return grid_sum<NV>(v, part, sh, st, round, spin);
    }
    template <int NV>
    __device__ __forceinline__ bool sumf(float *v, float *sh) {
        return grid_sum_f<NV>(v, part, sh, st, round, spin);
    }
    __device__ __forceinline__ void finish() {}
};

namespace cg = cooperative_groups;

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// Sum NV values (already block-summed, valid in every thread) over the CTAs
// of the cluster: thread 0 publishes them in `mine` (this reduction's buffer
// of two, used alternately as in grid_sum), the cluster barrier, then warp 0
// reads every CTA's copy in rank order and sums with a fixed shuffle tree.
template <int NV, typename T>
__device__ __forceinline__ void cluster_combine(T *v, T (*pub)[4], int par, T *sh) {
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) pub[par][k] = v[k];
    cluster_barrier();
    cg::cluster_group cl = cg::this_cluster();
    const int nb = (int)cl.num_blocks();
    if (threadIdx.x < 32) {
        T a[NV];
        for (int k = 0; k < NV; k++) a[k] = T(0);
        if ((int)threadIdx.x < nb) {
            const T *rp = cl.map_shared_rank(&pub[par][0], (unsigned)threadIdx.x);
            for (int k = 0; k < NV; k++) a[k] = rp[k];
        }
        for (int k = 0; k < NV; k++) a[k] = warp_sum(a[k]);
        if (threadIdx.x == 0)
            for (int k = 0; k < NV; k++) sh[k] = a[k];
    }
    __syncthreads();
    for (int k = 0; k < NV; k++) v[k] = sh[k];
    __syncthreads();
}

struct ClusterSync {
    SolveState *st;
    double *part;     // unused: partial sums live in shared memory
    long long spin;   // unused: the cluster barrier is a hardware barrier
    int round;
    __device__ __forceinline__ bool barrier() {
        cluster_barrier();
        return true;
    }
    template <int NV>
    __device__ __forceinline__ bool sum(double *v, double *sh) {
        __shared__ double pub[2][4];
        block_sum<NV>(v, sh);
        cluster_combine<NV, double>(v, pub, round++ & 1, sh);
        return true;
    }
    template <int NV>
    __device__ __forceinline__ bool sumf(float *v, float *sh) {
        __shared__ float pub[2][4];
        block_sum_f<NV>(v, sh);
        cluster_combine<NV, float>(v, pub, round++ & 1, sh);
        return true;
    }
    __device__ __forceinline__ void finish() { cluster_barrier(); }
};

template <bool CL>
using SyncOf = typename std::conditional<CL, ClusterSync, GridSync>::type;

constexpr int kClT = 1024;   // threads per CTA of the cluster solvers

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
template <int TPR, int U, bool PIPE, bool CL = false>
__global__ void __launch_bounds__(CL ? kClT : PTPB, CL ? 1 : (PIPE && U >= 8 ? 2 : 4)) k_pcg64(int n, const int32_t *rowptr, const int32_t *cols,
                                                const double *vals, const double *b, double *x, const double *dinv,
                                                double *r, double *z, double *p, double *q, double *partial,
                                                SolveState *st, double abstol, double reltol, int maxit, int guess,
                                                long long spin) {
    __shared__ double sh[32 * 4];
    SyncOf<CL> sy{st, partial, spin, 0};
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsz = gridDim.x * blockDim.x;
    // r = b - A x  (or b)
    if (guess) spmv_grid<TPR, U, PIPE, double, double, double, false, true>(n, rowptr, cols, vals, x, r, nullptr, b);
    if (!sy.barrier()) return;
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
    if (!sy.template sum<3>(v, sh)) return;
    double rz = v[0], rr = v[1];
    const double bn = sqrt(v[2]);
    const double tol = fmax(abstol, reltol * bn);
    int it = 0;
    bool conv = sqrt(rr) <= tol;
    while (!conv && it < maxit) {
        double d[1];
        d[0] = spmv_grid<TPR, U, PIPE, double, double, double, true, false>(n, rowptr, cols, vals, p, q, p, nullptr);
        if (!sy.template sum<1>(d, sh)) return;
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
        if (!sy.template sum<2>(w, sh)) return;
        it++;
        rr = w[1];
        conv = sqrt(rr) <= tol;
        if (conv) break;
        const double beta = w[0] / rz;
        rz = w[0];
        for (int i = gtid; i < n; i += gsz) p[i] = z[i] + beta * p[i];
        if (!sy.barrier()) return;
    }
    // true residual in FP64
    if (!sy.barrier()) return;
    double t[1];
    t[0] = spmv_grid<TPR, U, PIPE, double, double, double, true, true>(n, rowptr, cols, vals, x, r, nullptr, b);
    if (!sy.template sum<1>(t, sh)) return;
    if (gtid == 0) {
        st->iters = it;
        st->outer = 0;
        st->relres = sqrt(t[0]) / (bn > 0 ? bn : 1.0);
        if (st->status == 0 && !(sqrt(t[0]) <= fmax(tol, 0.0) || conv)) st->status = GRMP_ERR_NOT_CONVERGED;
    }
    sy.finish();
}

// ------------------------------------------------------------------ FP64 BiCGStab
// Jacobi right-preconditioned BiCGStab (van der Vorst 1992) for the
// non-symmetric systems of a Newton step (the Jacobian of a NonlinearForm),
// where the reference hands the matrix to a sparse LU.  Per iteration:
//   p = r + beta (p - omega v), ph = D^-1 p;  v = A ph;  alpha = rho / (rh, v)
//   s = r - alpha v, sh = D^-1 s;  t = A sh;  omega = (t, s) / (t, t)
//   x += alpha ph + omega sh;  r = s - omega t;  rho' = (rh, r)
// Five grid-wide synchronisations; every wait is bounded (`spin`).
template <int TPR, int U>
__global__ void __launch_bounds__(PTPB, 4) k_bicgstab64(int n, const int32_t *rowptr, const int32_t *cols,
                                                         const double *vals, const double *b, double *x,
                                                         const double *dinv, double *r, double *rh, double *p,
                                                         double *v, double *s, double *t, double *ph, double *shv,
                                                         double *partial, SolveState *st, double abstol,
                                                         double reltol, int maxit, int guess, long long spin) {
    __shared__ double sh[32 * 4];
    int round = 0;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsz = gridDim.x * blockDim.x;
    if (guess) spmv_grid<TPR, U, false, double, double, double, false, true>(n, rowptr, cols, vals, x, r, nullptr, b);
    if (!grid_barrier(&st->bar, gridDim.x, &st->status, spin)) return;
    double w3[3] = {0, 0, 0};
    for (int i = gtid; i < n; i += gsz) {
        const double ri = guess ? r[i] : b[i];
        if (!guess) {
            r[i] = ri;
            x[i] = 0.0;
        }
        rh[i] = ri;
        p[i] = 0.0;
        v[i] = 0.0;
        w3[0] += ri * ri;
        w3[1] += ri * ri;
        w3[2] += b[i] * b[i];
    }
    if (!grid_sum<3>(w3, partial, sh, st, round, spin)) return;
    double rho = w3[0], rr = w3[1];
    const double bn = sqrt(w3[2]);
    const double tol = fmax(abstol, reltol * bn);
    double alpha = 1.0, omega = 1.0, beta = 0.0;
    int it = 0;
    bool conv = sqrt(rr) <= tol;
    while (!conv && it < maxit) {
        for (int i = gtid; i < n; i += gsz) {
            const double pi = r[i] + beta * (p[i] - omega * v[i]);
            p[i] = pi;
            ph[i] = dinv[i] * pi;
        }
        if (!grid_barrier(&st->bar, gridDim.x, &st->status, spin)) return;
        double d[1];
        d[0] = spmv_grid<TPR, U, false, double, double, double, true, false>(n, rowptr, cols, vals, ph, v, rh, nullptr);
        if (!grid_sum<1>(d, partial, sh, st, round, spin)) return;
        if (!(d[0] != 0.0) || !isfinite(d[0])) {
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        alpha = rho / d[0];
        double ss[1] = {0};
        for (int i = gtid; i < n; i += gsz) {
            const double si = r[i] - alpha * v[i];
            s[i] = si;
            shv[i] = dinv[i] * si;
            ss[0] += si * si;
        }
        if (!grid_sum<1>(ss, partial, sh, st, round, spin)) return;
        if (sqrt(ss[0]) <= tol) {   // converged on the half step
            for (int i = gtid; i < n; i += gsz) {
                x[i] += alpha * ph[i];
                r[i] = s[i];
            }
            it++;
            conv = true;
            break;
        }
        double ts[2] = {0, 0};
        spmv_rows<TPR, U, false, double>(
            n, rowptr, CsrSource<double>{cols, vals}, [&](int c) { return shv[c]; },
            [&](int row, double tv) {
                t[row] = tv;
                ts[0] += tv * s[row];
                ts[1] += tv * tv;
            });
        if (!grid_sum<2>(ts, partial, sh, st, round, spin)) return;
        if (!(ts[1] > 0.0) || !isfinite(ts[1])) {
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        omega = ts[0] / ts[1];
        double w2[2] = {0, 0};
        for (int i = gtid; i < n; i += gsz) {
            x[i] += alpha * ph[i] + omega * shv[i];
            const double ri = s[i] - omega * t[i];
            r[i] = ri;
            w2[0] += rh[i] * ri;
            w2[1] += ri * ri;
        }
        if (!grid_sum<2>(w2, partial, sh, st, round, spin)) return;
        it++;
        rr = w2[1];
        conv = sqrt(rr) <= tol;
        if (!conv && (!(w2[0] != 0.0) || !(omega != 0.0))) {   // breakdown
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        beta = (w2[0] / rho) * (alpha / omega);
        rho = w2[0];
    }
    if (!grid_barrier(&st->bar, gridDim.x, &st->status, spin)) return;
    double tr[1];
    tr[0] = spmv_grid<TPR, U, false, double, double, double, true, true>(n, rowptr, cols, vals, x, r, nullptr, b);
    if (!grid_sum<1>(tr, partial, sh, st, round, spin)) return;
    if (gtid == 0) {
        st->iters = it;
        st->outer = 0;
        st->relres = sqrt(tr[0]) / (bn > 0 ? bn : 1.0);
        if (st->status == 0 && !(sqrt(tr[0]) <= fmax(tol, 0.0) || conv)) st->status = GRMP_ERR_NOT_CONVERGED;
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
                                               const float2 *cur, float2 *nxt, float *q, float beta) {
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
            nxt[r] = make_float2(me.x, pn);
            q[r] = s;
            dacc += pn * s;
        });
    return dacc;
}

// SpMV policy of the mixed solver: the grid-strided row loop over the packed
// FP32 pairs (fused_zp) and the FP64 residual b - A x (resid64).
template <int TPR, int U, bool PIPE>
struct RowsSpmv {
    int n;
    const int32_t *rowptr, *cols;
    const double *vals64;
    const int2 *pack32;
    __device__ __forceinline__ float fused_zp(const float2 *cur, float2 *nxt, float *q, float beta) {
        return spmv_fused_zp<TPR, U, PIPE>(n, rowptr, pack32, cur, nxt, q, beta);
    }
    __device__ __forceinline__ double resid64(const double *x, double *r64, const double *b) {
        return spmv_grid<TPR, U, PIPE, double, double, double, true, true>(n, rowptr, cols, vals64, x, r64, nullptr, b);
    }
};

// The mixed PCG iteration; `sp` supplies the two SpMV forms.  Returns early
// (every thread of a block alike) when a grid barrier fails.
//
// (preconditioned residual, search direction) pairs are double-buffered:
// `cur` holds (z_k, p_{k-1}); the SpMV gathers p_k = z_k + beta p_{k-1} on
// the fly, the owner of row i stores the pair (z_k, p_k) into nxt[i]; the
// vector phase (four rows per thread, 16-byte loads) reads p_k from nxt[i],
// updates x, r and writes z_{k+1} over the pair's first half.
template <class SP, class SY>
__device__ __forceinline__ void pcg_mixed_body(SP &sp, SY &sy, int n, const double *b, double *x, const float *dinv,
                                               float *r, float *q, float *xc, float2 *zp0, float2 *zp1, double *r64,
                                               SolveState *st, double abstol, double reltol, double delta, int maxit,
                                               int maxouter, int guess) {
    __shared__ double sh[32 * 4];
    __shared__ float shf[32 * 4];
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsz = gridDim.x * blockDim.x;
    // FP64 residual of the initial guess
    double v[2] = {0, 0};
    if (guess) {
        v[0] = sp.resid64(x, r64, b);
    } else {
        for (int i = gtid; i < n; i += gsz) {
            x[i] = 0.0;
            r64[i] = b[i];
            v[0] += b[i] * b[i];
        }
    }
    for (int i = gtid; i < n; i += gsz) v[1] += b[i] * b[i];
    if (!sy.template sum<2>(v, sh)) return;
    const double bn = sqrt(v[1]);
    const double tol = fmax(abstol, reltol * bn);
    double rn64 = sqrt(v[0]);
    int it = 0, outer = 0;
    bool conv = rn64 <= tol;
    // FP32 state from the FP64 residual; p_{-1} = 0
    float wf = 0.f;
    for (int i = gtid; i < n; i += gsz) {
        const float ri = (float)r64[i];
        const float zi = dinv[i] * ri;
        r[i] = ri;
        zp0[i] = make_float2(zi, 0.f);
        xc[i] = 0.0f;
        wf += ri * zi;
    }
    float w[1] = {wf};
    if (!sy.template sumf<1>(w, shf)) return;
    // inner-iteration scalars in FP32 (the FP64 pipe is scarce)
    float rz = w[0];
    float rmax = (float)rn64;
    const float tolf = (float)tol, deltaf = (float)delta;
    double prev_rn64 = rn64;
    int stall = 0;
    float beta = 0.f;
    float2 *cur = zp0, *nxt = zp1;
    const int n4 = n >> 2;
    while (!conv && it < maxit && outer < maxouter) {
        float d[1] = {sp.fused_zp(cur, nxt, q, beta)};
        if (!sy.template sumf<1>(d, shf)) return;   // barrier 1
        const float pq = d[0];
        if (!(pq > 0.f) || !isfinite(pq)) {
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        const float alpha = rz / pq;
        // vector phase, four rows per thread: two (z, p) pairs per 16-byte load
        float uf0 = 0.f, uf1 = 0.f;
        {
            float4 *nx4 = reinterpret_cast<float4 *>(nxt);
            float4 *xc4 = reinterpret_cast<float4 *>(xc);
            float4 *r4 = reinterpret_cast<float4 *>(r);
            const float4 *q4 = reinterpret_cast<const float4 *>(q);
            const float4 *di4 = reinterpret_cast<const float4 *>(dinv);
            for (int i = gtid; i < n4; i += gsz) {
                float4 a = nx4[2 * i], c = nx4[2 * i + 1];
                const float4 qq = q4[i], dd = di4[i];
                float4 rr = r4[i], xx = xc4[i];
                xx.x += alpha * a.y;
                xx.y += alpha * a.w;
                xx.z += alpha * c.y;
                xx.w += alpha * c.w;
                rr.x -= alpha * qq.x;
                rr.y -= alpha * qq.y;
                rr.z -= alpha * qq.z;
                rr.w -= alpha * qq.w;
                a.x = dd.x * rr.x;
                a.z = dd.y * rr.y;
                c.x = dd.z * rr.z;
                c.z = dd.w * rr.w;
                xc4[i] = xx;
                r4[i] = rr;
                nx4[2 * i] = a;
                nx4[2 * i + 1] = c;
                uf0 += rr.x * a.x + rr.y * a.z + rr.z * c.x + rr.w * c.z;
                uf1 += rr.x * rr.x + rr.y * rr.y + rr.z * rr.z + rr.w * rr.w;
            }
            for (int i = 4 * n4 + gtid; i < n; i += gsz) {
                float2 e = nxt[i];
                xc[i] += alpha * e.y;
                const float ri = r[i] - alpha * q[i];
                r[i] = ri;
                e.x = dinv[i] * ri;
                nxt[i] = e;
                uf0 += ri * e.x;
                uf1 += ri * ri;
            }
        }
        float u[2] = {uf0, uf1};
        if (!sy.template sumf<2>(u, shf)) return;   // barrier 2
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
            if (!sy.barrier()) return;
            double t[1];
            t[0] = sp.resid64(x, r64, b);
            if (!sy.template sum<1>(t, sh)) return;
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
            float yf = 0.f;
            for (int i = gtid; i < n; i += gsz) {
                const float ri = (float)r64[i];
                const float zi = dinv[i] * ri;
                r[i] = ri;
                nxt[i].x = zi;
                yf += ri * zi;
            }
            float y[1] = {yf};
            if (!sy.template sumf<1>(y, shf)) return;
            rz_new = y[0];
            rmax = (float)rn64;
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

template <int TPR, int U, bool PIPE, bool CL = false>
__global__ void __launch_bounds__(CL ? kClT : PTPB, CL ? 1 : (PIPE ? (U >= 8 ? 3 : (U >= 4 ? 4 : 6)) : (U >= 8 ? 4 : 5))) k_pcg_mixed(int n, const int32_t *rowptr, const int32_t *cols,
                                                    const double *vals64, const int2 *pack32, const double *b,
                                                    double *x, const float *dinv, float *r, float *q, float *xc,
                                                    float2 *zp0, float2 *zp1, double *r64, double *partial,
                                                    SolveState *st, double abstol, double reltol, double delta,
                                                    int maxit, int maxouter, int guess, long long spin) {
    RowsSpmv<TPR, U, PIPE> sp{n, rowptr, cols, vals64, pack32};
    SyncOf<CL> sy{st, partial, spin, 0};
    pcg_mixed_body(sp, sy, n, b, x, dinv, r, q, xc, zp0, zp1, r64, st, abstol, reltol, delta, maxit, maxouter, guess);
    sy.finish();
}

// ------------------------------------------------------------ duo mixed PCG
// FP32 SpMV fused with the search-direction update over the two-run 16-bit
// column copy (duo records, the matrix's own numbering): groups of TPR lanes
// per row as in spmv_rows, each lane with U duos (2U entries: one float2 and
// one 32-bit offset word per duo) in flight, software pipelined over the
// grid-strided rows (the next row's first chunk and the record of the row
// after it are loaded before the current row's gathers).  Per row one int4
// record {first duo, base1, base2, split | duos << 16}; entry e of the row has
// column (e < split ? base1 : base2) + its offset.  Summation order per row:
// chunk by chunk, duo u = 0..U-1, entry 0 then 1, then the lane reduction.
struct DuoRow {
    int kb, e, b1, b2, split;
};

__device__ __forceinline__ DuoRow duo_row(const int4 *__restrict__ meta, int r, int n) {
    DuoRow d{0, 0, 0, 0, 0};
    if (r < n) {
        const int4 m = __ldg(meta + r);
        d.kb = m.x;
        d.e = m.x + (m.w >> 16);
        d.b1 = m.y;
        d.b2 = m.z;
        d.split = m.w & 0xffff;
    }
    return d;
}

template <int U, int TPR>
__device__ __forceinline__ void duo_chunk(const float2 *__restrict__ val, const uint32_t *__restrict__ off,
                                          const DuoRow &d, int k, float2 *v, uint32_t *o) {
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int idx = k + u * TPR;
        if (idx < d.e) {
            v[u] = __ldg(val + idx);
            o[u] = __ldg(off + idx);
        } else {
            v[u] = make_float2(0.f, 0.f);
            o[u] = 0u;
        }
    }
}

// columns of duo idx (entries 2 (idx - kb) and 2 (idx - kb) + 1 of the row)
__device__ __forceinline__ void duo_cols(const DuoRow &d, int idx, uint32_t o, int &c0, int &c1) {
    const int e0 = 2 * (idx - d.kb);
    c0 = (e0 < d.split ? d.b1 : d.b2) + (int)(o & 0xffffu);
    c1 = (e0 + 1 < d.split ? d.b1 : d.b2) + (int)(o >> 16);
}

template <int TPR, int U>
__device__ __forceinline__ float duo_fused_zp(int n, const int4 *__restrict__ meta, const uint32_t *__restrict__ off,
                                              const float2 *__restrict__ val, const float2 *cur, float2 *nxt,
                                              float *q, float beta) {
    constexpr int RPW = 32 / TPR;
    constexpr int CH = TPR * U;   // duos of a row per chunk
    const int lane = threadIdx.x & (TPR - 1);
    const int gin = (threadIdx.x & 31) / TPR;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int stride = ((gridDim.x * blockDim.x) >> 5) * RPW;
    auto gp = [&](int c) {
        const float2 g = cur[c];
        return __fmaf_rn(beta, g.y, g.x);
    };
    float dacc = 0.f;
    int r = warp * RPW + gin;
    DuoRow d = duo_row(meta, r, n);
    DuoRow dn = duo_row(meta, r + stride, n);
    float2 v[U];
    uint32_t o[U];
    duo_chunk<U, TPR>(val, off, d, d.kb + lane, v, o);
    for (int base = warp * RPW; base < n; base += stride) {
        float2 vn[U];
        uint32_t on[U];
        duo_chunk<U, TPR>(val, off, dn, dn.kb + lane, vn, on);
        const DuoRow d2 = duo_row(meta, r + 2 * stride, n);
        float s = 0.f;
#pragma unroll
        for (int u = 0; u < U; u++) {
            int c0, c1;
            duo_cols(d, d.kb + lane + u * TPR, o[u], c0, c1);
            s += v[u].x * gp(c0);
            s += v[u].y * gp(c1);
        }
        for (int k = d.kb + lane + CH; k < d.e; k += CH) {   // rows longer than one chunk
            float2 v2[U];
            uint32_t o2[U];
            duo_chunk<U, TPR>(val, off, d, k, v2, o2);
#pragma unroll
            for (int u = 0; u < U; u++) {
                int c0, c1;
                duo_cols(d, k + u * TPR, o2[u], c0, c1);
                s += v2[u].x * gp(c0);
                s += v2[u].y * gp(c1);
            }
        }
#pragma unroll
        for (int w = TPR / 2; w > 0; w >>= 1) s += __shfl_xor_sync(0xffffffffu, s, w);
        if (r < n && lane == 0) {
            const float2 me = cur[r];
            const float pn = __fmaf_rn(beta, me.y, me.x);
            nxt[r] = make_float2(me.x, pn);
            q[r] = s;
            dacc += pn * s;
        }
        r += stride;
        d = dn;
        dn = d2;
#pragma unroll
        for (int u = 0; u < U; u++) {
            v[u] = vn[u];
            o[u] = on[u];
        }
    }
    return dacc;
}

// SpMV policy over the duo copy; the FP64 residual from the CSR arrays.
template <int TPR, int U>
struct DuoSpmv {
    int n;
    const int32_t *rowptr, *cols;
    const double *vals64;
    const int4 *meta;
    const uint32_t *off;
    const float2 *val;
    __device__ __forceinline__ float fused_zp(const float2 *cur, float2 *nxt, float *q, float beta) {
        return duo_fused_zp<TPR, U>(n, meta, off, val, cur, nxt, q, beta);
    }
    __device__ __forceinline__ double resid64(const double *x, double *r64, const double *b) {
        return spmv_grid<4, 4, true, double, double, double, true, true>(n, rowptr, cols, vals64, x, r64, nullptr, b);
    }
};

template <int TPR, int U, bool CL = false>
__global__ void __launch_bounds__(CL ? kClT : PTPB, CL ? 1 : (U >= 4 ? 3 : 4)) k_pcg_mixed_duo(
    int n, const int32_t *rowptr, const int32_t *cols, const double *vals64, const int4 *meta, const uint32_t *off,
    const float2 *val, const double *b, double *x, const float *dinv, float *r, float *q, float *xc, float2 *zp0,
    float2 *zp1, double *r64, double *partial, SolveState *st, double abstol, double reltol, double delta, int maxit,
    int maxouter, int guess, long long spin) {
    DuoSpmv<TPR, U> sp{n, rowptr, cols, vals64, meta, off, val};
    SyncOf<CL> sy{st, partial, spin, 0};
    pcg_mixed_body(sp, sy, n, b, x, dinv, r, q, xc, zp0, zp1, r64, st, abstol, reltol, delta, maxit, maxouter, guess);
    sy.finish();
}

// ------------------------------------------------ scaled duo mixed PCG (keep)
// The mixed solver's inner iteration on the Jacobi-scaled FP32 system
// S A32 S y = S r,  S = diag(1 / sqrt(a32_ii)) (A32: the FP32-assembled
// matrix): unpreconditioned CG on S A32 S is Jacobi-PCG on A32,
// with z = r, so the (z, p) pair is (r, p) and neither a separate residual
// array nor the inverse diagonal is streamed.  The row loop gives every row
// group a fixed list of rows (first row + j * stride, j < J); the SpMV phase
// keeps each row's S A32 S p (ALL: also r and p) in shared memory, in slots
// [J][groups of the block], and the vector phase, run over all threads of
// the block after the p.q reduction, updates the rows from there (p
// recomputed from the pair with the SpMV's own fmaf).  Per row and iteration
// the vector streams left are the own pair (read), the FP32 correction (read,
// write) and the next pair (write) -- against nine 4-byte words of the
// unscaled solver.  The FP64 refinement is unchanged: x += S xc, r64 = b - A x
// with the FP64 matrix, the scaled FP32 residual S r64.
template <int TPR, int U, bool ALL>
__device__ __forceinline__ float duo_zp_keep(int n, const int4 *__restrict__ meta, const uint32_t *__restrict__ off,
                                             const float2 *__restrict__ val, const float2 *cur, float beta, float *kr,
                                             float *kp, float *kq) {
    constexpr int RPW = 32 / TPR;
    constexpr int CH = TPR * U;
    constexpr int G = PTPB / TPR;
    const int lane = threadIdx.x & (TPR - 1);
    const int gin = (threadIdx.x & 31) / TPR;
    const int g = threadIdx.x / TPR;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int stride = ((gridDim.x * blockDim.x) >> 5) * RPW;
    auto gp = [&](int c) {
        const float2 v = cur[c];
        return __fmaf_rn(beta, v.y, v.x);
    };
    float dacc = 0.f;
    int r = warp * RPW + gin;
    int j = 0;
    DuoRow d = duo_row(meta, r, n);
    DuoRow dn = duo_row(meta, r + stride, n);
    float2 v[U];
    uint32_t o[U];
    duo_chunk<U, TPR>(val, off, d, d.kb + lane, v, o);
    for (int base = warp * RPW; base < n; base += stride, j++) {
        float2 vn[U];
        uint32_t on[U];
        duo_chunk<U, TPR>(val, off, dn, dn.kb + lane, vn, on);
        const DuoRow d2 = duo_row(meta, r + 2 * stride, n);
        float s = 0.f;
#pragma unroll
        for (int u = 0; u < U; u++) {
            int c0, c1;
            duo_cols(d, d.kb + lane + u * TPR, o[u], c0, c1);
            s += v[u].x * gp(c0);
            s += v[u].y * gp(c1);
        }
        for (int k = d.kb + lane + CH; k < d.e; k += CH) {   // rows longer than one chunk
            float2 v2[U];
            uint32_t o2[U];
            duo_chunk<U, TPR>(val, off, d, k, v2, o2);
#pragma unroll
            for (int u = 0; u < U; u++) {
                int c0, c1;
                duo_cols(d, k + u * TPR, o2[u], c0, c1);
                s += v2[u].x * gp(c0);
                s += v2[u].y * gp(c1);
            }
        }
#pragma unroll
        for (int w = TPR / 2; w > 0; w >>= 1) s += __shfl_xor_sync(0xffffffffu, s, w);
        if (r < n && lane == 0) {
            const float2 me = cur[r];
            const float pn = __fmaf_rn(beta, me.y, me.x);
            const int k = j * G + g;
            if (ALL) {
                kr[k] = me.x;
                kp[k] = pn;
            }
            kq[k] = s;
            dacc += pn * s;
        }
        r += stride;
        d = dn;
        dn = d2;
#pragma unroll
        for (int u = 0; u < U; u++) {
            v[u] = vn[u];
            o[u] = on[u];
        }
    }
    return dacc;
}

template <int TPR, int U, bool ALL, int MINB = (U >= 4 ? 3 : 4)>
__global__ void __launch_bounds__(PTPB, MINB) k_pcg_mixed_duo_keep(
    int n, const int32_t *rowptr, const int32_t *cols, const double *vals64, const int4 *meta, const uint32_t *off,
    const float2 *sval, const double *b, double *x, const double *sc, float *xc, float2 *zp0, float2 *zp1,
    double *r64, double *partial, SolveState *st, double abstol, double reltol, double delta, int maxit,
    int maxouter, int guess, long long spin, int J) {
    extern __shared__ float keep[];
    constexpr int G = PTPB / TPR, RPW = 32 / TPR, VB = 8;
    // ALL: r, p and A p per slot; else A p only (r and p from the pair)
    float *kq = keep, *kr = keep + (size_t)J * G, *kp = keep + 2 * (size_t)J * G;
    __shared__ double sh[32 * 4];
    __shared__ float shf[32 * 4];
    GridSync sy{st, partial, spin, 0};
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsz = gridDim.x * blockDim.x;
    // slot k = j * G + g of this block holds row  blockIdx.x * G + g + j * stride
    // (group g's j-th row in the SpMV row loop)
    const int stride = (gsz >> 5) * RPW;
    const int rbase = blockIdx.x * G;
    const int nslot = J * G;
    auto resid64 = [&]() {
        return spmv_grid<4, 4, true, double, double, double, true, true>(n, rowptr, cols, vals64, x, r64, nullptr, b);
    };
    // FP64 residual of the initial guess
    double v[2] = {0, 0};
    if (guess) {
        v[0] = resid64();
    } else {
        for (int i = gtid; i < n; i += gsz) {
            x[i] = 0.0;
            r64[i] = b[i];
            v[0] += b[i] * b[i];
        }
    }
    for (int i = gtid; i < n; i += gsz) v[1] += b[i] * b[i];
    if (!sy.template sum<2>(v, sh)) return;
    const double bn = sqrt(v[1]);
    const double tol = fmax(abstol, reltol * bn);
    double rn64 = sqrt(v[0]);
    int it = 0, outer = 0;
    bool conv = rn64 <= tol;
    // scaled FP32 residual S r64; p_{-1} = 0
    float wf = 0.f;
    for (int i = gtid; i < n; i += gsz) {
        const float ri = (float)(sc[i] * r64[i]);
        zp0[i] = make_float2(ri, 0.f);
        xc[i] = 0.0f;
        wf += ri * ri;
    }
    float w[1] = {wf};
    if (!sy.template sumf<1>(w, shf)) return;
    float rz = w[0];
    float rmax = sqrtf(rz);
    // the refinement also runs once the unscaled residual, estimated from the
    // scaled one with the ratio seen at the last refinement, is below tol
    float ratio = rmax > 0.f ? (float)(rn64 / (double)rmax) : 1.f;
    const float tolf = (float)tol;
    const float deltaf = (float)delta;
    double prev_rn64 = rn64;
    int stall = 0;
    float beta = 0.f;
    float2 *cur = zp0, *nxt = zp1;
    while (!conv && it < maxit && outer < maxouter) {
        float d[1] = {duo_zp_keep<TPR, U, ALL>(n, meta, off, sval, cur, beta, kr, kp, kq)};
        if (!sy.template sumf<1>(d, shf)) return;   // barrier 1
        const float pq = d[0];
        if (!(pq > 0.f) || !isfinite(pq)) {
            if (gtid == 0) atomicCAS(&st->status, 0, (int)GRMP_ERR_NAN);
            break;
        }
        const float alpha = rz / pq;
        float uf = 0.f;
        // the block's slots over all its threads (consecutive threads,
        // consecutive rows), VB independent correction loads in flight
        for (int k0 = threadIdx.x; k0 < nslot; k0 += PTPB * VB) {
            float xv[VB];
            float2 cv[VB];
            int rr[VB];
#pragma unroll
            for (int t = 0; t < VB; t++) {
                const int k = k0 + t * PTPB;
                rr[t] = k < nslot ? rbase + (k % G) + (k / G) * stride : n;
                xv[t] = rr[t] < n ? xc[rr[t]] : 0.f;
                if (!ALL) cv[t] = rr[t] < n ? cur[rr[t]] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int t = 0; t < VB; t++) {
                if (rr[t] < n) {
                    const int k = k0 + t * PTPB;
                    // p_k as the SpMV formed it (same fmaf): identical values
                    const float pk = ALL ? kp[k] : __fmaf_rn(beta, cv[t].y, cv[t].x);
                    const float rn = (ALL ? kr[k] : cv[t].x) - alpha * kq[k];
                    xc[rr[t]] = xv[t] + alpha * pk;
                    nxt[rr[t]] = make_float2(rn, pk);
                    uf += rn * rn;
                }
            }
        }
        float u[1] = {uf};
        if (!sy.template sumf<1>(u, shf)) return;   // barrier 2
        it++;
        float rz_new = u[0];
        const float rn32 = sqrtf(rz_new);
        bool restart = false;
        if (rn32 <= deltaf * rmax || ratio * rn32 <= tolf || it >= maxit) {
            // refinement: fold S xc into x, recompute b - A x in FP64
            for (int i = gtid; i < n; i += gsz) {
                x[i] += sc[i] * (double)xc[i];
                xc[i] = 0.0f;
            }
            if (!sy.barrier()) return;
            double t[1] = {resid64()};
            if (!sy.template sum<1>(t, sh)) return;
            outer++;
            rn64 = sqrt(t[0]);
            conv = rn64 <= tol;
            if (conv || it >= maxit) break;
            // as in pcg_mixed_body: restart the inner CG when the true residual
            // stops falling, give up after 16 refinements without progress
            restart = rn64 > 0.5 * prev_rn64;
            stall = (rn64 > 0.9 * prev_rn64) ? stall + 1 : 0;
            prev_rn64 = rn64;
            if (stall >= 16) break;
            float yf = 0.f;
            for (int i = gtid; i < n; i += gsz) {
                const float ri = (float)(sc[i] * r64[i]);
                nxt[i].x = ri;
                yf += ri * ri;
            }
            float y[1] = {yf};
            if (!sy.template sumf<1>(y, shf)) return;
            rz_new = y[0];
            rmax = sqrtf(rz_new);
            ratio = rmax > 0.f ? (float)(rn64 / (double)rmax) : 1.f;
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

// values of the duo copy from the CSR FP32 values (one thread per duo)
__global__ void k_duo_fill(long long nduo, const int32_t *src, const float *vals32, float2 *val) {
    const long long d = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= nduo) return;
    const int s = __ldg(src + d);
    const int k = s >= 0 ? s : -1 - s;
    val[d] = make_float2(__ldg(vals32 + k), s >= 0 ? __ldg(vals32 + k + 1) : 0.f);
}

// ------------------------------------------------------------ staged mixed PCG
// The FP32 matrix re-laid out in fixed-size row windows (kStgRec bytes each):
//   int row0, int nrows | uint16 local row offsets [nrows + 1] | pad to 16 B |
//   int2 (column, FP32 value bits) entries of rows row0 .. row0 + nrows - 1.
// Windows are packed greedily with whole rows.  Each block of the staged
// kernel owns a contiguous range of windows and streams them, iteration after
// iteration, through a ring of S shared-memory stages with one bulk async
// copy per window (cp.async.bulk, completion counted on an mbarrier): warp 0
// issues the copies, the other warps compute rows out of shared memory, so
// the only global loads left on the compute warps are the gathers of the
// search direction, which hit L1/L2.  The stream never stops at iteration
// boundaries: the copies of the next iteration's first windows are issued as
// soon as their stages are released, and land during the vector phase and
// the grid barriers.
constexpr int kStgRec = 32768;

__host__ __device__ __forceinline__ int stg_header_bytes(int nrows) { return (8 + 2 * (nrows + 1) + 15) & ~15; }

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, long long limit) {
    for (long long spins = 0; spins < limit; spins++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

template <int TPR, int U, int NT, int S>
struct StagedSpmv {
    static constexpr int NC = NT / 32 - 1;   // compute warps
    static constexpr int RPW = 32 / TPR;
    // FP64 residual: plain grid-strided rows from the CSR arrays
    int n;
    const int32_t *rowptr, *cols;
    const double *vals64;
    // window stream
    const char *rec;
    char *stage;            // S x kStgRec bytes of shared memory
    uint64_t *full, *empty;
    int jb, cnt;            // this block's windows
    unsigned consumed;      // windows consumed so far (all threads)
    unsigned issued;        // windows issued so far (issuing thread only)
    int *status;
    long long spin;         // polls of a bounded mbarrier wait

    __device__ __forceinline__ bool issue_one() {
        const unsigned qn = issued, s = qn % S;
        if (qn >= (unsigned)S && !mbar_wait(&empty[s], (qn / S - 1) & 1, spin)) return false;
        mbar_arrive_expect_tx(&full[s], kStgRec);
        bulk_load(stage + (size_t)s * kStgRec, rec + (size_t)(jb + (int)(qn % (unsigned)cnt)) * kStgRec, kStgRec,
                  &full[s]);
        issued = qn + 1;
        return true;
    }
    // first S windows, before the first SpMV
    __device__ __forceinline__ void prologue() {
        if (threadIdx.x == 0 && cnt > 0)
            for (int m = 0; m < S; m++)
                if (!issue_one()) {
                    atomicCAS(status, 0, (int)GRMP_ERR_TIMEOUT);
                    break;
                }
    }
    // wait (bounded) for the copies still in flight before the block exits:
    // the last copy issued into each stage (copies into one stage are
    // serialised by its release barrier).  This wait keeps the library's
    // default bound even when the context's limit is lower: a copy in flight
    // lands within microseconds, and the block must not leave before it does.
    __device__ __forceinline__ void drain() {
        if (threadIdx.x == 0 && cnt > 0)
            for (unsigned qn = issued > (unsigned)S ? issued - S : 0u; qn < issued; qn++)
                if (!mbar_wait(&full[qn % S], (qn / S) & 1, spin > GRMP_SPIN_LIMIT ? spin : GRMP_SPIN_LIMIT)) break;
        __syncthreads();
    }

    __device__ __forceinline__ float fused_zp(const float2 *cur, float2 *nxt, float *q, float beta) {
        float dacc = 0.f;
        const int warp = threadIdx.x >> 5;
        if (cnt <= 0) return dacc;
        if (warp == 0) {
            if (threadIdx.x == 0) {
                for (int m = 0; m < cnt; m++)
                    if (!issue_one()) {
                        atomicCAS(status, 0, (int)GRMP_ERR_TIMEOUT);
                        break;
                    }
            }
            __syncwarp();
        } else {
            const int cw = warp - 1;
            const int lane = threadIdx.x & (TPR - 1);
            const int gin = (threadIdx.x & 31) / TPR;
            int T = 0;   // row steps of the windows before this one
            for (int m = 0; m < cnt; m++) {
                const unsigned qn = consumed + m, s = qn % S;
                if (!mbar_wait(&full[s], (qn / S) & 1, spin)) {
                    atomicCAS(status, 0, (int)GRMP_ERR_TIMEOUT);
                    break;
                }
                const char *w = stage + (size_t)s * kStgRec;
                const int row0 = reinterpret_cast<const int *>(w)[0];
                const int nr = reinterpret_cast<const int *>(w)[1];
                const uint16_t *lrp = reinterpret_cast<const uint16_t *>(w + 8);
                const int2 *ent = reinterpret_cast<const int2 *>(w + stg_header_bytes(nr));
                const int steps = (nr + RPW - 1) / RPW;
                int j = cw - T % NC;
                if (j < 0) j += NC;
                for (; j < steps; j += NC) {
                    const int i = j * RPW + gin;
                    float sum = 0.f;
                    if (i < nr) {
                        const int kb = lrp[i], e = lrp[i + 1];
                        for (int k = kb + lane; k < e; k += TPR * U) {
                            int c[U];
                            float v[U];
#pragma unroll
                            for (int u = 0; u < U; u++) {
                                const int idx = k + u * TPR;
                                if (idx < e) {
                                    const int2 pe = ent[idx];
                                    c[u] = pe.x;
                                    v[u] = __int_as_float(pe.y);
                                } else {
                                    c[u] = 0;
                                    v[u] = 0.f;
                                }
                            }
#pragma unroll
                            for (int u = 0; u < U; u++) {
                                const float2 g = cur[c[u]];
                                sum += v[u] * __fmaf_rn(beta, g.y, g.x);
                            }
                        }
                    }
#pragma unroll
                    for (int o = TPR / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                    if (i < nr && lane == 0) {
                        const int r = row0 + i;
                        const float2 me = cur[r];
                        const float pn = __fmaf_rn(beta, me.y, me.x);
                        nxt[r] = make_float2(me.x, pn);
                        q[r] = sum;
                        dacc += pn * sum;
                    }
                }
                T += steps;
                __syncwarp();
                if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);
            }
        }
        consumed += cnt;
        return dacc;
    }
    __device__ __forceinline__ double resid64(const double *x, double *r64, const double *b) {
        return spmv_grid<TPR, 4, false, double, double, double, true, true>(n, rowptr, cols, vals64, x, r64, nullptr, b);
    }
};

template <int TPR, int U, int NT, int S>
__global__ void __launch_bounds__(NT, 2048 / NT / 2) k_pcg_mixed_staged(int n, const int32_t *rowptr, const int32_t *cols,
                                                            const double *vals64, const char *rec, int nwin,
                                                            const double *b, double *x, const float *dinv,
                                                            float *r, float *q, float *xc, float2 *zp0,
                                                            float2 *zp1, double *r64,
                                                            double *partial, SolveState *st, double abstol,
                                                            double reltol, double delta, int maxit, int maxouter,
                                                            int guess, long long spin) {
    extern __shared__ __align__(128) char stage_smem[];
    __shared__ __align__(8) uint64_t bars[2 * S];
    using SP = StagedSpmv<TPR, U, NT, S>;
    SP sp;
    sp.n = n;
    sp.rowptr = rowptr;
    sp.cols = cols;
    sp.vals64 = vals64;
    sp.rec = rec;
    sp.stage = stage_smem;
    sp.full = bars;
    sp.empty = bars + S;
    sp.jb = (int)((long long)blockIdx.x * nwin / gridDim.x);
    sp.cnt = (int)((long long)(blockIdx.x + 1) * nwin / gridDim.x) - sp.jb;
    sp.consumed = 0;
    sp.issued = 0;
    sp.status = &st->status;
    sp.spin = spin;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&sp.full[s], 1);
            mbar_init(&sp.empty[s], SP::NC);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    sp.prologue();
    GridSync sy{st, partial, spin, 0};
    pcg_mixed_body(sp, sy, n, b, x, dinv, r, q, xc, zp0, zp1, r64, st, abstol, reltol, delta, maxit, maxouter, guess);
    sp.drain();
}

// fills the window records from the packed FP32 pairs (one block per window)
__global__ void k_stage_fill(const int32_t *win_row0, const int32_t *rowptr, const int2 *pack, char *rec) {
    const int j = blockIdx.x;
    const int r0 = win_row0[j], nr = win_row0[j + 1] - r0;
    char *w = rec + (size_t)j * kStgRec;
    const int base = rowptr[r0];
    if (threadIdx.x == 0) {
        reinterpret_cast<int *>(w)[0] = r0;
        reinterpret_cast<int *>(w)[1] = nr;
    }
    uint16_t *lrp = reinterpret_cast<uint16_t *>(w + 8);
    for (int i = threadIdx.x; i <= nr; i += blockDim.x) lrp[i] = (uint16_t)(rowptr[r0 + i] - base);
    const int ne = rowptr[r0 + nr] - base;
    int2 *ent = reinterpret_cast<int2 *>(w + stg_header_bytes(nr));
    for (int k = threadIdx.x; k < ne; k += blockDim.x) ent[k] = pack[base + k];
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
// flight per lane), encoded 100*TPR + U; + 10000: software-pipelined row
// loop; + 20000: staged windows, 512 threads x 3 stages per block; + 30000:
// staged windows, 1024 threads x 6 stages (the staged ones: mixed solves only).
// (The cluster configurations 7xxxx / 8xxxx are not timed: on systems of
// 20,000 rows and more, where the autotuner runs, the grid-wide solvers are
// faster; the row-length heuristic uses them for the smallest mixed solves.)
constexpr int kConfigs[] = {208,   404,   408,   804,   1602,  10204, 10404, 10408, 10804, 10402,
                            10802, 20204, 20408, 20804, 30408, 30804, 60404, 60208, 60802, 60408, 64208, 64404,
                            65208, 65404, 66404};

inline bool staged_config(int cfg) { return cfg >= 20000 && cfg < 60000; }
inline bool duo_config(int cfg) { return (cfg >= 60000 && cfg < 70000) || cfg >= 80000; }
inline bool cluster_config(int cfg) { return cfg >= 70000; }
inline bool scaled_config(int cfg) { return cfg >= 64000 && cfg < 67000; }

// Window layout of the staged SpMV, built once per matrix pattern from the
// row pointers (greedy: whole rows while header + entries fit one record).
int stage_build(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    std::vector<int32_t> rp((size_t)n + 1);
    cudaError_t e = cudaMemcpyAsync(rp.data(), A->d_rowptr, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "staged SpMV: row pointer download");
    std::vector<int32_t> row0;
    int r = 0;
    while (r < n) {
        const int start = r;
        long long ne = 0;
        while (r < n) {
            const int len = rp[r + 1] - rp[r];
            if (stg_header_bytes(r - start + 1) + 8 * (ne + len) > kStgRec) break;
            ne += len;
            r++;
        }
        if (r == start) {
            A->stg_state = -1;
            return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "staged SpMV: row %d has %d entries, more than a window holds",
                             r, rp[r + 1] - rp[r]);
        }
        row0.push_back(start);
    }
    row0.push_back(n);
    const int nwin = (int)row0.size() - 1;
    int32_t *d_row0 = nullptr;
    char *d_rec = nullptr;
    const size_t rec_bytes = std::max<size_t>(1, (size_t)nwin) * kStgRec;
    int rc = grmp_alloc(ctx, (void **)&d_row0, row0.size() * 4);
    if (rc) return rc;
    rc = grmp_alloc(ctx, (void **)&d_rec, rec_bytes);
    if (rc) {
        grmp_free(ctx, d_row0, row0.size() * 4);
        return rc;
    }
    e = cudaMemcpyAsync(d_row0, row0.data(), row0.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_rec, 0, rec_bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);   // row0 is a host vector
    if (e != cudaSuccess) {
        grmp_free(ctx, d_row0, row0.size() * 4);
        grmp_free(ctx, d_rec, rec_bytes);
        return grmp_cuda_fail(ctx, e, "staged SpMV: window upload");
    }
    A->d_stg_row0 = d_row0;
    A->d_stg_rec = d_rec;
    A->stg_rec_bytes = rec_bytes;
    A->stg_nwin = nwin;
    A->stg_state = 1;
    return GRMP_OK;
}

void stage_fill(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    if (A->stg_nwin <= 0) return;
    k_stage_fill<<<A->stg_nwin, 256, 0, ctx->stream>>>(A->d_stg_row0, A->d_rowptr, (const int2 *)A->d_pack32,
                                                       A->d_stg_rec);
    GRMP_LAUNCHED(ctx);
}

// The packed (column, FP32 value) pairs (and the staged windows copied from
// them) for the values of the current solve.
int ensure_pack32(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    if (A->pack_fresh) return GRMP_OK;
    if (!A->d_pack32) {
        int rc = grmp_alloc(ctx, &A->d_pack32, (size_t)A->nnz * 8);
        if (rc) return rc;
    }
    k_pack32<<<(unsigned)((A->nnz + 255) / 256), 256, 0, ctx->stream>>>(A->nnz, A->d_cols, A->d_vals32,
                                                                       (int2 *)A->d_pack32);
    GRMP_LAUNCHED(ctx);
    if (A->stg_state == 1) stage_fill(A);   // the staged windows hold a copy of the pairs
    A->pack_fresh = true;
    return GRMP_OK;
}

// The duo copy: layout once per pattern (host), values per solve (device).
int duo_build_dev(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    std::vector<int32_t> rp((size_t)n + 1), ci((size_t)A->nnz);
    cudaError_t e = cudaMemcpyAsync(rp.data(), A->d_rowptr, rp.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ci.data(), A->d_cols, ci.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "duo layout: pattern download");
    DuoLayout L;
    if (duo_build(n, rp.data(), ci.data(), &L)) {
        A->duo_state = -1;
        A->duo_span = L.max_span;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "duo layout: a column run spans %d columns (more than 65535)",
                         L.max_span);
    }
    A->duo_nduo = L.nduo;
    int rc = grmp_upload(ctx, (int32_t **)&A->d_duo_meta, L.meta.data(), L.meta.size());
    if (!rc) rc = grmp_upload(ctx, &A->d_duo_off, L.off.data(), L.off.size());
    if (!rc) rc = grmp_upload(ctx, &A->d_duo_src, L.src.data(), L.src.size());
    if (!rc) rc = grmp_alloc(ctx, &A->d_duo_val, (size_t)L.nduo * 8);
    if (!rc) {
        e = cudaStreamSynchronize(ctx->stream);   // the host vectors are freed on return
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "duo layout: upload");
    }
    if (rc) {
        grmp_duo_free(A);
        return rc;
    }
    A->duo_span = L.max_span;
    A->duo_state = 1;
    return GRMP_OK;
}

// The duo layout (once per pattern); with `values`, also the unscaled FP32
// values of the current solve.
int ensure_duo(grmp_matrix A, bool values = true) {
    grmp_context ctx = A->space->mesh->ctx;
    if (A->duo_state == 0) {
        int rc = duo_build_dev(A);
        if (rc) return rc;
    }
    if (A->duo_state < 0)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "duo layout: a column run spans %d columns (more than 65535)",
                         A->duo_span);
    if (values && !A->duo_fresh) {
        k_duo_fill<<<(unsigned)((A->duo_nduo + 255) / 256), 256, 0, ctx->stream>>>(A->duo_nduo, A->d_duo_src,
                                                                                   A->d_vals32,
                                                                                   (float2 *)A->d_duo_val);
        GRMP_LAUNCHED(ctx);
        A->duo_fresh = true;
    }
    return GRMP_OK;
}

// The Jacobi-scaled duo values of the FP32-assembled values (scaled
// solver: the inner iteration is Jacobi-PCG on the FP32 matrix, run as CG on
// S A32 S): the row scales s_i = 1 / sqrt(a32_ii) in FP64, then each duo's
// two values a32_ij * s_i * s_j formed in FP64 and rounded once to FP32.
// *bad is set for a non-positive or non-finite diagonal entry.
__global__ void k_duo_scales(int n, const int32_t *rowptr, const int32_t *cols, const float *vals, double *sc,
                             int *bad) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double d = 0.0;
    for (int k = rowptr[r]; k < rowptr[r + 1]; k++)
        if (cols[k] == r) d = (double)vals[k];
    if (!(d > 0.0) || !isfinite(d)) {
        atomicExch(bad, 1);
        sc[r] = 0.0;
        return;
    }
    sc[r] = 1.0 / sqrt(d);
}

// 16 lanes per row over the row's duos (contiguous in the duo arrays and,
// through their source positions, in the CSR arrays): coalesced loads and
// stores
__global__ void k_duo_fill_scaled(int n, const int4 *meta, const int32_t *src, const int32_t *cols,
                                  const float *vals, const double *sc, float2 *sval) {
    const int r = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 4);
    const int l = threadIdx.x & 15;
    if (r >= n) return;
    const int4 m = meta[r];
    const double sr = sc[r];
    const int d1 = m.x + (m.w >> 16);
    for (int d = m.x + l; d < d1; d += 16) {
        const int s = src[d];
        const int k = s >= 0 ? s : -1 - s;
        const float v0 = (float)((double)vals[k] * sr * sc[cols[k]]);
        const float v1 = s >= 0 ? (float)((double)vals[k + 1] * sr * sc[cols[k + 1]]) : 0.f;
        sval[d] = make_float2(v0, v1);
    }
}

int ensure_duo_scaled(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    int rc = ensure_duo(A, false);
    if (rc) return rc;
    if (!A->d_duo_sval) {
        rc = grmp_alloc(ctx, &A->d_duo_sval, (size_t)A->duo_nduo * 8);
        if (!rc) rc = grmp_alloc(ctx, (void **)&A->d_duo_sc, (size_t)A->nrows * 8);
        if (rc) {
            grmp_free(ctx, A->d_duo_sval, (size_t)A->duo_nduo * 8);
            A->d_duo_sval = nullptr;
            return rc;
        }
    }
    if (!A->duo_sfresh) {
        const int n = A->nrows;
        int *bad = nullptr;
        rc = grmp_alloc(ctx, (void **)&bad, 4);
        if (rc) return rc;
        cudaMemsetAsync(bad, 0, 4, ctx->stream);
        k_duo_scales<<<nblk(n), 256, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals32, A->d_duo_sc, bad);
        GRMP_LAUNCHED(ctx);
        k_duo_fill_scaled<<<nblk((long long)n * 16), 256, 0, ctx->stream>>>(
            n, (const int4 *)A->d_duo_meta, A->d_duo_src, A->d_cols, A->d_vals32, A->d_duo_sc,
            (float2 *)A->d_duo_sval);
        GRMP_LAUNCHED(ctx);
        int hbad = 0;
        cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        grmp_free(ctx, bad, 4);
        if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "scaled duo values");
        if (hbad) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: non-positive or non-finite diagonal entry");
        A->duo_sfresh = true;
    }
    return GRMP_OK;
}

int heuristic_tpr(grmp_matrix A) {
    double avg = (double)A->nnz / (double)std::max(1, A->nrows);
    if (avg <= 3) return 2;
    if (avg <= 6) return 4;
    if (avg <= 14) return 8;
    if (avg <= 40) return 16;
    return 32;
}

// Configuration from the mean row length alone (no timing): the autotuner's
// usual choices on FEM matrices -- plain row loops for FP64 (FP64-pipe bound,
// more loads in flight do not help), the pipelined row loop for FP32 -- and,
// for mixed solves of at most kClusterRows rows, the one-cluster solver
// (measured on 2D P1 systems of 1,089 and 4,225 rows: 6.8 and 7.5 us per
// iteration against 7.8 and 8.2 for the best grid-wide configuration; on
// 15,625 rows of 3D P2 the grid-wide solver is faster).
constexpr int kClusterRows = 8192;

int heuristic_config(grmp_matrix A, bool mixed) {
    double avg = (double)A->nnz / (double)std::max(1, A->nrows);
    if (mixed && A->nrows <= kClusterRows) return avg <= 10 ? 70204 : 70404;
    if (mixed) {
        if (avg <= 8) return 10204;
        if (avg <= 20) return 10404;
        return 10408;
    }
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

// Cluster size of a cluster solver: 16 CTAs (non-portable size) where such
// a cluster fits on this GPU, else the portable 8.  Returns 0 when neither
// fits.  (Sets the kernel's non-portable-size attribute, which a launch with
// 16 CTAs needs.)
template <typename K>
int cluster_ctas(K kern) {
    int c = 0;
    for (int want : {16, 8}) {
        if (want > 8 &&
            cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t lc{};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)want;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.gridDim = dim3((unsigned)want);
        lc.blockDim = dim3(kClT);
        lc.attrs = at;
        lc.numAttrs = 1;
        int ncl = 0;
        if (cudaOccupancyMaxActiveClusters(&ncl, (const void *)kern, &lc) != cudaSuccess) {
            cudaGetLastError();
            ncl = 0;
        }
        if (ncl >= 1) {
            c = want;
            break;
        }
    }
    return c;
}

// One cluster of `ctas` CTAs of kClT threads on the context's stream.
template <typename K>
cudaError_t launch_cluster(grmp_context ctx, K kern, int ctas, void **args) {
    cudaLaunchConfig_t lc{};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.gridDim = dim3((unsigned)ctas);
    lc.blockDim = dim3(kClT);
    lc.dynamicSmemBytes = 0;
    lc.stream = ctx->stream;
    lc.attrs = at;
    lc.numAttrs = 1;
    return cudaLaunchKernelExC(&lc, (const void *)kern, args);
}

// Persistent launch of a solver kernel: a cooperative grid (CL false) or one
// cluster (CL true).  *grid receives the number of CTAs.
template <bool CL, typename K>
cudaError_t launch_persistent(grmp_context ctx, K kern, int n, int want, void **args, int *grid) {
    if (CL) {
        const int c = cluster_ctas(kern);
        *grid = c;
        if (c < 1) return cudaErrorInvalidConfiguration;
        return launch_cluster(ctx, kern, c, args);
    }
    *grid = coop_grid(ctx, kern, n, want);
    return cudaLaunchCooperativeKernel((void *)kern, *grid, PTPB, args, 0, ctx->stream);
}

template <int TPR, int U, bool PIPE, bool CL = false>
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
        auto kern = k_pcg64<TPR, U, PIPE, CL>;
        double *dinv = (double *)work, *r = (double *)(work + lay.vec), *z = (double *)(work + 2 * lay.vec);
        double *pp = (double *)(work + 3 * lay.vec), *q = (double *)(work + 4 * lay.vec);
        double *part = (double *)(work + lay.off_part);
        int nn = n, mi = p->maxiter;
        double at = p->abstol, rt = p->reltol;
        const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
        const double *vv = A->d_vals64, *bb = bvec;
        double *xx = xvec;
        long long spin = ctx->wait_limit;
        void *args[] = {&nn, &rp, &ci, &vv, &bb, &xx, &dinv, &r, &z, &pp, &q, &part, &dst, &at, &rt, &mi, &guess, &spin};
        cudaEventRecord(e0, ctx->stream);
        e = launch_persistent<CL>(ctx, kern, n, p->grid_blocks, args, &grid);
        GRMP_LAUNCHED(ctx);
        cudaEventRecord(e1, ctx->stream);
    } else {
        const int prc = ensure_pack32(A);
        if (prc) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return prc;
        }
        auto kern = k_pcg_mixed<TPR, U, PIPE, CL>;
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
        long long spin = ctx->wait_limit;
        void *args[] = {&nn, &rp, &ci, &v64, &v32, &bb, &xx, &dinv, &r, &q, &xc, &zp0, &zp1, &r64, &part, &dst,
                        &at, &rt, &dl, &mi, &mo, &guess, &spin};
        cudaEventRecord(e0, ctx->stream);
        e = launch_persistent<CL>(ctx, kern, n, p->grid_blocks, args, &grid);
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
    out->spmv_config = 100 * TPR + U + (CL ? 70000 : (PIPE ? 10000 : 0));
    out->grid_blocks = grid;
    out->solve_ms = ms;
    if (hs.status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, GRMP_ERR_NOT_CONVERGED, "PCG: %d iterations, relative residual %.3e", hs.iters, hs.relres);
    if (hs.status == GRMP_ERR_TIMEOUT) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "PCG: a grid barrier wait timed out");
    if (hs.status == GRMP_ERR_NAN) return grmp_fail(ctx, GRMP_ERR_NAN, "PCG: breakdown (non-positive or non-finite p.Ap)");
    return hs.status;
}

template <int TPR, int U, int NT, int S>
int launch_pcg_staged(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p,
                      grmp_solve_stats *out, char *work, SolveState *dst, WorkLayout lay) {
    grmp_context ctx = A->space->mesh->ctx;
    const int cfg = (NT == 512 ? 20000 : 30000) + 100 * TPR + U;
    if (p->mode != GRMP_SOLVE_MIXED)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "spmv_config %d: staged configurations are for mixed solves", cfg);
    const int prc = ensure_pack32(A);
    if (prc) return prc;
    if (A->stg_state == 0) {
        int rc = stage_build(A);
        if (rc) return rc;
        stage_fill(A);
    }
    if (A->stg_state < 0)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "spmv_config %d: a row does not fit a staged window", cfg);
    const int n = A->nrows;
    auto kern = k_pcg_mixed_staged<TPR, U, NT, S>;
    const int dyn = S * kStgRec;
    cudaError_t e = cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, dyn);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "staged PCG: occupancy");
    if (per_sm < 1) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "spmv_config %d: does not fit an SM", cfg);
    const int maxg = std::min(per_sm * ctx->num_sms, kPartStride / 4);
    int grid = std::min(maxg, std::max(A->stg_nwin, nblk(n, NT)));
    if (p->grid_blocks > 0) grid = std::min(grid, p->grid_blocks);
    grid = std::max(1, grid);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(dst, 0, sizeof(SolveState), ctx->stream);
    float *dinv = (float *)work, *r = (float *)(work + lay.vec), *q = (float *)(work + 2 * lay.vec);
    float *xc = (float *)(work + 3 * lay.vec);
    float2 *zp0 = (float2 *)(work + 4 * lay.vec), *zp1 = (float2 *)(work + 6 * lay.vec);
    double *r64 = (double *)(work + lay.off_r64);
    double *part = (double *)(work + lay.off_part);
    int nn = n, nw = A->stg_nwin, mi = p->maxiter, mo = p->max_outer > 0 ? p->max_outer : 1000;
    int guess = p->use_initial_guess ? 1 : 0;
    double at = p->abstol, rt = p->reltol, dl = p->inner_reltol > 0 && p->inner_reltol < 1 ? p->inner_reltol : 0.1;
    const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
    const double *v64 = A->d_vals64, *bb = bvec;
    const char *rec = A->d_stg_rec;
    double *xx = xvec;
    long long spin = ctx->wait_limit;
    void *args[] = {&nn, &rp, &ci, &v64, &rec, &nw, &bb, &xx, &dinv, &r, &q, &xc, &zp0, &zp1, &r64, &part, &dst,
                    &at, &rt, &dl, &mi, &mo, &guess, &spin};
    cudaEventRecord(e0, ctx->stream);
    e = cudaLaunchCooperativeKernel((void *)kern, grid, NT, args, (size_t)dyn, ctx->stream);
    GRMP_LAUNCHED(ctx);
    cudaEventRecord(e1, ctx->stream);
    SolveState hs;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "staged PCG launch");
    out->status = hs.status;
    out->iterations = hs.iters;
    out->outer_iterations = hs.outer;
    out->final_relres = hs.relres;
    out->spmv_config = cfg;
    out->grid_blocks = grid;
    out->solve_ms = ms;
    if (hs.status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, GRMP_ERR_NOT_CONVERGED, "PCG: %d iterations, relative residual %.3e", hs.iters, hs.relres);
    if (hs.status == GRMP_ERR_TIMEOUT) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "PCG: a barrier wait timed out");
    if (hs.status == GRMP_ERR_NAN) return grmp_fail(ctx, GRMP_ERR_NAN, "PCG: breakdown (non-positive or non-finite p.Ap)");
    return hs.status;
}

// Mixed solve over the duo copy (configurations 60000 + 100 * lanes + duos in flight).
template <int TPR, int U, bool CL = false>
int launch_pcg_duo(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p, grmp_solve_stats *out,
                   char *work, SolveState *dst, WorkLayout lay) {
    grmp_context ctx = A->space->mesh->ctx;
    const int cfg = (CL ? 80000 : 60000) + 100 * TPR + U;
    if (p->mode != GRMP_SOLVE_MIXED)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "spmv_config %d: duo configurations are for mixed solves", cfg);
    int rc = ensure_duo(A);
    if (rc) return rc;
    const int n = A->nrows;
    auto kern = k_pcg_mixed_duo<TPR, U, CL>;
    int grid = 0;
    float *dinv = (float *)work, *r = (float *)(work + lay.vec), *q = (float *)(work + 2 * lay.vec);
    float *xc = (float *)(work + 3 * lay.vec);
    float2 *zp0 = (float2 *)(work + 4 * lay.vec), *zp1 = (float2 *)(work + 6 * lay.vec);
    double *r64 = (double *)(work + lay.off_r64);
    double *part = (double *)(work + lay.off_part);
    int nn = n, mi = p->maxiter, mo = p->max_outer > 0 ? p->max_outer : 1000;
    int guess = p->use_initial_guess ? 1 : 0;
    double at = p->abstol, rt = p->reltol, dl = p->inner_reltol > 0 && p->inner_reltol < 1 ? p->inner_reltol : 0.1;
    const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
    const int4 *mt = (const int4 *)A->d_duo_meta;
    const uint32_t *of = A->d_duo_off;
    const float2 *vl = (const float2 *)A->d_duo_val;
    const double *v64 = A->d_vals64, *bb = bvec;
    double *xx = xvec;
    long long spin = ctx->wait_limit;
    void *args[] = {&nn, &rp, &ci, &v64, &mt, &of, &vl, &bb, &xx, &dinv, &r, &q, &xc, &zp0, &zp1, &r64, &part, &dst,
                    &at, &rt, &dl, &mi, &mo, &guess, &spin};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(dst, 0, sizeof(SolveState), ctx->stream);
    cudaEventRecord(e0, ctx->stream);
    cudaError_t e = launch_persistent<CL>(ctx, kern, n, p->grid_blocks, args, &grid);
    GRMP_LAUNCHED(ctx);
    cudaEventRecord(e1, ctx->stream);
    SolveState hs;
    std::memset(&hs, 0, sizeof(hs));
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "duo PCG launch");
    out->status = hs.status;
    out->iterations = hs.iters;
    out->outer_iterations = hs.outer;
    out->final_relres = hs.relres;
    out->spmv_config = cfg;
    out->grid_blocks = grid;
    out->solve_ms = ms;
    if (hs.status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, GRMP_ERR_NOT_CONVERGED, "PCG: %d iterations, relative residual %.3e", hs.iters, hs.relres);
    if (hs.status == GRMP_ERR_TIMEOUT) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "PCG: a grid barrier wait timed out");
    if (hs.status == GRMP_ERR_NAN) return grmp_fail(ctx, GRMP_ERR_NAN, "PCG: breakdown (non-positive or non-finite p.Ap)");
    return hs.status;
}

// Mixed solve over the Jacobi-scaled duo copy with the row state kept in
// shared memory (configurations 64000 + 100 * lanes + duos in flight).  Each
// block keeps 12 bytes per row of its rows: about 12 n / (number of SMs)
// bytes per SM whatever the grid, so systems beyond about 2.8 M rows do not
// fit (GRMP_ERR_UNSUPPORTED).
template <int TPR, int U, bool ALL, int MINB = (U >= 4 ? 3 : 4)>
int launch_pcg_duo_keep(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p,
                        grmp_solve_stats *out, char *work, SolveState *dst, WorkLayout lay) {
    grmp_context ctx = A->space->mesh->ctx;
    // 64xxx: r, p, A p kept, 3 blocks/SM; 65xxx / 66xxx: A p kept, at least
    // 3 / 4 blocks per SM (registers capped to match: 80 / 64)
    const int cfg = (ALL ? 64000 : 62000 + 1000 * MINB) + 100 * TPR + U;
    constexpr int KW = ALL ? 3 : 1;   // words kept per row
    if (p->mode != GRMP_SOLVE_MIXED)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "spmv_config %d: duo configurations are for mixed solves", cfg);
    int rc = ensure_duo_scaled(A);
    if (rc) return rc;
    const int n = A->nrows;
    constexpr int G = PTPB / TPR;
    auto kern = k_pcg_mixed_duo_keep<TPR, U, ALL, MINB>;
    int dev_max = 0;
    cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PTPB, 0);
    int grid = 0, J = 0;
    size_t smem = 0;
    for (int bps = std::max(1, per_sm); bps >= 1 && !grid; bps--) {
        int gtry = bps * ctx->num_sms;
        if (p->grid_blocks > 0) gtry = std::min(gtry, p->grid_blocks);
        const long long stride = (long long)gtry * G;
        const int jt = (int)((n + stride - 1) / stride);
        const size_t sb = (size_t)KW * jt * G * 4;
        if ((long long)sb > dev_max) continue;
        if (cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb) !=
            cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, PTPB, sb);
        if ((long long)occ * ctx->num_sms >= gtry) {
            grid = gtry;
            J = jt;
            smem = sb;
        }
    }
    if (!grid)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "spmv_config %d: %d rows of row state do not fit shared memory",
                         cfg, n);
    float *xc = (float *)(work + 3 * lay.vec);
    float2 *zp0 = (float2 *)(work + 4 * lay.vec), *zp1 = (float2 *)(work + 6 * lay.vec);
    double *r64 = (double *)(work + lay.off_r64);
    double *part = (double *)(work + lay.off_part);
    int nn = n, mi = p->maxiter, mo = p->max_outer > 0 ? p->max_outer : 1000;
    int guess = p->use_initial_guess ? 1 : 0;
    double at = p->abstol, rt = p->reltol, dl = p->inner_reltol > 0 && p->inner_reltol < 1 ? p->inner_reltol : 0.1;
    const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
    const int4 *mt = (const int4 *)A->d_duo_meta;
    const uint32_t *of = A->d_duo_off;
    const float2 *vl = (const float2 *)A->d_duo_sval;
    const double *v64 = A->d_vals64, *bb = bvec, *scl = A->d_duo_sc;
    double *xx = xvec;
    long long spin = ctx->wait_limit;
    void *args[] = {&nn, &rp, &ci, &v64, &mt, &of, &vl, &bb, &xx, &scl, &xc, &zp0, &zp1, &r64, &part, &dst,
                    &at, &rt, &dl, &mi, &mo, &guess, &spin, &J};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(dst, 0, sizeof(SolveState), ctx->stream);
    cudaEventRecord(e0, ctx->stream);
    cudaError_t e = cudaLaunchCooperativeKernel((void *)kern, grid, PTPB, args, smem, ctx->stream);
    GRMP_LAUNCHED(ctx);
    cudaEventRecord(e1, ctx->stream);
    SolveState hs;
    std::memset(&hs, 0, sizeof(hs));
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "scaled duo PCG launch");
    out->status = hs.status;
    out->iterations = hs.iters;
    out->outer_iterations = hs.outer;
    out->final_relres = hs.relres;
    out->spmv_config = cfg;
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
        case 64208: return launch_pcg_duo_keep<2, 8, true>(A, b, x, p, st, work, dst, lay);
        case 64404: return launch_pcg_duo_keep<4, 4, true>(A, b, x, p, st, work, dst, lay);
        case 65208: return launch_pcg_duo_keep<2, 8, false>(A, b, x, p, st, work, dst, lay);
        case 65404: return launch_pcg_duo_keep<4, 4, false>(A, b, x, p, st, work, dst, lay);
        case 66404: return launch_pcg_duo_keep<4, 4, false, 4>(A, b, x, p, st, work, dst, lay);
        case 70204: return launch_pcg<2, 4, true, true>(A, b, x, p, st, work, dst, lay);
        case 70404: return launch_pcg<4, 4, true, true>(A, b, x, p, st, work, dst, lay);
        case 70802: return launch_pcg<8, 2, true, true>(A, b, x, p, st, work, dst, lay);
        case 80204: return launch_pcg_duo<2, 4, true>(A, b, x, p, st, work, dst, lay);
        case 80404: return launch_pcg_duo<4, 4, true>(A, b, x, p, st, work, dst, lay);
        case 60404: return launch_pcg_duo<4, 4>(A, b, x, p, st, work, dst, lay);
        case 60208: return launch_pcg_duo<2, 8>(A, b, x, p, st, work, dst, lay);
        case 60802: return launch_pcg_duo<8, 2>(A, b, x, p, st, work, dst, lay);
        case 60408: return launch_pcg_duo<4, 8>(A, b, x, p, st, work, dst, lay);
        case 20204: return launch_pcg_staged<2, 4, 512, 3>(A, b, x, p, st, work, dst, lay);
        case 20408: return launch_pcg_staged<4, 8, 512, 3>(A, b, x, p, st, work, dst, lay);
        case 20804: return launch_pcg_staged<8, 4, 512, 3>(A, b, x, p, st, work, dst, lay);
        case 30408: return launch_pcg_staged<4, 8, 1024, 6>(A, b, x, p, st, work, dst, lay);
        case 30804: return launch_pcg_staged<8, 4, 1024, 6>(A, b, x, p, st, work, dst, lay);
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
// the one with the lowest time per iteration; then, for that configuration,
// the persistent grid: as many blocks as fit, one or two per SM (fewer
// blocks make the grid barriers cheaper, which wins on problems whose
// iteration is short).  The persistent kernel's occupancy, barriers and
// vector phases are part of what is measured.  *grid_out: 0 = as many
// blocks as fit.
int autotune_config(grmp_matrix A, const grmp_vector_s *b, const grmp_solve_params *p, char *work, SolveState *dst,
                    WorkLayout lay, int *grid_out) {
    grmp_context ctx = A->space->mesh->ctx;
    const bool mixed = p->mode == GRMP_SOLVE_MIXED;
    *grid_out = 0;
    if (A->nrows < 20000) return heuristic_config(A, mixed);
    double *xs = nullptr;
    if (grmp_alloc(ctx, (void **)&xs, (size_t)A->nrows * 8)) return heuristic_config(A, mixed);
    grmp_solve_params q = *p;
    q.maxiter = 48;
    q.use_initial_guess = 0;
    q.reltol = 0.0;
    q.abstol = 0.0;
    q.grid_blocks = 0;
    // per configuration: one untimed launch (first launch of the
    // instantiation), then the faster of two timed ones
    auto trial = [&](int cfg) {
        grmp_solve_stats s{};
        dispatch_pcg(cfg, A, b->d, xs, &q, &s, work, dst, lay);
        double best = 1e30;
        for (int rep = 0; rep < 2; rep++) {
            s = grmp_solve_stats{};
            dispatch_pcg(cfg, A, b->d, xs, &q, &s, work, dst, lay);
            if (s.iterations > 0) best = std::min(best, (double)s.solve_ms / s.iterations);
        }
        return best;
    };
    int best = heuristic_config(A, mixed);
    double bt = 1e30;
    for (int cfg : kConfigs) {
        if (staged_config(cfg) && (p->mode != GRMP_SOLVE_MIXED || A->stg_state < 0)) continue;
        if (duo_config(cfg) && (p->mode != GRMP_SOLVE_MIXED || A->duo_state < 0)) continue;
        const double per = trial(cfg);
        if (per < bt) {
            bt = per;
            best = cfg;
        }
    }
    for (int g : {ctx->num_sms, 2 * ctx->num_sms}) {
        if (cluster_config(best)) break;   // one cluster: no grid size to choose
        q.grid_blocks = g;
        const double per = trial(best);
        if (per < 0.97 * bt) {   // keep the default unless a smaller grid is clearly faster
            bt = per;
            *grid_out = g;
        }
    }
    grmp_free(ctx, xs, (size_t)A->nrows * 8);
    ctx->last_error.clear();
    return best;
}

template <int TPR, int U>
int launch_bicgstab_t(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p,
                      grmp_solve_stats *out, char *work, SolveState *dst, WorkLayout lay) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    auto kern = k_bicgstab64<TPR, U>;
    const int grid = coop_grid(ctx, kern, n, p->grid_blocks);
    double *dinv = (double *)work;
    double *vv[8];
    for (int k = 0; k < 8; k++) vv[k] = (double *)(work + (size_t)(k + 1) * lay.vec);
    double *part = (double *)(work + lay.off_part);
    int nn = n, mi = p->maxiter, guess = p->use_initial_guess ? 1 : 0;
    double at = p->abstol, rt = p->reltol;
    const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
    const double *vals = A->d_vals64, *bb = bvec;
    double *xx = xvec;
    long long spin = ctx->wait_limit;
    void *args[] = {&nn, &rp, &ci, &vals, &bb, &xx, &dinv, &vv[0], &vv[1], &vv[2], &vv[3], &vv[4], &vv[5], &vv[6],
                    &vv[7], &part, &dst, &at, &rt, &mi, &guess, &spin};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(dst, 0, sizeof(SolveState), ctx->stream);
    cudaEventRecord(e0, ctx->stream);
    cudaError_t e = cudaLaunchCooperativeKernel((void *)kern, grid, PTPB, args, 0, ctx->stream);
    GRMP_LAUNCHED(ctx);
    cudaEventRecord(e1, ctx->stream);
    SolveState hs;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "persistent BiCGStab launch");
    out->status = hs.status;
    out->iterations = hs.iters;
    out->final_relres = hs.relres;
    out->spmv_config = 100 * TPR + U;
    out->grid_blocks = grid;
    out->solve_ms = ms;
    if (hs.status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, GRMP_ERR_NOT_CONVERGED, "BiCGStab: %d iterations, relative residual %.3e", hs.iters,
                         hs.relres);
    if (hs.status == GRMP_ERR_TIMEOUT) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "BiCGStab: a grid barrier wait timed out");
    if (hs.status == GRMP_ERR_NAN) return grmp_fail(ctx, GRMP_ERR_NAN, "BiCGStab: breakdown");
    return hs.status;
}

int launch_bicgstab(grmp_matrix A, const double *b, double *x, const grmp_solve_params *p, grmp_solve_stats *st,
                    char *work, SolveState *dst, WorkLayout lay) {
    switch (heuristic_tpr(A)) {
        case 2: return launch_bicgstab_t<2, 4>(A, b, x, p, st, work, dst, lay);
        case 4: return launch_bicgstab_t<4, 4>(A, b, x, p, st, work, dst, lay);
        case 8: return launch_bicgstab_t<8, 4>(A, b, x, p, st, work, dst, lay);
        default: return launch_bicgstab_t<16, 2>(A, b, x, p, st, work, dst, lay);
    }
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
    //   MIXED: dinv r q xc (float), (z, p) pairs x2 | r64 (double) | partials | state
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t pbytes = (size_t)2 * kPartStride * 8;   // two alternating partial-sum buffers
    size_t vec = mixed ? al((size_t)n * 4) : al((size_t)n * 8);
    const bool bicg = p->mode == GRMP_SOLVE_BICGSTAB;
    // MIXED: dinv, r, q, xc (float) + two (z, p) float2 pair buffers; BICGSTAB: dinv r rh p v s t ph sh
    size_t nvec = mixed ? 8 : (bicg ? 9 : 5);
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
    // Jacobi preconditioner (not for the Jacobi-scaled configurations, which
    // form and check their own row scales)
    const int known = p->spmv_config != 0 ? p->spmv_config : (mixed ? A->tuned_cfg32 : A->tuned_cfg);
    if (!(mixed && scaled_config(known))) {
        int *bad = nullptr;
        int rc = grmp_alloc(ctx, (void **)&bad, 4);
        if (rc) return rc;
        cudaMemsetAsync(bad, 0, 4, ctx->stream);
        if (mixed)
            k_dinv<float><<<nblk(n), 256, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals32, (float *)work, bad);
        else
            k_dinv<double><<<nblk(n), 256, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, (double *)work,
                                                             bad);
        GRMP_LAUNCHED(ctx);
        int hbad = 0;
        cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        grmp_free(ctx, bad, 4);
        if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "jacobi diagonal");
        if (hbad) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: non-positive or non-finite diagonal entry");
    }
    if (bicg) return launch_bicgstab(A, b->d, x->d, p, st, work, dst, lay);
    // the FP32 copies (packed pairs and staged windows, duo values) are
    // refreshed by the first launch that reads them: the values may have been
    // reassembled since the last solve
    A->pack_fresh = false;
    A->duo_fresh = false;
    A->duo_sfresh = false;
    int cfg = p->spmv_config;
    grmp_solve_params q = *p;
    if (cfg == 0) {   // autotuned once per matrix and solver mode (configuration and grid)
        int &slot = mixed ? A->tuned_cfg32 : A->tuned_cfg;
        int &gslot = mixed ? A->tuned_grid32 : A->tuned_grid;
        if (!slot) slot = autotune_config(A, b, p, work, dst, lay, &gslot);
        cfg = slot;
        if (q.grid_blocks <= 0) q.grid_blocks = gslot;
    } else if (cfg < 0) {   // heuristic from the row length: no timing, independent of other work on the GPU
        cfg = heuristic_config(A, mixed);
    }
    return dispatch_pcg(cfg, A, b->d, x->d, &q, st, work, dst, lay);
}

int grmp_spmv_impl(grmp_matrix A, int precision, grmp_vector x, grmp_vector y) {
    grmp_context ctx = A->space->mesh->ctx;
    int n = A->nrows;
    int tpr = A->tuned_cfg ? (A->tuned_cfg % 10000) / 100 : heuristic_tpr(A);
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
// Failure-detection check of the bounded waits (grmp_selftest_wait_timeout):
// every block waits on a shared-memory mbarrier that nothing completes, then
// block 0 leaves while the others wait at a grid barrier it never reaches.
// Both waits give up after `spin` polls and record GRMP_ERR_TIMEOUT; the
// kernel then ends normally, so the context stays usable.
namespace {
__global__ void k_wait_selftest(GridBarrier *bar, int *grid_status, int *mbar_status, long long spin) {
    __shared__ __align__(8) uint64_t mb;
    if (threadIdx.x == 0) {
        mbar_init(&mb, 1);   // one arrival expected; none is ever made
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(&mb, 0, spin)) atomicCAS(mbar_status, 0, (int)GRMP_ERR_TIMEOUT);
    __syncthreads();
    if (blockIdx.x == 0) return;   // the block that never arrives
    grid_barrier(bar, gridDim.x, grid_status, spin);
}
}  // namespace

extern "C" int grmp_selftest_wait_timeout(grmp_context ctx, int64_t polls, int32_t *grid_status,
                                          int32_t *mbar_status) {
    if (!ctx || !ctx->stream || polls < 0 || !grid_status || !mbar_status) return GRMP_ERR_INVALID_ARG;
    cudaError_t se = cudaSetDevice(ctx->device);
    if (se != cudaSuccess) return grmp_cuda_fail(ctx, se, "wait self-test: cudaSetDevice");
    std::lock_guard<std::mutex> lk(ctx->mu);
    struct Words {
        GridBarrier bar;
        int grid_status, mbar_status;
    };
    Words *d = nullptr;
    int rc = grmp_alloc(ctx, (void **)&d, sizeof(Words));
    if (rc) return rc;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wait_selftest, 128, 0);
    const int grid = std::max(2, std::min(2, per_sm) * ctx->num_sms);
    GridBarrier *bar = &d->bar;
    int *gs = &d->grid_status, *ms = &d->mbar_status;
    long long spin = (long long)polls;
    void *args[] = {&bar, &gs, &ms, &spin};
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(Words), ctx->stream);
    if (e == cudaSuccess) e = cudaLaunchCooperativeKernel((void *)k_wait_selftest, grid, 128, args, 0, ctx->stream);
    GRMP_LAUNCHED(ctx);
    Words h;
    std::memset(&h, 0, sizeof(h));
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, d, sizeof(Words));
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "wait self-test launch");
    *grid_status = h.grid_status;
    *mbar_status = h.mbar_status;
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

template <int TPR, int U, bool PIPE, bool CL = false>
cudaError_t launch_pcg64_static(grmp_matrix A, const double *bvec, double *xvec, const grmp_solve_params *p,
                                int grid_blocks, char *work, int *grid_out) {
    grmp_context ctx = A->space->mesh->ctx;
    auto kern = k_pcg64<TPR, U, PIPE, CL>;
    double *dinv = (double *)work, *r = (double *)(work + kNaVec), *z = (double *)(work + 2 * kNaVec);
    double *pp = (double *)(work + 3 * kNaVec), *q = (double *)(work + 4 * kNaVec);
    double *part = (double *)(work + 5 * kNaVec);
    SolveState *dst = (SolveState *)(work + kNaState);
    int nn = A->nrows, mi = p->maxiter, guess = p->use_initial_guess ? 1 : 0;
    double at = p->abstol, rt = p->reltol;
    const int32_t *rp = A->d_rowptr, *ci = A->d_cols;
    const double *vv = A->d_vals64, *bb = bvec;
    double *xx = xvec;
    long long spin = ctx->wait_limit;
    void *args[] = {&nn, &rp, &ci, &vv, &bb, &xx, &dinv, &r, &z, &pp, &q, &part, &dst, &at, &rt, &mi, &guess, &spin};
    cudaError_t e = launch_persistent<CL>(ctx, kern, A->nrows, grid_blocks, args, grid_out);
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
    if (!(p->reltol >= 0) || !(p->abstol >= 0) || p->maxiter <= 0)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: invalid tolerance or maxiter");
    if (A->nrows > GRMP_NOALLOC_MAX_ROWS)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: %d rows exceed the fixed scratch limit of %d rows",
                         A->nrows, GRMP_NOALLOC_MAX_ROWS);
    if (!A->has64) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "noalloc solve: FP64 values not assembled");
    const auto t0 = std::chrono::steady_clock::now();
    cudaError_t se = cudaSetDevice(ctx->device);
    if (se != cudaSuccess) return grmp_cuda_fail(ctx, se, "noalloc solve: cudaSetDevice");
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
    // spmv_config 0 takes grmp_solve's tuned configuration and grid when there are
    // any (so both entry points run the same launch), else the heuristic
    int cfg = p->spmv_config;
    int gb = p->grid_blocks;
    if (cfg <= 0) {
        cfg = A->tuned_cfg ? A->tuned_cfg : heuristic_config(A, false);
        if (A->tuned_cfg && gb <= 0) gb = A->tuned_grid;
    }
    int grid = 0;
    switch (cfg) {
        case 208: e = launch_pcg64_static<2, 8, false>(A, b->d, x->d, p, gb, work, &grid); break;
        case 404: e = launch_pcg64_static<4, 4, false>(A, b->d, x->d, p, gb, work, &grid); break;
        case 408: e = launch_pcg64_static<4, 8, false>(A, b->d, x->d, p, gb, work, &grid); break;
        case 804: e = launch_pcg64_static<8, 4, false>(A, b->d, x->d, p, gb, work, &grid); break;
        case 1602: e = launch_pcg64_static<16, 2, false>(A, b->d, x->d, p, gb, work, &grid); break;
        case 10204: e = launch_pcg64_static<2, 4, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 10404: e = launch_pcg64_static<4, 4, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 10408: e = launch_pcg64_static<4, 8, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 10804: e = launch_pcg64_static<8, 4, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 10402: e = launch_pcg64_static<4, 2, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 10802: e = launch_pcg64_static<8, 2, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 70204: e = launch_pcg64_static<2, 4, true, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 70404: e = launch_pcg64_static<4, 4, true, true>(A, b->d, x->d, p, gb, work, &grid); break;
        case 70802: e = launch_pcg64_static<8, 2, true, true>(A, b->d, x->d, p, gb, work, &grid); break;
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

// Frees the duo copy of a matrix (any part of it may be absent).
void grmp_duo_free(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    const size_t nd = (size_t)A->duo_nduo;
    grmp_free(ctx, A->d_duo_meta, ((size_t)A->nrows + 1) * 16);
    grmp_free(ctx, A->d_duo_off, nd * 4);
    grmp_free(ctx, A->d_duo_src, nd * 4);
    grmp_free(ctx, A->d_duo_val, nd * 8);
    grmp_free(ctx, A->d_duo_sval, nd * 8);
    grmp_free(ctx, A->d_duo_sc, (size_t)A->nrows * 8);
    A->d_duo_meta = A->d_duo_val = A->d_duo_sval = nullptr;
    A->d_duo_sc = nullptr;
    A->d_duo_off = nullptr;
    A->d_duo_src = nullptr;
    A->duo_state = 0;
    A->duo_fresh = false;
    A->duo_sfresh = false;
}
