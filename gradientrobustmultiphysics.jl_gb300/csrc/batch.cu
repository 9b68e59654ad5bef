// Batched iterated-penalty Stokes solver: many independent Bernardi-Raugel /
// P0 problems, one thread block per problem, all in one launch.
//
// Reference: solve_fixpoint_subiterations! (src/solvers.jl:1018-1250) with
// subiterations [[1],[2]] on the operators of
// examples/Example221_StokesIterated2D.jl:80-90 (without the convection term):
//   velocity update  (nu grad u, grad v) + lambda (div R u, div R v)
//                      = (f, R v) + (p, div v)            [R: BR -> RT0]
//   pressure update  (p_new, q) = (p, q) - lambda (div u, q)  on P0
//   FixedIntegralMean(2, 0): the pressure has zero mean (src/globalconstraints.jl:23-44).
// The velocity system is solved by Jacobi-PCG (FP64, or FP32 inside FP64
// refinement) warm-started from the previous sweep's velocity.
//
// Scheduling: a persistent grid of blocks pulls problems from a work queue
// sorted by size (largest first).  A problem never spans blocks, all its
// reductions are block reductions in a fixed order, so its result does not
// depend on which block runs it or on the rest of the batch.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <numeric>
#include <thread>
#include <tuple>

#include "grmp_internal.h"
#include "mf_device.cuh"
#include "nd_symbolic.h"

int grmp_br_divergence(grmp_space s, double **Dv, double **vol);

namespace {

struct BatchDev {
    int nprob;
    const int32_t *order, *row_off, *cell_off;
    const int32_t *rowptr, *cols;
    const double *v64;
    const float *v32;
    const int32_t *inc_ptr, *inc_cell;
    const uint8_t *inc_loc;
    const int32_t *celldofs;
    const double *Dv, *vol;
    const uint8_t *fixed;
    const double *bf;
    double *u, *p;
    // workspace (per row / per cell)
    double *rhs, *r64, *dinv64, *w64a, *w64b, *w64c;
    float *dinv32, *r32, *q32, *xc32;
    float2 *zp0, *zp1;
    // split-penalty inner operator (MIXED, split_penalty = 1)
    float *z32, *p32, *s32, *Dv32, *w32;
    int *queue;
    int *iters, *sweeps_done, *status, *fallbacks;
    double *relres;
    double lambda, sweep_tol, reltol, delta;
    int sweeps, maxit, mixed, split;
    int ld;   // local velocity DoFs per cell: 9 (H1BR{2}) or 16 (H1BR{3})
};

// sum_I Dv[c][I] u[celldofs[c][I]] in ascending I (int_T div u for the
// cell's velocity DoFs)
template <int LD, typename T, typename V>
__device__ __forceinline__ T cell_div_t(const T *Dv, const int32_t *celldofs, const V *u, int c) {
    T a = T(0);
#pragma unroll
    for (int I = 0; I < LD; I++) a += Dv[(size_t)c * LD + I] * u[celldofs[(size_t)c * LD + I]];
    return a;
}
template <typename T, typename V>
__device__ __forceinline__ T cell_div(const BatchDev &d, const T *Dv, const V *u, int c) {
    return d.ld == 9 ? cell_div_t<9>(Dv, d.celldofs, u, c) : cell_div_t<16>(Dv, d.celldofs, u, c);
}

template <int NV>
__device__ __forceinline__ void bsum(double *v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; k++)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < NV; k++) sh[wid * NV + k] = v[k];
    __syncthreads();
    // warp 0 adds the per-warp values (fixed shuffle tree) and publishes the
    // totals; the other threads do not repeat those FP64 additions
    if (wid == 0) {
        double a[NV];
        for (int k = 0; k < NV; k++) a[k] = lane < nw ? sh[lane * NV + k] : 0.0;
        for (int k = 0; k < NV; k++)
            for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
        if (lane == 0)
            for (int k = 0; k < NV; k++) sh[k] = a[k];
    }
    __syncthreads();
    for (int k = 0; k < NV; k++) v[k] = sh[k];
    __syncthreads();
}

__device__ __forceinline__ void bmax1(double *v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v[0] = fmax(v[0], __shfl_xor_sync(0xffffffffu, v[0], o));
    __syncthreads();
    if (lane == 0) sh[wid] = v[0];
    __syncthreads();
    if (wid == 0) {
        double a = lane < nw ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
        if (lane == 0) sh[0] = a;
    }
    __syncthreads();
    v[0] = sh[0];
    __syncthreads();
}

// rows [r0, r1) of y = A x (or y = b - A x with RESID) by the block; returns
// this thread's part of sum w.y (DOT) or of sum y^2 (RESID)
template <int TPR, typename V, typename X, bool RESID>
__device__ __forceinline__ double block_spmv(const BatchDev &d, int r0, int r1, const V *vals, const X *x, X *y,
                                             const X *w, const double *b) {
    constexpr int RPW = 32 / TPR;
    constexpr int U = TPR >= 16 ? 2 : 4;
    using A = typename std::conditional<sizeof(V) == 8, double, float>::type;
    const int lane = threadIdx.x & (TPR - 1), gin = (threadIdx.x & 31) / TPR;
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    double dot = 0;
    for (int base = r0 + warp * RPW; base < r1; base += nwarps * RPW) {
        const int r = base + gin;
        A s = 0;
        if (r < r1) {
            const int kb = __ldg(d.rowptr + r), e = __ldg(d.rowptr + r + 1);
            for (int k = kb + lane; k < e; k += TPR * U) {
                int c[U];
                A v[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int idx = k + u * TPR;
                    const bool ok = idx < e;
                    c[u] = ok ? __ldg(d.cols + idx) : r;
                    v[u] = ok ? (A)__ldg(vals + idx) : A(0);
                }
#pragma unroll
                for (int u = 0; u < U; u++) s += v[u] * (A)x[c[u]];
            }
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (r < r1 && lane == 0) {
            if (RESID) {
                const double v = b[r] - (double)s;
                y[r] = (X)v;
                dot += v * v;
            } else {
                y[r] = (X)s;
                if (w) dot += (double)w[r] * (double)s;
            }
        }
    }
    return dot;
}

template <int TPR>
__device__ __forceinline__ float block_spmv_zp(const BatchDev &d, int r0, int r1, const float2 *cur, float *nxt_f,
                                               float *q, float beta) {
    constexpr int RPW = 32 / TPR;
    constexpr int U = TPR >= 16 ? 2 : 4;
    const int lane = threadIdx.x & (TPR - 1), gin = (threadIdx.x & 31) / TPR;
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    float dacc = 0.f;
    for (int base = r0 + warp * RPW; base < r1; base += nwarps * RPW) {
        const int r = base + gin;
        float s = 0.f;
        if (r < r1) {
            const int kb = __ldg(d.rowptr + r), e = __ldg(d.rowptr + r + 1);
            for (int k = kb + lane; k < e; k += TPR * U) {
                int c[U];
                float v[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int idx = k + u * TPR;
                    const bool ok = idx < e;
                    c[u] = ok ? __ldg(d.cols + idx) : r;
                    v[u] = ok ? __ldg(d.v32 + idx) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const float2 g = cur[c[u]];
                    s += v[u] * __fmaf_rn(beta, g.y, g.x);
                }
            }
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (r < r1 && lane == 0) {
            const float2 me = cur[r];
            const float pn = __fmaf_rn(beta, me.y, me.x);
            nxt_f[2 * r + 1] = pn;
            q[r] = s;
            dacc += pn * s;
        }
    }
    return dacc;
}

// FP32 Jacobi-PCG inside FP64 refinement on rows [r0, r1); x (FP64) holds the
// initial guess and the result.  Returns iterations; *relres = final FP64
// relative residual; *ok = converged.
template <int TPR>
__device__ int block_pcg_mixed(const BatchDev &d, int r0, int r1, const double *rhs, double *x, double *sh,
                               double *relres, bool *ok) {
    const int tid = threadIdx.x, bs = blockDim.x;
    double v[2] = {0, 0};
    v[0] = block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, x, d.r64, nullptr, rhs);
    for (int i = r0 + tid; i < r1; i += bs) v[1] += rhs[i] * rhs[i];
    bsum<2>(v, sh);
    const double bn = sqrt(v[1]);
    const double tol = d.reltol * bn;
    double rn64 = sqrt(v[0]);
    bool conv = rn64 <= tol || bn == 0.0;
    int it = 0;
    float wf0 = 0.f, wf1 = 0.f;
    for (int i = r0 + tid; i < r1; i += bs) {
        const float ri = (float)d.r64[i];
        const float zi = d.dinv32[i] * ri;
        d.r32[i] = ri;
        d.zp0[i] = make_float2(zi, 0.f);
        d.xc32[i] = 0.f;
        wf0 += ri * zi;
        wf1 += ri * ri;
    }
    double w[2] = {(double)wf0, (double)wf1};
    bsum<2>(w, sh);
    double rz = w[0], rmax = sqrt(w[1]), prev = rn64;
    int stall = 0;
    float beta = 0.f;
    float2 *cur = d.zp0, *nxt = d.zp1;
    while (!conv && it < d.maxit) {
        float *nxt_f = reinterpret_cast<float *>(nxt);
        double pq[1] = {(double)block_spmv_zp<TPR>(d, r0, r1, cur, nxt_f, d.q32, beta)};
        bsum<1>(pq, sh);
        if (!(pq[0] > 0) || !isfinite(pq[0])) break;
        const float alpha = (float)(rz / pq[0]);
        float u0 = 0.f, u1 = 0.f;
        for (int i = r0 + tid; i < r1; i += bs) {
            const float pi = nxt_f[2 * i + 1];
            d.xc32[i] += alpha * pi;
            const float ri = d.r32[i] - alpha * d.q32[i];
            d.r32[i] = ri;
            const float zi = d.dinv32[i] * ri;
            nxt_f[2 * i] = zi;
            u0 += ri * zi;
            u1 += ri * ri;
        }
        double u[2] = {(double)u0, (double)u1};
        bsum<2>(u, sh);
        it++;
        double rz_new = u[0];
        const double rn32 = sqrt(u[1]);
        bool restart = false;
        if (rn32 <= d.delta * rmax || rn32 <= tol || it >= d.maxit) {
            for (int i = r0 + tid; i < r1; i += bs) {
                x[i] += (double)d.xc32[i];
                d.xc32[i] = 0.f;
            }
            __syncthreads();
            double t[1] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, x, d.r64, nullptr, rhs)};
            bsum<1>(t, sh);
            rn64 = sqrt(t[0]);
            conv = rn64 <= tol;
            if (conv || it >= d.maxit) break;
            restart = rn64 > 0.5 * prev;
            stall = rn64 > 0.9 * prev ? stall + 1 : 0;
            prev = rn64;
            if (stall >= 16) break;
            float y0 = 0.f, y1 = 0.f;
            for (int i = r0 + tid; i < r1; i += bs) {
                const float ri = (float)d.r64[i];
                const float zi = d.dinv32[i] * ri;
                d.r32[i] = ri;
                nxt_f[2 * i] = zi;
                y0 += ri * zi;
                y1 += ri * ri;
            }
            double y[2] = {(double)y0, (double)y1};
            bsum<2>(y, sh);
            rz_new = y[0];
            rmax = sqrt(y[1]);
        }
        beta = restart ? 0.f : (float)(rz_new / rz);
        rz = rz_new;
        float2 *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    *relres = bn > 0 ? rn64 / bn : 0.0;
    *ok = conv;
    return it;
}

// Inner FP32 operator with the penalty in factored form:
//   q = L32 p + sum_T w_T D_T^T (D_T . p),   w_T = lambda / |T|,
// L32 = FP32 values of (nu grad u, grad v) with Dirichlet rows eliminated,
// D_T[I] = int_T div phi_I with the entries of Dirichlet DoFs zeroed.
// Cells first (s_T = w_T D_T . p), then rows gather the matrix part and the
// incident cells' D_T[loc] s_T.  Returns this thread's part of p.q.
template <int TPR>
__device__ __forceinline__ float block_apply_split(const BatchDev &d, int r0, int r1, int c0, int c1) {
    constexpr int RPW = 32 / TPR;
    constexpr int U = TPR >= 16 ? 2 : 4;
    const int tid = threadIdx.x, bs = blockDim.x;
    const float *p = d.p32;
    for (int c = c0 + tid; c < c1; c += bs) {
        const float a = cell_div(d, (const float *)d.Dv32, p, c);
        d.s32[c] = d.w32[c] * a;
    }
    __syncthreads();
    const int lane = threadIdx.x & (TPR - 1), gin = (threadIdx.x & 31) / TPR;
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    float dacc = 0.f;
    for (int base = r0 + warp * RPW; base < r1; base += nwarps * RPW) {
        const int r = base + gin;
        float sm = 0.f;
        if (r < r1) {
            const int kb = __ldg(d.rowptr + r), e = __ldg(d.rowptr + r + 1);
            for (int k = kb + lane; k < e; k += TPR * U) {
                int c[U];
                float v[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int idx = k + u * TPR;
                    const bool ok = idx < e;
                    c[u] = ok ? __ldg(d.cols + idx) : r;
                    v[u] = ok ? __ldg(d.v32 + idx) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < U; u++) sm += v[u] * p[c[u]];
            }
            const int qb = d.inc_ptr[r], qe = d.inc_ptr[r + 1];
            for (int q = qb + lane; q < qe; q += TPR) {
                const int cell = d.inc_cell[q];
                sm += d.Dv32[(size_t)cell * d.ld + d.inc_loc[q]] * d.s32[cell];
            }
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
        if (r < r1 && lane == 0) {
            d.q32[r] = sm;
            dacc += p[r] * sm;
        }
    }
    return dacc;
}

// FP32 Jacobi-PCG on the split-penalty operator inside FP64 refinement
// (outer residual rhs - A64 x with the assembled FP64 matrix).  Same
// reliable-update and restart rules as block_pcg_mixed.
template <int TPR>
__device__ int block_pcg_mixed_split(const BatchDev &d, int r0, int r1, int c0, int c1, const double *rhs,
                                     double *x, double *sh, double *relres, bool *ok) {
    const int tid = threadIdx.x, bs = blockDim.x;
    double v[2] = {0, 0};
    v[0] = block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, x, d.r64, nullptr, rhs);
    for (int i = r0 + tid; i < r1; i += bs) v[1] += rhs[i] * rhs[i];
    bsum<2>(v, sh);
    const double bn = sqrt(v[1]);
    const double tol = d.reltol * bn;
    double rn64 = sqrt(v[0]);
    bool conv = rn64 <= tol || bn == 0.0;
    int it = 0;
    float wf0 = 0.f, wf1 = 0.f;
    for (int i = r0 + tid; i < r1; i += bs) {
        const float ri = (float)d.r64[i];
        const float zi = d.dinv32[i] * ri;
        d.r32[i] = ri;
        d.p32[i] = zi;
        d.xc32[i] = 0.f;
        wf0 += ri * zi;
        wf1 += ri * ri;
    }
    double w[2] = {(double)wf0, (double)wf1};
    bsum<2>(w, sh);
    double rz = w[0], rmax = sqrt(w[1]), prev = rn64;
    int stall = 0;
    while (!conv && it < d.maxit) {
        double pq[1] = {(double)block_apply_split<TPR>(d, r0, r1, c0, c1)};
        bsum<1>(pq, sh);
        if (!(pq[0] > 0) || !isfinite(pq[0])) break;
        const float alpha = (float)(rz / pq[0]);
        float u0 = 0.f, u1 = 0.f;
        for (int i = r0 + tid; i < r1; i += bs) {
            d.xc32[i] += alpha * d.p32[i];
            const float ri = d.r32[i] - alpha * d.q32[i];
            d.r32[i] = ri;
            const float zi = d.dinv32[i] * ri;
            d.z32[i] = zi;
            u0 += ri * zi;
            u1 += ri * ri;
        }
        double u[2] = {(double)u0, (double)u1};
        bsum<2>(u, sh);
        it++;
        double rz_new = u[0];
        const double rn32 = sqrt(u[1]);
        bool restart = false;
        if (rn32 <= d.delta * rmax || rn32 <= tol || it >= d.maxit) {
            for (int i = r0 + tid; i < r1; i += bs) {
                x[i] += (double)d.xc32[i];
                d.xc32[i] = 0.f;
            }
            __syncthreads();
            double t[1] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, x, d.r64, nullptr, rhs)};
            bsum<1>(t, sh);
            rn64 = sqrt(t[0]);
            conv = rn64 <= tol;
            if (conv || it >= d.maxit) break;
            restart = rn64 > 0.5 * prev;
            stall = rn64 > 0.9 * prev ? stall + 1 : 0;
            prev = rn64;
            if (stall >= 16) break;
            float y0 = 0.f, y1 = 0.f;
            for (int i = r0 + tid; i < r1; i += bs) {
                const float ri = (float)d.r64[i];
                const float zi = d.dinv32[i] * ri;
                d.r32[i] = ri;
                d.z32[i] = zi;
                y0 += ri * zi;
                y1 += ri * ri;
            }
            double y[2] = {(double)y0, (double)y1};
            bsum<2>(y, sh);
            rz_new = y[0];
            rmax = sqrt(y[1]);
        }
        const float beta = restart ? 0.f : (float)(rz_new / rz);
        rz = rz_new;
        for (int i = r0 + tid; i < r1; i += bs) d.p32[i] = __fmaf_rn(beta, d.p32[i], d.z32[i]);
        __syncthreads();
    }
    *relres = bn > 0 ? rn64 / bn : 0.0;
    *ok = conv;
    return it;
}

// Plain FP64 Jacobi-PCG on rows [r0, r1); w64a = z, w64b = p, w64c = q.
template <int TPR>
__device__ int block_pcg64(const BatchDev &d, int r0, int r1, const double *rhs, double *x, double *sh,
                           double *relres, bool *ok) {
    const int tid = threadIdx.x, bs = blockDim.x;
    double *z = d.w64a, *p = d.w64b, *q = d.w64c, *r = d.r64;
    double v[1] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, x, r, nullptr, rhs)};
    bsum<1>(v, sh);
    double w[3] = {0, 0, 0};
    for (int i = r0 + tid; i < r1; i += bs) {
        const double zi = d.dinv64[i] * r[i];
        z[i] = zi;
        p[i] = zi;
        w[0] += r[i] * zi;
        w[1] += r[i] * r[i];
        w[2] += rhs[i] * rhs[i];
    }
    bsum<3>(w, sh);
    const double bn = sqrt(w[2]), tol = d.reltol * bn;
    double rz = w[0], rr = w[1];
    bool conv = sqrt(rr) <= tol || bn == 0.0;
    int it = 0;
    while (!conv && it < d.maxit) {
        double pq[1] = {block_spmv<TPR, double, double, false>(d, r0, r1, d.v64, p, q, p, nullptr)};
        bsum<1>(pq, sh);
        if (!(pq[0] > 0) || !isfinite(pq[0])) break;
        const double alpha = rz / pq[0];
        double u[2] = {0, 0};
        for (int i = r0 + tid; i < r1; i += bs) {
            x[i] += alpha * p[i];
            const double ri = r[i] - alpha * q[i];
            r[i] = ri;
            const double zi = d.dinv64[i] * ri;
            z[i] = zi;
            u[0] += ri * zi;
            u[1] += ri * ri;
        }
        bsum<2>(u, sh);
        it++;
        rr = u[1];
        conv = sqrt(rr) <= tol;
        if (conv) break;
        const double beta = u[0] / rz;
        rz = u[0];
        for (int i = r0 + tid; i < r1; i += bs) p[i] = z[i] + beta * p[i];
        __syncthreads();
    }
    *relres = bn > 0 ? sqrt(rr) / bn : 0.0;
    *ok = conv;
    return it;
}

// rhs = (f, R v) + (p, div v) on the free rows of one problem
__device__ __forceinline__ void block_sweep_rhs(const BatchDev &d, int r0, int r1) {
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        double acc = d.bf[i];
        if (!d.fixed[i])
            for (int q = d.inc_ptr[i]; q < d.inc_ptr[i + 1]; q++) {
                const int cell = d.inc_cell[q];
                acc += d.Dv[(size_t)cell * d.ld + d.inc_loc[q]] * d.p[cell];
            }
        d.rhs[i] = acc;
    }
    __syncthreads();
}

// Pressure update p <- p - lambda (1/|T|) int_T div u, then zero mean.
// Returns true when the sweep tolerance is met (change of p from the
// divergence <= sweep_tol * |p|, both in the volume-weighted norm).
__device__ __forceinline__ bool block_pressure_update(const BatchDev &d, int c0, int c1, double *sh) {
    const int tid = threadIdx.x, bs = blockDim.x;
    double m[3] = {0, 0, 0};   // sum vol*p_new, sum vol
    for (int c = c0 + tid; c < c1; c += bs) {
        const double dv = cell_div(d, d.Dv, (const double *)d.u, c);
        const double dp = d.lambda * dv / d.vol[c];
        const double pn = d.p[c] - dp;
        d.p[c] = pn;
        m[0] += d.vol[c] * pn;
        m[1] += d.vol[c];
    }
    bsum<2>(m, sh);
    const double mean = m[0] / m[1];
    double cmp[2] = {0, 0};
    for (int c = c0 + tid; c < c1; c += bs) {
        const double pn = d.p[c] - mean;
        d.p[c] = pn;
        cmp[1] += d.vol[c] * pn * pn;
    }
    // change of the pressure in this sweep (after the mean shift) from the divergence
    for (int c = c0 + tid; c < c1; c += bs) {
        const double dv = cell_div(d, d.Dv, (const double *)d.u, c);
        const double dp = d.lambda * dv / d.vol[c];
        cmp[0] += d.vol[c] * dp * dp;
    }
    bsum<2>(cmp, sh);
    return d.sweep_tol > 0 && sqrt(cmp[0]) <= d.sweep_tol * sqrt(cmp[1]);
}

template <int TPR>
__global__ void __launch_bounds__(512, 2) k_stokes_batch(BatchDev d) {
    __shared__ double sh[32 * 4];
    __shared__ int slot;
    const int tid = threadIdx.x, bs = blockDim.x;
    while (true) {
        if (tid == 0) slot = atomicAdd(d.queue, 1);
        __syncthreads();
        const int k = slot;
        __syncthreads();
        if (k >= d.nprob) break;
        const int pid = d.order[k];
        const int r0 = d.row_off[pid], r1 = d.row_off[pid + 1];
        const int c0 = d.cell_off[pid], c1 = d.cell_off[pid + 1];
        // Jacobi diagonal, zero initial state
        for (int i = r0 + tid; i < r1; i += bs) {
            double dg = 1.0;
            for (int kk = d.rowptr[i]; kk < d.rowptr[i + 1]; kk++)
                if (d.cols[kk] == i) dg = d.v64[kk];
            d.dinv64[i] = 1.0 / dg;
            if (d.mixed && d.split) {
                d.dinv32[i] = (float)(1.0 / dg);   // diagonal of the whole operator
            } else if (d.mixed) {
                float df = 1.f;
                for (int kk = d.rowptr[i]; kk < d.rowptr[i + 1]; kk++)
                    if (d.cols[kk] == i) df = d.v32[kk];
                d.dinv32[i] = 1.f / df;
            }
            d.u[i] = 0.0;
        }
        for (int c = c0 + tid; c < c1; c += bs) {
            d.p[c] = 0.0;
            if (d.mixed && d.split) {
                for (int I = 0; I < d.ld; I++) {
                    const size_t k = (size_t)c * d.ld + I;
                    d.Dv32[k] = d.fixed[d.celldofs[k]] ? 0.f : (float)d.Dv[k];
                }
                d.w32[c] = (float)(d.lambda / d.vol[c]);
            }
        }
        __syncthreads();
        int total_it = 0, sweep = 0, nfall = 0;
        double worst = 0.0;
        bool all_ok = true;
        for (sweep = 0; sweep < d.sweeps; sweep++) {
            block_sweep_rhs(d, r0, r1);
            double rr;
            bool ok;
            int it = !d.mixed ? block_pcg64<TPR>(d, r0, r1, d.rhs, d.u, sh, &rr, &ok)
                     : d.split ? block_pcg_mixed_split<TPR>(d, r0, r1, c0, c1, d.rhs, d.u, sh, &rr, &ok)
                               : block_pcg_mixed<TPR>(d, r0, r1, d.rhs, d.u, sh, &rr, &ok);
            if (d.mixed && !ok) {
                // FP32 stalled (or hit the cap): finish this sweep in FP64 from the same iterate
                __syncthreads();
                it += block_pcg64<TPR>(d, r0, r1, d.rhs, d.u, sh, &rr, &ok);
                nfall++;
            }
            total_it += it;
            worst = fmax(worst, rr);
            all_ok = all_ok && ok;
            __syncthreads();
            if (block_pressure_update(d, c0, c1, sh)) {
                sweep++;
                break;
            }
        }
        if (tid == 0) {
            d.iters[pid] = total_it;
            d.sweeps_done[pid] = sweep;
            d.relres[pid] = worst;
            d.fallbacks[pid] = nfall;
            d.status[pid] = all_ok ? 0 : (int)GRMP_ERR_NOT_CONVERGED;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------
// Direct mode: one multifrontal Cholesky factorisation per problem (nested-
// dissection assembly tree from nd_symbolic.cpp), reused by every sweep.

struct DNode {
    int s, f, front_off, child_off, nchild, entry_off, nentry, ext_off;
    long long L_off, U_off, uv_off;
};

// A sweep whose refined residual stagnates (FP64 rounding floor of an
// ill-conditioned system) counts as solved when the normwise backward error
// ||r|| / (||A||_inf ||u|| + ||rhs||) is at most this: the computed velocity
// is then the exact solution of a system within this relative distance.
constexpr double kDirectBackwardMax = 1e-13;

// MIXED_DIRECT: CG iterations a sweep may take with the FP32 factor before
// the problem is refactored in FP64 (the penalty systems that an FP32
// factor still resolves need 3-25 per sweep; slower convergence means the
// FP32 factor is too inexact for the problem's conditioning)
constexpr int kMixedCgCap = 100;

struct DirectDev {
    const DNode *node;
    const int32_t *front, *child, *ent_rel, *ent_pos, *ext;
    const int32_t *prob_node0, *prob_nnodes;
    // level schedule of each problem's tree: levels lvl_ptr[prob_lvl0 + l ..
    // + l + 1) index lvl_nodes (node ids, children always in lower levels)
    const int32_t *lvl_ptr, *lvl_nodes, *prob_lvl0, *prob_nlev;
    double *work;                                   // per resident block: [F | U | L | uv | group fronts]
    long long slot_doubles, F_doubles, U_doubles, L_doubles, uv_doubles;
    int max_f, max_s, max_solves;
    int fact_groups;                                // thread groups factoring small fronts concurrently
};

// fronts up to this size are factored by a group of warps (several groups
// per block work on one tree level at the same time)
constexpr int kGroupFront = 96;

// fronts up to this size are solved by one warp (forward and backward)
constexpr int kWarpFront = 96;

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Numeric factorisation of one node by thread group g: assemble the front
// F (original entries + the children's update matrices), eliminate its own
// DoFs (blocked right-looking dense Cholesky), keep the factor columns and
// the update matrix.  Returns false on a non-positive pivot.  Every entry's
// arithmetic is independent of the group's size.
template <typename T>
__device__ bool mf_factor_node(const BatchDev &d, const DirectDev &m, const DNode &nd, long long nnz0, T *F,
                               T *U, T *L, T *colk, T *P, ThreadGroup g) {
    const int lane = threadIdx.x & 31, gw = g.tid >> 5, gnw = g.size >> 5;
    const int f = nd.f, s = nd.s;
    for (long long q = g.tid; q < (long long)f * f; q += g.size) F[q] = 0.0;
    g.sync();
    for (int e = g.tid; e < nd.nentry; e += g.size)
        F[m.ent_pos[nd.entry_off + e]] = (T)d.v64[nnz0 + m.ent_rel[nd.entry_off + e]];
    g.sync();
    for (int q = 0; q < nd.nchild; q++) {
        const DNode cn = m.node[m.child[nd.child_off + q]];
        const int sc = cn.f - cn.s;
        const T *Uc = U + cn.U_off;
        const int32_t *ex = m.ext + cn.ext_off;
        for (int a = gw; a < sc; a += gnw) {
            const long long pa = (long long)ex[a] * f;
            for (int b = lane; b <= a; b += 32) F[pa + ex[b]] += Uc[(long long)a * sc + b];
        }
        g.sync();
    }
    if (!front_cholesky<T>(F, f, s, colk, P, kPanelStride, g)) return false;
    T *Lt = L + nd.L_off;
    for (long long q = g.tid; q < (long long)f * s; q += g.size) {
        const int i = (int)(q / s), j = (int)(q - (long long)i * s);
        Lt[q] = j <= i ? F[(long long)i * f + j] : 0.0;
    }
    const int sc = f - s;
    T *Ut = U + nd.U_off;
    for (long long q = g.tid; q < (long long)sc * sc; q += g.size) {
        const int a = (int)(q / sc), b = (int)(q - (long long)a * sc);
        if (b <= a) Ut[q] = F[(long long)(s + a) * f + s + b];
    }
    g.sync();
    return true;
}

// Numeric factorisation of one problem, level by level from the leaves:
// fronts of at most kGroupFront rows by m.fact_groups groups of warps in
// parallel (each with its own front scratch Fg, pivot column and panel
// shares of colk and P), larger fronts by the whole block one after another.
template <typename T>
__device__ bool mf_factor_lv(const BatchDev &d, const DirectDev &m, int lv0, int nlev, long long nnz0, T *F,
                             T *U, T *L, T *colk, T *P, T *Fg, int *fail) {
    const int ng = m.fact_groups;
    const int gsize = blockDim.x / ng, gid = threadIdx.x / gsize;
    const ThreadGroup grp{(int)threadIdx.x - gid * gsize, gsize, 1 + gid};
    T *gF = Fg + (long long)gid * kGroupFront * kGroupFront;
    T *gcolk = colk + gid * kGroupFront;
    T *gP = P + (long long)gid * kGroupFront * kPanelStride;
    if (threadIdx.x == 0) *fail = 0;
    __syncthreads();
    for (int l = 0; l < nlev; l++) {
        const int a = m.lvl_ptr[lv0 + l], b = m.lvl_ptr[lv0 + l + 1];
        if (ng > 1)
            for (int i = a + gid; i < b; i += ng) {
                const DNode nd = m.node[m.lvl_nodes[i]];
                if (nd.f <= kGroupFront && !mf_factor_node(d, m, nd, nnz0, gF, U, L, gcolk, gP, grp) && grp.tid == 0)
                    atomicOr(fail, 1);
            }
        __syncthreads();
        if (*(volatile int *)fail) return false;
        for (int i = a; i < b; i++) {
            const DNode nd = m.node[m.lvl_nodes[i]];
            if ((ng == 1 || nd.f > kGroupFront) && !mf_factor_node(d, m, nd, nnz0, F, U, L, colk, P, whole_block()))
                return false;
        }
    }
    return true;
}

// Level-scheduled solve w <- A^{-1} w.  Forward (leaves up): every node
// forms its front vector from its own entries of w and its children's update
// vectors (extend-add, children in tree order), eliminates its s pivots
// (y into w), and leaves the remaining f - s entries as its own update
// vector; backward (root down): every node solves its pivots from its
// ancestors' values already in w.  Nodes of one level are independent, so
// fronts of at most kWarpFront rows go one per warp in parallel and the
// larger ones through the whole block; one block barrier per level.  Fixed
// order everywhere, no atomics: bit-reproducible.
template <typename T>
__device__ void mf_fwd_warp(const DirectDev &m, const DNode &nd, T *w, const T *L, T *uv, T *v,
                            int lane) {
    const int f = nd.f, s = nd.s;
    const int32_t *fr = m.front + nd.front_off;
    const T *Lt = L + nd.L_off;
    for (int k = lane; k < f; k += 32) v[k] = k < s ? w[fr[k]] : 0.0;
    __syncwarp();
    for (int q = 0; q < nd.nchild; q++) {
        const DNode cn = m.node[m.child[nd.child_off + q]];
        const int sc = cn.f - cn.s;
        const int32_t *ex = m.ext + cn.ext_off;
        const T *uc = uv + cn.uv_off;
        for (int a = lane; a < sc; a += 32) v[ex[a]] += uc[a];
        __syncwarp();
    }
    // column-oriented elimination; the next column of L (rows below its
    // diagonal, up to three per lane) and its diagonal entry are loaded
    // while the current column is applied
    T lc[3], ln[3], dk = s > 0 ? Lt[0] : 1.0, dn = 1.0;
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const int j = 1 + lane + 32 * t;
        lc[t] = (s > 0 && j < f) ? Lt[(long long)j * s] : 0.0;
    }
    for (int k = 0; k < s; k++) {
        const bool more = k + 1 < s;
#pragma unroll
        for (int t = 0; t < 3; t++) {
            const int j = k + 2 + lane + 32 * t;
            ln[t] = (more && j < f) ? Lt[(long long)j * s + k + 1] : 0.0;
        }
        if (more) dn = Lt[(long long)(k + 1) * s + k + 1];
        const T yk = v[k] / dk;
#pragma unroll
        for (int t = 0; t < 3; t++) {
            const int j = k + 1 + lane + 32 * t;
            if (j < f) v[j] -= lc[t] * yk;
        }
        __syncwarp();
        if (lane == 0) v[k] = yk;
        __syncwarp();
#pragma unroll
        for (int t = 0; t < 3; t++) lc[t] = ln[t];
        dk = dn;
    }
    for (int k = lane; k < s; k += 32) w[fr[k]] = v[k];
    T *uo = uv + nd.uv_off;
    for (int j = lane; j < f - s; j += 32) uo[j] = v[s + j];
    __syncwarp();
}

template <typename T>
__device__ void mf_bwd_warp(const DirectDev &m, const DNode &nd, T *w, const T *L, T *v, int lane) {
    const int f = nd.f, s = nd.s, sc = f - s;
    const int32_t *fr = m.front + nd.front_off;
    const T *Lt = L + nd.L_off;
    T *xs = v + s;
    for (int i = lane; i < sc; i += 32) xs[i] = w[fr[s + i]];
    __syncwarp();
    for (int k = lane; k < s; k += 32) {
        T acc = w[fr[k]];
        for (int i = 0; i < sc; i++) acc -= Lt[(long long)(s + i) * s + k] * xs[i];
        v[k] = acc;
    }
    __syncwarp();
    // row k of L11 (entries left of its diagonal, up to three per lane since
    // s <= kWarpFront) and the next diagonal are loaded one step ahead
    T rc[3], rn[3], dk = s > 0 ? Lt[(long long)(s - 1) * s + s - 1] : 1.0, dn = 1.0;
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const int j = lane + 32 * t;
        rc[t] = (s > 0 && j < s - 1) ? Lt[(long long)(s - 1) * s + j] : 0.0;
    }
    for (int k = s - 1; k >= 0; k--) {
        const bool more = k > 0;
#pragma unroll
        for (int t = 0; t < 3; t++) {
            const int j = lane + 32 * t;
            rn[t] = (more && j < k - 1) ? Lt[(long long)(k - 1) * s + j] : 0.0;
        }
        if (more) dn = Lt[(long long)(k - 1) * s + k - 1];
        const T xk = v[k] / dk;
#pragma unroll
        for (int t = 0; t < 3; t++) {
            const int j = lane + 32 * t;
            if (j < k) v[j] -= rc[t] * xk;
        }
        __syncwarp();
        if (lane == 0) v[k] = xk;
        __syncwarp();
#pragma unroll
        for (int t = 0; t < 3; t++) rc[t] = rn[t];
        dk = dn;
    }
    for (int k = lane; k < s; k += 32) w[fr[k]] = v[k];
    __syncwarp();
}

// one large front by the whole block (fv: shared front vector, max_f)
template <typename T>
__device__ void mf_fwd_block(const DirectDev &m, const DNode &nd, T *w, const T *L, T *uv, T *fv,
                             T *tile) {
    const int tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
    const int f = nd.f, s = nd.s;
    const int32_t *fr = m.front + nd.front_off;
    const T *Lt = L + nd.L_off;
    for (int k = tid; k < f; k += bs) fv[k] = k < s ? w[fr[k]] : 0.0;
    __syncthreads();
    for (int q = 0; q < nd.nchild; q++) {
        const DNode cn = m.node[m.child[nd.child_off + q]];
        const int sc = cn.f - cn.s;
        const int32_t *ex = m.ext + cn.ext_off;
        const T *uc = uv + cn.uv_off;
        for (int a = tid; a < sc; a += bs) fv[ex[a]] += uc[a];
        __syncthreads();
    }
    for (int kb = 0; kb < s; kb += 32) {
        const int nbk = min(32, s - kb);
        if (kb > 0)
            for (int r = warp; r < nbk; r += nw) {
                const T *Li = Lt + (long long)(kb + r) * s;
                T acc = 0.0;
                for (int j = lane; j < kb; j += 32) acc += Li[j] * fv[j];
                acc = warp_sum_t(acc);
                if (lane == 0) fv[kb + r] -= acc;
            }
        for (int q = tid; q < nbk * nbk; q += bs) {
            const int r = q / nbk, c = q - r * nbk;
            tile[r * 33 + c] = c <= r ? Lt[(long long)(kb + r) * s + kb + c] : 0.0;
        }
        __syncthreads();
        if (warp == 0) {
            T vv = lane < nbk ? fv[kb + lane] : 0.0;
            for (int c = 0; c < nbk; c++) {
                const T yc = __shfl_sync(0xffffffffu, vv, c) / tile[c * 33 + c];
                if (lane == c) vv = yc;
                else if (lane > c && lane < nbk) vv -= tile[lane * 33 + c] * yc;
            }
            if (lane < nbk) fv[kb + lane] = vv;
        }
        __syncthreads();
    }
    for (int k = tid; k < s; k += bs) w[fr[k]] = fv[k];
    T *uo = uv + nd.uv_off;
    for (int i = s + warp; i < f; i += nw) {
        const T *Li = Lt + (long long)i * s;
        T acc = 0.0;
        for (int k = lane; k < s; k += 32) acc += Li[k] * fv[k];
        acc = warp_sum_t(acc);
        if (lane == 0) uo[i - s] = fv[i] - acc;
    }
    __syncthreads();
}

template <typename T>
__device__ void mf_bwd_block(const DirectDev &m, const DNode &nd, T *w, const T *L, T *ys, T *xs,
                             T *tile) {
    const int tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int f = nd.f, s = nd.s, sc = f - s;
    const int32_t *fr = m.front + nd.front_off;
    const T *Lt = L + nd.L_off;
    for (int i = tid; i < sc; i += bs) xs[i] = w[fr[s + i]];
    __syncthreads();
    for (int k = tid; k < s; k += bs) {
        T acc = w[fr[k]];
        for (int i = 0; i < sc; i++) acc -= Lt[(long long)(s + i) * s + k] * xs[i];
        ys[k] = acc;
    }
    __syncthreads();
    for (int kb = ((s + 31) / 32 - 1) * 32; kb >= 0; kb -= 32) {
        const int nbk = min(32, s - kb);
        for (int q = tid; q < nbk * nbk; q += bs) {
            const int r = q / nbk, c = q - r * nbk;
            tile[r * 33 + c] = c <= r ? Lt[(long long)(kb + r) * s + kb + c] : 0.0;
        }
        __syncthreads();
        if (warp == 0) {
            T vv = lane < nbk ? ys[kb + lane] : 0.0;
            for (int c = nbk - 1; c >= 0; c--) {
                const T xc = __shfl_sync(0xffffffffu, vv, c) / tile[c * 33 + c];
                if (lane == c) vv = xc;
                else if (lane < c) vv -= tile[c * 33 + lane] * xc;
            }
            if (lane < nbk) ys[kb + lane] = vv;
        }
        __syncthreads();
        for (int k = tid; k < kb; k += bs) {
            T acc = 0.0;
            for (int r = 0; r < nbk; r++) acc += Lt[(long long)(kb + r) * s + k] * ys[kb + r];
            ys[k] -= acc;
        }
        __syncthreads();
    }
    for (int k = tid; k < s; k += bs) w[fr[k]] = ys[k];
    __syncthreads();
}

template <typename T>
__device__ void mf_solve_lv(const DirectDev &m, int lv0, int nlev, T *w, const T *L, T *uv,
                            T *fv, T *ys, T *xs, T *tile, T *wbuf) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    T *v = wbuf + warp * kWarpFront;
    for (int l = 0; l < nlev; l++) {
        const int a = m.lvl_ptr[lv0 + l], b = m.lvl_ptr[lv0 + l + 1];
        for (int i = a + warp; i < b; i += nw) {
            const DNode nd = m.node[m.lvl_nodes[i]];
            if (nd.f <= kWarpFront) mf_fwd_warp(m, nd, w, L, uv, v, lane);
        }
        __syncthreads();
        for (int i = a; i < b; i++) {
            const DNode nd = m.node[m.lvl_nodes[i]];
            if (nd.f > kWarpFront) mf_fwd_block(m, nd, w, L, uv, fv, tile);
        }
    }
    for (int l = nlev - 1; l >= 0; l--) {
        const int a = m.lvl_ptr[lv0 + l], b = m.lvl_ptr[lv0 + l + 1];
        for (int i = a; i < b; i++) {
            const DNode nd = m.node[m.lvl_nodes[i]];
            if (nd.f > kWarpFront) mf_bwd_block(m, nd, w, L, ys, xs, tile);
        }
        for (int i = a + warp; i < b; i += nw) {
            const DNode nd = m.node[m.lvl_nodes[i]];
            if (nd.f <= kWarpFront) mf_bwd_warp(m, nd, w, L, v, lane);
        }
        __syncthreads();
    }
}

// z = M^{-1} r for rows [r0, r1) with the FP32 factor: r rounded into the
// problem's FP32 work vector, the level-scheduled FP32 solve, z back in FP64.
__device__ void mf_prec32(const BatchDev &d, const DirectDev &m, int pid, int r0, int r1, const double *r, double *z,
                          const float *L, float *uv, float *fv, float *ys, float *xs, float *tile, float *wbuf) {
    float *w = d.r32 + r0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) w[i - r0] = (float)r[i];
    __syncthreads();
    mf_solve_lv<float>(m, m.prob_lvl0[pid], m.prob_nlev[pid], w, L, uv, fv, ys, xs, tile, wbuf);
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) z[i] = (double)w[i - r0];
    __syncthreads();
}

// MIXED = false: FP64 factorisation, each sweep refined against the FP64
// matrix.  MIXED = true: FP32 factorisation (GB300's FP32 rate is ~64x its
// FP64 rate), each sweep solved by FP64 conjugate gradients on the FP64
// matrix preconditioned by the FP32 factor, warm-started from the previous
// sweep's velocity; a problem whose FP32 factorisation meets a non-positive
// pivot, or whose preconditioned CG stalls above the tolerance, is factored
// again in FP64 and finishes in the FP64 mode (counted in fallbacks).
template <int TPR, bool MIXED>
__global__ void __launch_bounds__(512, 1) k_stokes_direct(BatchDev d, DirectDev m) {
    extern __shared__ double dsm[];
    __shared__ double sh[32 * 4];
    __shared__ int slot;
    double *colk = dsm;                 // factor: column k of the front; solve: a large front's vector
    double *ys = dsm + m.max_f;
    double *tile = ys + m.max_s;
    double *P = tile + 32 * 33;         // factor: the current panel's rows below it; solve: structure values
    double *wbuf = P + (long long)m.max_f * kPanelStride;   // solve: one small front per warp
    double *F = m.work + (long long)blockIdx.x * m.slot_doubles;
    double *U = F + m.F_doubles, *L = U + m.U_doubles, *uvw = L + m.L_doubles, *Fg = uvw + m.uv_doubles;
    __shared__ int fail_flag;
    const int tid = threadIdx.x, bs = blockDim.x;
    while (true) {
        if (tid == 0) slot = atomicAdd(d.queue, 1);
        __syncthreads();
        const int k = slot;
        __syncthreads();
        if (k >= d.nprob) break;
        const int pid = d.order[k];
        const int r0 = d.row_off[pid], r1 = d.row_off[pid + 1];
        const int c0 = d.cell_off[pid], c1 = d.cell_off[pid + 1];
        for (int i = r0 + tid; i < r1; i += bs) d.u[i] = 0.0;
        for (int c = c0 + tid; c < c1; c += bs) d.p[c] = 0.0;
        __syncthreads();
        bool use32 = MIXED;
        int nfall = 0;
        bool fact_ok = false;
        if (MIXED) {
            fact_ok = mf_factor_lv<float>(d, m, m.prob_lvl0[pid], m.prob_nlev[pid], (long long)d.rowptr[r0], (float *)F,
                                          (float *)U, (float *)L, (float *)colk, (float *)P, (float *)Fg, &fail_flag);
            __syncthreads();
            if (!fact_ok) {
                use32 = false;
                nfall = 1;
            }
        }
        if (!use32)
            fact_ok = mf_factor_lv<double>(d, m, m.prob_lvl0[pid], m.prob_nlev[pid], (long long)d.rowptr[r0], F, U, L,
                                           colk, P, Fg, &fail_flag);
        __syncthreads();
        // ||A||_inf of the problem (for the normwise backward error of a solve)
        double an[1] = {0.0};
        for (int i = r0 + tid; i < r1; i += bs) {
            double rs = 0.0;
            for (int kk = d.rowptr[i]; kk < d.rowptr[i + 1]; kk++) rs += fabs(d.v64[kk]);
            an[0] = fmax(an[0], rs);
        }
        bmax1(an, sh);
        const double anorm = an[0];
        int nsolve = 0, sweep = 0;
        double worst = 0.0;
        bool all_ok = fact_ok;
        if (fact_ok)
            for (sweep = 0; sweep < d.sweeps; sweep++) {
                block_sweep_rhs(d, r0, r1);
                double bb[1] = {0.0};
                for (int i = r0 + tid; i < r1; i += bs) bb[0] += d.rhs[i] * d.rhs[i];
                bsum<1>(bb, sh);
                const double bn = sqrt(bb[0]);
                double rel = 0.0, prev = INFINITY, eta = 0.0;
                bool floor = false;
                bool done32 = false;
                if (MIXED && use32) {
                    // FP64 CG preconditioned by the FP32 factor (x = u, r = rhs - A u)
                    double *z = d.w64a, *pp = d.w64b, *q = d.w64c, *r = d.r64;
                    double v[1] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, d.u, r, nullptr, d.rhs)};
                    bsum<1>(v, sh);
                    rel = bn > 0 ? sqrt(v[0]) / bn : 0.0;
                    if (rel <= d.reltol) done32 = true;
                    double rz = 0.0, best = rel;
                    int since = 0, restarts = 0;
                    int cg_its = 0;
                    for (int it = 0; !done32 && cg_its < kMixedCgCap; it++, cg_its++) {
                        mf_prec32(d, m, pid, r0, r1, r, z, (const float *)L, (float *)uvw, (float *)colk, (float *)ys,
                                  (float *)P, (float *)tile, (float *)wbuf);
                        double w1[1] = {0.0};
                        for (int i = r0 + tid; i < r1; i += bs) w1[0] += r[i] * z[i];
                        bsum<1>(w1, sh);
                        const double beta = it == 0 ? 0.0 : w1[0] / rz;
                        rz = w1[0];
                        for (int i = r0 + tid; i < r1; i += bs) pp[i] = z[i] + beta * (it == 0 ? 0.0 : pp[i]);
                        __syncthreads();
                        double pq[1] = {block_spmv<TPR, double, double, false>(d, r0, r1, d.v64, pp, q, pp, nullptr)};
                        bsum<1>(pq, sh);
                        if (!(pq[0] > 0.0) || !isfinite(pq[0])) break;
                        const double alpha = rz / pq[0];
                        double w2[1] = {0.0};
                        for (int i = r0 + tid; i < r1; i += bs) {
                            d.u[i] += alpha * pp[i];
                            const double ri = r[i] - alpha * q[i];
                            r[i] = ri;
                            w2[0] += ri * ri;
                        }
                        bsum<1>(w2, sh);
                        nsolve++;
                        rel = bn > 0 ? sqrt(w2[0]) / bn : 0.0;
                        if (rel <= d.reltol) {   // confirm with the true residual
                            double t[1] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, d.u, r, nullptr,
                                                                                 d.rhs)};
                            bsum<1>(t, sh);
                            rel = bn > 0 ? sqrt(t[0]) / bn : 0.0;
                            if (rel <= d.reltol) {
                                done32 = true;
                                break;
                            }
                            if (++restarts > 3) break;
                            it = -1;   // restart from the true residual
                        }
                        if (rel < 0.5 * best) {
                            best = rel;
                            since = 0;
                        } else if (++since >= 20) {
                            break;   // stalled
                        }
                    }
                    if (!done32 && cg_its < kMixedCgCap) {
                        // a stall at the FP64 floor of an ill-conditioned system is accepted by backward error
                        double t[2] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, d.u, r, nullptr, d.rhs),
                                       0.0};
                        for (int i = r0 + tid; i < r1; i += bs) t[1] += d.u[i] * d.u[i];
                        bsum<2>(t, sh);
                        rel = bn > 0 ? sqrt(t[0]) / bn : 0.0;
                        eta = sqrt(t[0]) / (anorm * sqrt(t[1]) + bn + 1e-300);
                        if (eta <= kDirectBackwardMax) {
                            floor = true;
                            done32 = true;
                        }
                    }
                    if (!done32) {
                        // fall back: factor in FP64 and finish this problem in the FP64 mode
                        use32 = false;
                        nfall = 1;
                        fact_ok = mf_factor_lv<double>(d, m, m.prob_lvl0[pid], m.prob_nlev[pid],
                                                       (long long)d.rowptr[r0], F, U, L, colk, P, Fg, &fail_flag);
                        __syncthreads();
                        if (!fact_ok) {
                            all_ok = false;
                            break;
                        }
                    }
                }
                if (!done32) {
                    for (int ref = 0;; ref++) {
                        // r = rhs - A u (FP64, assembled matrix); stop at reltol or when the
                        // residual stops falling (the FP64 floor of an ill-conditioned
                        // system), else u += A^{-1} r
                        double v[2] = {block_spmv<TPR, double, double, true>(d, r0, r1, d.v64, d.u, d.r64, nullptr, d.rhs),
                                       0.0};
                        for (int i = r0 + tid; i < r1; i += bs) v[1] += d.u[i] * d.u[i];
                        bsum<2>(v, sh);
                        rel = bn > 0 ? sqrt(v[0]) / bn : 0.0;
                        eta = sqrt(v[0]) / (anorm * sqrt(v[1]) + bn + 1e-300);   // normwise backward error
                        if (rel <= d.reltol) break;
                        if (ref > 0 && rel > 0.5 * prev) {
                            floor = true;
                            break;
                        }
                        if (ref >= m.max_solves) break;
                        prev = rel;
                        mf_solve_lv<double>(m, m.prob_lvl0[pid], m.prob_nlev[pid], d.r64 + r0, L, uvw, colk, ys, P, tile,
                                            wbuf);
                        for (int i = r0 + tid; i < r1; i += bs) d.u[i] += d.r64[i];
                        __syncthreads();
                        nsolve++;
                    }
                }
                worst = fmax(worst, rel);
                all_ok = all_ok && (rel <= d.reltol || (floor && eta <= kDirectBackwardMax));
                if (block_pressure_update(d, c0, c1, sh)) {
                    sweep++;
                    break;
                }
            }
        if (tid == 0) {
            d.iters[pid] = nsolve;
            d.sweeps_done[pid] = sweep;
            d.relres[pid] = fact_ok ? worst : INFINITY;
            d.fallbacks[pid] = nfall;
            d.status[pid] = !fact_ok ? (int)GRMP_ERR_NAN : (all_ok ? 0 : (int)GRMP_ERR_NOT_CONVERGED);
        }
        __syncthreads();
    }
}

// 64-bit fingerprint of each problem's local pattern (row lengths and
// row-relative columns), summed over nonzeros so the reduction order does
// not matter.
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__global__ void k_pattern_hash(int nprob, const int32_t *row_off, const int32_t *rowptr, const int32_t *cols,
                               unsigned long long *hash) {
    const int pid = blockIdx.x;
    if (pid >= nprob) return;
    const int r0 = row_off[pid], r1 = row_off[pid + 1];
    const long long nnz0 = rowptr[r0];
    unsigned long long h = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
            h += mix64(((unsigned long long)(k - nnz0) << 32) ^ (unsigned long long)(uint32_t)(cols[k] - r0) ^
                       ((unsigned long long)(i - r0) << 52));
    atomicAdd(hash + pid, h);
}

// bad[p] = 1 when problem p's local pattern differs from problem rep[p]'s
__global__ void k_pattern_equal(int nprob, const int32_t *row_off, const int32_t *rowptr, const int32_t *cols,
                                const int32_t *rep, int *bad) {
    const int pid = blockIdx.x;
    if (pid >= nprob) return;
    const int q = rep[pid];
    if (q == pid) return;
    const int r0 = row_off[pid], s0 = row_off[q];
    const int n = row_off[pid + 1] - r0;
    if (n != row_off[q + 1] - s0) {
        if (threadIdx.x == 0) bad[pid] = 1;
        return;
    }
    const long long a0 = rowptr[r0], b0 = rowptr[s0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ka = rowptr[r0 + i], kb = rowptr[s0 + i];
        const int la = rowptr[r0 + i + 1] - ka, lb = rowptr[s0 + i + 1] - kb;
        if (la != lb || ka - a0 != kb - b0) {
            bad[pid] = 1;
            continue;
        }
        for (int j = 0; j < la; j++)
            if (cols[ka + j] - r0 != cols[kb + j] - s0) bad[pid] = 1;
    }
}

__global__ void k_check_blocks(int nprob, const int32_t *row_off, const int32_t *rowptr, const int32_t *cols,
                               int *bad) {
    int pid = blockIdx.x;
    if (pid >= nprob) return;
    const int r0 = row_off[pid], r1 = row_off[pid + 1];
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
            if (cols[k] < r0 || cols[k] >= r1) atomicExch(bad, 1);
}

}  // namespace

// ---------------------------------------------------------------- direct-mode symbolic cache

struct DirectCache {
    std::vector<int32_t> row_offsets;
    std::vector<std::pair<void *, size_t>> bufs;
    const DNode *node = nullptr;
    const int32_t *front = nullptr, *child = nullptr, *ent_rel = nullptr, *ent_pos = nullptr, *ext = nullptr;
    const int32_t *prob_node0 = nullptr, *prob_nnodes = nullptr;
    const int32_t *lvl_ptr = nullptr, *lvl_nodes = nullptr, *prob_lvl0 = nullptr, *prob_nlev = nullptr;
    long long max_U = 0, max_L = 0, max_uv = 0;
    int max_f = 0, max_s = 0, groups = 0;
};

namespace {

template <typename T>
int upload_vec(grmp_context ctx, DirectCache &C, const std::vector<T> &v, const T **out) {
    T *p = nullptr;
    const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
    int rc = grmp_alloc(ctx, (void **)&p, bytes);
    if (rc) return rc;
    C.bufs.push_back({p, bytes});
    if (!v.empty()) {
        cudaError_t e = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "direct cache upload");
    }
    *out = p;
    return GRMP_OK;
}

// Group problems by local pattern (device fingerprint, then a device
// comparison against the group's first problem), analyse one pattern per
// group on the host cores, upload the concatenated trees.
int build_direct_cache(grmp_matrix A, int np, const int32_t *row_off, const int32_t *drow) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    std::vector<int32_t> rowptr(n + 1);
    cudaError_t e = cudaMemcpyAsync(rowptr.data(), A->d_rowptr, (size_t)(n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    unsigned long long *dh = nullptr;
    int32_t *drep = nullptr;
    int *dbad = nullptr;
    int rc = grmp_alloc(ctx, (void **)&dh, (size_t)np * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&drep, (size_t)np * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&dbad, (size_t)np * 4);
    auto cleanup = [&]() {
        grmp_free(ctx, dh, (size_t)np * 8);
        grmp_free(ctx, drep, (size_t)np * 4);
        grmp_free(ctx, dbad, (size_t)np * 4);
    };
    if (rc) {
        cleanup();
        return rc;
    }
    std::vector<unsigned long long> h(np);
    cudaMemsetAsync(dh, 0, (size_t)np * 8, ctx->stream);
    k_pattern_hash<<<np, 256, 0, ctx->stream>>>(np, drow, A->d_rowptr, A->d_cols, dh);
    GRMP_LAUNCHED(ctx);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), dh, (size_t)np * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cleanup();
        return grmp_cuda_fail(ctx, e, "direct: pattern fingerprints");
    }
    std::vector<int32_t> rep(np);
    {
        std::vector<std::pair<std::pair<long long, long long>, unsigned long long>> keys;
        std::vector<std::tuple<long long, long long, unsigned long long, int>> seen;
        for (int k = 0; k < np; k++) {
            const long long nk = row_off[k + 1] - row_off[k];
            const long long zk = (long long)rowptr[row_off[k + 1]] - rowptr[row_off[k]];
            int r = k;
            for (auto &t : seen)
                if (std::get<0>(t) == nk && std::get<1>(t) == zk && std::get<2>(t) == h[k]) {
                    r = std::get<3>(t);
                    break;
                }
            if (r == k) seen.emplace_back(nk, zk, h[k], k);
            rep[k] = r;
        }
    }
    std::vector<int> bad(np, 0);
    cudaMemcpyAsync(drep, rep.data(), (size_t)np * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(dbad, 0, (size_t)np * 4, ctx->stream);
    k_pattern_equal<<<np, 256, 0, ctx->stream>>>(np, drow, A->d_rowptr, A->d_cols, drep, dbad);
    GRMP_LAUNCHED(ctx);
    e = cudaMemcpyAsync(bad.data(), dbad, (size_t)np * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "direct: pattern comparison");
    for (int k = 0; k < np; k++)
        if (bad[k]) rep[k] = k;   // fingerprint collision: own analysis
    std::vector<int> reps;
    std::vector<int> group_of(np, -1);
    for (int k = 0; k < np; k++)
        if (rep[k] == k) {
            group_of[k] = (int)reps.size();
            reps.push_back(k);
        }
    for (int k = 0; k < np; k++) group_of[k] = group_of[rep[k]];
    // local patterns of the representatives
    const int ng = (int)reps.size();
    std::vector<std::vector<int32_t>> lrp(ng), lci(ng);
    for (int g = 0; g < ng; g++) {
        const int r0 = row_off[reps[g]], r1 = row_off[reps[g] + 1];
        const long long z0 = rowptr[r0], z1 = rowptr[r1];
        lrp[g].resize(r1 - r0 + 1);
        for (int i = 0; i <= r1 - r0; i++) lrp[g][i] = (int32_t)(rowptr[r0 + i] - z0);
        lci[g].resize(z1 - z0);
        e = cudaMemcpyAsync(lci[g].data(), A->d_cols + z0, (size_t)(z1 - z0) * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "direct: pattern download");
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "direct: pattern download");
    for (int g = 0; g < ng; g++) {
        const int r0 = row_off[reps[g]];
        for (auto &c : lci[g]) c -= r0;
    }
    std::vector<NdSymbolic> S(ng);
    std::vector<int> src(ng, 0);
    {
        const int nthr = std::max(1, std::min<int>(ng, (int)std::thread::hardware_concurrency()));
        std::atomic<int> next{0};
        std::vector<std::thread> pool;
        for (int w = 0; w < nthr; w++)
            pool.emplace_back([&]() {
                for (int g = next++; g < ng; g = next++)
                    src[g] = nd_symbolic_build((int)lrp[g].size() - 1, lrp[g].data(), lci[g].data(), &S[g]);
            });
        for (auto &t : pool) t.join();
    }
    for (int g = 0; g < ng; g++)
        if (src[g]) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "direct: symbolic analysis failed (%d)", src[g]);
    // concatenate
    DirectCache *C = new DirectCache;
    C->row_offsets.assign(row_off, row_off + np + 1);
    C->groups = ng;
    std::vector<DNode> node;
    std::vector<int32_t> front, child, ent_rel, ent_pos, ext, gnode0(ng), pn0(np), pnn(np);
    std::vector<int32_t> lvl_ptr, lvl_nodes, glvl0(ng), gnlev(ng), pl0(np), pnl(np);
    for (int g = 0; g < ng; g++) {
        const NdSymbolic &Sg = S[g];
        const int nbase = (int)node.size(), fbase = (int)front.size(), cbase = (int)child.size();
        const int ebase = (int)ent_rel.size(), xbase = (int)ext.size();
        gnode0[g] = nbase;
        const int lbase = (int)lvl_nodes.size();
        glvl0[g] = (int)lvl_ptr.size();
        gnlev[g] = (int)Sg.level_ptr.size() - 1;
        for (int32_t lp : Sg.level_ptr) lvl_ptr.push_back(lbase + lp);
        for (int32_t t : Sg.level_nodes) lvl_nodes.push_back(t + nbase);
        C->max_uv = std::max<long long>(C->max_uv, Sg.uv_size);
        for (const NdNode &q : Sg.node) {
            DNode dn;
            dn.s = q.s;
            dn.f = q.f;
            dn.front_off = q.front_off + fbase;
            dn.child_off = q.child_off + cbase;
            dn.nchild = q.nchild;
            dn.entry_off = q.entry_off + ebase;
            dn.nentry = q.nentry;
            dn.ext_off = q.ext_off + xbase;
            dn.L_off = q.L_off;
            dn.U_off = q.U_off;
            dn.uv_off = Sg.uv_off[&q - Sg.node.data()];
            node.push_back(dn);
        }
        front.insert(front.end(), Sg.front.begin(), Sg.front.end());
        for (int c : Sg.child) child.push_back(c + nbase);
        ent_rel.insert(ent_rel.end(), Sg.ent_rel.begin(), Sg.ent_rel.end());
        ent_pos.insert(ent_pos.end(), Sg.ent_pos.begin(), Sg.ent_pos.end());
        ext.insert(ext.end(), Sg.ext.begin(), Sg.ext.end());
        C->max_f = std::max(C->max_f, Sg.max_f);
        C->max_s = std::max(C->max_s, Sg.max_s);
        C->max_U = std::max<long long>(C->max_U, Sg.U_size);
        C->max_L = std::max<long long>(C->max_L, Sg.L_size);
    }
    for (int k = 0; k < np; k++) {
        pn0[k] = gnode0[group_of[k]];
        pnn[k] = S[group_of[k]].nnodes;
        pl0[k] = glvl0[group_of[k]];
        pnl[k] = gnlev[group_of[k]];
    }
    A->direct = C;
    rc = upload_vec(ctx, *C, node, &C->node);
    if (!rc) rc = upload_vec(ctx, *C, front, &C->front);
    if (!rc) rc = upload_vec(ctx, *C, child, &C->child);
    if (!rc) rc = upload_vec(ctx, *C, ent_rel, &C->ent_rel);
    if (!rc) rc = upload_vec(ctx, *C, ent_pos, &C->ent_pos);
    if (!rc) rc = upload_vec(ctx, *C, ext, &C->ext);
    if (!rc) rc = upload_vec(ctx, *C, pn0, &C->prob_node0);
    if (!rc) rc = upload_vec(ctx, *C, pnn, &C->prob_nnodes);
    if (!rc) rc = upload_vec(ctx, *C, lvl_ptr, &C->lvl_ptr);
    if (!rc) rc = upload_vec(ctx, *C, lvl_nodes, &C->lvl_nodes);
    if (!rc) rc = upload_vec(ctx, *C, pl0, &C->prob_lvl0);
    if (!rc) rc = upload_vec(ctx, *C, pnl, &C->prob_nlev);
    if (!rc) {
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "direct cache upload");
    }
    if (rc) grmp_direct_cache_free(A);
    return rc;
}

}  // namespace

void grmp_direct_cache_free(grmp_matrix A) {
    if (!A || !A->direct) return;
    grmp_context ctx = A->space->mesh->ctx;
    for (auto &b : A->direct->bufs) grmp_free(ctx, b.first, b.second);
    delete A->direct;
    A->direct = nullptr;
}

extern "C" int grmp_stokes_batch_solve(grmp_matrix A, grmp_vector bf, grmp_vector u, grmp_vector p,
                                       const grmp_stokes_batch_params *prm, int32_t *iters_out,
                                       grmp_stokes_batch_stats *stats) {
    if (!A || !bf || !u || !p || !prm || !stats) return GRMP_ERR_INVALID_ARG;
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    std::memset(stats, 0, sizeof(*stats));
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int np = prm->nproblems;
    if (s->fe != GRMP_FE_H1BR) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "batched Stokes needs an H1BR space");
    if (np <= 0 || !prm->row_offsets || !prm->cell_offsets) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: offsets");
    if (prm->row_offsets[0] != 0 || prm->row_offsets[np] != A->nrows || prm->cell_offsets[0] != 0 ||
        prm->cell_offsets[np] != m->ncells)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: offsets must cover all rows and cells");
    for (int k = 0; k < np; k++)
        if (prm->row_offsets[k + 1] <= prm->row_offsets[k] || prm->cell_offsets[k + 1] <= prm->cell_offsets[k])
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: empty or decreasing problem range");
    if (bf->n != A->nrows || u->n != A->nrows || p->n != m->ncells)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: vector sizes");
    if (!A->has64 || (prm->mode == GRMP_SOLVE_MIXED && !A->has32) || !A->d_fixed || !A->eliminated)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: assemble FP64 (and FP32 for MIXED) and eliminate Dirichlet rows first");
    if (prm->sweeps <= 0 || prm->maxiter <= 0 || !(prm->reltol > 0))
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: sweeps, maxiter and reltol must be positive");
    if (prm->mode < GRMP_SOLVE_FP64 || prm->mode > GRMP_SOLVE_MIXED_DIRECT)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: mode %d", prm->mode);
    const int n = A->nrows, nc = m->ncells;
    // problem order: largest first (longest processing time first)
    std::vector<int32_t> order(np);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return prm->row_offsets[a + 1] - prm->row_offsets[a] > prm->row_offsets[b + 1] - prm->row_offsets[b];
    });
    // device buffers
    std::vector<std::pair<void *, size_t>> bufs;
    auto take = [&](size_t bytes) -> void * {
        void *q = nullptr;
        if (grmp_alloc(ctx, &q, bytes)) return nullptr;
        bufs.push_back({q, bytes});
        return q;
    };
    auto release = [&]() {
        for (auto &b : bufs) grmp_free(ctx, b.first, b.second);
        bufs.clear();
    };
    BatchDev d;
    std::memset(&d, 0, sizeof(d));
    int32_t *dorder = (int32_t *)take((size_t)np * 4), *drow = (int32_t *)take((size_t)(np + 1) * 4);
    int32_t *dcell = (int32_t *)take((size_t)(np + 1) * 4);
    d.rhs = (double *)take((size_t)n * 8);
    d.r64 = (double *)take((size_t)n * 8);
    d.dinv64 = (double *)take((size_t)n * 8);
    d.w64a = (double *)take((size_t)n * 8);
    d.w64b = (double *)take((size_t)n * 8);
    d.w64c = (double *)take((size_t)n * 8);
    d.dinv32 = (float *)take((size_t)n * 4);
    d.r32 = (float *)take((size_t)n * 4);
    d.q32 = (float *)take((size_t)n * 4);
    d.xc32 = (float *)take((size_t)n * 4);
    d.zp0 = (float2 *)take((size_t)n * 8);
    d.zp1 = (float2 *)take((size_t)n * 8);
    const bool split = prm->mode == GRMP_SOLVE_MIXED && prm->split_penalty;
    if (split) {
        d.z32 = (float *)take((size_t)n * 4);
        d.p32 = (float *)take((size_t)n * 4);
        d.s32 = (float *)take((size_t)nc * 4);
        d.Dv32 = (float *)take((size_t)nc * s->ldofs * 4);
        d.w32 = (float *)take((size_t)nc * 4);
    }
    d.queue = (int *)take(64);
    d.fallbacks = (int *)take((size_t)np * 4);
    d.iters = (int *)take((size_t)np * 4);
    d.sweeps_done = (int *)take((size_t)np * 4);
    d.status = (int *)take((size_t)np * 4);
    d.relres = (double *)take((size_t)np * 8);
    int *bad = (int *)take(4);
    double *Dv = nullptr, *vol = nullptr;
    bool okalloc = dorder && drow && dcell && d.rhs && d.r64 && d.dinv64 && d.w64a && d.w64b && d.w64c && d.dinv32 &&
                   d.r32 && d.q32 && d.xc32 && d.zp0 && d.zp1 && d.queue && d.iters && d.sweeps_done && d.status &&
                   d.relres && bad && d.fallbacks && (!split || (d.z32 && d.p32 && d.s32 && d.Dv32 && d.w32));
    int rc = okalloc ? GRMP_OK : GRMP_ERR_OUT_OF_MEMORY;
    if (!rc) rc = grmp_br_divergence(s, &Dv, &vol);
    if (rc) {
        release();
        grmp_free(ctx, Dv, (size_t)nc * s->ldofs * 8);
        grmp_free(ctx, vol, (size_t)nc * 8);
        return rc;
    }
    cudaMemcpyAsync(dorder, order.data(), (size_t)np * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(drow, prm->row_offsets, (size_t)(np + 1) * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dcell, prm->cell_offsets, (size_t)(np + 1) * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(d.queue, 0, 64, ctx->stream);
    cudaMemsetAsync(bad, 0, 4, ctx->stream);
    // the problems must not couple (block-diagonal system)
    k_check_blocks<<<np, 128, 0, ctx->stream>>>(np, drow, A->d_rowptr, A->d_cols, bad);
    GRMP_LAUNCHED(ctx);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess || hbad) {
        release();
        grmp_free(ctx, Dv, (size_t)nc * s->ldofs * 8);
        grmp_free(ctx, vol, (size_t)nc * 8);
        return e != cudaSuccess ? grmp_cuda_fail(ctx, e, "batch check")
                                : grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "batch: a row couples two problems");
    }
    d.nprob = np;
    d.order = dorder;
    d.row_off = drow;
    d.cell_off = dcell;
    d.rowptr = A->d_rowptr;
    d.cols = A->d_cols;
    d.v64 = A->d_vals64;
    d.v32 = A->d_vals32;
    d.inc_ptr = s->d_inc_ptr;
    d.inc_cell = s->d_inc_cell;
    d.inc_loc = s->d_inc_loc;
    d.celldofs = s->d_celldofs;
    d.ld = s->ldofs;
    d.Dv = Dv;
    d.vol = vol;
    d.fixed = A->d_fixed;
    d.bf = bf->d;
    d.u = u->d;
    d.p = p->d;
    d.lambda = prm->lambda;
    d.sweep_tol = prm->sweep_tol;
    d.reltol = prm->reltol;
    d.delta = prm->inner_reltol > 0 && prm->inner_reltol < 1 ? prm->inner_reltol : 0.1;
    d.sweeps = prm->sweeps;
    d.maxit = prm->maxiter;
    d.mixed = prm->mode == GRMP_SOLVE_MIXED ? 1 : 0;
    d.split = split ? 1 : 0;
    int threads = prm->block_threads > 0 ? prm->block_threads : 512;
    threads = std::max(64, std::min(512, threads / 32 * 32));
    // lanes per row from the average row length
    double avg = (double)A->nnz / std::max(1, n);
    int tpr = avg <= 6 ? 4 : (avg <= 14 ? 8 : 16);
    int per_sm = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    void *dwork = nullptr;
    size_t dwork_bytes = 0;
    const bool direct = prm->mode == GRMP_SOLVE_DIRECT || prm->mode == GRMP_SOLVE_MIXED_DIRECT;
    if (direct) {
        // symbolic analysis once per distinct local pattern, cached in the matrix
        if (!A->direct || A->direct->row_offsets != std::vector<int32_t>(prm->row_offsets, prm->row_offsets + np + 1)) {
            grmp_direct_cache_free(A);
            rc = build_direct_cache(A, np, prm->row_offsets, drow);
        }
        DirectDev m;
        std::memset(&m, 0, sizeof(m));
        if (!rc) {
            DirectCache &C = *A->direct;
            m.node = C.node;
            m.front = C.front;
            m.child = C.child;
            m.ent_rel = C.ent_rel;
            m.ent_pos = C.ent_pos;
            m.ext = C.ext;
            m.prob_node0 = C.prob_node0;
            m.prob_nnodes = C.prob_nnodes;
            m.lvl_ptr = C.lvl_ptr;
            m.lvl_nodes = C.lvl_nodes;
            m.prob_lvl0 = C.prob_lvl0;
            m.prob_nlev = C.prob_nlev;
            m.F_doubles = (long long)C.max_f * C.max_f;
            m.U_doubles = C.max_U;
            m.L_doubles = C.max_L;
            m.uv_doubles = std::max<long long>(1, C.max_uv);
            // groups of 128 threads factoring small fronts concurrently, as many as
            // the pivot-column and panel buffers (sized for the largest front) hold
            m.fact_groups = std::max(1, std::min(4, C.max_f / kGroupFront));
            m.slot_doubles = m.F_doubles + m.U_doubles + C.max_L + m.uv_doubles +
                             (m.fact_groups > 1 ? (long long)m.fact_groups * kGroupFront * kGroupFront : 0);
            m.max_f = C.max_f;
            m.max_s = C.max_s;
            m.max_solves = 4;
        }
        const size_t smem =
            ((size_t)m.max_f + m.max_s + 32 * 33 + (size_t)m.max_f * kPanelStride + 16 * (size_t)kWarpFront) * 8;
        const bool mx = prm->mode == GRMP_SOLVE_MIXED_DIRECT;
        auto kern = mx ? (tpr == 4 ? k_stokes_direct<4, true> : (tpr == 8 ? k_stokes_direct<8, true> : k_stokes_direct<16, true>))
                       : (tpr == 4 ? k_stokes_direct<4, false>
                                   : (tpr == 8 ? k_stokes_direct<8, false> : k_stokes_direct<16, false>));
        if (!rc && smem > 220 * 1024)
            rc = grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "batch direct: front of %d DoFs too large", m.max_f);
        if (!rc) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 512, smem);
            int grid = std::max(1, std::min(np, std::max(1, per_sm) * ctx->num_sms));
            // one workspace slot per resident block; fewer blocks when memory is short
            size_t freeb = 0, totalb = 0;
            cudaMemGetInfo(&freeb, &totalb);
            size_t allow = (size_t)(0.8 * (double)freeb);
            if (ctx->budget) allow = std::min(allow, ctx->budget > ctx->in_use ? ctx->budget - ctx->in_use : (size_t)0);
            const size_t slot_bytes = (size_t)m.slot_doubles * 8;
            grid = (int)std::min<size_t>((size_t)grid, std::max<size_t>(1, allow / std::max<size_t>(1, slot_bytes)));
            dwork_bytes = (size_t)grid * slot_bytes;
            rc = grmp_alloc(ctx, &dwork, dwork_bytes);
            if (!rc) {
                m.work = (double *)dwork;
                cudaEventRecord(e0, ctx->stream);
                kern<<<grid, 512, smem, ctx->stream>>>(d, m);
                GRMP_LAUNCHED(ctx);
                cudaEventRecord(e1, ctx->stream);
            }
        }
        if (rc) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            release();
            grmp_free(ctx, Dv, (size_t)nc * s->ldofs * 8);
            grmp_free(ctx, vol, (size_t)nc * 8);
            return rc;
        }
    } else {
        auto kern = tpr == 4 ? k_stokes_batch<4> : (tpr == 8 ? k_stokes_batch<8> : k_stokes_batch<16>);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0);
        int grid = std::max(1, std::min(np, std::max(1, per_sm) * ctx->num_sms));
        cudaEventRecord(e0, ctx->stream);
        kern<<<grid, threads, 0, ctx->stream>>>(d);
        GRMP_LAUNCHED(ctx);
        cudaEventRecord(e1, ctx->stream);
    }
    std::vector<int> it(np), sw(np), st(np), fb(np);
    std::vector<double> rr(np);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(it.data(), d.iters, (size_t)np * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sw.data(), d.sweeps_done, (size_t)np * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st.data(), d.status, (size_t)np * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rr.data(), d.relres, (size_t)np * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fb.data(), d.fallbacks, (size_t)np * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release();
    grmp_free(ctx, dwork, dwork_bytes);
    grmp_free(ctx, Dv, (size_t)nc * s->ldofs * 8);
    grmp_free(ctx, vol, (size_t)nc * 8);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "batched Stokes");
    stats->solve_ms = ms;
    for (int k = 0; k < np; k++) {
        stats->total_iterations += it[k];
        stats->max_iterations = std::max(stats->max_iterations, it[k]);
        stats->max_sweeps = std::max(stats->max_sweeps, sw[k]);
        stats->max_relres = std::max(stats->max_relres, rr[k]);
        stats->fp64_fallbacks += fb[k];
        if (st[k]) stats->failed_problems++;
    }
    if (iters_out) std::memcpy(iters_out, it.data(), (size_t)np * 4);
    stats->status = stats->failed_problems ? GRMP_ERR_NOT_CONVERGED : GRMP_OK;
    if (stats->status)
        return grmp_fail(ctx, stats->status,
                         direct
                             ? "batch: %d of %d problems failed (non-positive pivot or residual above reltol, worst %.2e)"
                             : "batch: %d of %d problems hit the iteration cap (worst relres %.2e)",
                         stats->failed_problems, np, stats->max_relres);
    return GRMP_OK;
}
