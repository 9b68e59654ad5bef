// Single-problem sparse direct solvers on the device (grmp_solve with
// mode GRMP_SOLVE_DIRECT or GRMP_SOLVE_MIXED_DIRECT).
//
// The reference solves every linear system with a sparse direct solver
// (UMFPACK through LinearSolve.jl, src/solvers.jl:89-101).  Here the matrix
// gets a multifrontal Cholesky factorisation over a nested-dissection tree
// (symbolic analysis: nd_symbolic.cpp, once per pattern, cached in the
// matrix).  The tree is processed level by level (a node's children are in
// lower levels), one kernel launch per level, one thread block per front, so
// the many small fronts near the leaves run in parallel across the GPU.
//  * DIRECT: FP64 factorisation, forward/backward solves, residual
//    refinement against the assembled FP64 matrix.
//  * MIXED_DIRECT: the factorisation and the triangular solves run in FP32
//    (the GB300 FP32 pipe is about 64x the FP64 rate) and precondition an
//    FP64 conjugate-gradient iteration on the assembled FP64 matrix, whose
//    residual decides convergence.
// Forward solves pass each front's contribution to its ancestors as an update
// vector read by the parent (no scatter, no atomics): results are
// reproducible run to run.
#include <algorithm>
#include <cmath>
#include <vector>

#include "grmp_internal.h"
#include "mf_device.cuh"
#include "nd_symbolic.h"

namespace {

constexpr int kTB = 256;   // threads per block of the level kernels

struct MfNode {
    int s, f, front_off, child_off, nchild, entry_off, nentry, ext_off;
    long long L_off, U_off, uv_off;
};

struct MfDev {
    const MfNode *node;
    const int32_t *front, *child, *ent_rel, *ent_pos, *ext, *lvl_nodes;
};

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) { return warp_sum_t<double>(v); }

// ---------------------------------------------------------------- factor
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_factor_level(MfDev m, int lb, int count, const double *vals, T *L, T *U,
                                                         T *Fpool, long long fslot, T *Ppool, long long pslot,
                                                         int *err) {
    extern __shared__ unsigned char mf_smem[];
    T *colk = reinterpret_cast<T *>(mf_smem);
    const int tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
    T *F = Fpool + (long long)blockIdx.x * fslot;
    T *P = Ppool + (long long)blockIdx.x * pslot;
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int t = m.lvl_nodes[lb + q];
        const MfNode nd = m.node[t];
        const int f = nd.f, s = nd.s;
        for (long long k = tid; k < (long long)f * f; k += bs) F[k] = T(0);
        __syncthreads();
        for (int e = tid; e < nd.nentry; e += bs) F[m.ent_pos[nd.entry_off + e]] = (T)vals[m.ent_rel[nd.entry_off + e]];
        __syncthreads();
        for (int c = 0; c < nd.nchild; c++) {
            const MfNode cn = m.node[m.child[nd.child_off + c]];
            const int sc = cn.f - cn.s;
            const T *Uc = U + cn.U_off;
            const int32_t *ex = m.ext + cn.ext_off;
            for (int a = warp; a < sc; a += nw) {
                const long long pa = (long long)ex[a] * f;
                for (int b = lane; b <= a; b += 32) F[pa + ex[b]] += Uc[(long long)a * sc + b];
            }
            __syncthreads();
        }
        if (!front_cholesky<T>(F, f, s, colk, P, kPanelStride)) {
            if (tid == 0) atomicCAS(err, 0, t + 1);
            __syncthreads();
            continue;
        }
        T *Lt = L + nd.L_off;
        for (long long k = tid; k < (long long)f * s; k += bs) {
            const int i = (int)(k / s), j = (int)(k - (long long)i * s);
            Lt[k] = j <= i ? F[(long long)i * f + j] : T(0);
        }
        const int sc = f - s;
        T *Ut = U + nd.U_off;
        for (long long k = tid; k < (long long)sc * sc; k += bs) {
            const int a = (int)(k / sc), b = (int)(k - (long long)a * sc);
            if (b <= a) Ut[k] = F[(long long)(s + a) * f + s + b];
        }
        __syncthreads();
    }
}

// Large fronts by a group of blocks of the whole grid (cooperative launch,
// bounded grid barriers): group_factor_wide below.
struct CoopState {
    GridBarrier bar;
    int status;   // GRMP_ERR_TIMEOUT if a barrier wait gave up
    int abort;    // non-positive pivot found
};

// Body of the grouped large-front factorisation: `grank` = this block's
// rank in the group, `gblocks` = blocks in the group, `sync()` = the group's
// barrier (returns false when a bounded wait gave up), `abort` = the group's
// pivot-failure flag (global memory, zero on entry).
// Wide-panel variant for the grid-wide path (the fronts near the root of
// the tree, up to a few thousand rows): panels of kWide columns, so that a
// front of f rows takes f / kWide steps with two group barriers each.
// (a) every block factors the kWide x kWide diagonal block itself in shared
// memory (identical arithmetic in every block, so no barrier and no copy
// are needed before (b)); (b) one thread per row below solves it against the
// diagonal block (L21 = A21 L11^-T, kept in registers, written to F and to
// the panel buffer P); (c) the trailing lower triangle is cut into
// kWide x kWide tiles, one per block at a time, each computed from the two
// panel slices staged in shared memory by 4x4 register tiles (16 FMAs per
// 8 shared loads) and subtracted from F once.  Each entry's arithmetic is
// fixed (sum over the panel's columns in order, then one subtraction), so
// results do not depend on the grid size.
constexpr int kWide = 64;
constexpr int kWideStride = kWide + 1;

template <typename T, typename Sync>
__device__ void group_factor_wide(MfDev m, int t, const double *vals, T *L, T *U, T *F, T *P, int grank, int gblocks,
                                  Sync sync, int *abort, int *err, T *sm) {
    T *Dg = sm;                          // diagonal block [kWide][kWideStride]
    T *Ta = sm + kWide * kWideStride;    // panel rows of tile row bi
    T *Tb = Ta + kWide * kWideStride;    // panel rows of tile column bj
    const long long gtid = (long long)grank * blockDim.x + threadIdx.x, gsz = (long long)gblocks * blockDim.x;
    const int tid = threadIdx.x, bs = blockDim.x, lane = tid & 31;
    const long long gwarp = gtid >> 5, nwarps = gsz >> 5;
    const MfNode nd = m.node[t];
    const int f = nd.f, s = nd.s;
    for (long long k = gtid; k < (long long)f * f; k += gsz) F[k] = T(0);
    if (!sync()) return;
    for (long long e = gtid; e < nd.nentry; e += gsz) F[m.ent_pos[nd.entry_off + e]] = (T)vals[m.ent_rel[nd.entry_off + e]];
    if (!sync()) return;
    for (int c = 0; c < nd.nchild; c++) {
        const MfNode cn = m.node[m.child[nd.child_off + c]];
        const int sc = cn.f - cn.s;
        const T *Uc = U + cn.U_off;
        const int32_t *ex = m.ext + cn.ext_off;
        for (long long a = gwarp; a < sc; a += nwarps) {
            const long long pa = (long long)ex[a] * f;
            for (int b = lane; b <= a; b += 32) F[pa + ex[b]] += Uc[a * sc + b];
        }
        if (!sync()) return;
    }
    for (int k0 = 0; k0 < s; k0 += kWide) {
        const int kw = min(kWide, s - k0), k1 = k0 + kw, mrows = f - k1;
        // (a) the diagonal block, in every block
        for (int q = tid; q < kWide * kWide; q += bs) {
            const int r = q / kWide, c = q - r * kWide;
            Dg[r * kWideStride + c] = (r < kw && c <= r) ? F[(long long)(k0 + r) * f + k0 + c] : T(0);
        }
        __syncthreads();
        bool bad = false;
        for (int c = 0; c < kw; c++) {
            const T dcc = Dg[c * kWideStride + c];
            if (!(dcc > T(0)) || !isfinite((double)dcc)) {   // the same value in every thread and block
                bad = true;
                break;
            }
            const T dk = sqrt(dcc);
            __syncthreads();
            for (int r = c + 1 + tid; r < kw; r += bs) Dg[r * kWideStride + c] /= dk;
            if (tid == 0) Dg[c * kWideStride + c] = dk;
            __syncthreads();
            const int w = kw - c - 1;
            for (int q = tid; q < w * w; q += bs) {
                const int r = c + 1 + q / w, cc = c + 1 + q % w;
                if (cc <= r) Dg[r * kWideStride + cc] -= Dg[r * kWideStride + c] * Dg[cc * kWideStride + c];
            }
            __syncthreads();
        }
        if (bad) {   // every block sees it: leave without a further barrier
            if (tid == 0) {
                *(volatile int *)abort = 1;
                atomicCAS(err, 0, t + 1);
            }
            return;
        }
        // (b) rows below the diagonal block
        for (long long i = k1 + gtid; i < f; i += gsz) {
            T x[kWide];
            T *Fi = F + i * f + k0;
#pragma unroll
            for (int j = 0; j < kWide; j++) {
                if (j < kw) {
                    T a = Fi[j];
#pragma unroll
                    for (int l = 0; l < j; l++) a -= x[l] * Dg[j * kWideStride + l];
                    x[j] = a / Dg[j * kWideStride + j];
                } else {
                    x[j] = T(0);
                }
            }
            T *Pi = P + (i - k1) * kWideStride;
#pragma unroll
            for (int j = 0; j < kWide; j++)
                if (j < kw) {
                    Fi[j] = x[j];
                    Pi[j] = x[j];
                }
        }
        if (!sync()) return;
        // the factored diagonal block goes back into F only now: before the
        // barrier other blocks may still be reading the unfactored one in (a)
        if (grank == 0)
            for (int q = tid; q < kw * kw; q += bs) {
                const int r = q / kw, c = q - r * kw;
                if (c <= r) F[(long long)(k0 + r) * f + k0 + c] = Dg[r * kWideStride + c];
            }
        // (c) trailing update in kWide x kWide tiles of the lower triangle
        const int nt = (mrows + kWide - 1) / kWide;
        const long long ntiles = (long long)nt * (nt + 1) / 2;
        const int ty = tid / 16, tx = tid % 16;   // 16 x 16 threads, 4 x 4 entries each
        for (long long q = grank; q < ntiles; q += gblocks) {
            int bi = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
            while ((long long)(bi + 1) * (bi + 2) / 2 <= q) bi++;
            while ((long long)bi * (bi + 1) / 2 > q) bi--;
            const int bj = (int)(q - (long long)bi * (bi + 1) / 2);
            for (int e = tid; e < kWide * kWide; e += bs) {
                const int r = e / kWide, c = e - r * kWide;
                const int ia = bi * kWide + r, ib = bj * kWide + r;
                Ta[r * kWideStride + c] = (ia < mrows && c < kw) ? P[(long long)ia * kWideStride + c] : T(0);
                Tb[r * kWideStride + c] = (ib < mrows && c < kw) ? P[(long long)ib * kWideStride + c] : T(0);
            }
            __syncthreads();
            if (tid < 256) {
                T acc[4][4];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
                for (int tt = 0; tt < kw; tt++) {
                    T xa[4], yb[4];
#pragma unroll
                    for (int a = 0; a < 4; a++) {
                        xa[a] = Ta[(ty * 4 + a) * kWideStride + tt];
                        yb[a] = Tb[(tx * 4 + a) * kWideStride + tt];
                    }
#pragma unroll
                    for (int a = 0; a < 4; a++)
#pragma unroll
                        for (int b = 0; b < 4; b++) acc[a][b] += xa[a] * yb[b];
                }
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const int i = bi * kWide + ty * 4 + a;
                    if (i >= mrows) break;
                    T *Fi = F + (long long)(k1 + i) * f + k1;
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const int j = bj * kWide + tx * 4 + b;
                        if (j <= i) Fi[j] -= acc[a][b];
                    }
                }
            }
            __syncthreads();   // the tiles are reloaded next
        }
        if (!sync()) return;
    }
    T *Lt = L + nd.L_off;
    for (long long k = gtid; k < (long long)f * s; k += gsz) {
        const int i = (int)(k / s), j = (int)(k - (long long)i * s);
        Lt[k] = j <= i ? F[(long long)i * f + j] : T(0);
    }
    const int sc = f - s;
    T *Ut = U + nd.U_off;
    for (long long k = gtid; k < (long long)sc * sc; k += gsz) {
        const int a = (int)(k / sc), b = (int)(k - (long long)a * sc);
        if (b <= a) Ut[k] = F[(long long)(s + a) * f + s + b];
    }
}

// The large fronts of one level by the whole grid split into `ngroups`
// groups (block b belongs to group b % ngroups, so every group spans all
// SMs evenly); group g factors fronts g, g + ngroups, ... of the level, each
// group with its own bounded barrier, front and panel buffers.  One
// cooperative launch per level.
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_group_factor(MfDev m, int lb, int count, int ngroups, const double *vals,
                                                         T *L, T *U, T *Fpool, long long fslot, T *Ppool,
                                                         long long pslot, CoopState *cs, int *err) {
    const int g = blockIdx.x % ngroups, grank = blockIdx.x / ngroups;
    const int gblocks = (gridDim.x - g + ngroups - 1) / ngroups;
    CoopState *c = cs + g;
    extern __shared__ unsigned char mf_gsmem[];
    T *sm = reinterpret_cast<T *>(mf_gsmem);
    auto sync = [&]() { return grid_barrier(&c->bar, gblocks, &c->status); };
    for (int q = g; q < count; q += ngroups) {
        group_factor_wide<T>(m, m.lvl_nodes[lb + q], vals, L, U, Fpool + g * fslot, Ppool + g * pslot, grank, gblocks,
                             sync, &c->abort, err, sm);
        if (*(volatile int *)&c->abort || *(volatile int *)&c->status) return;
        if (!sync()) return;   // buffers reused by the group's next front
    }
}

// ---------------------------------------------------------------- solves
// Forward: ys = w[own] minus the children's update entries for own DoFs,
// L11 y = ys, and the node's update vector = children's entries for its
// structure + L21 y.
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_forward_level(MfDev m, int lb, int count, const T *L, T *uv, T *w,
                                                          int maxs) {
    extern __shared__ unsigned char mf_smem[];
    T *ys = reinterpret_cast<T *>(mf_smem);
    T *tile = ys + maxs;   // 32 x 33
    const int tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int t = m.lvl_nodes[lb + q];
        const MfNode nd = m.node[t];
        const int f = nd.f, s = nd.s, sc = f - s;
        const int32_t *fr = m.front + nd.front_off;
        const T *Lt = L + nd.L_off;
        T *ut = uv + nd.uv_off;
        for (int k = tid; k < s; k += bs) ys[k] = w[fr[k]];
        for (int i = tid; i < sc; i += bs) ut[i] = T(0);
        __syncthreads();
        for (int c = 0; c < nd.nchild; c++) {
            const MfNode cn = m.node[m.child[nd.child_off + c]];
            const int scc = cn.f - cn.s;
            const T *uc = uv + cn.uv_off;
            const int32_t *ex = m.ext + cn.ext_off;
            for (int a = tid; a < scc; a += bs) {
                const int pos = ex[a];
                if (pos < s) ys[pos] -= uc[a];
                else ut[pos - s] += uc[a];
            }
            __syncthreads();
        }
        for (int kb = 0; kb < s; kb += 32) {
            const int nbk = min(32, s - kb);
            if (kb > 0)
                for (int r = warp; r < nbk; r += nw) {
                    const T *Li = Lt + (long long)(kb + r) * s;
                    T acc = T(0);
                    for (int j = lane; j < kb; j += 32) acc += Li[j] * ys[j];
                    acc = warp_sum_t<T>(acc);
                    if (lane == 0) ys[kb + r] -= acc;
                }
            for (int k = tid; k < nbk * nbk; k += bs) {
                const int r = k / nbk, c = k - r * nbk;
                tile[r * 33 + c] = c <= r ? Lt[(long long)(kb + r) * s + kb + c] : T(0);
            }
            __syncthreads();
            if (warp == 0) {
                T v = lane < nbk ? ys[kb + lane] : T(0);
                for (int c = 0; c < nbk; c++) {
                    const T yc = __shfl_sync(0xffffffffu, v, c) / tile[c * 33 + c];
                    if (lane == c) v = yc;
                    else if (lane > c && lane < nbk) v -= tile[lane * 33 + c] * yc;
                }
                if (lane < nbk) ys[kb + lane] = v;
            }
            __syncthreads();
        }
        for (int k = tid; k < s; k += bs) w[fr[k]] = ys[k];
        for (int i = warp; i < sc; i += nw) {
            const T *Li = Lt + (long long)(s + i) * s;
            T acc = T(0);
            for (int k = lane; k < s; k += 32) acc += Li[k] * ys[k];
            acc = warp_sum_t<T>(acc);
            if (lane == 0) ut[i] += acc;
        }
        __syncthreads();
    }
}

// Backward: z = y_own - L21^T x_struct (ancestors already final), L11^T x = z.
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_backward_level(MfDev m, int lb, int count, const T *L, T *w, int maxs) {
    extern __shared__ unsigned char mf_smem[];
    T *ys = reinterpret_cast<T *>(mf_smem);
    T *tile = ys + maxs;
    T *xs = tile + 32 * 33;
    const int tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int t = m.lvl_nodes[lb + q];
        const MfNode nd = m.node[t];
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
            for (int k = tid; k < nbk * nbk; k += bs) {
                const int r = k / nbk, c = k - r * nbk;
                tile[r * 33 + c] = c <= r ? Lt[(long long)(kb + r) * s + kb + c] : T(0);
            }
            __syncthreads();
            if (warp == 0) {
                T v = lane < nbk ? ys[kb + lane] : T(0);
                for (int c = nbk - 1; c >= 0; c--) {
                    const T xc = __shfl_sync(0xffffffffu, v, c) / tile[c * 33 + c];
                    if (lane == c) v = xc;
                    else if (lane < c) v -= tile[c * 33 + lane] * xc;
                }
                if (lane < nbk) ys[kb + lane] = v;
            }
            __syncthreads();
            for (int k = tid; k < kb; k += bs) {
                T acc = T(0);
                for (int r = 0; r < nbk; r++) acc += Lt[(long long)(kb + r) * s + k] * ys[kb + r];
                ys[k] -= acc;
            }
            __syncthreads();
        }
        for (int k = tid; k < s; k += bs) w[fr[k]] = ys[k];
        __syncthreads();
    }
}

// ---------------------------------------------------------------- inverse-based solves
// For the FP32 preconditioner, applied once per CG iteration, each front
// keeps Q = [L11^-1 ; G] with G = L21 L11^-1 (same f x s layout as its
// factor columns).  Forward:  y_own = L11^-1 b_own,  u_struct += G b_own;
// backward: x_own = L11^-T y_own - G^T x_struct.  Every output is one dot
// product: a level is one or two fully parallel launches, with no
// sequential triangular chain inside a front.

// index idx in [lo, hi) with pref[idx] <= item < pref[idx + 1]
__device__ __forceinline__ int find_seg(const long long *pref, int lo, int hi, long long item) {
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pref[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// L11^-1 by 32 x 32 blocks: one thread block per (front, block column c).
// X_cc solves L_cc X = I; for b > c, X_bc solves L_bb X = -sum_{m=c}^{b-1} L_bm X_mc
// (the sum as a small GEMM by all threads, the 32-column triangular solve by
// one warp, each lane a column).  Block columns are independent.
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_invert(MfDev m, const long long *bcol, int nn, const T *L, T *Q) {
    __shared__ T Lbb[32][33];
    __shared__ T Tb[32][33];
    __shared__ T Ls[32][33];   // slab of L_b,[k0, k0+32)
    __shared__ T Xs[32][33];   // slab of X_[k0, k0+32),c
    const long long item = blockIdx.x;
    const int idx = find_seg(bcol, 0, nn, item);
    const MfNode nd = m.node[m.lvl_nodes[idx]];
    const int s = nd.s, c = (int)(item - bcol[idx]);
    const T *Lt = L + nd.L_off;
    T *Qt = Q + nd.L_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nbk = (s + 31) / 32;
    const int c0 = c * 32, cw = min(32, s - c0);
    for (int b = c; b < nbk; b++) {
        const int b0 = b * 32, bw = min(32, s - b0);
        // Tb = (b == c ? I : -sum_m L_bm X_mc), Lbb = L_bb.  The sum runs over
        // k in [c0, b0) (whole 32-slabs) with both factors staged in shared
        // memory, k ascending as a plain loop would take it.
        for (int q = tid; q < 32 * 32; q += blockDim.x) {
            const int r = q >> 5, cc = q & 31;
            Tb[r][cc] = (b == c && r == cc && r < bw) ? T(1) : T(0);
            Lbb[r][cc] = (r < bw && cc <= r) ? Lt[(long long)(b0 + r) * s + b0 + cc] : T(0);
        }
        if (b > c) {
            for (int k0 = c0; k0 < b0; k0 += 32) {
                __syncthreads();
                for (int q = tid; q < 32 * 32; q += blockDim.x) {
                    const int r = q >> 5, cc = q & 31;
                    Ls[r][cc] = r < bw ? Lt[(long long)(b0 + r) * s + k0 + cc] : T(0);
                    Xs[r][cc] = cc < cw ? Qt[(long long)(k0 + r) * s + c0 + cc] : T(0);
                }
                __syncthreads();
                for (int q = tid; q < 32 * 32; q += blockDim.x) {
                    const int r = q >> 5, cc = q & 31;
                    T acc = Tb[r][cc];
#pragma unroll 8
                    for (int kk = 0; kk < 32; kk++) acc -= Ls[r][kk] * Xs[kk][cc];
                    Tb[r][cc] = acc;
                }
            }
        }
        __syncthreads();
        if (warp == 0 && lane < cw) {   // forward substitution, column `lane`
            for (int r = 0; r < bw; r++) {
                T v = Tb[r][lane];
                for (int k = 0; k < r; k++) v -= Lbb[r][k] * Tb[k][lane];
                Tb[r][lane] = v / Lbb[r][r];
            }
        }
        __syncthreads();
        for (int q = tid; q < bw * cw; q += blockDim.x) {
            const int r = q / cw, cc = q - r * cw;
            Qt[(long long)(b0 + r) * s + c0 + cc] = Tb[r][cc];
        }
        __syncthreads();
    }
}

// G = L21 L11^-1 of every front, as tiles of 64 x 64 entries (rows i of the
// structure part, columns k): a 256-thread block per tile, the product over
// m in 32-wide slabs of L21 (64 x 32) and L11^-1 (32 x 64) staged in shared
// memory, 4 x 4 outputs per thread.  L11^-1 is lower triangular and only
// its blocks on or below the diagonal are stored, so entries with m < k are
// read as zero.  Tiles: {level-order front index, first row, first column}.
constexpr int kGmT = 64, kGmK = 32;

template <typename T>
__global__ void __launch_bounds__(256) k_mf_gmat(MfDev m, const int4 *tiles, long long ntiles, const T *L, T *Q) {
    __shared__ T As[kGmK][kGmT + 1];   // As[mm][i]
    __shared__ T Bs[kGmK][kGmT + 1];   // Bs[mm][k]
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // 16 x 16 threads, 4 x 4 outputs each
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int4 tl = tiles[t];
        const MfNode nd = m.node[m.lvl_nodes[tl.x]];
        const int s = nd.s, sc = nd.f - nd.s, i0 = tl.y, k0 = tl.z;
        const T *L21 = L + nd.L_off + (long long)s * s;   // row i of the structure part: L21 + i * s
        const T *Qt = Q + nd.L_off;
        T acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] = T(0);
        for (int m0 = k0; m0 < s; m0 += kGmK) {
            for (int q = threadIdx.x; q < kGmK * kGmT; q += 256) {
                const int mm = q % kGmK, ii = q / kGmK;   // A: consecutive threads along m (row-major L21)
                const int gi = i0 + ii, gm = m0 + mm;
                As[mm][ii] = (gi < sc && gm < s) ? L21[(long long)gi * s + gm] : T(0);
                const int kk = q % kGmT, m2 = q / kGmT;    // B: consecutive threads along k (row-major Q)
                const int gk = k0 + kk, gm2 = m0 + m2;
                Bs[m2][kk] = (gk < s && gm2 < s && gm2 >= gk) ? Qt[(long long)gm2 * s + gk] : T(0);
            }
            __syncthreads();
#pragma unroll 8
            for (int mm = 0; mm < kGmK; mm++) {
                T av[4], bv[4];
#pragma unroll
                for (int a = 0; a < 4; a++) av[a] = As[mm][ty * 4 + a];
#pragma unroll
                for (int b = 0; b < 4; b++) bv[b] = Bs[mm][tx * 4 + b];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) acc[a][b] += av[a] * bv[b];
            }
            __syncthreads();
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int gi = i0 + ty * 4 + a;
            if (gi >= sc) continue;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int gk = k0 + tx * 4 + b;
                if (gk < s) Q[nd.L_off + (long long)(s + gi) * s + gk] = acc[a][b];
            }
        }
    }
}

// forward, part 1 (block per front): the children's update entries, own ones
// subtracted from w in place, structure ones summed into the front's update vector
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_gather_level(MfDev m, int lb, int count, T *uv, T *w) {
    const int tid = threadIdx.x, bs = blockDim.x;
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const MfNode nd = m.node[m.lvl_nodes[lb + q]];
        const int s = nd.s, sc = nd.f - nd.s;
        const int32_t *fr = m.front + nd.front_off;
        T *ut = uv + nd.uv_off;
        for (int i = tid; i < sc; i += bs) ut[i] = T(0);
        __syncthreads();
        for (int c = 0; c < nd.nchild; c++) {
            const MfNode cn = m.node[m.child[nd.child_off + c]];
            const int scc = cn.f - cn.s;
            const T *uc = uv + cn.uv_off;
            const int32_t *ex = m.ext + cn.ext_off;
            for (int a = tid; a < scc; a += bs) {
                const int pos = ex[a];
                if (pos < s) w[fr[pos]] -= uc[a];
                else ut[pos - s] += uc[a];
            }
            __syncthreads();
        }
    }
}

// forward, part 2 (warp per row of Q over the level): y_own, update vector
template <typename T>
__global__ void __launch_bounds__(kTB) k_mf_qmul_level(MfDev m, const long long *qrow, int lb, int cnt, const T *Q,
                                                       T *uv, const T *w, T *wy) {
    const long long r0 = qrow[lb], nrows = qrow[lb + cnt] - r0;
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarp = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long it = gw; it < nrows; it += nwarp) {
        const int idx = find_seg(qrow, lb, lb + cnt, r0 + it);
        const MfNode nd = m.node[m.lvl_nodes[idx]];
        const int s = nd.s, r = (int)(r0 + it - qrow[idx]);
        const int32_t *fr = m.front + nd.front_off;
        const T *Qr = Q + nd.L_off + (long long)r * s;
        const int kend = r < s ? r + 1 : s;
        T acc = T(0);
        for (int k = lane; k < kend; k += 32) acc += Qr[k] * w[fr[k]];
        acc = warp_sum_t<T>(acc);
        if (lane == 0) {
            if (r < s) wy[fr[r]] = acc;
            else uv[nd.uv_off + r - s] += acc;
        }
    }
}

// backward: x_k = sum_j Q[j][k] y_j - sum_i G[i][k] x_struct_i over the
// level's tiles of 32 consecutive own columns of one front (`bcol`: the
// prefix of tiles per front in level order).  A block of 32 x 32 threads
// takes a tile: lane tx = column kb + tx, warp ty = rows kb + ty, kb + ty +
// 32, ...; all lanes of a warp read the same row of Q (32 consecutive
// columns: one coalesced line) and the same right-hand value, skipping rows
// above their column's diagonal; the 32 partial sums of a column are added in
// a fixed order.
constexpr int kQtT = 1024;

template <typename T>
__global__ void __launch_bounds__(kQtT) k_mf_qtmul_level(MfDev m, const long long *bcol, int lb, int cnt, const T *Q,
                                                         const T *wy, T *wx) {
    __shared__ T part[32][33];
    const long long t0 = bcol[lb], ntiles = bcol[lb + cnt] - t0;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int idx = find_seg(bcol, lb, lb + cnt, t0 + t);
        const MfNode nd = m.node[m.lvl_nodes[idx]];
        const int s = nd.s, f = nd.f;
        const int kb = (int)(t0 + t - bcol[idx]) * 32;
        const int k = kb + tx;
        const int32_t *fr = m.front + nd.front_off;
        const T *Qk = Q + nd.L_off + k;
        T acc = T(0);
        if (k < s)
            for (int j = kb + ty; j < f; j += 32) {
                const T v = j < s ? wy[fr[j]] : -wx[fr[j]];
                if (j >= k) acc += Qk[(long long)j * s] * v;
            }
        part[ty][tx] = acc;
        __syncthreads();
        if (ty == 0 && k < s) {
            T sum = T(0);
            for (int g = 0; g < 32; g++) sum += part[g][tx];
            wx[fr[k]] = sum;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- vector kernels
// r = b - A x (FP64), per-block partial sums of r^2 (fixed order)
__global__ void k_resid(int n, const int32_t *rowptr, const int32_t *cols, const double *vals, const double *x,
                        const double *b, double *r, double *part) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double acc2 = 0.0;
    for (int row = blockIdx.x * nw + warp; row < n; row += gridDim.x * nw) {
        double s = 0.0;
        for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) s += vals[k] * x[cols[k]];
        s = warp_sum_d(s);
        if (lane == 0) {
            const double v = b[row] - s;
            r[row] = v;
            acc2 += v * v;
        }
    }
    if (lane == 0) sh[warp] = acc2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// q = A p (FP64) and partial sums of p.q
__global__ void k_apply_dot(int n, const int32_t *rowptr, const int32_t *cols, const double *vals, const double *p,
                            double *q, double *part) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double acc = 0.0;
    for (int row = blockIdx.x * nw + warp; row < n; row += gridDim.x * nw) {
        double s = 0.0;
        for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) s += vals[k] * p[cols[k]];
        s = warp_sum_d(s);
        if (lane == 0) {
            q[row] = s;
            acc += p[row] * s;
        }
    }
    if (lane == 0) sh[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

template <typename T>
__global__ void k_to(int n, const double *a, T *b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (T)a[i];
}

// x += alpha p, r -= alpha q, partial sums of r^2
__global__ void k_cg_update(int n, double alpha, const double *p, const double *q, double *x, double *r,
                            double *part) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * q[i];
        r[i] = ri;
        acc += ri * ri;
    }
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// z = (double) zf, partial sums of r.z
template <typename T>
__global__ void k_from_dot(int n, const T *zf, const double *r, double *z, double *part) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double zi = (double)zf[i];
        z[i] = zi;
        acc += r[i] * zi;
    }
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// partial sums of a.b
__global__ void k_dot(int n, const double *a, const double *b, double *part) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += a[i] * b[i];
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        part[blockIdx.x] = t;
    }
}

// per-block maxima of the row sums of |A| (||A||_inf)
__global__ void k_rownorm(int n, const int32_t *rowptr, const double *vals, double *part) {
    __shared__ double sh[32];
    double mx = 0.0;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = rowptr[row]; k < rowptr[row + 1]; k++) s += fabs(vals[k]);
        mx = fmax(mx, s);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmax(t, sh[w]);
        part[blockIdx.x] = t;
    }
}

__global__ void k_xpby(int n, const double *z, double beta, double *p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + beta * p[i];
}

template <typename T>
__global__ void k_add_from(int n, const T *w, double *x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)w[i];
}

}  // namespace

// ---------------------------------------------------------------- host side

struct MfCache {
    std::vector<std::pair<void *, size_t>> bufs;   // symbolic arrays
    MfDev dev{};
    std::vector<int32_t> level_ptr, level_maxf, level_small;   // level_small[l]: fronts below kBigFront first
    std::vector<int32_t> level_nodes_host;                     // same order as dev.lvl_nodes
    int nnodes = 0, max_f = 0, max_s = 0;
    long long L_size = 0, U_size = 0, uv_size = 0;
    long long fpool = 0, ppool = 0;   // elements of the per-launch front / panel pools
    // numeric storage of the current precision (sizeof(T) = esize)
    int esize = 0;
    void *L = nullptr, *U = nullptr, *uv = nullptr, *F = nullptr, *P = nullptr, *w = nullptr;
    size_t Lb = 0, Ub = 0, uvb = 0, Fb = 0, Pb = 0, wb = 0;
    // inverse-based FP32 preconditioner: Q = [L11^-1; L21 L11^-1] per front, two more vectors
    void *Q = nullptr, *wy = nullptr, *wx = nullptr;
    size_t Qb = 0;
    // prefixes over fronts in level order: rows (f), own columns (s), G entries (sc * s)
    const long long *qrow = nullptr, *scol = nullptr, *bcol = nullptr;
    std::vector<long long> bcol_host;   // the same prefix of 32-column tiles, for launch sizes
    const int4 *gtiles = nullptr;       // 64 x 64 tiles of every front's L21 L11^-1
    long long total_cols = 0, total_gtiles = 0, total_bcols = 0;
    // the preconditioner's level launches (w -> wx), captured once per numeric storage
    cudaGraphExec_t apply_graph = nullptr;
    int apply_kernels = 0;
};

namespace {

constexpr int kMaxGrid = 2 * 152;
constexpr int kBigFront = 1024;   // fronts from this size up are factored by the whole grid
constexpr int kCoopFront = 256;   // ... and from this size up in levels with fewer than kFillLevel fronts
constexpr int kFillLevel = 152;
constexpr int kGroups64 = 4;      // concurrent large fronts per level launch, FP64 (FP64 pipe bound: many SMs each)
constexpr int kGroups32 = 16;     // ... FP32

template <typename V>
int mf_upload(grmp_context ctx, MfCache &C, const std::vector<V> &v, const V **out) {
    V *p = nullptr;
    const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(V);
    int rc = grmp_alloc(ctx, (void **)&p, bytes);
    if (rc) return rc;
    C.bufs.push_back({p, bytes});
    if (!v.empty()) {
        cudaError_t e = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "multifrontal upload");
    }
    *out = p;
    return GRMP_OK;
}

void mf_free_numeric(grmp_context ctx, MfCache &C) {
    if (C.apply_graph) cudaGraphExecDestroy(C.apply_graph);
    C.apply_graph = nullptr;
    grmp_free(ctx, C.L, C.Lb);
    grmp_free(ctx, C.U, C.Ub);
    grmp_free(ctx, C.uv, C.uvb);
    grmp_free(ctx, C.F, C.Fb);
    grmp_free(ctx, C.P, C.Pb);
    grmp_free(ctx, C.w, C.wb);
    grmp_free(ctx, C.Q, C.Qb);
    grmp_free(ctx, C.wy, C.wb);
    grmp_free(ctx, C.wx, C.wb);
    C.L = C.U = C.uv = C.F = C.P = C.w = C.Q = C.wy = C.wx = nullptr;
    C.Lb = C.Ub = C.uvb = C.Fb = C.Pb = C.wb = C.Qb = 0;
    C.esize = 0;
}

int mf_build(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    std::vector<int32_t> rp(n + 1), ci((size_t)A->nnz);
    cudaError_t e = cudaMemcpyAsync(rp.data(), A->d_rowptr, (size_t)(n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ci.data(), A->d_cols, (size_t)A->nnz * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "multifrontal: pattern download");
    NdSymbolic S;
    int src = nd_symbolic_build(n, rp.data(), ci.data(), &S);
    if (src) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "multifrontal: symbolic analysis failed (%d)", src);
    MfCache *C = new MfCache;
    std::vector<MfNode> node(S.nnodes);
    for (int t = 0; t < S.nnodes; t++) {
        const NdNode &q = S.node[t];
        node[t] = MfNode{q.s, q.f, q.front_off, q.child_off, q.nchild, q.entry_off, q.nentry, q.ext_off,
                         (long long)q.L_off, (long long)q.U_off, (long long)S.uv_off[t]};
    }
    C->nnodes = S.nnodes;
    C->max_f = S.max_f;
    C->max_s = S.max_s;
    C->L_size = S.L_size;
    C->U_size = S.U_size;
    C->uv_size = S.uv_size;
    C->level_ptr = S.level_ptr;
    C->level_maxf = S.level_maxf;
    const int nl = (int)S.level_ptr.size() - 1;
    // within each level: fronts below kBigFront first (one block each), then the big ones
    // (one cooperative launch each, the whole grid on one front)
    std::vector<int32_t> order = S.level_nodes;
    C->level_small.assign(nl, 0);
    for (int l = 0; l < nl; l++) {
        auto b0 = order.begin() + S.level_ptr[l], b1 = order.begin() + S.level_ptr[l + 1];
        // a level too sparse to fill the GPU with one front per block sends its
        // mid-size and large fronts to the whole grid
        const bool sparse = S.level_ptr[l + 1] - S.level_ptr[l] < kFillLevel;
        auto mid = std::stable_partition(b0, b1, [&](int32_t t) {
            return S.node[t].f < (sparse ? kCoopFront : kBigFront);
        });
        C->level_small[l] = (int)(mid - b0);
        const long long nbig = (long long)(b1 - mid);
        const long long g = std::max<long long>(std::min<long long>(std::max(1, C->level_small[l]), kMaxGrid), nbig);
        long long mf = 0;
        for (auto it2 = b0; it2 != b1; ++it2) mf = std::max<long long>(mf, S.node[*it2].f);
        C->fpool = std::max(C->fpool, g * mf * mf);
        C->ppool = std::max(C->ppool, g * mf * kWideStride);   // the grid-wide path's panels are kWide wide
    }
    C->level_nodes_host = order;
    std::vector<long long> qrow(S.nnodes + 1, 0), scol(S.nnodes + 1, 0), bcol(S.nnodes + 1, 0);
    std::vector<int4> gtiles;
    for (int i = 0; i < S.nnodes; i++) {
        const NdNode &q = S.node[order[i]];
        qrow[i + 1] = qrow[i] + q.f;
        scol[i + 1] = scol[i] + q.s;
        bcol[i + 1] = bcol[i] + (q.s + 31) / 32;
        for (int i0 = 0; i0 < q.f - q.s; i0 += kGmT)
            for (int k0 = 0; k0 < q.s; k0 += kGmT) gtiles.push_back(make_int4(i, i0, k0, 0));
    }
    C->total_cols = scol[S.nnodes];
    C->total_gtiles = (long long)gtiles.size();
    C->total_bcols = bcol[S.nnodes];
    C->bcol_host = bcol;
    A->mf = C;
    int rc = mf_upload(ctx, *C, node, &C->dev.node);
    if (!rc) rc = mf_upload(ctx, *C, S.front, &C->dev.front);
    if (!rc) rc = mf_upload(ctx, *C, S.child, &C->dev.child);
    if (!rc) rc = mf_upload(ctx, *C, S.ent_rel, &C->dev.ent_rel);
    if (!rc) rc = mf_upload(ctx, *C, S.ent_pos, &C->dev.ent_pos);
    if (!rc) rc = mf_upload(ctx, *C, S.ext, &C->dev.ext);
    if (!rc) rc = mf_upload(ctx, *C, order, &C->dev.lvl_nodes);
    if (!rc) rc = mf_upload(ctx, *C, qrow, &C->qrow);
    if (!rc) rc = mf_upload(ctx, *C, scol, &C->scol);
    if (!rc) rc = mf_upload(ctx, *C, gtiles, &C->gtiles);
    if (!rc) rc = mf_upload(ctx, *C, bcol, &C->bcol);
    if (!rc) {
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "multifrontal upload");
    }
    if (rc) grmp_mf_cache_free(A);
    return rc;
}

template <typename T>
int mf_numeric(grmp_matrix A, int *grid_out) {
    grmp_context ctx = A->space->mesh->ctx;
    MfCache &C = *A->mf;
    // shared memory of the solve kernels: own values, a 32x33 tile and the structure values
    if (((size_t)C.max_s + 32 * 33 + C.max_f) * sizeof(T) > 220 * 1024)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "direct solve: front of %d DoFs exceeds shared memory", C.max_f);
    if (C.esize != (int)sizeof(T)) {
        mf_free_numeric(ctx, C);
        C.Lb = std::max<size_t>(1, C.L_size) * sizeof(T);
        C.Ub = std::max<size_t>(1, C.U_size) * sizeof(T);
        C.uvb = std::max<size_t>(1, C.uv_size) * sizeof(T);
        C.Fb = std::max<size_t>(1, C.fpool) * sizeof(T);
        C.Pb = std::max<size_t>(1, C.ppool) * sizeof(T);
        C.wb = (size_t)A->nrows * sizeof(T);
        int rc = grmp_alloc(ctx, &C.L, C.Lb);
        if (!rc) rc = grmp_alloc(ctx, &C.U, C.Ub);
        if (!rc) rc = grmp_alloc(ctx, &C.uv, C.uvb);
        if (!rc) rc = grmp_alloc(ctx, &C.F, C.Fb);
        if (!rc) rc = grmp_alloc(ctx, &C.P, C.Pb);
        if (!rc) rc = grmp_alloc(ctx, &C.w, C.wb);
        if (rc) {
            mf_free_numeric(ctx, C);
            return rc;
        }
        C.esize = sizeof(T);
    }
    int *derr = nullptr;
    int rc = grmp_alloc(ctx, (void **)&derr, 4);
    if (rc) return rc;
    cudaMemsetAsync(derr, 0, 4, ctx->stream);
    const size_t smem = (size_t)C.max_f * sizeof(T);
    cudaFuncSetAttribute(k_mf_factor_level<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int nl = (int)C.level_ptr.size() - 1;
    int gmax = 0, coop_grid = 0, ncs = 0;
    bool timed_out = false;
    CoopState *cs = nullptr;
    cudaError_t e = cudaSuccess;
    for (int l = 0; l < nl; l++) {
        const int lb = C.level_ptr[l], cnt = C.level_ptr[l + 1] - lb, nsmall = C.level_small[l];
        if (nsmall > 0) {
            const int g = std::min(nsmall, kMaxGrid);
            const long long mf = C.level_maxf[l];
            gmax = std::max(gmax, g);
            k_mf_factor_level<T><<<g, kTB, smem, ctx->stream>>>(C.dev, lb, nsmall, A->d_vals64, (T *)C.L, (T *)C.U,
                                                                (T *)C.F, mf * mf, (T *)C.P, mf * kPanelStride, derr);
            GRMP_LAUNCHED(ctx);
        }
        const int nbig = cnt - nsmall;
        if (nbig > 0) {
            // one cooperative launch for the level's large fronts; FP64 fronts get more SMs each
            const int ng = std::min(nbig, sizeof(T) == 8 ? kGroups64 : kGroups32);
            if (!cs || ng > ncs) {
                grmp_free(ctx, cs, (size_t)ncs * sizeof(CoopState));
                ncs = std::max(ng, kGroups32);
                rc = grmp_alloc(ctx, (void **)&cs, (size_t)ncs * sizeof(CoopState));
                if (rc) break;
            }
            const size_t gsmem = (size_t)3 * kWide * kWideStride * sizeof(T);
            if (!coop_grid) {
                int per_sm = 0;
                cudaFuncSetAttribute(k_mf_group_factor<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsmem);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mf_group_factor<T>, kTB, gsmem);
                coop_grid = std::max(1, std::min(per_sm, 4)) * ctx->num_sms;
            }
            cudaMemsetAsync(cs, 0, (size_t)ng * sizeof(CoopState), ctx->stream);
            MfDev dv = C.dev;
            int lbb = lb + nsmall, cntb = nbig, ngv = ng;
            const double *vv = A->d_vals64;
            T *Lp = (T *)C.L, *Up = (T *)C.U, *Fp = (T *)C.F, *Pp = (T *)C.P;
            long long mf = C.level_maxf[l], fs = mf * mf, ps = mf * kWideStride;
            void *args[] = {&dv, &lbb, &cntb, &ngv, &vv, &Lp, &Up, &Fp, &fs, &Pp, &ps, &cs, &derr};
            e = cudaLaunchCooperativeKernel((void *)k_mf_group_factor<T>, coop_grid, kTB, args, gsmem, ctx->stream);
            GRMP_LAUNCHED(ctx);
            gmax = std::max(gmax, coop_grid);
            if (e == cudaSuccess) {   // a timed-out barrier of any group fails the factorisation
                std::vector<CoopState> hc(ng);
                e = cudaMemcpyAsync(hc.data(), cs, (size_t)ng * sizeof(CoopState), cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                for (auto &h : hc) timed_out = timed_out || h.status != 0;
            }
        }
        if (rc || e != cudaSuccess) break;
    }
    int herr = 0;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, derr, 4);
    grmp_free(ctx, cs, (size_t)ncs * sizeof(CoopState));
    if (rc) return rc;
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "multifrontal factorisation");
    if (timed_out) return grmp_fail(ctx, GRMP_ERR_TIMEOUT, "multifrontal factorisation: a grid barrier wait timed out");
    if (herr)
        return grmp_fail(ctx, GRMP_ERR_NAN, "multifrontal %s factorisation: non-positive pivot in front %d",
                         sizeof(T) == 4 ? "FP32" : "FP64", herr - 1);
    *grid_out = gmax;
    return GRMP_OK;
}

// Q = [L11^-1; L21 L11^-1] of every front from the current factor (FP32 preconditioner)
template <typename T>
int mf_build_inverse(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    MfCache &C = *A->mf;
    if (!C.Q) {
        C.Qb = std::max<size_t>(1, C.L_size) * sizeof(T);
        int rc = grmp_alloc(ctx, &C.Q, C.Qb);
        if (!rc) rc = grmp_alloc(ctx, &C.wy, C.wb);
        if (!rc) rc = grmp_alloc(ctx, &C.wx, C.wb);
        if (rc) return rc;
    }
    if (C.total_bcols > 0) {
        k_mf_invert<T><<<(unsigned)C.total_bcols, kTB, 0, ctx->stream>>>(C.dev, C.bcol, C.nnodes, (const T *)C.L,
                                                                        (T *)C.Q);
        GRMP_LAUNCHED(ctx);
    }
    if (C.total_gtiles > 0) {
        const int gg = (int)std::min<long long>(C.total_gtiles, 8LL * ctx->num_sms);
        k_mf_gmat<T><<<gg, 256, 0, ctx->stream>>>(C.dev, C.gtiles, C.total_gtiles, (const T *)C.L, (T *)C.Q);
        GRMP_LAUNCHED(ctx);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "multifrontal inverse");
    return GRMP_OK;
}

// wx <- A^{-1} w with the inverse-based factor (w is overwritten): the level
// launches, in order
template <typename T>
int mf_enqueue_inverse(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    MfCache &C = *A->mf;
    const int nl = (int)C.level_ptr.size() - 1;
    const int grid = 4 * ctx->num_sms;
    int k = 0;
    for (int l = 0; l < nl; l++) {
        const int lb = C.level_ptr[l], cnt = C.level_ptr[l + 1] - lb;
        k_mf_gather_level<T><<<std::min(cnt, kMaxGrid), kTB, 0, ctx->stream>>>(C.dev, lb, cnt, (T *)C.uv, (T *)C.w);
        k_mf_qmul_level<T><<<grid, kTB, 0, ctx->stream>>>(C.dev, C.qrow, lb, cnt, (const T *)C.Q, (T *)C.uv,
                                                         (const T *)C.w, (T *)C.wy);
        k += 2;
    }
    for (int l = nl - 1; l >= 0; l--) {
        const int lb = C.level_ptr[l], cnt = C.level_ptr[l + 1] - lb;
        const long long tiles = C.bcol_host[lb + cnt] - C.bcol_host[lb];
        const int tgrid = (int)std::max<long long>(1, std::min<long long>(tiles, 2LL * ctx->num_sms));
        k_mf_qtmul_level<T><<<tgrid, kQtT, 0, ctx->stream>>>(C.dev, C.bcol, lb, cnt, (const T *)C.Q, (const T *)C.wy,
                                                            (T *)C.wx);
        k++;
    }
    return k;
}

// The sequence is replayed once per CG iteration with the same buffers, so it
// is captured into a CUDA graph at the first application after the numeric
// storage was (re)allocated and replayed from then on.
template <typename T>
int mf_apply_inverse(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    MfCache &C = *A->mf;
    if (!C.apply_graph) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            C.apply_kernels = mf_enqueue_inverse<T>(A);
            e = cudaStreamEndCapture(ctx->stream, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&C.apply_graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            C.apply_graph = nullptr;
            return grmp_cuda_fail(ctx, e, "preconditioner graph capture");
        }
    }
    cudaError_t e = cudaGraphLaunch(C.apply_graph, ctx->stream);
    ctx->launches += (uint64_t)C.apply_kernels;
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "preconditioner graph launch");
    return GRMP_OK;
}

// w <- A^{-1} w with the current factor (level launches)
template <typename T>
void mf_apply(grmp_matrix A) {
    grmp_context ctx = A->space->mesh->ctx;
    MfCache &C = *A->mf;
    const int nl = (int)C.level_ptr.size() - 1;
    const size_t smem_f = ((size_t)C.max_s + 32 * 33) * sizeof(T);
    const size_t smem_b = ((size_t)C.max_s + 32 * 33 + C.max_f) * sizeof(T);
    cudaFuncSetAttribute(k_mf_forward_level<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f);
    cudaFuncSetAttribute(k_mf_backward_level<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
    for (int l = 0; l < nl; l++) {
        const int lb = C.level_ptr[l], cnt = C.level_ptr[l + 1] - lb;
        k_mf_forward_level<T><<<std::min(cnt, kMaxGrid), kTB, smem_f, ctx->stream>>>(C.dev, lb, cnt, (const T *)C.L,
                                                                                     (T *)C.uv, (T *)C.w, C.max_s);
        GRMP_LAUNCHED(ctx);
    }
    for (int l = nl - 1; l >= 0; l--) {
        const int lb = C.level_ptr[l], cnt = C.level_ptr[l + 1] - lb;
        k_mf_backward_level<T><<<std::min(cnt, kMaxGrid), kTB, smem_b, ctx->stream>>>(C.dev, lb, cnt,
                                                                                      (const T *)C.L, (T *)C.w,
                                                                                      C.max_s);
        GRMP_LAUNCHED(ctx);
    }
}

double host_sum(grmp_context ctx, const double *dpart, int nb, cudaError_t *e) {
    std::vector<double> h(nb);
    *e = cudaMemcpyAsync(h.data(), dpart, (size_t)nb * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (*e == cudaSuccess) *e = cudaStreamSynchronize(ctx->stream);
    double s = 0.0;
    for (double v : h) s += v;   // fixed order
    return s;
}

}  // namespace

void grmp_mf_cache_free(grmp_matrix A) {
    if (!A || !A->mf) return;
    grmp_context ctx = A->space->mesh->ctx;
    mf_free_numeric(ctx, *A->mf);
    for (auto &b : A->mf->bufs) grmp_free(ctx, b.first, b.second);
    delete A->mf;
    A->mf = nullptr;
}

// grmp_solve for the direct modes; called with the context locked.
int grmp_mf_solve(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *p, grmp_solve_stats *st) {
    grmp_context ctx = A->space->mesh->ctx;
    const int n = A->nrows;
    const bool mixed = p->mode == GRMP_SOLVE_MIXED_DIRECT;
    if (!A->has64) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "solve: FP64 values not assembled");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    int rc = A->mf ? GRMP_OK : mf_build(A);
    int grid = 0;
    if (!rc) rc = mixed ? mf_numeric<float>(A, &grid) : mf_numeric<double>(A, &grid);
    if (!rc && mixed) rc = mf_build_inverse<float>(A);
    const int nb = 2 * ctx->num_sms, tb = 256;
    double *r = nullptr, *z = nullptr, *pp = nullptr, *q = nullptr, *part = nullptr;
    const size_t vb = (size_t)n * 8;
    if (!rc) rc = grmp_alloc(ctx, (void **)&r, vb);
    if (!rc) rc = grmp_alloc(ctx, (void **)&z, vb);
    if (!rc) rc = grmp_alloc(ctx, (void **)&pp, vb);
    if (!rc) rc = grmp_alloc(ctx, (void **)&q, vb);
    if (!rc) rc = grmp_alloc(ctx, (void **)&part, (size_t)nb * 8);
    auto cleanup = [&]() {
        grmp_free(ctx, r, vb);
        grmp_free(ctx, z, vb);
        grmp_free(ctx, pp, vb);
        grmp_free(ctx, q, vb);
        grmp_free(ctx, part, (size_t)nb * 8);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    };
    if (rc) {
        cleanup();
        return rc;
    }
    MfCache &C = *A->mf;
    cudaError_t e = cudaSuccess;
    const int gv = (n + tb - 1) / tb;
    if (!p->use_initial_guess) cudaMemsetAsync(x->d, 0, vb, ctx->stream);
    k_dot<<<nb, tb, 0, ctx->stream>>>(n, b->d, b->d, part);
    GRMP_LAUNCHED(ctx);
    const double bn = sqrt(host_sum(ctx, part, nb, &e));
    const double tol = std::max(p->abstol, p->reltol * bn);
    int it = 0, status = GRMP_ERR_NOT_CONVERGED;
    double rn = 0.0;
    if (!mixed) {
        // FP64 factor: x += A^{-1} (b - A x) until reltol or the residual stops falling
        double prev = INFINITY;
        for (;; it++) {
            k_resid<<<nb, tb, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, x->d, b->d, r, part);
            GRMP_LAUNCHED(ctx);
            rn = sqrt(host_sum(ctx, part, nb, &e));
            if (e != cudaSuccess) break;
            if (rn <= tol || bn == 0.0) {
                status = GRMP_OK;
                break;
            }
            if ((it > 0 && rn > 0.5 * prev) || it >= std::min(p->maxiter, 8)) {
                // the residual stopped falling (FP64 floor of an ill-conditioned system):
                // accept when the normwise backward error ||r|| / (||A|| ||x|| + ||b||) is at rounding level
                k_rownorm<<<nb, tb, 0, ctx->stream>>>(n, A->d_rowptr, A->d_vals64, part);
                GRMP_LAUNCHED(ctx);
                std::vector<double> hm(nb);
                if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), part, (size_t)nb * 8, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                double anorm = 0.0;
                for (double v : hm) anorm = std::max(anorm, v);
                k_dot<<<nb, tb, 0, ctx->stream>>>(n, x->d, x->d, part);
                GRMP_LAUNCHED(ctx);
                const double xn = sqrt(host_sum(ctx, part, nb, &e));
                const double eta = rn / (anorm * xn + bn + 1e-300);
                status = (it > 0 && rn > 0.5 * prev && eta <= 1e-13) ? GRMP_OK : GRMP_ERR_NOT_CONVERGED;
                break;
            }
            prev = rn;
            cudaMemcpyAsync(C.w, r, vb, cudaMemcpyDeviceToDevice, ctx->stream);
            mf_apply<double>(A);
            k_add_from<double><<<gv, tb, 0, ctx->stream>>>(n, (const double *)C.w, x->d);
            GRMP_LAUNCHED(ctx);
        }
    } else {
        // FP64 conjugate gradients preconditioned by the FP32 factorisation
        k_resid<<<nb, tb, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, x->d, b->d, r, part);
        GRMP_LAUNCHED(ctx);
        rn = sqrt(host_sum(ctx, part, nb, &e));
        auto precond = [&]() -> double {   // z = M^{-1} r, returns r.z
            k_to<float><<<gv, tb, 0, ctx->stream>>>(n, r, (float *)C.w);
            GRMP_LAUNCHED(ctx);
            if (mf_apply_inverse<float>(A)) e = cudaErrorUnknown;
            k_from_dot<float><<<nb, tb, 0, ctx->stream>>>(n, (const float *)C.wx, r, z, part);
            GRMP_LAUNCHED(ctx);
            return host_sum(ctx, part, nb, &e);
        };
        // CG with restarts from the true FP64 residual: when the recurrence
        // residual has converged but b - A x has not, restart from x (at most
        // 3 times); a residual that no longer falls is accepted when its
        // normwise backward error is at FP64 rounding level.
        double prev_true = INFINITY;
        for (int restart = 0; restart < 4 && e == cudaSuccess; restart++) {
            double rz = rn <= tol ? 0.0 : precond();
            cudaMemcpyAsync(pp, z, vb, cudaMemcpyDeviceToDevice, ctx->stream);
            status = GRMP_ERR_NOT_CONVERGED;
            while (e == cudaSuccess) {
                if (rn <= tol || bn == 0.0) {
                    status = GRMP_OK;
                    break;
                }
                if (it >= p->maxiter) break;
                k_apply_dot<<<nb, tb, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, pp, q, part);
                GRMP_LAUNCHED(ctx);
                const double pq = host_sum(ctx, part, nb, &e);
                if (!(pq > 0.0) || !std::isfinite(pq)) {
                    status = GRMP_ERR_NAN;
                    break;
                }
                const double alpha = rz / pq;
                k_cg_update<<<nb, tb, 0, ctx->stream>>>(n, alpha, pp, q, x->d, r, part);
                GRMP_LAUNCHED(ctx);
                rn = sqrt(host_sum(ctx, part, nb, &e));
                it++;
                if (rn <= tol) continue;
                const double rz_new = precond();
                k_xpby<<<gv, tb, 0, ctx->stream>>>(n, z, rz_new / rz, pp);
                GRMP_LAUNCHED(ctx);
                rz = rz_new;
            }
            if (e != cudaSuccess || status == GRMP_ERR_NAN) break;
            // the true FP64 residual of the iterate (r becomes b - A x)
            k_resid<<<nb, tb, 0, ctx->stream>>>(n, A->d_rowptr, A->d_cols, A->d_vals64, x->d, b->d, r, part);
            GRMP_LAUNCHED(ctx);
            rn = sqrt(host_sum(ctx, part, nb, &e));
            if (rn <= 2.0 * tol) {
                status = GRMP_OK;
                break;
            }
            if (rn > 0.5 * prev_true || it >= p->maxiter) {
                k_rownorm<<<nb, tb, 0, ctx->stream>>>(n, A->d_rowptr, A->d_vals64, part);
                GRMP_LAUNCHED(ctx);
                std::vector<double> hm(nb);
                if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), part, (size_t)nb * 8, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                double anorm = 0.0;
                for (double v : hm) anorm = std::max(anorm, v);
                k_dot<<<nb, tb, 0, ctx->stream>>>(n, x->d, x->d, part);
                GRMP_LAUNCHED(ctx);
                const double xn = sqrt(host_sum(ctx, part, nb, &e));
                status = rn / (anorm * xn + bn + 1e-300) <= 1e-13 ? GRMP_OK : GRMP_ERR_NOT_CONVERGED;
                break;
            }
            prev_true = rn;
            status = GRMP_ERR_NOT_CONVERGED;
        }
    }
    cudaEventRecord(e1, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cleanup();
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "multifrontal solve");
    st->status = status;
    st->iterations = it;
    st->outer_iterations = 0;
    st->spmv_config = 0;
    st->grid_blocks = grid;
    st->final_relres = bn > 0 ? rn / bn : 0.0;
    st->solve_ms = ms;
    if (status == GRMP_ERR_NOT_CONVERGED)
        return grmp_fail(ctx, status, "direct solve: relative residual %.3e after %d steps", st->final_relres, it);
    if (status == GRMP_ERR_NAN) return grmp_fail(ctx, status, "direct solve: breakdown of the preconditioned CG");
    return status;
}
