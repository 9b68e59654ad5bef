// Dense kernels of the multifrontal Cholesky factorisation, shared by the
// batched Stokes solver (one problem per block, FP64) and the single-problem
// direct solvers (FP64, or FP32 as a preconditioner).
#pragma once

constexpr int kPanel = 16;
constexpr int kPanelStride = kPanel + 1;   // panel row stride (spreads shared-memory banks)

// The threads that run one dense front operation: the whole block
// (barrier 0 = __syncthreads) or a contiguous range of warps synchronised by
// the named barrier `bar` (1..15).
struct ThreadGroup {
    int tid, size, bar;
    __device__ __forceinline__ void sync() const {
        if (bar == 0) __syncthreads();
        else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(size) : "memory");
    }
};
__device__ __forceinline__ ThreadGroup whole_block() { return ThreadGroup{(int)threadIdx.x, (int)blockDim.x, 0}; }

// Partial Cholesky of a front F (f x f, lower part, row-major): eliminate
// its first s columns.  Blocked right-looking: a panel of kPanel columns
// (all rows from the panel's diagonal down) is copied to shared memory P and
// factored there column by column, written back, and the trailing lower
// triangle receives one rank-kPanel update per panel from 4x4 register
// tiles reading the panel from P, so F is read and written once per panel
// instead of once per column.  Returns false on a non-positive pivot.  The
// arithmetic of every entry is independent of the thread group's size.
// P holds (f - k0) x kPanel values with row stride ps (shared or global memory).

template <typename T>
__device__ bool front_cholesky(T *F, int f, int s, T *colk, T *P, int ps, ThreadGroup g = whole_block()) {
    const int tid = g.tid, bs = g.size;
    for (int k0 = 0; k0 < s; k0 += kPanel) {
        const int kw = min(kPanel, s - k0), k1 = k0 + kw, mp = f - k0;
        // panel: rows k0..f-1, columns k0..k1-1, factored in shared memory
        for (int q = tid; q < mp * kw; q += bs) {
            const int i = q / kw, t = q - i * kw;
            P[i * ps + t] = F[(long long)(k0 + i) * f + k0 + t];
        }
        g.sync();
        for (int c = 0; c < kw; c++) {
            const T dcc = P[c * ps + c];
            if (!(dcc > T(0)) || !isfinite((double)dcc)) return false;   // uniform: same value in every thread
            const T dk = sqrt(dcc);
            for (int i = c + 1 + tid; i < mp; i += bs) {
                const T v = P[i * ps + c] / dk;
                P[i * ps + c] = v;
                colk[i] = v;
            }
            g.sync();
            if (tid == 0) P[c * ps + c] = dk;
            for (int i = c + 1 + tid; i < mp; i += bs) {
                const T lic = colk[i];
                const int jmax = min(i, kw - 1);
                for (int j = c + 1; j <= jmax; j++) P[i * ps + j] -= lic * colk[j];
            }
            g.sync();
        }
        for (int q = tid; q < mp * kw; q += bs) {
            const int i = q / kw, t = q - i * kw;
            if (t <= i) F[(long long)(k0 + i) * f + k0 + t] = P[i * ps + t];
        }
        // trailing lower triangle: rank-kw update from 4x4 register tiles
        const int m = f - k1;
        const T *Pt = P + kw * ps;   // panel rows k1..f-1
        const int nt = (m + 3) >> 2;
        const long long ntiles = (long long)nt * (nt + 1) / 2;
        for (long long q = tid; q < ntiles; q += bs) {
            int bi = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
            while ((long long)(bi + 1) * (bi + 2) / 2 <= q) bi++;
            while ((long long)bi * (bi + 1) / 2 > q) bi--;
            const int bj = (int)(q - (long long)bi * (bi + 1) / 2);
            const int i0 = bi * 4, j0 = bj * 4;
            T acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = T(0);
            for (int t = 0; t < kw; t++) {
                T x[4], y[4];
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    x[a] = i0 + a < m ? Pt[(i0 + a) * ps + t] : T(0);
                    y[a] = j0 + a < m ? Pt[(j0 + a) * ps + t] : T(0);
                }
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) acc[a][b] += x[a] * y[b];
            }
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int i = i0 + a;
                if (i >= m) break;
                T *Fi = F + (long long)(k1 + i) * f + k1;
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int j = j0 + b;
                    if (j <= i) Fi[j] -= acc[a][b];
                }
            }
        }
        g.sync();
    }
    return true;
}

