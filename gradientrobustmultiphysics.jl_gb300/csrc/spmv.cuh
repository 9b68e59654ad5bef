// Warp-stream CSR SpMV core shared by the persistent and the batched solvers.
//
// A warp owns RPW = 8 consecutive rows at a time.  Their nonzeros form one
// contiguous range [ka, kb) of the CSR arrays; the warp streams it in chunks
// of CHUNK entries with fully coalesced loads (lane l reads entries
// c0 + 32 j + l, j = 0..CHUNK/32-1, all independent, so every lane keeps
// CHUNK/32 column and value loads and CHUNK/32 gathers in flight), writes the
// products to a per-warp shared-memory buffer, and four lanes per row sum
// that row's segment.  Rows of any length work (a row may span chunks); the
// summation order of a row is fixed by its length, so results are
// reproducible run to run.
#pragma once

#include "grmp_internal.h"

namespace spmv {

constexpr int RPW = 8;   // rows per warp step (4 lanes per row in the segmented sum)

// gather(c) -> A: value of the input vector at column c
// epilogue(r, acc): consumes the row result (lane with sub == 0 only)
template <int CHUNK, typename V, typename A, typename Gather, typename Epi>
__device__ __forceinline__ void warp_stream(int r0, int r1, int gw, int nw, const int32_t *__restrict__ rowptr,
                                            const int32_t *__restrict__ cols, const V *__restrict__ vals,
                                            A *wbuf, Gather gather, Epi epi) {
    static_assert(CHUNK % 32 == 0, "chunk must be a multiple of the warp size");
    constexpr int J = CHUNK / 32;
    const int lane = threadIdx.x & 31;
    const int sub = lane & 3, rl = lane >> 2;
    for (int base = r0 + gw * RPW; base < r1; base += nw * RPW) {
        const int r = base + rl;
        const bool valid = r < r1;
        const int rs = valid ? __ldg(rowptr + r) : 0;
        const int re = valid ? __ldg(rowptr + r + 1) : 0;
        const int ka = __ldg(rowptr + base);
        const int kb = __ldg(rowptr + min(base + RPW, r1));
        A acc = 0;
        for (int c0 = ka; c0 < kb; c0 += CHUNK) {
            int cc[J];
            A vv[J];
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int k = c0 + j * 32 + lane;
                const bool ok = k < kb;
                cc[j] = ok ? __ldg(cols + k) : -1;
                vv[j] = ok ? (A)__ldg(vals + k) : A(0);
            }
#pragma unroll
            for (int j = 0; j < J; j++) wbuf[j * 32 + lane] = cc[j] >= 0 ? vv[j] * gather(cc[j]) : A(0);
            __syncwarp();
            const int lo = max(rs, c0) - c0, hi = min(re, c0 + CHUNK) - c0;
            for (int t = lo + sub; t < hi; t += 4) acc += wbuf[t];
            __syncwarp();
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (valid && sub == 0) epi(r, acc);
    }
}

}  // namespace spmv
