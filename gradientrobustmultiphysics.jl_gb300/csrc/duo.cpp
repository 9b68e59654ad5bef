// Two-run 16-bit column layout of the mixed solver's FP32 matrix copy (host
// construction, rows split over threads).
#include "duo.h"

#include <algorithm>
#include <climits>
#include <thread>

int duo_build(int n, const int32_t *rowptr, const int32_t *cols, DuoLayout *L) {
    L->n = n;
    L->meta.assign(4 * ((size_t)n + 1), 0);
    int64_t nd = 0;
    for (int i = 0; i < n; i++) {
        const int len = rowptr[i + 1] - rowptr[i];
        if (len > 65535) return 1;
        L->meta[4 * (size_t)i] = (int32_t)nd;
        nd += (len + 1) / 2;
        if (nd > INT32_MAX) return 1;
    }
    L->meta[4 * (size_t)n] = (int32_t)nd;
    L->nduo = nd;
    L->off.assign((size_t)nd, 0);
    L->src.assign((size_t)nd, 0);
    const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<int> span(nt, 0);
    auto work = [&](int t) {
        const int lo = (int)((long long)n * t / nt), hi = (int)((long long)n * (t + 1) / nt);
        int myspan = 0;
        for (int i = lo; i < hi; i++) {
            const int kb = rowptr[i], ke = rowptr[i + 1], len = ke - kb;
            int split = len;   // one run unless a gap splits the row
            int64_t gap = -1;
            for (int k = kb + 1; k < ke; k++) {
                const int64_t g = (int64_t)cols[k] - cols[k - 1];
                if (g > gap) {
                    gap = g;
                    split = k - kb;
                }
            }
            const int b1 = len ? cols[kb] : 0;
            const int b2 = split < len ? cols[kb + split] : b1;
            const int s1 = split > 0 ? cols[kb + split - 1] - b1 : 0;
            const int s2 = split < len ? cols[ke - 1] - b2 : 0;
            myspan = std::max(myspan, std::max(s1, s2));
            const int d0 = L->meta[4 * (size_t)i], ndu = (len + 1) / 2;
            L->meta[4 * (size_t)i + 1] = b1;
            L->meta[4 * (size_t)i + 2] = b2;
            L->meta[4 * (size_t)i + 3] = split | (ndu << 16);
            auto code = [&](int e) -> uint32_t {
                if (e >= len) return 0u;   // padding: offset 0 from base2
                const int c = cols[kb + e] - (e < split ? b1 : b2);
                return (uint32_t)(c > 65535 ? 65535 : c);
            };
            for (int d = 0; d < ndu; d++) {
                L->off[(size_t)d0 + d] = code(2 * d) | (code(2 * d + 1) << 16);
                L->src[(size_t)d0 + d] = 2 * d + 1 < len ? kb + 2 * d : -1 - (kb + 2 * d);
            }
        }
        span[t] = myspan;
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; t++) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    L->max_span = *std::max_element(span.begin(), span.end());
    return L->max_span > 65535 ? 1 : 0;
}
