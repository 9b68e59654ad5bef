// Nested-dissection ordering and multifrontal symbolic analysis of one
// problem's sparsity pattern (host side of the batched direct solver).
//
// The reference solves every iterated-penalty sweep with a sparse direct
// solver (UMFPACK through LinearSolve.jl, src/solvers.jl:89-101); on the GPU
// each problem of a batch gets a multifrontal Cholesky factorisation, done
// once and reused by every sweep.  This file computes, for a symmetric
// pattern:
//   * a nested-dissection elimination order: level-set separators of a
//     breadth-first search started at a pseudo-peripheral DoF, recursively,
//     down to leaves of at most kLeaf DoFs;
//   * the assembly tree in post-order (children before parents, which is
//     the elimination order), each node with its front = its own DoFs
//     followed by its structure (later-eliminated DoFs coupled to them);
//   * for every node the map of original matrix entries into its front and
//     the map of each child's update matrix into the parent's front;
//   * storage offsets of the factor columns and update matrices.
// Everything depends on the pattern only, so problems with equal local
// patterns share one analysis.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "nd_symbolic.h"

namespace {

constexpr int kLeaf = 48;

struct Builder {
    int n;
    const int32_t *rp, *ci;      // local CSR (columns local, includes the diagonal)
    std::vector<int> stamp;      // membership stamps
    int cur = 0;
    std::vector<int> level, queue;
    NdSymbolic *S;
    std::vector<std::vector<int>> own;   // own DoFs per node (creation = post-order)
    std::vector<std::vector<int>> kids;

    int bfs(const std::vector<int> &set, int start, int setstamp, std::vector<int> &order_out) {
        // returns the eccentricity of `start` in the subgraph; order_out = BFS order
        order_out.clear();
        ++cur;
        const int visit = cur;
        order_out.push_back(start);
        level[start] = 0;
        stamp[start] = visit;
        int far = 0;
        for (size_t h = 0; h < order_out.size(); h++) {
            const int v = order_out[h];
            for (int k = rp[v]; k < rp[v + 1]; k++) {
                const int w = ci[k];
                if (w == v || stamp[w] != setstamp) continue;
                stamp[w] = visit;
                level[w] = level[v] + 1;
                far = std::max(far, level[w]);
                order_out.push_back(w);
            }
        }
        // restore the set stamp for the members reached
        for (int v : order_out) stamp[v] = setstamp;
        return far;
    }

    int dissect(std::vector<int> set) {
        if ((int)set.size() <= kLeaf) return leaf(std::move(set));
        ++cur;
        const int setstamp = cur;
        for (int v : set) stamp[v] = setstamp;
        std::vector<int> ord;
        // pseudo-peripheral start: repeat BFS from a farthest DoF while the eccentricity grows
        int start = set[0];
        int ecc = bfs(set, start, setstamp, ord);
        if (ord.size() < set.size()) {
            // disconnected: split off the component of set[0]
            std::vector<int> a = ord, b;
            ++cur;
            for (int v : a) stamp[v] = cur;
            for (int v : set)
                if (stamp[v] != cur) b.push_back(v);
            int ca = dissect(std::move(a));
            int cb = dissect(std::move(b));
            return join({}, {ca, cb});
        }
        for (int rep = 0; rep < 4; rep++) {
            int cand = ord.back();
            std::vector<int> o2;
            int e2 = bfs(set, cand, setstamp, o2);
            if (e2 <= ecc) break;
            ecc = e2;
            start = cand;
            ord.swap(o2);
        }
        bfs(set, start, setstamp, ord);   // levels from the chosen start
        if (ecc < 2) return leaf(std::move(set));
        // median level as the separator
        std::vector<int> cnt(ecc + 1, 0);
        for (int v : ord) cnt[level[v]]++;
        int acc = 0, L = 1;
        const int half = (int)set.size() / 2;
        for (int l = 0; l <= ecc; l++) {
            acc += cnt[l];
            if (acc >= half) {
                L = l;
                break;
            }
        }
        L = std::min(std::max(L, 1), ecc - 1);
        std::vector<int> a, b, sep;
        for (int v : ord) {
            if (level[v] < L) a.push_back(v);
            else if (level[v] > L) b.push_back(v);
            else sep.push_back(v);
        }
        std::vector<int> ch;
        if (!a.empty()) ch.push_back(dissect(std::move(a)));
        if (!b.empty()) ch.push_back(dissect(std::move(b)));
        return join(std::move(sep), std::move(ch));
    }

    int leaf(std::vector<int> set) { return join(std::move(set), {}); }

    int join(std::vector<int> mine, std::vector<int> children) {
        own.push_back(std::move(mine));
        kids.push_back(std::move(children));
        return (int)own.size() - 1;
    }
};

}  // namespace

int nd_symbolic_build(int n, const int32_t *rowptr, const int32_t *cols, NdSymbolic *S) {
    *S = NdSymbolic();
    if (n <= 0) return 1;
    Builder B;
    B.n = n;
    B.rp = rowptr;
    B.ci = cols;
    B.stamp.assign(n, 0);
    B.level.assign(n, 0);
    B.S = S;
    std::vector<int> all(n);
    for (int i = 0; i < n; i++) all[i] = i;
    B.dissect(std::move(all));
    const int nn = (int)B.own.size();
    // elimination order = own lists in node (post-)order
    std::vector<int> order(n, -1), node_of(n, -1);
    std::vector<int> last(nn, -1);   // last elimination index in the node's subtree
    int k = 0;
    for (int t = 0; t < nn; t++) {
        for (int v : B.own[t]) {
            order[v] = k++;
            node_of[v] = t;
        }
        int l = B.own[t].empty() ? -1 : order[B.own[t].back()];
        for (int c : B.kids[t]) l = std::max(l, last[c]);
        last[t] = l;
    }
    if (k != n) return 2;
    // structures, bottom-up
    std::vector<std::vector<int>> strct(nn);
    std::vector<int> mark(n, -1);
    for (int t = 0; t < nn; t++) {
        std::vector<int> &st = strct[t];
        auto add = [&](int j) {
            if (order[j] > last[t] && mark[j] != t) {
                mark[j] = t;
                st.push_back(j);
            }
        };
        for (int v : B.own[t])
            for (int q = rowptr[v]; q < rowptr[v + 1]; q++) add(cols[q]);
        for (int c : B.kids[t])
            for (int j : strct[c]) add(j);
        std::sort(st.begin(), st.end(), [&](int a, int b) { return order[a] < order[b]; });
    }
    // parents
    std::vector<int> parent(nn, -1);
    for (int t = 0; t < nn; t++)
        for (int c : B.kids[t]) parent[c] = t;
    // fronts, maps, offsets
    S->n = n;
    S->nnodes = nn;
    S->perm.resize(n);
    for (int v = 0; v < n; v++) S->perm[order[v]] = v;
    std::vector<int> pos(n, -1);
    int64_t Loff = 0, Uoff = 0;
    S->node.resize(nn);
    for (int t = 0; t < nn; t++) {
        NdNode &nd = S->node[t];
        nd.s = (int)B.own[t].size();
        nd.f = nd.s + (int)strct[t].size();
        nd.parent = parent[t];
        nd.front_off = (int)S->front.size();
        for (int v : B.own[t]) S->front.push_back(v);
        for (int v : strct[t]) S->front.push_back(v);
        nd.child_off = (int)S->child.size();
        nd.nchild = (int)B.kids[t].size();
        for (int c : B.kids[t]) S->child.push_back(c);
        nd.L_off = Loff;
        Loff += (int64_t)nd.f * nd.s;
        nd.U_off = Uoff;
        const int64_t sc = nd.f - nd.s;
        Uoff += sc * sc;
        S->max_f = std::max(S->max_f, nd.f);
        S->max_s = std::max(S->max_s, nd.s);
        // original entries (r, c) with c in own(t), order[r] >= order[c]
        for (int i = 0; i < nd.f; i++) pos[S->front[nd.front_off + i]] = i;
        nd.entry_off = (int)S->ent_rel.size();
        for (int v : B.own[t])
            for (int q = rowptr[v]; q < rowptr[v + 1]; q++) {
                const int r = cols[q];
                if (order[r] < order[v]) continue;
                if (pos[r] < 0) return 3;
                S->ent_rel.push_back(q - rowptr[0]);
                S->ent_pos.push_back(pos[r] * nd.f + pos[v]);
            }
        nd.nentry = (int)S->ent_rel.size() - nd.entry_off;
        // children's structures into this front
        for (int c : B.kids[t]) {
            NdNode &cn = S->node[c];
            cn.ext_off = (int)S->ext.size();
            for (int j : strct[c]) {
                if (pos[j] < 0) return 4;
                S->ext.push_back(pos[j]);
            }
        }
        for (int i = 0; i < nd.f; i++) pos[S->front[nd.front_off + i]] = -1;
    }
    S->L_size = Loff;
    S->U_size = Uoff;
    // level schedule (height above the leaves) and update-vector offsets
    std::vector<int> height(nn, 0);
    int maxh = 0;
    for (int t = 0; t < nn; t++) {
        for (int c : B.kids[t]) height[t] = std::max(height[t], height[c] + 1);
        maxh = std::max(maxh, height[t]);
    }
    S->level_ptr.assign(maxh + 2, 0);
    for (int t = 0; t < nn; t++) S->level_ptr[height[t] + 1]++;
    for (int l = 0; l <= maxh; l++) S->level_ptr[l + 1] += S->level_ptr[l];
    S->level_nodes.resize(nn);
    S->level_maxf.assign(maxh + 1, 0);
    std::vector<int> fill(S->level_ptr.begin(), S->level_ptr.end() - 1);
    for (int t = 0; t < nn; t++) {
        S->level_nodes[fill[height[t]]++] = t;
        S->level_maxf[height[t]] = std::max(S->level_maxf[height[t]], S->node[t].f);
    }
    S->uv_off.resize(nn);
    int64_t uo = 0;
    for (int t = 0; t < nn; t++) {
        S->uv_off[t] = uo;
        uo += S->node[t].f - S->node[t].s;
    }
    S->uv_size = uo;
    return 0;
}
