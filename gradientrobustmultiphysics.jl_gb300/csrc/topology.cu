// Mesh topology and DoF maps built on the device: the entity enumeration of
// the grid (edges; faces with the cells that share them), the CellDofs of
// H1P1 / H1P2 spaces (the dofmap of FESpace{FEType}(xgrid),
// src/dofmaps.jl:201-330, patterns "N1" of src/fedefs/h1_p1.jl and "N1F1" /
// "N1E1" of src/fedefs/h1_p2.jl:33-35) and the DoFs on boundary faces of any
// space (the BFaceDofs collected by boundarydata!, src/boundarydata.jl:200-260,
// all boundary regions).
//
// Numbering (the ExtendableGrids role, restated here and in the host mesh
// module identically): an edge or face is the sorted tuple of its vertices,
// and entities are numbered in the lexicographic order of those tuples.
// Enumeration without a global sort: every (cell, local entity) is filed
// under its smallest vertex (a counting pass, an exclusive scan and a fill
// pass), each vertex's bucket is sorted and deduplicated by one thread (a
// few dozen entries on simplex meshes), and the entity id is the number of
// distinct entities under smaller vertices plus the rank inside the bucket.
// The result does not depend on the order in which the atomics fill a
// bucket.
#include <vector>

#include "grmp_internal.h"

namespace {

constexpr int TPB = 256;
inline int nblk(long long n) { return (int)((n + TPB - 1) / TPB); }

__constant__ int kTriEdges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
__constant__ int kTetEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
__constant__ int kTetFaces[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};

// entity kinds: 2D edges (= faces), 3D edges, 3D faces
struct EntKind {
    int dim, k, nloc;   // cell dimension, vertices per entity, entities per cell
};

__device__ __forceinline__ void ent_tuple(const int32_t *cells, EntKind e, long long idx, int t[3]) {
    const long long c = idx / e.nloc;
    const int l = (int)(idx % e.nloc);
    const int32_t *cv = cells + c * (e.dim + 1);
    if (e.k == 2) {
        const int a = e.dim == 2 ? cv[kTriEdges[l][0]] : cv[kTetEdges[l][0]];
        const int b = e.dim == 2 ? cv[kTriEdges[l][1]] : cv[kTetEdges[l][1]];
        t[0] = min(a, b);
        t[1] = max(a, b);
        t[2] = 0;
    } else {
        int a = cv[kTetFaces[l][0]], b = cv[kTetFaces[l][1]], d = cv[kTetFaces[l][2]];
        if (a > b) { int s = a; a = b; b = s; }
        if (b > d) { int s = b; b = d; d = s; }
        if (a > b) { int s = a; a = b; b = s; }
        t[0] = a, t[1] = b, t[2] = d;
    }
}

// key of an entity inside the bucket of its smallest vertex
__device__ __forceinline__ long long ent_key(const int t[3], int k, int nverts) {
    return k == 2 ? (long long)t[1] : (long long)t[1] * nverts + t[2];
}

__global__ void k_ent_count(long long n, const int32_t *cells, EntKind e, int32_t *cnt) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int t[3];
    ent_tuple(cells, e, i, t);
    atomicAdd(&cnt[t[0]], 1);
}

__global__ void k_ent_fill(long long n, const int32_t *cells, EntKind e, int nverts, const int32_t *off,
                           int32_t *fill, long long *bucket) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int t[3];
    ent_tuple(cells, e, i, t);
    const int pos = off[t[0]] + atomicAdd(&fill[t[0]], 1);
    bucket[pos] = ent_key(t, e.k, nverts);
}

// per vertex: sort its bucket, keep the distinct keys in front with their
// multiplicities (the number of cells sharing the entity)
__global__ void k_ent_dedupe(int nverts, const int32_t *off, long long *bucket, int32_t *mult, int32_t *ucount) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nverts) return;
    const int b = off[v], e = off[v + 1];
    for (int i = b + 1; i < e; i++) {
        const long long key = bucket[i];
        int j = i - 1;
        while (j >= b && bucket[j] > key) {
            bucket[j + 1] = bucket[j];
            j--;
        }
        bucket[j + 1] = key;
    }
    int u = 0;
    for (int i = b; i < e; i++) {
        if (u > 0 && bucket[b + u - 1] == bucket[i]) {
            mult[b + u - 1]++;
        } else {
            bucket[b + u] = bucket[i];
            mult[b + u] = 1;
            u++;
        }
    }
    ucount[v] = u;
}

// entity id of every (cell, local entity); optionally whether it is a
// boundary entity (owned by one cell)
__global__ void k_ent_lookup(long long n, const int32_t *cells, EntKind e, int nverts, const int32_t *off,
                             const long long *bucket, const int32_t *mult, const int32_t *ucount,
                             const int32_t *ubase, int32_t *cell_ent, uint8_t *bnd) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int t[3];
    ent_tuple(cells, e, i, t);
    const long long key = ent_key(t, e.k, nverts);
    int lo = off[t[0]], hi = off[t[0]] + ucount[t[0]] - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (bucket[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    if (cell_ent) cell_ent[i] = ubase[t[0]] + (lo - off[t[0]]);
    if (bnd) bnd[i] = mult[lo] == 1 ? 1 : 0;
}

// CellDofs: per component the nv vertex DoFs, then (H1P2) the ne edge DoFs
__global__ void k_celldofs(int ncells, const int32_t *cells, int nv, const int32_t *cell_edges, int ne, int ncomp,
                           int nverts, int coffset, int32_t *celldofs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const int nb = nv + ne;
    int32_t *out = celldofs + (size_t)c * nb * ncomp;
    for (int k = 0; k < ncomp; k++) {
        for (int v = 0; v < nv; v++) out[k * nb + v] = cells[(size_t)c * nv + v] + k * coffset;
        for (int l = 0; l < ne; l++) out[k * nb + nv + l] = nverts + cell_edges[(size_t)c * ne + l] + k * coffset;
    }
}

// mark the DoFs that lie on boundary faces, through the space's CellDofs:
// the face's vertex DoFs (every component), its edge DoFs (H1P2) and its
// face bubble (H1BR)
__global__ void k_mark_boundary(long long n, int dim, int fe, int ncomp, int ldofs, const int32_t *celldofs,
                                const uint8_t *bnd, uint8_t *flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !bnd[i]) return;
    const int nloc = dim + 1;
    const long long c = i / nloc;
    const int f = (int)(i % nloc);
    const int32_t *cd = celldofs + c * ldofs;
    const int nv = dim + 1;
    int fv[3], nfv = dim;
    for (int j = 0; j < nfv; j++) fv[j] = dim == 2 ? kTriEdges[f][j] : kTetFaces[f][j];
    if (fe == GRMP_FE_H1P1 || fe == GRMP_FE_H1P2 || fe == GRMP_FE_H1BR) {
        const int nb = fe == GRMP_FE_H1P1 ? nv : (fe == GRMP_FE_H1BR ? nv : (dim == 2 ? 6 : 10));
        for (int k = 0; k < ncomp; k++)
            for (int j = 0; j < nfv; j++) flag[cd[k * nb + fv[j]]] = 1;
        if (fe == GRMP_FE_H1P2) {
            for (int k = 0; k < ncomp; k++) {
                if (dim == 2) {
                    flag[cd[k * nb + nv + f]] = 1;   // the face is the edge f
                } else {
                    for (int l = 0; l < 6; l++) {
                        int on = 0;
                        for (int j = 0; j < 3; j++) on += (kTetEdges[l][0] == fv[j]) + (kTetEdges[l][1] == fv[j]);
                        if (on == 2) flag[cd[k * nb + nv + l]] = 1;
                    }
                }
            }
        }
        if (fe == GRMP_FE_H1BR) flag[cd[ncomp * nv + f]] = 1;
    }
}

struct DevBuf {
    grmp_context ctx;
    std::vector<std::pair<void *, size_t>> held;
    template <typename T>
    int get(T **p, size_t count) {
        int rc = grmp_alloc(ctx, (void **)p, count * sizeof(T) + (count == 0 ? 8 : 0));
        if (!rc) held.push_back({*p, count * sizeof(T) + (count == 0 ? 8 : 0)});
        return rc;
    }
    ~DevBuf() {
        for (auto &h : held) grmp_free(ctx, h.first, h.second);
    }
};

// Enumerate one entity kind of the mesh.  cell_ent (optional) receives the
// entity id of every (cell, local entity), bnd (optional) whether it lies on
// the boundary; *count the number of distinct entities.
int enumerate(grmp_mesh m, EntKind e, int32_t *cell_ent, uint8_t *bnd, int32_t *count) {
    grmp_context ctx = m->ctx;
    const long long n = (long long)m->ncells * e.nloc;
    if (n >= (1LL << 31)) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "topology: too many cell entities");
    DevBuf buf{ctx, {}};
    int32_t *cnt, *off, *fill, *mult, *ucount, *ubase;
    long long *bucket;
    const int nv = m->nverts;
    int rc = buf.get(&cnt, nv);
    if (!rc) rc = buf.get(&off, (size_t)nv + 1);
    if (!rc) rc = buf.get(&fill, nv);
    if (!rc) rc = buf.get(&ucount, nv);
    if (!rc) rc = buf.get(&ubase, (size_t)nv + 1);
    if (!rc) rc = buf.get(&mult, (size_t)n);
    if (!rc) rc = buf.get(&bucket, (size_t)n);
    if (rc) return rc;
    cudaMemsetAsync(cnt, 0, (size_t)nv * 4, ctx->stream);
    cudaMemsetAsync(fill, 0, (size_t)nv * 4, ctx->stream);
    k_ent_count<<<nblk(n), TPB, 0, ctx->stream>>>(n, m->d_cells, e, cnt);
    GRMP_LAUNCHED(ctx);
    int32_t total = 0;
    rc = grmp_scan_i32(ctx, cnt, off, nv, &total);
    if (rc) return rc;
    cudaMemcpyAsync(off + nv, &total, 4, cudaMemcpyHostToDevice, ctx->stream);
    k_ent_fill<<<nblk(n), TPB, 0, ctx->stream>>>(n, m->d_cells, e, nv, off, fill, bucket);
    GRMP_LAUNCHED(ctx);
    k_ent_dedupe<<<nblk(nv), TPB, 0, ctx->stream>>>(nv, off, bucket, mult, ucount);
    GRMP_LAUNCHED(ctx);
    int32_t nent = 0;
    rc = grmp_scan_i32(ctx, ucount, ubase, nv, &nent);
    if (rc) return rc;
    k_ent_lookup<<<nblk(n), TPB, 0, ctx->stream>>>(n, m->d_cells, e, nv, off, bucket, mult, ucount, ubase, cell_ent,
                                                   bnd);
    GRMP_LAUNCHED(ctx);
    GRMP_CUDA(ctx, cudaGetLastError());
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *count = nent;
    return GRMP_OK;
}

EntKind edge_kind(int dim) { return dim == 2 ? EntKind{2, 2, 3} : EntKind{3, 2, 6}; }
EntKind face_kind(int dim) { return dim == 2 ? EntKind{2, 2, 3} : EntKind{3, 3, 4}; }

}  // namespace

int grmp_space_create_on_device(grmp_mesh mesh, int fe_kind, int ncomponents, grmp_space *out, int32_t *ndofs_out) {
    if (!mesh || !out) return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    grmp_context ctx = mesh->ctx;
    const int dim = mesh->dim;
    if (!((fe_kind == GRMP_FE_H1P1 || fe_kind == GRMP_FE_H1P2) && ncomponents >= 1 && ncomponents <= 3))
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "device dofmap: H1P1 / H1P2 with 1-3 components (got %d, %d)",
                         fe_kind, ncomponents);
    cudaSetDevice(ctx->device);
    const int nv = dim + 1;
    int ne = 0;
    int32_t nedges = 0;
    int32_t *cell_edges = nullptr;
    DevBuf buf{ctx, {}};
    int rc = GRMP_OK;
    if (fe_kind == GRMP_FE_H1P2) {
        const EntKind e = edge_kind(dim);
        ne = e.nloc;
        rc = buf.get(&cell_edges, (size_t)mesh->ncells * ne);
        if (!rc) rc = enumerate(mesh, e, cell_edges, nullptr, &nedges);
        if (rc) return rc;
    }
    const long long coffset = (long long)mesh->nverts + nedges;
    if (coffset * ncomponents >= (1LL << 31)) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "device dofmap: too many DoFs");
    const int ldofs = (nv + ne) * ncomponents;
    if (ldofs != grmp_fe_ldofs(fe_kind, dim, ncomponents))
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "device dofmap: local DoF count");
    grmp_space s = new (std::nothrow) grmp_space_s();
    if (!s) return GRMP_ERR_OUT_OF_MEMORY;
    s->mesh = mesh;
    s->fe = fe_kind;
    s->ncomp = ncomponents;
    s->ldofs = ldofs;
    s->nb = grmp_fe_nb(fe_kind, dim);
    s->ndofs = (int32_t)(coffset * ncomponents);
    rc = grmp_alloc(ctx, (void **)&s->d_celldofs, (size_t)mesh->ncells * ldofs * 4);
    if (!rc) {
        k_celldofs<<<nblk(mesh->ncells), TPB, 0, ctx->stream>>>(mesh->ncells, mesh->d_cells, nv, cell_edges, ne,
                                                                 ncomponents, mesh->nverts, (int)coffset, s->d_celldofs);
        GRMP_LAUNCHED(ctx);
        rc = grmp_build_incidence(s);
    }
    if (!rc) GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (rc) {
        grmp_space_destroy(s);
        return rc;
    }
    *out = s;
    if (ndofs_out) *ndofs_out = s->ndofs;
    return GRMP_OK;
}

int grmp_space_celldofs(grmp_space s, int32_t *celldofs) {
    if (!s || !celldofs) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = s->mesh->ctx;
    cudaSetDevice(ctx->device);
    GRMP_CUDA(ctx, cudaMemcpyAsync(celldofs, s->d_celldofs, (size_t)s->mesh->ncells * s->ldofs * 4,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GRMP_OK;
}

int grmp_space_boundary_dofs(grmp_space s, int32_t capacity, int32_t *fixed, int32_t *nfixed) {
    if (!s || !nfixed || capacity < 0) return GRMP_ERR_INVALID_ARG;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    cudaSetDevice(ctx->device);
    *nfixed = 0;
    if (s->fe == GRMP_FE_L2P0) return GRMP_OK;
    if (!(s->fe == GRMP_FE_H1P1 || s->fe == GRMP_FE_H1P2 || s->fe == GRMP_FE_H1BR))
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "boundary DoFs: element %d", s->fe);
    const EntKind e = face_kind(m->dim);
    const long long n = (long long)m->ncells * e.nloc;
    DevBuf buf{ctx, {}};
    uint8_t *bnd, *flag;
    int rc = buf.get(&bnd, (size_t)n);
    if (!rc) rc = buf.get(&flag, (size_t)s->ndofs);
    int32_t nf = 0;
    if (!rc) rc = enumerate(m, e, nullptr, bnd, &nf);
    if (rc) return rc;
    cudaMemsetAsync(flag, 0, (size_t)s->ndofs, ctx->stream);
    k_mark_boundary<<<nblk(n), TPB, 0, ctx->stream>>>(n, m->dim, s->fe, s->ncomp, s->ldofs, s->d_celldofs, bnd, flag);
    GRMP_LAUNCHED(ctx);
    std::vector<uint8_t> h((size_t)s->ndofs);
    GRMP_CUDA(ctx, cudaMemcpyAsync(h.data(), flag, h.size(), cudaMemcpyDeviceToHost, ctx->stream));
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int32_t k = 0;
    for (int32_t i = 0; i < s->ndofs; i++)
        if (h[i]) {
            if (fixed && k < capacity) fixed[k] = i;
            k++;
        }
    *nfixed = k;
    if (fixed && k > capacity)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "boundary DoFs: %d do not fit the capacity %d", k, capacity);
    return GRMP_OK;
}
