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

// outward unit normal and measure of local face l of cell c, as the host
// mesh module builds them: 2D (t_y, -t_x) with t = P1 - P0, 3D
// (P1 - P0) x (P2 - P0), normalised and turned away from the cell centroid
__device__ void face_outward(const double *coords, const int32_t *cells, int dim, long long c, int l, double n[3],
                             double &meas) {
    const int32_t *cv = cells + c * (dim + 1);
    double X[4][3], P[3][3];
    for (int v = 0; v <= dim; v++)
        for (int k = 0; k < dim; k++) X[v][k] = coords[(size_t)cv[v] * dim + k];
    for (int j = 0; j < dim; j++)
        for (int k = 0; k < dim; k++) P[j][k] = X[dim == 2 ? kTriEdges[l][j] : kTetFaces[l][j]][k];
    double cc[3] = {0, 0, 0}, fm[3] = {0, 0, 0};
    for (int k = 0; k < dim; k++) {
        for (int v = 0; v <= dim; v++) cc[k] += X[v][k];
        cc[k] /= (dim + 1);
        for (int j = 0; j < dim; j++) fm[k] += P[j][k];
        fm[k] /= dim;
    }
    // products rounded before they are subtracted or summed (no FMA
    // contraction): an axis-aligned face then gets exactly zero normal
    // components, as on the host, and the drop-zero pattern of a BR space
    // built here is the host-built one's
    double nr[3] = {0, 0, 0};
    if (dim == 2) {
        nr[0] = P[1][1] - P[0][1];
        nr[1] = -(P[1][0] - P[0][0]);
    } else {
        double a[3], b[3];
        for (int k = 0; k < 3; k++) {
            a[k] = P[1][k] - P[0][k];
            b[k] = P[2][k] - P[0][k];
        }
        nr[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
        nr[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
        nr[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
    }
    double ln = 0;
    for (int k = 0; k < dim; k++) ln = __dadd_rn(ln, __dmul_rn(nr[k], nr[k]));
    ln = sqrt(ln);
    double d = 0;
    for (int k = 0; k < dim; k++) {
        nr[k] /= ln;
        d = __dadd_rn(d, __dmul_rn(nr[k], fm[k] - cc[k]));
    }
    const double sg = d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0);
    for (int k = 0; k < 3; k++) n[k] = k < dim ? nr[k] * sg : 0.0;
    meas = dim == 2 ? ln : 0.5 * ln;
}

// the owner of a face is the lowest-numbered cell that has it
__global__ void k_face_owner(long long n, int nloc, const int32_t *cell_faces, int32_t *owner) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicMin(&owner[cell_faces[i]], (int32_t)(i / nloc));
}

// the face normal is the owner's outward normal; the measure the owner's
__global__ void k_face_geom(long long n, int dim, const double *coords, const int32_t *cells,
                            const int32_t *cell_faces, const int32_t *owner, double *normals, double *vols) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nloc = dim + 1;
    const long long c = i / nloc;
    const int f = cell_faces[i];
    if (owner[f] != c) return;
    double nn[3], meas;
    face_outward(coords, cells, dim, c, (int)(i % nloc), nn, meas);
    for (int k = 0; k < dim; k++) normals[(size_t)f * dim + k] = nn[k];
    vols[f] = meas;
}

// +1 where the cell's outward normal agrees with the face normal, else -1
__global__ void k_face_signs(long long n, int dim, const double *coords, const int32_t *cells,
                             const int32_t *cell_faces, const double *normals, int8_t *signs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nloc = dim + 1;
    double nn[3], meas;
    face_outward(coords, cells, dim, i / nloc, (int)(i % nloc), nn, meas);
    const int f = cell_faces[i];
    double d = 0;
    for (int k = 0; k < dim; k++) d += nn[k] * normals[(size_t)f * dim + k];
    signs[i] = d > 0 ? 1 : -1;
}

// H1BR CellDofs: the vertex DoFs of each component, then the faces
__global__ void k_celldofs_br(int ncells, const int32_t *cells, int dim, int nverts, const int32_t *cell_faces,
                              int32_t *celldofs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const int nv = dim + 1;
    int32_t *out = celldofs + (size_t)c * (dim * nv + nv);
    for (int k = 0; k < dim; k++)
        for (int v = 0; v < nv; v++) out[k * nv + v] = cells[(size_t)c * nv + v] + k * nverts;
    for (int l = 0; l < nv; l++) out[dim * nv + l] = dim * nverts + cell_faces[(size_t)c * nv + l];
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

int grmp_mesh_build_faces(grmp_mesh m) {
    if (!m) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = m->ctx;
    cudaSetDevice(ctx->device);
    const int dim = m->dim, nloc = dim + 1;
    const long long n = (long long)m->ncells * nloc;
    int32_t *cf = nullptr, *owner = nullptr;
    double *nrm = nullptr, *vol = nullptr;
    int8_t *sg = nullptr;
    int32_t nf = 0;
    int rc = grmp_alloc(ctx, (void **)&cf, (size_t)n * 4);
    if (!rc) rc = enumerate(m, face_kind(dim), cf, nullptr, &nf);
    if (!rc) rc = grmp_alloc(ctx, (void **)&owner, (size_t)nf * 4);
    if (!rc) rc = grmp_alloc(ctx, (void **)&nrm, (size_t)nf * dim * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&vol, (size_t)nf * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)&sg, (size_t)n);
    if (!rc) {
        cudaMemsetAsync(owner, 0x7f, (size_t)nf * 4, ctx->stream);   // 0x7f7f7f7f: above every cell id
        k_face_owner<<<nblk(n), TPB, 0, ctx->stream>>>(n, nloc, cf, owner);
        GRMP_LAUNCHED(ctx);
        k_face_geom<<<nblk(n), TPB, 0, ctx->stream>>>(n, dim, m->d_coords, m->d_cells, cf, owner, nrm, vol);
        GRMP_LAUNCHED(ctx);
        k_face_signs<<<nblk(n), TPB, 0, ctx->stream>>>(n, dim, m->d_coords, m->d_cells, cf, nrm, sg);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "mesh faces");
    }
    grmp_free(ctx, owner, (size_t)nf * 4);
    if (rc) {
        grmp_free(ctx, cf, (size_t)n * 4);
        grmp_free(ctx, nrm, (size_t)nf * dim * 8);
        grmp_free(ctx, vol, (size_t)nf * 8);
        grmp_free(ctx, sg, (size_t)n);
        return rc;
    }
    grmp_free(ctx, m->d_cell_faces, (size_t)n * 4);
    grmp_free(ctx, m->d_face_normals, (size_t)m->nfaces * dim * 8);
    grmp_free(ctx, m->d_face_volumes, (size_t)m->nfaces * 8);
    grmp_free(ctx, m->d_cell_face_signs, (size_t)n);
    grmp_free(ctx, m->d_cell_nbr, (size_t)n * 4);
    grmp_free(ctx, m->d_face_cells, (size_t)m->nfaces * 8);
    m->d_cell_nbr = m->d_face_cells = nullptr;
    m->nfaces = nf;
    m->d_cell_faces = cf;
    m->d_face_normals = nrm;
    m->d_face_volumes = vol;
    m->d_cell_face_signs = sg;
    return GRMP_OK;
}

int grmp_mesh_faces(grmp_mesh m, int32_t *nfaces, int32_t *cell_faces, double *face_normals, double *face_volumes,
                    int8_t *cell_face_signs) {
    if (!m || !nfaces) return GRMP_ERR_INVALID_ARG;
    grmp_context ctx = m->ctx;
    cudaSetDevice(ctx->device);
    *nfaces = m->nfaces;
    if (m->nfaces == 0) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "mesh faces: none set or built");
    const size_t nl = (size_t)m->ncells * (m->dim + 1);
    if (cell_faces) GRMP_CUDA(ctx, cudaMemcpyAsync(cell_faces, m->d_cell_faces, nl * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (face_normals)
        GRMP_CUDA(ctx, cudaMemcpyAsync(face_normals, m->d_face_normals, (size_t)m->nfaces * m->dim * 8,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    if (face_volumes)
        GRMP_CUDA(ctx, cudaMemcpyAsync(face_volumes, m->d_face_volumes, (size_t)m->nfaces * 8, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    if (cell_face_signs)
        GRMP_CUDA(ctx, cudaMemcpyAsync(cell_face_signs, m->d_cell_face_signs, nl, cudaMemcpyDeviceToHost, ctx->stream));
    GRMP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GRMP_OK;
}

int grmp_space_create_on_device(grmp_mesh mesh, int fe_kind, int ncomponents, grmp_space *out, int32_t *ndofs_out) {
    if (!mesh || !out) return GRMP_ERR_INVALID_ARG;
    *out = nullptr;
    grmp_context ctx = mesh->ctx;
    const int dim = mesh->dim;
    const bool br = fe_kind == GRMP_FE_H1BR && ncomponents == dim;
    if (!(br || ((fe_kind == GRMP_FE_H1P1 || fe_kind == GRMP_FE_H1P2) && ncomponents >= 1 && ncomponents <= 3)))
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED,
                         "device dofmap: H1P1 / H1P2 with 1-3 components or H1BR{dim} (got %d, %d)", fe_kind,
                         ncomponents);
    cudaSetDevice(ctx->device);
    if (br) {   // vertex DoFs per component, then one bubble per face (pattern "N1f1")
        int rc = mesh->nfaces ? GRMP_OK : grmp_mesh_build_faces(mesh);
        if (rc) return rc;
        const long long nd = (long long)dim * mesh->nverts + mesh->nfaces;
        if (nd >= (1LL << 31)) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "device dofmap: too many DoFs");
        grmp_space s = new (std::nothrow) grmp_space_s();
        if (!s) return GRMP_ERR_OUT_OF_MEMORY;
        s->mesh = mesh;
        s->fe = fe_kind;
        s->ncomp = ncomponents;
        s->ldofs = grmp_fe_ldofs(fe_kind, dim, ncomponents);
        s->nb = grmp_fe_nb(fe_kind, dim);
        s->ndofs = (int32_t)nd;
        rc = grmp_alloc(ctx, (void **)&s->d_celldofs, (size_t)mesh->ncells * s->ldofs * 4);
        if (!rc) {
            k_celldofs_br<<<nblk(mesh->ncells), TPB, 0, ctx->stream>>>(mesh->ncells, mesh->d_cells, dim, mesh->nverts,
                                                                        mesh->d_cell_faces, s->d_celldofs);
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
