// Bernardi-Raugel H1BR{2} velocity element with the RT0 reconstruction:
// drop-zero mask (reference operation order), fast assembly, reconstructed
// right-hand side and the cell divergences used by the iterated-penalty
// Stokes solver.
//
// Local DoFs of a triangle (src/fedefs/h1v_br.jl:33 pattern "N1f1"):
// 0-2 P1 component 1 at the nodes, 3-5 P1 component 2, 6-8 the face bubbles.
// Scalar basis (tables of grmp_tables, fe = H1BR): 0-2 the P1 functions,
// 3-5 the bubbles 6 x1 r, 6 x2 x1, 6 r x2 (:117-130).  Coefficients
// (:150-162): 1 for the P1 DoFs, the global unit normal n_F of face f for
// bubble f (both components).  RT0 reconstruction R (9 x 3,
// src/reconstructions.jl:381-403): R[3k+node][f] = (|F|/2) n_F[k] for the two
// nodes of face f = (f, f+1 mod 3), R[6+f][f] = |F|.
#include <cmath>

#include "element.cuh"
#include "grmp_internal.h"

int grmp_prepare_terms(grmp_space s, int nterms, const grmp_bilinear_term *terms, TermsDev *td,
                       std::vector<std::pair<void *, size_t>> &keep);
void grmp_release(grmp_context ctx, std::vector<std::pair<void *, size_t>> &keep);

namespace {

constexpr int TPB = 128;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

struct BrMeshDev {
    const double *coords;
    const int32_t *cells, *cell_faces;
    const double *fnormals, *fvolumes;
    const int8_t *signs;
};

struct BrTerm {
    int op;            // GRMP_OP_LAPLACE or GRMP_OP_RDIVRDIV
    int symmetric;
    double factor;
    const double *coef;  // per-cell coefficient or nullptr
};

struct BrTerms {
    int n;
    BrTerm t[GRMP_MAX_TERMS];
    // quadrature (order 2) and the scalar basis derivative table
    int nq;
    double w[4];
    double dref[4][6][2];
};

__device__ __forceinline__ void br_load_cell(const BrMeshDev &m, int cell, double X[6], double nrm[3][2],
                                             double fv[3], double sg[3]) {
    for (int v = 0; v < 3; v++)
        for (int k = 0; k < 2; k++) X[v * 2 + k] = m.coords[(size_t)m.cells[(size_t)cell * 3 + v] * 2 + k];
    for (int f = 0; f < 3; f++) {
        int F = m.cell_faces[(size_t)cell * 3 + f];
        nrm[f][0] = m.fnormals[(size_t)F * 2];
        nrm[f][1] = m.fnormals[(size_t)F * 2 + 1];
        fv[f] = m.fvolumes[F];
        sg[f] = (double)m.signs[(size_t)cell * 3 + f];
    }
}

// scalar basis index and component coefficient of local DoF `dof` for component c
__device__ __forceinline__ int br_scalar(int dof) { return dof < 3 ? dof : (dof < 6 ? dof - 3 : dof - 3); }
__device__ __forceinline__ double br_coef(int dof, int c, const double nrm[3][2]) {
    if (dof < 3) return c == 0 ? 1.0 : 0.0;
    if (dof < 6) return c == 1 ? 1.0 : 0.0;
    return nrm[dof - 6][c];
}

__device__ __forceinline__ void br_rt0(const double fv[3], const double nrm[3][2], double R[9][3], bool rn) {
    for (int i = 0; i < 9; i++)
        for (int f = 0; f < 3; f++) R[i][f] = 0.0;
    for (int f = 0; f < 3; f++) {
        const int nodes[2] = {f, (f + 1) % 3};
        for (int n = 0; n < 2; n++)
            for (int k = 0; k < 2; k++)
                R[3 * k + nodes[n]][f] = rn ? __dmul_rn(__dmul_rn(0.5, fv[f]), nrm[f][k]) : 0.5 * fv[f] * nrm[f][k];
        R[6 + f][f] = fv[f];
    }
}

// ------------------------------------------------------------------ mask (reference order)
__global__ void k_br_mask(int ncells, BrMeshDev m, BrTerms terms, uint32_t *mask) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[6], nrm[3][2], fv[3], sg[3];
    br_load_cell(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry_rn<2>(X, A, G, vol);
    const double det = __dsub_rn(__dmul_rn(A[0][0], A[1][1]), __dmul_rn(A[0][1], A[1][0]));
    uint32_t mk[9];
    for (int i = 0; i < 9; i++) mk[i] = 0;
    for (int ti = 0; ti < terms.n; ti++) {
        const BrTerm &t = terms.t[ti];
        if (t.op == GRMP_OP_LAPLACE) {
            // Gradient with coefficients, src/feevaluator_h1.jl:77-94
            double cv[4][9][4];
            for (int q = 0; q < terms.nq; q++)
                for (int dof = 0; dof < 9; dof++)
                    for (int c = 0; c < 2; c++)
                        for (int k = 0; k < 2; k++) {
                            const bool has = (dof < 3 && c == 0) || (dof >= 3 && dof < 6 && c == 1) || dof >= 6;
                            const int sidx = br_scalar(dof);
                            double s = 0.0;
                            for (int j = 0; j < 2; j++)
                                s = __dadd_rn(s, __dmul_rn(G[k][j], has ? terms.dref[q][sidx][j] : 0.0));
                            s = __dmul_rn(s, dof < 6 ? 1.0 : nrm[dof - 6][c]);
                            cv[q][dof][k + 2 * c] = s;
                        }
            const double coef = t.coef ? t.coef[cell] : 1.0;
            const double itemfactor = __dmul_rn(vol, t.coef ? 1.0 : t.factor);
            for (int i = 0; i < 9; i++)
                for (int j = t.symmetric ? i : 0; j < 9; j++) {
                    double loc = 0.0;
                    for (int q = 0; q < terms.nq; q++) {
                        double tt = 0.0;
                        for (int k = 0; k < 4; k++) {
                            const double res = t.coef ? __dmul_rn(coef, cv[q][i][k]) : cv[q][i][k];
                            tt = __dadd_rn(tt, __dmul_rn(res, cv[q][j][k]));
                        }
                        loc = __dadd_rn(loc, __dmul_rn(terms.w[q], tt));
                    }
                    if (__dmul_rn(loc, itemfactor) != 0.0) {
                        mk[i] |= 1u << j;
                        if (t.symmetric) mk[j] |= 1u << i;
                    }
                }
        } else {
            // ReconstructionDivergence, src/feevaluator_h1.jl:409-437
            double R[9][3];
            br_rt0(fv, nrm, R, true);
            double dv[9];
            for (int i = 0; i < 9; i++) {
                double s = 0.0;
                for (int j = 0; j < 3; j++)
                    if (R[i][j] != 0.0)
                        for (int jd = 0; jd < 2; jd++) s = __dadd_rn(s, __dmul_rn(__dmul_rn(R[i][j], 1.0), sg[j]));
                dv[i] = __ddiv_rn(s, det);
            }
            const double coef = t.coef ? t.coef[cell] : 1.0;
            const double itemfactor = __dmul_rn(vol, t.coef ? 1.0 : t.factor);
            for (int i = 0; i < 9; i++)
                for (int j = t.symmetric ? i : 0; j < 9; j++) {
                    double loc = 0.0;
                    for (int q = 0; q < terms.nq; q++) {
                        const double res = t.coef ? __dmul_rn(coef, dv[i]) : dv[i];
                        const double tt = __dadd_rn(0.0, __dmul_rn(res, dv[j]));
                        loc = __dadd_rn(loc, __dmul_rn(terms.w[q], tt));
                    }
                    if (__dmul_rn(loc, itemfactor) != 0.0) {
                        mk[i] |= 1u << j;
                        if (t.symmetric) mk[j] |= 1u << i;
                    }
                }
        }
    }
    for (int i = 0; i < 9; i++) mask[(size_t)cell * 9 + i] = mk[i];
}

// ------------------------------------------------------------------ fast assembly
// Per-cell factors (FP64, stored as T): [0..2]  scaled G^T G (Laplace), [3..8]
// face normals, [9] lambda*vol (divergence term), [10..18] div R phi_I.
constexpr int BR_NF = 19;

template <typename T>
__global__ void k_br_factors(int ncells, BrMeshDev m, BrTerms terms, T *fac) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[6], nrm[3][2], fv[3], sg[3];
    br_load_cell(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry<2, double>(X, G, vol, A);
    const double det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    double f[BR_NF];
    for (int i = 0; i < BR_NF; i++) f[i] = 0.0;
    for (int ti = 0; ti < terms.n; ti++) {
        const BrTerm &t = terms.t[ti];
        const double scale = vol * t.factor * (t.coef ? t.coef[cell] : 1.0);
        if (t.op == GRMP_OP_LAPLACE) {
            f[0] += scale * (G[0][0] * G[0][0] + G[1][0] * G[1][0]);
            f[1] += scale * (G[0][0] * G[0][1] + G[1][0] * G[1][1]);
            f[2] += scale * (G[0][1] * G[0][1] + G[1][1] * G[1][1]);
        } else {
            double R[9][3];
            br_rt0(fv, nrm, R, false);
            for (int i = 0; i < 9; i++) {
                double s = 0;
                for (int j = 0; j < 3; j++) s += R[i][j] * 2.0 * sg[j];
                f[10 + i] = s / det;
            }
            f[9] += scale;
        }
    }
    for (int fc = 0; fc < 3; fc++) {
        f[3 + 2 * fc] = nrm[fc][0];
        f[4 + 2 * fc] = nrm[fc][1];
    }
    T *out = fac + (size_t)cell * BR_NF;
    for (int i = 0; i < BR_NF; i++) out[i] = (T)f[i];
}

// S^{ps}_{ab} of the BR scalar basis (6x6, three p<=s pairs) in shared memory
template <typename T, typename S>
__global__ void __launch_bounds__(128) k_br_rows(int32_t nrows, const int32_t *__restrict__ inc_ptr,
                                                  const int32_t *__restrict__ inc_cell,
                                                  const uint8_t *__restrict__ inc_loc, const S *__restrict__ slot,
                                                  const int32_t *__restrict__ rowptr, const T *__restrict__ fac,
                                                  const T *__restrict__ gtens, T *__restrict__ vals) {
    __shared__ T tens[3 * 36];
    for (int i = threadIdx.x; i < 3 * 36; i += blockDim.x) tens[i] = gtens[i];
    __syncthreads();
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    T *rv = vals + rowptr[row];
    const int nnz = rowptr[row + 1] - rowptr[row];
    for (int k = 0; k < nnz; k++) rv[k] = T(0);
    const S DROP = (S)~(S)0;
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) {
        const int cell = inc_cell[p];
        const int I = inc_loc[p];
        const T *cf = fac + (size_t)cell * BR_NF;
        T f[BR_NF];
#pragma unroll
        for (int i = 0; i < BR_NF; i++) f[i] = cf[i];
        const S *sl = slot + (size_t)p * 9;
        const int sI = I < 3 ? I : I - 3;
        // coefficient vector of DoF I
        const T cI0 = I < 3 ? T(1) : (I < 6 ? T(0) : f[3 + 2 * (I - 6)]);
        const T cI1 = I < 3 ? T(0) : (I < 6 ? T(1) : f[4 + 2 * (I - 6)]);
#pragma unroll
        for (int J = 0; J < 9; J++) {
            const S s = sl[J];
            if (s == DROP) continue;
            const int sJ = J < 3 ? J : J - 3;
            const T cJ0 = J < 3 ? T(1) : (J < 6 ? T(0) : f[3 + 2 * (J - 6)]);
            const T cJ1 = J < 3 ? T(0) : (J < 6 ? T(1) : f[4 + 2 * (J - 6)]);
            const T cdot = cI0 * cJ0 + cI1 * cJ1;
            const int ab = sI * 6 + sJ;
            const T lap = f[0] * tens[ab] + f[1] * tens[36 + ab] + f[2] * tens[72 + ab];
            rv[s] += cdot * lap + f[9] * f[10 + I] * f[10 + J];
        }
    }
}

// ------------------------------------------------------------------ reconstructed rhs (FP64)
struct BrRhs {
    const double *par;     // [ngroups][nt][5] polynomial terms (component, coef, e1, e2, e3)
    int nt;                // terms per group
    const int32_t *group;  // [ncells] group of each cell (nullptr: one group)
    double factor;
    int nq;
    double xref[64][2];
    double w[64];
};

// loc[cell][I] = factor*vol * sum_q w_q f(x_q) . (R Piola RT0)_I (x_q)
// (src/feevaluator_h1.jl:342-381; src/assemblypatterns/linearform.jl:181-220)
// BR -> BDM1 reconstruction coefficients (src/reconstructions.jl:351-379):
// column 2f = RT0 function of face f, 2f+1 = its linear-moment BDM1 function.
__device__ __forceinline__ void br_bdm1(const double fv[3], const double nrm[3][2], const double sg[3], double R[9][6]) {
    const double c[2] = {-1.0 / 12.0, 1.0 / 12.0};
    for (int i = 0; i < 9; i++)
        for (int j = 0; j < 6; j++) R[i][j] = 0.0;
    for (int f = 0; f < 3; f++) {
        const int nodes[2] = {f, (f + 1) % 3};
        for (int n = 0; n < 2; n++)
            for (int k = 0; k < 2; k++) {
                R[3 * k + nodes[n]][2 * f] = 0.5 * fv[f] * nrm[f][k];
                R[3 * k + nodes[n]][2 * f + 1] = c[n] * fv[f] * nrm[f][k] * sg[f];
            }
        R[6 + f][2 * f] = fv[f];
    }
}

// b += factor (f, R v) with R = BR -> RT0 (NR = 3) or BR -> BDM1 (NR = 6):
// ReconstructionIdentity (src/feevaluator_h1.jl:342-381) with the Piola
// transform of the H(div) basis (RT0: src/fedefs/hdiv_rt0.jl:67-116,
// BDM1: src/fedefs/hdiv_bdm1.jl:81-92, 160-172; cell-face signs on the RT0
// functions only).
template <int NR>
__global__ void k_br_rhs_cells(int ncells, BrMeshDev m, BrRhs r, double *loc) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[6], nrm[3][2], fv[3], sg[3];
    br_load_cell(m, cell, X, nrm, fv, sg);
    double A[2][2];
    for (int k = 0; k < 2; k++)
        for (int j = 0; j < 2; j++) A[k][j] = X[(j + 1) * 2 + k] - X[k];
    const double det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    const double vol = fabs(det) / 2.0;
    double R[9][NR];
    if constexpr (NR == 3) {
        br_rt0(fv, nrm, R, false);
    } else {
        br_bdm1(fv, nrm, sg, R);
    }
    const double *par = r.par + (size_t)(r.group ? r.group[cell] : 0) * r.nt * 5;
    double lb[9];
    for (int i = 0; i < 9; i++) lb[i] = 0;
    for (int q = 0; q < r.nq; q++) {
        const double xi = r.xref[q][0], eta = r.xref[q][1];
        double rt[NR][2], cf[NR];
        if constexpr (NR == 3) {
            rt[0][0] = xi, rt[0][1] = eta - 1;
            rt[1][0] = xi, rt[1][1] = eta;
            rt[2][0] = xi - 1, rt[2][1] = eta;
            for (int j = 0; j < NR; j++) cf[j] = sg[j];
        } else {
            rt[0][0] = xi, rt[0][1] = eta - 1;
            rt[1][0] = 6 * xi, rt[1][1] = 6 - 12 * xi - 6 * eta;
            rt[2][0] = xi, rt[2][1] = eta;
            rt[3][0] = -6 * xi, rt[3][1] = 6 * eta;
            rt[4][0] = xi - 1, rt[4][1] = eta;
            rt[5][0] = 6 * (xi - 1) + 12 * eta, rt[5][1] = -6 * eta;
            for (int j = 0; j < NR; j++) cf[j] = (j % 2 == 0) ? sg[j / 2] : 1.0;   // signs on RT0 only
        }
        double te[NR][2];
        for (int j = 0; j < NR; j++)
            for (int k = 0; k < 2; k++) te[j][k] = (A[k][0] * rt[j][0] + A[k][1] * rt[j][1]) * (cf[j] / det);
        double x[2];
        for (int k = 0; k < 2; k++) x[k] = X[k] + A[k][0] * xi + A[k][1] * eta;
        double f[2] = {0, 0};
        for (int t = 0; t < r.nt; t++) {
            const int c = (int)par[5 * t];
            double v = par[5 * t + 1];
            if (par[5 * t + 2] != 0) v *= poly_pow(x[0], par[5 * t + 2]);
            if (par[5 * t + 3] != 0) v *= poly_pow(x[1], par[5 * t + 3]);
            f[c] += v;
        }
        for (int i = 0; i < 9; i++) {
            double cv0 = 0, cv1 = 0;
            for (int j = 0; j < NR; j++) {
                cv0 += R[i][j] * te[j][0];
                cv1 += R[i][j] * te[j][1];
            }
            lb[i] += (f[0] * cv0 + f[1] * cv1) * r.w[q];
        }
    }
    const double itemfactor = r.factor * vol;
    for (int i = 0; i < 9; i++) loc[(size_t)cell * 9 + i] = lb[i] * itemfactor;
}

__global__ void k_gather_rows_br(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell,
                                 const uint8_t *inc_loc, const double *loc, double *b) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    double acc = b[row];
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) acc += loc[(size_t)inc_cell[p] * 9 + inc_loc[p]];
    b[row] = acc;
}

// Dv[cell][I] = int_T div phi_I (Divergence with coefficients,
// src/feevaluator_h1.jl:133-145; the gradient of every BR function is at
// most linear, so the midpoint value times |T| is exact); vol[cell] = |T|.
__global__ void k_br_div(int ncells, BrMeshDev m, BrTerms terms, double *Dv, double *vol_out) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[6], nrm[3][2], fv[3], sg[3];
    br_load_cell(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry<2, double>(X, G, vol, A);
    // gradients of the scalar basis at the midpoint (1/3, 1/3)
    const double l = 1.0 / 3.0;
    const double dref[6][2] = {{-1, -1}, {1, 0}, {0, 1},
                               {6 * (1 - 2 * l - l), -6 * l}, {6 * l, 6 * l}, {-6 * l, 6 * (1 - l - 2 * l)}};
    for (int I = 0; I < 9; I++) {
        const int s = I < 3 ? I : I - 3;
        double d = 0;
        for (int c = 0; c < 2; c++) {
            const double coef = br_coef(I, c, nrm);
            if (coef == 0.0) continue;
            for (int j = 0; j < 2; j++) d += G[c][j] * dref[s][j] * coef;
        }
        Dv[(size_t)cell * 9 + I] = d * vol;
    }
    vol_out[cell] = vol;
}

int br_terms(grmp_space s, int nterms, const grmp_bilinear_term *terms, BrTerms *bt,
             std::vector<std::pair<void *, size_t>> &keep) {
    grmp_context ctx = s->mesh->ctx;
    std::memset(bt, 0, sizeof(*bt));
    bt->n = nterms;
    for (int i = 0; i < nterms; i++) {
        const grmp_bilinear_term &t = terms[i];
        if (t.op_kind != GRMP_OP_LAPLACE && t.op_kind != GRMP_OP_RDIVRDIV)
            return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR: only Laplace and reconstruction-divergence terms");
        if (t.bonus_quadorder != 0) return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR: bonus_quadorder must be 0");
        bt->t[i].op = t.op_kind;
        bt->t[i].symmetric = t.symmetric ? 1 : 0;
        bt->t[i].factor = t.factor;
        bt->t[i].coef = nullptr;
        if (t.cell_coef) {
            if (t.coef_on_device) {
                bt->t[i].coef = t.cell_coef;
            } else {
                double *dc = nullptr;
                int rc = grmp_upload(ctx, &dc, t.cell_coef, (size_t)s->mesh->ncells);
                if (rc) return rc;
                keep.push_back({dc, (size_t)s->mesh->ncells * 8});
                bt->t[i].coef = dc;
            }
        }
    }
    RefTables *rt = new RefTables;
    int rc = grmp_tables(2, GRMP_FE_H1BR, 2, rt);   // polyorder 2 - derivative 1, twice
    if (rc || rt->nq > 4) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR tables");
    }
    bt->nq = rt->nq;
    for (int q = 0; q < rt->nq; q++) {
        bt->w[q] = rt->w[q];
        for (int a = 0; a < 6; a++)
            for (int j = 0; j < 2; j++) bt->dref[q][a][j] = rt->derivs[q][a][j];
    }
    delete rt;
    return GRMP_OK;
}

BrMeshDev br_mesh(grmp_mesh m) {
    return BrMeshDev{m->d_coords, m->d_cells, m->d_cell_faces, m->d_face_normals, m->d_face_volumes,
                     m->d_cell_face_signs};
}

template <typename T>
int br_assemble_t(grmp_matrix A, const BrTerms &bt) {
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    // S^{ps} tensors of the scalar basis from the order-2 rule
    std::vector<T> tens(3 * 36);
    for (int pair = 0, p = 0; p < 2; p++)
        for (int q2 = p; q2 < 2; q2++, pair++)
            for (int a = 0; a < 6; a++)
                for (int b = 0; b < 6; b++) {
                    double acc = 0;
                    for (int q = 0; q < bt.nq; q++) {
                        acc += bt.w[q] * bt.dref[q][a][p] * bt.dref[q][b][q2];
                        if (p != q2) acc += bt.w[q] * bt.dref[q][a][q2] * bt.dref[q][b][p];
                    }
                    tens[pair * 36 + a * 6 + b] = (T)acc;
                }
    T *dtens = nullptr;
    int rc = grmp_upload(ctx, &dtens, tens.data(), tens.size());
    if (rc) return rc;
    size_t fbytes = (size_t)m->ncells * BR_NF * sizeof(T);
    if (A->cellfac_bytes < fbytes) {
        grmp_free(ctx, A->d_cellfac, A->cellfac_bytes);
        A->cellfac_bytes = 0;
        rc = grmp_alloc(ctx, &A->d_cellfac, fbytes);
        if (rc) {
            grmp_free(ctx, dtens, tens.size() * sizeof(T));
            return rc;
        }
        A->cellfac_bytes = fbytes;
    }
    T *fac = (T *)A->d_cellfac;
    k_br_factors<T><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br_mesh(m), bt, fac);
    GRMP_LAUNCHED(ctx);
    T **vals = sizeof(T) == 8 ? (T **)&A->d_vals64 : (T **)&A->d_vals32;
    if (!*vals) {
        rc = grmp_alloc(ctx, (void **)vals, (size_t)A->nnz * sizeof(T));
        if (rc) {
            grmp_free(ctx, dtens, tens.size() * sizeof(T));
            return rc;
        }
    }
    if (A->slot_bytes == 1)
        k_br_rows<T, uint8_t><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell,
                                                                     s->d_inc_loc, (const uint8_t *)A->d_slot,
                                                                     A->d_rowptr, fac, dtens, *vals);
    else
        k_br_rows<T, uint16_t><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell,
                                                                      s->d_inc_loc, (const uint16_t *)A->d_slot,
                                                                      A->d_rowptr, fac, dtens, *vals);
    GRMP_LAUNCHED(ctx);
    cudaError_t e = cudaGetLastError();
    grmp_free(ctx, dtens, tens.size() * sizeof(T));
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "H1BR assembly");
    if (sizeof(T) == 8) A->has64 = true; else A->has32 = true;
    return GRMP_OK;
}

}  // namespace

// ---------------------------------------------------------------------- entry points used by pattern/assemble
int grmp_br3_mask(grmp_space s, int nterms, const grmp_bilinear_term *terms, uint32_t *mask);
int grmp_br3_assemble(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision);
int grmp_br3_rhs(grmp_space s, const grmp_rhs *rhs, grmp_vector b);
int grmp_br3_divergence(grmp_space s, double **Dv, double **vol);

int grmp_br_mask(grmp_space s, int nterms, const grmp_bilinear_term *terms, uint32_t *mask) {
    if (s->mesh->dim == 3) return grmp_br3_mask(s, nterms, terms, mask);
    grmp_context ctx = s->mesh->ctx;
    BrTerms bt;
    std::vector<std::pair<void *, size_t>> keep;
    int rc = br_terms(s, nterms, terms, &bt, keep);
    if (!rc) {
        k_br_mask<<<nblk(s->mesh->ncells, 64), 64, 0, ctx->stream>>>(s->mesh->ncells, br_mesh(s->mesh), bt, mask);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "H1BR mask");
    }
    grmp_release(ctx, keep);
    return rc;
}

int grmp_br_assemble(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision) {
    if (A->space->mesh->dim == 3) return grmp_br3_assemble(A, nterms, terms, precision);
    grmp_context ctx = A->space->mesh->ctx;
    BrTerms bt;
    std::vector<std::pair<void *, size_t>> keep;
    int rc = br_terms(A->space, nterms, terms, &bt, keep);
    if (!rc) rc = precision == GRMP_FP64 ? br_assemble_t<double>(A, bt) : br_assemble_t<float>(A, bt);
    cudaStreamSynchronize(ctx->stream);
    grmp_release(ctx, keep);
    return rc;
}

// b += (f, R v) with f polynomial (optionally one polynomial per cell group)
int grmp_br_rhs(grmp_space s, const grmp_rhs *rhs, grmp_vector b) {
    if (s->mesh->dim == 3) return grmp_br3_rhs(s, rhs, b);
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    if (rhs->kind != GRMP_RHS_POLY || rhs->ncomponents != 2)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR reconstructed rhs: 2-component polynomial data only");
    long long ng = rhs->cell_group ? rhs->ngroups : 1;
    if (ng <= 0 || rhs->nparams % (5 * ng)) return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: parameter layout");
    int nt = (int)(rhs->nparams / (5 * ng));
    for (long long t = 0; t < ng * nt; t++)
        if (rhs->params[5 * t] < 0 || rhs->params[5 * t] > 1)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: polynomial component out of range");
    if (rhs->cell_group)
        for (int c = 0; c < m->ncells; c++)
            if (rhs->cell_group[c] < 0 || rhs->cell_group[c] >= ng)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: cell group out of range");
    BrRhs r;
    std::memset(&r, 0, sizeof(r));
    RefTables *rt = new RefTables;
    int rc = grmp_tables(2, GRMP_FE_H1BR, 2 + rhs->bonus_quadorder, rt);
    if (rc || rt->nq > 64) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no rule of order %d", 2 + rhs->bonus_quadorder);
    }
    r.nq = rt->nq;
    for (int q = 0; q < rt->nq; q++) {
        r.xref[q][0] = rt->xref[q][0];
        r.xref[q][1] = rt->xref[q][1];
        r.w[q] = rt->w[q];
    }
    delete rt;
    r.nt = nt;
    r.factor = rhs->factor;
    double *dpar = nullptr;
    int32_t *dgrp = nullptr;
    rc = grmp_upload(ctx, &dpar, rhs->params, (size_t)rhs->nparams);
    if (!rc && rhs->cell_group) rc = grmp_upload(ctx, &dgrp, rhs->cell_group, (size_t)m->ncells);
    size_t ncl = (size_t)m->ncells * 9;
    if (!rc && !s->d_locbuf) rc = grmp_alloc(ctx, (void **)&s->d_locbuf, ncl * 8);
    if (!rc) {
        r.par = dpar;
        r.group = dgrp;
        if (rhs->test_operator == 2)
            k_br_rhs_cells<6><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br_mesh(m), r, s->d_locbuf);
        else
            k_br_rhs_cells<3><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br_mesh(m), r, s->d_locbuf);
        GRMP_LAUNCHED(ctx);
        k_gather_rows_br<<<nblk(s->ndofs), TPB, 0, ctx->stream>>>(s->ndofs, s->d_inc_ptr, s->d_inc_cell,
                                                                  s->d_inc_loc, s->d_locbuf, b->d);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "H1BR rhs");
    }
    grmp_free(ctx, dpar, (size_t)rhs->nparams * 8);
    grmp_free(ctx, dgrp, (size_t)m->ncells * 4);
    return rc;
}

// cell divergence table Dv [ncells][ldofs] and cell volumes, allocated here
int grmp_br_divergence(grmp_space s, double **Dv, double **vol) {
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    if (m->dim == 3) return grmp_br3_divergence(s, Dv, vol);
    int rc = grmp_alloc(ctx, (void **)Dv, (size_t)m->ncells * 9 * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)vol, (size_t)m->ncells * 8);
    if (rc) return rc;
    BrTerms bt;
    std::memset(&bt, 0, sizeof(bt));
    k_br_div<<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br_mesh(m), bt, *Dv, *vol);
    GRMP_LAUNCHED(ctx);
    GRMP_CUDA(ctx, cudaGetLastError());
    return GRMP_OK;
}
