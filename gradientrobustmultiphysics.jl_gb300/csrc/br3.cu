// Bernardi-Raugel H1BR{3} velocity element on tetrahedra with the RT0 and
// BDM1 reconstructions: drop-zero mask (reference operation order), fast
// assembly of nu (grad u, grad v) + lambda (div R u, div R v) (the same for
// both reconstructions: the BDM1 functions beyond RT0 carry no flux, so the
// divergence is the RT0 one), and the reconstructed right-hand side
// (f, R v).
//
// Local DoFs of a tetrahedron (src/fedefs/h1v_br.jl:33 pattern "N1f1"):
// 0-11 the P1 functions, component-major (4 c + node), 12-15 the face
// bubbles of the faces [0,1,2], [0,1,3], [1,2,3], [0,2,3] (scalar basis 4-7,
// 60 x r y, 60 r x z, 60 x y z, 60 r y z with r = 1 - x - y - z, :221-233),
// each times the global unit normal n_F[c] in component c (:241-262).  RT0
// reconstruction R (16 x 4, src/reconstructions.jl:474-491):
// R[4k + node][f] = (|F|/3) n_F[k] for the three nodes of face f,
// R[12 + f][f] = |F|.  HDIVRT0{3} reference basis 2(x, y, z-1),
// 2(x, y-1, z), 2(x, y, z), 2(x-1, y, z) (src/fedefs/hdiv_rt0.jl:93-100),
// mapped by the Piola transform A phi / |det A| with the cell-face signs:
// the tetrahedra of a mesh may have either orientation, and dividing by
// |det A| makes the reconstruction's flux through every face the cell-face
// sign times the face moment whatever the orientation (the reconstructed
// divergence is then the cell mean of div u, which the iterated penalty
// needs).
#include <cmath>

#include "element.cuh"
#include "grmp_internal.h"

void grmp_release(grmp_context ctx, std::vector<std::pair<void *, size_t>> &keep);

namespace {

constexpr int TPB = 128;
inline int nblk(long long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

constexpr int kMaxQ3 = 11;   // the order-4 tetrahedral rule
__constant__ int kFaces3[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};

struct Br3MeshDev {
    const double *coords;
    const int32_t *cells, *cell_faces;
    const double *fnormals, *fvolumes;
    const int8_t *signs;
};

struct Br3Term {
    int op;              // GRMP_OP_LAPLACE or GRMP_OP_RDIVRDIV
    int symmetric;
    double factor;
    const double *coef;  // per-cell coefficient or nullptr
};

struct Br3Terms {
    int n;
    Br3Term t[GRMP_MAX_TERMS];
    int nq;                      // order-4 rule (both terms)
    double w[kMaxQ3];
    double dref[kMaxQ3][8][3];   // scalar basis derivatives
};

__device__ __forceinline__ void br3_load(const Br3MeshDev &m, int cell, double X[12], double nrm[4][3], double fv[4],
                                         double sg[4]) {
    for (int v = 0; v < 4; v++)
        for (int k = 0; k < 3; k++) X[v * 3 + k] = m.coords[(size_t)m.cells[(size_t)cell * 4 + v] * 3 + k];
    for (int f = 0; f < 4; f++) {
        const int F = m.cell_faces[(size_t)cell * 4 + f];
        for (int k = 0; k < 3; k++) nrm[f][k] = m.fnormals[(size_t)F * 3 + k];
        fv[f] = m.fvolumes[F];
        sg[f] = (double)m.signs[(size_t)cell * 4 + f];
    }
}

// det A with the operation order of the host restatement (cofactor expansion)
__device__ __forceinline__ double det3_rn(const double A[3][3]) {
    const double c00 = __dsub_rn(__dmul_rn(A[1][1], A[2][2]), __dmul_rn(A[1][2], A[2][1]));
    const double c01 = __dsub_rn(__dmul_rn(A[1][2], A[2][0]), __dmul_rn(A[1][0], A[2][2]));
    const double c02 = __dsub_rn(__dmul_rn(A[1][0], A[2][1]), __dmul_rn(A[1][1], A[2][0]));
    return __dadd_rn(__dadd_rn(__dmul_rn(A[0][0], c00), __dmul_rn(A[0][1], c01)), __dmul_rn(A[0][2], c02));
}

// scalar basis index of local DoF `dof` in component c (-1: none)
__device__ __forceinline__ int br3_scalar(int dof, int c) {
    if (dof < 12) return (dof / 4 == c) ? dof % 4 : -1;
    return 4 + (dof - 12);
}
__device__ __forceinline__ double br3_coef(int dof, int c, const double nrm[4][3]) {
    return dof < 12 ? 1.0 : nrm[dof - 12][c];
}

__device__ __forceinline__ void br3_rt0(const double fv[4], const double nrm[4][3], double R[16][4], bool rn) {
    for (int i = 0; i < 16; i++)
        for (int f = 0; f < 4; f++) R[i][f] = 0.0;
    for (int f = 0; f < 4; f++) {
        for (int n = 0; n < 3; n++)
            for (int k = 0; k < 3; k++)
                R[4 * k + kFaces3[f][n]][f] = rn ? __dmul_rn(__dmul_rn(1.0 / 3.0, fv[f]), nrm[f][k])
                                                 : (1.0 / 3.0) * fv[f] * nrm[f][k];
        R[12 + f][f] = fv[f];
    }
}

// ------------------------------------------------------------------ mask (reference order)
__global__ void k_br3_mask(int ncells, Br3MeshDev m, Br3Terms terms, uint32_t *mask) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[12], nrm[4][3], fv[4], sg[4];
    br3_load(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry_rn<3>(X, A, G, vol);
    uint32_t mk[16];
    for (int i = 0; i < 16; i++) mk[i] = 0;
    for (int ti = 0; ti < terms.n; ti++) {
        const Br3Term &t = terms.t[ti];
        const double coef = t.coef ? t.coef[cell] : 1.0;
        const double itemfactor = __dmul_rn(vol, t.coef ? 1.0 : t.factor);
        if (t.op == GRMP_OP_LAPLACE) {
            // Gradient with coefficients, src/feevaluator_h1.jl:77-94: loc[i][j] = sum_q w_q
            // sum_k res_i,k cv_j,k with cv[dof][k + 3c] = (sum_j G[k][j] dphi_j) * coef
            double loc[16][16];
            for (int i = 0; i < 16; i++)
                for (int j = 0; j < 16; j++) loc[i][j] = 0.0;
            for (int q = 0; q < terms.nq; q++) {
                double cv[16][9];
                for (int dof = 0; dof < 16; dof++)
                    for (int c = 0; c < 3; c++)
                        for (int k = 0; k < 3; k++) {
                            const int si = br3_scalar(dof, c);
                            double a = 0.0;
                            for (int jj = 0; jj < 3; jj++)
                                a = __dadd_rn(a, __dmul_rn(G[k][jj], si >= 0 ? terms.dref[q][si][jj] : 0.0));
                            cv[dof][k + 3 * c] = __dmul_rn(a, br3_coef(dof, c, nrm));
                        }
                for (int i = 0; i < 16; i++)
                    for (int j = t.symmetric ? i : 0; j < 16; j++) {
                        double tt = 0.0;
                        for (int kk = 0; kk < 9; kk++) {
                            const double res = t.coef ? __dmul_rn(coef, cv[i][kk]) : cv[i][kk];
                            tt = __dadd_rn(tt, __dmul_rn(res, cv[j][kk]));
                        }
                        loc[i][j] = __dadd_rn(loc[i][j], __dmul_rn(terms.w[q], tt));
                    }
            }
            for (int i = 0; i < 16; i++)
                for (int j = t.symmetric ? i : 0; j < 16; j++)
                    if (__dmul_rn(loc[i][j], itemfactor) != 0.0) {
                        mk[i] |= 1u << j;
                        if (t.symmetric) mk[j] |= 1u << i;
                    }
        } else {
            // ReconstructionDivergence, src/feevaluator_h1.jl:409-437 (dphi_hat = 2 per direction)
            double R[16][4];
            br3_rt0(fv, nrm, R, true);
            const double adet = fabs(det3_rn(A));
            double dv[16];
            for (int i = 0; i < 16; i++) {
                double s = 0.0;
                for (int j = 0; j < 4; j++)
                    if (R[i][j] != 0.0)
                        for (int jd = 0; jd < 3; jd++) s = __dadd_rn(s, __dmul_rn(__dmul_rn(R[i][j], 2.0), sg[j]));
                dv[i] = __ddiv_rn(s, adet);
            }
            for (int i = 0; i < 16; i++)
                for (int j = t.symmetric ? i : 0; j < 16; j++) {
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
    for (int i = 0; i < 16; i++) mask[(size_t)cell * 16 + i] = mk[i];
}

// ------------------------------------------------------------------ fast assembly
// Per-cell factors (FP64, stored as T): [0..5] scaled G^T G (p <= s pairs),
// [6..17] face normals, [18] lambda*vol, [19..34] div R phi_I.
constexpr int BR3_NF = 35;

template <typename T>
__global__ void k_br3_factors(int ncells, Br3MeshDev m, Br3Terms terms, T *fac) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[12], nrm[4][3], fv[4], sg[4];
    br3_load(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry<3, double>(X, G, vol, A);
    const double adet = 6.0 * vol;
    double f[BR3_NF];
    for (int i = 0; i < BR3_NF; i++) f[i] = 0.0;
    for (int ti = 0; ti < terms.n; ti++) {
        const Br3Term &t = terms.t[ti];
        const double scale = vol * t.factor * (t.coef ? t.coef[cell] : 1.0);
        if (t.op == GRMP_OP_LAPLACE) {
            int pr = 0;
            for (int p = 0; p < 3; p++)
                for (int s = p; s < 3; s++, pr++) {
                    double g = 0;
                    for (int k = 0; k < 3; k++) g += G[k][p] * G[k][s];
                    f[pr] += scale * g;
                }
        } else {
            double R[16][4];
            br3_rt0(fv, nrm, R, false);
            for (int i = 0; i < 16; i++) {
                double s = 0;
                for (int j = 0; j < 4; j++) s += R[i][j] * 6.0 * sg[j];
                f[19 + i] = s / adet;
            }
            f[18] += scale;
        }
    }
    for (int fc = 0; fc < 4; fc++)
        for (int k = 0; k < 3; k++) f[6 + 3 * fc + k] = nrm[fc][k];
    T *out = fac + (size_t)cell * BR3_NF;
    for (int i = 0; i < BR3_NF; i++) out[i] = (T)f[i];
}

// S^{ps}_{ab} of the BR3 scalar basis (8 x 8, six p <= s pairs) in shared
// memory; one thread per row walks the row's incident cells in ascending order
template <typename T, typename S>
__global__ void __launch_bounds__(128) k_br3_rows(int32_t nrows, const int32_t *__restrict__ inc_ptr,
                                                   const int32_t *__restrict__ inc_cell,
                                                   const uint8_t *__restrict__ inc_loc, const S *__restrict__ slot,
                                                   const int32_t *__restrict__ rowptr, const T *__restrict__ fac,
                                                   const T *__restrict__ gtens, T *__restrict__ vals) {
    __shared__ T tens[6 * 64];
    for (int i = threadIdx.x; i < 6 * 64; i += blockDim.x) tens[i] = gtens[i];
    __syncthreads();
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    T *rv = vals + rowptr[row];
    const int nnz = rowptr[row + 1] - rowptr[row];
    for (int k = 0; k < nnz; k++) rv[k] = T(0);
    const S DROP = (S)~(S)0;
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) {
        const int cell = inc_cell[p];
        const int I = inc_loc[p];
        const T *cf = fac + (size_t)cell * BR3_NF;
        T f[BR3_NF];
#pragma unroll
        for (int i = 0; i < BR3_NF; i++) f[i] = cf[i];
        const S *sl = slot + (size_t)p * 16;
        const int sI = I < 12 ? I % 4 : I - 8;
        T cI[3];
#pragma unroll
        for (int c = 0; c < 3; c++) cI[c] = I < 12 ? (I / 4 == c ? T(1) : T(0)) : f[6 + 3 * (I - 12) + c];
#pragma unroll
        for (int J = 0; J < 16; J++) {
            const S s = sl[J];
            if (s == DROP) continue;
            const int sJ = J < 12 ? J % 4 : J - 8;
            T cdot = T(0);
#pragma unroll
            for (int c = 0; c < 3; c++) cdot += cI[c] * (J < 12 ? (J / 4 == c ? T(1) : T(0)) : f[6 + 3 * (J - 12) + c]);
            const int ab = sI * 8 + sJ;
            T lap = T(0);
#pragma unroll
            for (int pr = 0; pr < 6; pr++) lap += f[pr] * tens[pr * 64 + ab];
            rv[s] += cdot * lap + f[18] * f[19 + I] * f[19 + J];
        }
    }
}

// ------------------------------------------------------------------ reconstructed rhs (FP64)
// BR -> BDM1 reconstruction (src/reconstructions.jl:493-535): R phi is the
// linear vector field whose normal-flux moments against P1 on every face
// equal those of phi (the functionals the reference's coefficients
// _P1_INTO_BDM1_COEFFS_3D encode; its orientation-dependent choice of two
// linear moments per face only selects a basis of the same space).  On face
// f with vertices V and moments m_a = int_F (phi . n_F) lambda_a, the
// field's normal components at the face's vertices are
// s_a = (12 / |F|) (m_a - (m_0 + m_1 + m_2) / 4); its value at vertex i
// solves n_F . w_i = s over the three faces at i.  W[dof][vertex][component].
__device__ void br3_bdm1_fields(const double fv[4], const double nrm[4][3], double W[16][4][3]) {
    for (int dof = 0; dof < 16; dof++) {
        double s[4][3];
        for (int f = 0; f < 4; f++) {
            double m[3] = {0.0, 0.0, 0.0};
            for (int a = 0; a < 3; a++) {
                const int va = kFaces3[f][a];
                if (dof < 12) {
                    const int k = dof / 4, p = dof % 4;
                    const bool on = kFaces3[f][0] == p || kFaces3[f][1] == p || kFaces3[f][2] == p;
                    if (on) m[a] = nrm[f][k] * fv[f] * (va == p ? 2.0 : 1.0) / 12.0;
                } else if (dof - 12 == f) {
                    m[a] = (nrm[f][0] * nrm[f][0] + nrm[f][1] * nrm[f][1] + nrm[f][2] * nrm[f][2]) * fv[f] / 3.0;
                }
            }
            const double mean = (m[0] + m[1] + m[2]) / 4.0;
            for (int a = 0; a < 3; a++) s[f][a] = (12.0 / fv[f]) * (m[a] - mean);
        }
        for (int i = 0; i < 4; i++) {
            double N[3][3], r[3];
            int row = 0;
            for (int f = 0; f < 4; f++)
                for (int a = 0; a < 3; a++)
                    if (kFaces3[f][a] == i) {
                        for (int k = 0; k < 3; k++) N[row][k] = nrm[f][k];
                        r[row++] = s[f][a];
                    }
            const double det = N[0][0] * (N[1][1] * N[2][2] - N[1][2] * N[2][1]) -
                               N[0][1] * (N[1][0] * N[2][2] - N[1][2] * N[2][0]) +
                               N[0][2] * (N[1][0] * N[2][1] - N[1][1] * N[2][0]);
            for (int c = 0; c < 3; c++) {   // Cramer's rule
                double M[3][3];
                for (int x = 0; x < 3; x++)
                    for (int y = 0; y < 3; y++) M[x][y] = (y == c) ? r[x] : N[x][y];
                W[dof][i][c] = (M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                                M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                                M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0])) /
                               det;
            }
        }
    }
}

struct Br3Rhs {
    const double *par;   // [ngroups][nt][5] polynomial terms (component, coef, e1, e2, e3)
    const int32_t *group;   // [ncells] group of each cell, or nullptr (one group)
    int nt;
    double factor;
    int bdm1;            // 0: RT0 reconstruction, 1: BDM1
    int nq;
    double xref[64][3];
    double w[64];
};

// loc[cell][I] = factor*vol * sum_q w_q f(x_q) . (R Piola RT0)_I (x_q)
// (ReconstructionIdentity, src/feevaluator_h1.jl:342-381)
__global__ void k_br3_rhs_cells(int ncells, Br3MeshDev m, Br3Rhs r, double *loc) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[12], nrm[4][3], fv[4], sg[4];
    br3_load(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry<3, double>(X, G, vol, A);
    const double adet = 6.0 * vol;
    double R[16][4];
    br3_rt0(fv, nrm, R, false);
    double lb[16];
    for (int i = 0; i < 16; i++) lb[i] = 0.0;
    if (r.bdm1) {
        double W[16][4][3];
        br3_bdm1_fields(fv, nrm, W);
        for (int q = 0; q < r.nq; q++) {
            const double lam[4] = {1.0 - r.xref[q][0] - r.xref[q][1] - r.xref[q][2], r.xref[q][0], r.xref[q][1],
                                   r.xref[q][2]};
            double x[3];
            for (int k = 0; k < 3; k++) {
                x[k] = X[k];
                for (int j = 0; j < 3; j++) x[k] += A[k][j] * r.xref[q][j];
            }
            double fq[3] = {0, 0, 0};
            const double *gpar = r.par + (r.group ? (size_t)r.group[cell] * r.nt * 5 : 0);
            for (int t = 0; t < r.nt; t++) {
                const double *pt = gpar + 5 * t;
                double v = pt[1];
                for (int j = 0; j < 3; j++)
                    if (pt[2 + j] != 0) v *= poly_pow(x[j], pt[2 + j]);
                fq[(int)pt[0]] += v;
            }
            for (int i = 0; i < 16; i++) {
                double t = 0;
                for (int k = 0; k < 3; k++)
                    t += fq[k] * (lam[0] * W[i][0][k] + lam[1] * W[i][1][k] + lam[2] * W[i][2][k] +
                                  lam[3] * W[i][3][k]);
                lb[i] += t * r.w[q];
            }
        }
        const double itemfactor = r.factor * vol;
        for (int i = 0; i < 16; i++) loc[(size_t)cell * 16 + i] = lb[i] * itemfactor;
        return;
    }
    for (int q = 0; q < r.nq; q++) {
        const double x0 = r.xref[q][0], y0 = r.xref[q][1], z0 = r.xref[q][2];
        const double rt[4][3] = {{2 * x0, 2 * y0, 2 * (z0 - 1)}, {2 * x0, 2 * (y0 - 1), 2 * z0},
                                 {2 * x0, 2 * y0, 2 * z0}, {2 * (x0 - 1), 2 * y0, 2 * z0}};
        double te[4][3];
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 3; k++) {
                double s = 0;
                for (int l = 0; l < 3; l++) s += A[k][l] * rt[j][l];
                te[j][k] = s * (sg[j] / adet);
            }
        double x[3];
        for (int k = 0; k < 3; k++) {
            x[k] = X[k];
            for (int j = 0; j < 3; j++) x[k] += A[k][j] * r.xref[q][j];
        }
        double fq[3] = {0, 0, 0};
        const double *gpar = r.par + (r.group ? (size_t)r.group[cell] * r.nt * 5 : 0);
        for (int t = 0; t < r.nt; t++) {
            const double *pt = gpar + 5 * t;
            double v = pt[1];
            for (int j = 0; j < 3; j++)
                if (pt[2 + j] != 0) v *= poly_pow(x[j], pt[2 + j]);
            fq[(int)pt[0]] += v;
        }
        for (int i = 0; i < 16; i++) {
            double cv[3] = {0, 0, 0};
            for (int j = 0; j < 4; j++)
                if (R[i][j] != 0)
                    for (int k = 0; k < 3; k++) cv[k] += R[i][j] * te[j][k];
            lb[i] += (fq[0] * cv[0] + fq[1] * cv[1] + fq[2] * cv[2]) * r.w[q];
        }
    }
    const double itemfactor = r.factor * vol;
    for (int i = 0; i < 16; i++) loc[(size_t)cell * 16 + i] = lb[i] * itemfactor;
}

__global__ void k_gather_rows_br3(int32_t nrows, const int32_t *inc_ptr, const int32_t *inc_cell,
                                  const uint8_t *inc_loc, const double *loc, double *b) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    double acc = b[row];
    for (int p = inc_ptr[row]; p < inc_ptr[row + 1]; p++) acc += loc[(size_t)inc_cell[p] * 16 + inc_loc[p]];
    b[row] = acc;
}

struct Br3DivTab {
    int nq;
    double w[4];
    double dref[4][8][3];
};

__global__ void k_br3_div(int ncells, Br3MeshDev m, Br3DivTab t, double *Dv, double *vol_out) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncells) return;
    double X[12], nrm[4][3], fv[4], sg[4];
    br3_load(m, cell, X, nrm, fv, sg);
    double A[3][3], G[3][3], vol;
    simplex_geometry<3, double>(X, G, vol, A);
    for (int I = 0; I < 16; I++) {
        double s = 0;
        for (int q = 0; q < t.nq; q++) {
            double cv = 0;
            for (int k = 0; k < 3; k++) {
                const int si = br3_scalar(I, k);
                if (si < 0) continue;
                const double coef = br3_coef(I, k, nrm);
                for (int j = 0; j < 3; j++) cv += G[k][j] * t.dref[q][si][j] * coef;
            }
            s += cv * t.w[q];
        }
        Dv[(size_t)cell * 16 + I] = s * vol;
    }
    vol_out[cell] = vol;
}

int br3_terms(grmp_space s, int nterms, const grmp_bilinear_term *terms, Br3Terms *bt,
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
    const int rc = grmp_tables(3, GRMP_FE_H1BR, 4, rt);   // 2 (polyorder 3 - derivative 1)
    if (rc || rt->nq > kMaxQ3 || rt->nb != 8) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR{3} tables");
    }
    bt->nq = rt->nq;
    for (int q = 0; q < rt->nq; q++) {
        bt->w[q] = rt->w[q];
        for (int a = 0; a < 8; a++)
            for (int j = 0; j < 3; j++) bt->dref[q][a][j] = rt->derivs[q][a][j];
    }
    delete rt;
    return GRMP_OK;
}

Br3MeshDev br3_mesh(grmp_mesh m) {
    return Br3MeshDev{m->d_coords, m->d_cells, m->d_cell_faces, m->d_face_normals, m->d_face_volumes,
                      m->d_cell_face_signs};
}

template <typename T>
int br3_assemble_t(grmp_matrix A, const Br3Terms &bt) {
    grmp_space s = A->space;
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    std::vector<T> tens(6 * 64);
    for (int pair = 0, p = 0; p < 3; p++)
        for (int q2 = p; q2 < 3; q2++, pair++)
            for (int a = 0; a < 8; a++)
                for (int b = 0; b < 8; b++) {
                    double acc = 0;
                    for (int q = 0; q < bt.nq; q++) {
                        acc += bt.w[q] * bt.dref[q][a][p] * bt.dref[q][b][q2];
                        if (p != q2) acc += bt.w[q] * bt.dref[q][a][q2] * bt.dref[q][b][p];
                    }
                    tens[pair * 64 + a * 8 + b] = (T)acc;
                }
    T *dtens = nullptr;
    int rc = grmp_upload(ctx, &dtens, tens.data(), tens.size());
    if (rc) return rc;
    const size_t fbytes = (size_t)m->ncells * BR3_NF * sizeof(T);
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
    k_br3_factors<T><<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br3_mesh(m), bt, fac);
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
        k_br3_rows<T, uint8_t><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell,
                                                                      s->d_inc_loc, (const uint8_t *)A->d_slot,
                                                                      A->d_rowptr, fac, dtens, *vals);
    else
        k_br3_rows<T, uint16_t><<<nblk(A->nrows), TPB, 0, ctx->stream>>>(A->nrows, s->d_inc_ptr, s->d_inc_cell,
                                                                       s->d_inc_loc, (const uint16_t *)A->d_slot,
                                                                       A->d_rowptr, fac, dtens, *vals);
    GRMP_LAUNCHED(ctx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    grmp_free(ctx, dtens, tens.size() * sizeof(T));
    if (e != cudaSuccess) return grmp_cuda_fail(ctx, e, "H1BR{3} assembly");
    if (sizeof(T) == 8) A->has64 = true; else A->has32 = true;
    return GRMP_OK;
}

}  // namespace

int grmp_br3_mask(grmp_space s, int nterms, const grmp_bilinear_term *terms, uint32_t *mask) {
    grmp_context ctx = s->mesh->ctx;
    Br3Terms bt;
    std::vector<std::pair<void *, size_t>> keep;
    int rc = br3_terms(s, nterms, terms, &bt, keep);
    if (!rc) {
        k_br3_mask<<<nblk(s->mesh->ncells, 64), 64, 0, ctx->stream>>>(s->mesh->ncells, br3_mesh(s->mesh), bt, mask);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "H1BR{3} mask");
    }
    grmp_release(ctx, keep);
    return rc;
}

int grmp_br3_assemble(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision) {
    grmp_context ctx = A->space->mesh->ctx;
    Br3Terms bt;
    std::vector<std::pair<void *, size_t>> keep;
    int rc = br3_terms(A->space, nterms, terms, &bt, keep);
    if (!rc) rc = precision == GRMP_FP64 ? br3_assemble_t<double>(A, bt) : br3_assemble_t<float>(A, bt);
    cudaStreamSynchronize(ctx->stream);
    grmp_release(ctx, keep);
    return rc;
}

// b += (f, R v) with f a 3-component polynomial
int grmp_br3_rhs(grmp_space s, const grmp_rhs *rhs, grmp_vector b) {
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    if (rhs->test_operator != 1 && rhs->test_operator != 2)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR{3} right-hand sides: the RT0 or BDM1 reconstruction only");
    if (rhs->kind != GRMP_RHS_POLY || rhs->ncomponents != 3)
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR{3} reconstructed rhs: 3-component polynomial data only");
    const long long ng = rhs->cell_group ? rhs->ngroups : 1;
    if (ng <= 0 || rhs->nparams <= 0 || rhs->nparams % (5 * ng) || !rhs->params)
        return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: parameter layout");
    const int nt = (int)(rhs->nparams / (5 * ng));
    for (long long t = 0; t < ng * nt; t++)
        if (rhs->params[5 * t] < 0 || rhs->params[5 * t] > 2)
            return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: polynomial component out of range");
    if (rhs->cell_group)
        for (int c = 0; c < m->ncells; c++)
            if (rhs->cell_group[c] < 0 || rhs->cell_group[c] >= ng)
                return grmp_fail(ctx, GRMP_ERR_INVALID_ARG, "rhs: cell group out of range");
    Br3Rhs r;
    std::memset(&r, 0, sizeof(r));
    RefTables *rt = new RefTables;
    int rc = grmp_tables(3, GRMP_FE_H1BR, 3 + rhs->bonus_quadorder, rt);
    if (rc || rt->nq > 64) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "no tetrahedral rule of order %d", 3 + rhs->bonus_quadorder);
    }
    r.nq = rt->nq;
    for (int q = 0; q < rt->nq; q++) {
        for (int k = 0; k < 3; k++) r.xref[q][k] = rt->xref[q][k];
        r.w[q] = rt->w[q];
    }
    delete rt;
    r.nt = nt;
    r.factor = rhs->factor;
    r.bdm1 = rhs->test_operator == 2;
    double *dpar = nullptr;
    int32_t *dgrp = nullptr;
    rc = grmp_upload(ctx, &dpar, rhs->params, (size_t)rhs->nparams);
    if (!rc && rhs->cell_group) rc = grmp_upload(ctx, &dgrp, rhs->cell_group, (size_t)m->ncells);
    const size_t ncl = (size_t)m->ncells * 16;
    if (!rc && !s->d_locbuf) rc = grmp_alloc(ctx, (void **)&s->d_locbuf, ncl * 8);
    if (!rc) {
        r.par = dpar;
        r.group = dgrp;
        k_br3_rhs_cells<<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br3_mesh(m), r, s->d_locbuf);
        GRMP_LAUNCHED(ctx);
        k_gather_rows_br3<<<nblk(s->ndofs), TPB, 0, ctx->stream>>>(s->ndofs, s->d_inc_ptr, s->d_inc_cell,
                                                                   s->d_inc_loc, s->d_locbuf, b->d);
        GRMP_LAUNCHED(ctx);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = grmp_cuda_fail(ctx, e, "H1BR{3} rhs");
    }
    grmp_free(ctx, dpar, (size_t)rhs->nparams * 8);
    grmp_free(ctx, dgrp, (size_t)m->ncells * 4);
    return rc;
}

// Cell divergence table of the batched Stokes solver: Dv[cell][I] =
// int_T div phi_I with the order-2 rule of the velocity-pressure coupling
// (BilinearForm([Divergence, Identity]): polyorder 3 - 1 + 0), vol[cell] = |T|.
int grmp_br3_divergence(grmp_space s, double **Dv, double **vol) {
    grmp_mesh m = s->mesh;
    grmp_context ctx = m->ctx;
    Br3DivTab t;
    std::memset(&t, 0, sizeof(t));
    RefTables *rt = new RefTables;
    int rc = grmp_tables(3, GRMP_FE_H1BR, 2, rt);
    if (rc || rt->nq > 4 || rt->nb != 8) {
        delete rt;
        return grmp_fail(ctx, GRMP_ERR_UNSUPPORTED, "H1BR{3} divergence tables");
    }
    t.nq = rt->nq;
    for (int q = 0; q < rt->nq; q++) {
        t.w[q] = rt->w[q];
        for (int a = 0; a < 8; a++)
            for (int j = 0; j < 3; j++) t.dref[q][a][j] = rt->derivs[q][a][j];
    }
    delete rt;
    rc = grmp_alloc(ctx, (void **)Dv, (size_t)m->ncells * 16 * 8);
    if (!rc) rc = grmp_alloc(ctx, (void **)vol, (size_t)m->ncells * 8);
    if (rc) return rc;
    k_br3_div<<<nblk(m->ncells), TPB, 0, ctx->stream>>>(m->ncells, br3_mesh(m), t, *Dv, *vol);
    GRMP_LAUNCHED(ctx);
    GRMP_CUDA(ctx, cudaGetLastError());
    return GRMP_OK;
}
