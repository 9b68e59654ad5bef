// Device-side element data shared by the pattern and assembly kernels.
#pragma once

#include "grmp_internal.h"

// Reference tables of one (element, quadrature order) pair in device memory.
struct TablesDev {
    int nq, nb, dim;
    const double *w;       // [nq]
    const double *xref;    // [nq][3]
    const double *vals;    // [nq][nb]
    const double *derivs;  // [nq][nb][dim]
};

// One operator term as seen by device code.
struct TermDev {
    int op;                // grmp_op_kind
    int symmetric;
    double factor;
    const double *cell_coef;   // [ncells] or nullptr
    double mu, lambda;
    TablesDev tab;
};

struct TermsDev {
    int n;
    TermDev t[GRMP_MAX_TERMS];
};

// Geometry of one simplex: A = [x1-x0, x2-x0(, x3-x0)] and G = A^{-T} =
// cof(A)/det(A) (the `L2GAinv` of src/feevaluator_h1.jl:61-74; this library's
// convention for ExtendableGrids' mapderiv!), volume |det|/d!.  The RN
// variant uses explicitly rounded operations (no FMA contraction) so that it
// reproduces the host restatement bit for bit.
template <int DIM>
__device__ __forceinline__ void simplex_geometry_rn(const double *X, double A[3][3], double G[3][3], double &vol) {
    for (int k = 0; k < DIM; k++)
        for (int j = 0; j < DIM; j++) A[k][j] = __dsub_rn(X[(j + 1) * DIM + k], X[k]);
    if (DIM == 2) {
        double d = __dsub_rn(__dmul_rn(A[0][0], A[1][1]), __dmul_rn(A[0][1], A[1][0]));
        G[0][0] = __ddiv_rn(A[1][1], d);
        G[0][1] = __ddiv_rn(-A[1][0], d);
        G[1][0] = __ddiv_rn(-A[0][1], d);
        G[1][1] = __ddiv_rn(A[0][0], d);
        vol = __ddiv_rn(fabs(d), 2.0);
    } else {
        double c00 = __dsub_rn(__dmul_rn(A[1][1], A[2][2]), __dmul_rn(A[1][2], A[2][1]));
        double c01 = __dsub_rn(__dmul_rn(A[1][2], A[2][0]), __dmul_rn(A[1][0], A[2][2]));
        double c02 = __dsub_rn(__dmul_rn(A[1][0], A[2][1]), __dmul_rn(A[1][1], A[2][0]));
        double c10 = __dsub_rn(__dmul_rn(A[0][2], A[2][1]), __dmul_rn(A[0][1], A[2][2]));
        double c11 = __dsub_rn(__dmul_rn(A[0][0], A[2][2]), __dmul_rn(A[0][2], A[2][0]));
        double c12 = __dsub_rn(__dmul_rn(A[0][1], A[2][0]), __dmul_rn(A[0][0], A[2][1]));
        double c20 = __dsub_rn(__dmul_rn(A[0][1], A[1][2]), __dmul_rn(A[0][2], A[1][1]));
        double c21 = __dsub_rn(__dmul_rn(A[0][2], A[1][0]), __dmul_rn(A[0][0], A[1][2]));
        double c22 = __dsub_rn(__dmul_rn(A[0][0], A[1][1]), __dmul_rn(A[0][1], A[1][0]));
        double d = __dadd_rn(__dadd_rn(__dmul_rn(A[0][0], c00), __dmul_rn(A[0][1], c01)), __dmul_rn(A[0][2], c02));
        G[0][0] = __ddiv_rn(c00, d); G[0][1] = __ddiv_rn(c01, d); G[0][2] = __ddiv_rn(c02, d);
        G[1][0] = __ddiv_rn(c10, d); G[1][1] = __ddiv_rn(c11, d); G[1][2] = __ddiv_rn(c12, d);
        G[2][0] = __ddiv_rn(c20, d); G[2][1] = __ddiv_rn(c21, d); G[2][2] = __ddiv_rn(c22, d);
        vol = __ddiv_rn(fabs(d), 6.0);
    }
}

// Fast geometry (contraction allowed): G and volume in precision T.
template <int DIM, typename T>
__device__ __forceinline__ void simplex_geometry(const double *X, T G[3][3], T &vol, T A[3][3]) {
    double Ad[3][3];
    for (int k = 0; k < DIM; k++)
        for (int j = 0; j < DIM; j++) Ad[k][j] = X[(j + 1) * DIM + k] - X[k];
    for (int k = 0; k < DIM; k++)
        for (int j = 0; j < DIM; j++) A[k][j] = (T)Ad[k][j];
    if (DIM == 2) {
        T d = A[0][0] * A[1][1] - A[0][1] * A[1][0];
        T id = T(1) / d;
        G[0][0] = A[1][1] * id;
        G[0][1] = -A[1][0] * id;
        G[1][0] = -A[0][1] * id;
        G[1][1] = A[0][0] * id;
        vol = fabs(d) * T(0.5);
    } else {
        T c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
        T c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
        T c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
        T c10 = A[0][2] * A[2][1] - A[0][1] * A[2][2];
        T c11 = A[0][0] * A[2][2] - A[0][2] * A[2][0];
        T c12 = A[0][1] * A[2][0] - A[0][0] * A[2][1];
        T c20 = A[0][1] * A[1][2] - A[0][2] * A[1][1];
        T c21 = A[0][2] * A[1][0] - A[0][0] * A[1][2];
        T c22 = A[0][0] * A[1][1] - A[0][1] * A[1][0];
        T d = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
        T id = T(1) / d;
        G[0][0] = c00 * id; G[0][1] = c01 * id; G[0][2] = c02 * id;
        G[1][0] = c10 * id; G[1][1] = c11 * id; G[1][2] = c12 * id;
        G[2][0] = c20 * id; G[2][1] = c21 * id; G[2][2] = c22 * id;
        vol = fabs(d) * T(1.0 / 6.0);
    }
}

// Voigt compression of SymmetricGradient (src/feevaluator.jl:228-231):
// gradient entry (component c, direction k) -> Voigt slot.
__device__ __forceinline__ int voigt_slot(int dim, int c, int k) {
    if (dim == 2) {
        const int m[4] = {0, 2, 2, 1};
        return m[k + c * 2];
    }
    const int m[9] = {0, 5, 4, 5, 1, 3, 4, 3, 2};
    return m[k + c * 3];
}

// x^e for the exponents of polynomial data: integer e in [1, 8] by
// repeated multiplication left to right (x*x*x, as Julia's literal powers
// x^2, x^3 of the reference's data functions evaluate), pow otherwise.
__host__ __device__ __forceinline__ double poly_pow(double x, double e) {
    const int k = (int)e;
    if ((double)k == e && k >= 1 && k <= 8) {
        double r = x;
        for (int i = 1; i < k; i++) r = r * x;
        return r;
    }
    return pow(x, e);
}

// Data functions of the linear forms and item integrators evaluated on device
// (constant, per cell, Fourier series, polynomial; grmp_rhs_kind).  f gets
// r.ncomp values.
struct RhsDev {
    int kind, ncomp;
    const double *par;
    long long npar;
    double factor;
    int nq, nb;
    const double *w, *xref, *vals;
};

__device__ __forceinline__ void rhs_eval(const RhsDev &r, int dim, int cell, const double *x, double *f) {
    if (r.kind == GRMP_RHS_CONST) {
        for (int c = 0; c < r.ncomp; c++) f[c] = r.par[c];
    } else if (r.kind == GRMP_RHS_CELL) {
        for (int c = 0; c < r.ncomp; c++) f[c] = r.par[(size_t)cell * r.ncomp + c];
    } else if (r.kind == GRMP_RHS_FOURIER) {
        int stride = 1 + dim, nm = (int)(r.npar / stride);
        double s = 0;
        for (int m = 0; m < nm; m++) {
            double arg = 0;
            for (int j = 0; j < dim; j++) arg += r.par[m * stride + 1 + j] * x[j];
            s += r.par[m * stride] * sinpi(arg);   // sin(pi arg), without rounding pi * arg first
        }
        f[0] = s;
        for (int c = 1; c < r.ncomp; c++) f[c] = 0;
    } else {
        for (int c = 0; c < r.ncomp; c++) f[c] = 0;
        int nt = (int)(r.npar / 5);
        for (int t = 0; t < nt; t++) {
            int c = (int)r.par[5 * t];
            double v = r.par[5 * t + 1];
            for (int j = 0; j < dim; j++) {
                double e = r.par[5 * t + 2 + j];
                if (e != 0) v *= poly_pow(x[j], e);
            }
            f[c] += v;
        }
    }
}
