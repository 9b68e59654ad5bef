/*
 * grmp.h -- C-ABI of the GB300 finite-element assembly + solve library
 * (libgrmp_gpu.so).
 *
 * The library replaces, for one GPU, the hot path of GradientRobustMultiPhysics.jl
 * v0.12.0: global assembly of BilinearForm / LinearForm operators and the sparse
 * linear solve behind solve!(Solution, Problem).  Each entry point cites the
 * reference interface it stands in for (paths are relative to the reference
 * project root).
 *
 * Conventions
 *  - Every function returns an int status (grmp_status); nothing throws.
 *    The text of the last error of a context is returned by grmp_last_error.
 *  - Handles are opaque and owned by the library; free them with the matching
 *    *_destroy call.  Host arrays passed in are copied before the call returns
 *    (a garbage-collected caller may move or free them afterwards).  Output
 *    host arrays are allocated by the caller.
 *  - Indices are 0-based int32.  The reference is 1-based: a Julia caller
 *    subtracts 1 (see the integration notes).
 *  - One context owns one CUDA stream; all work of a context is ordered on it.
 *    Handles of one context may be used from one host thread at a time.
 */
#ifndef GRMP_H
#define GRMP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef enum {
    GRMP_OK = 0,
    GRMP_ERR_INVALID_ARG = 1,    /* bad handle, size, index or option          */
    GRMP_ERR_OUT_OF_MEMORY = 2,  /* device allocation failed                  */
    GRMP_ERR_DEVICE = 3,         /* CUDA runtime error                        */
    GRMP_ERR_NOT_CONVERGED = 4,  /* iteration cap hit before the tolerance    */
    GRMP_ERR_UNSUPPORTED = 5,    /* element / operator combination not built  */
    GRMP_ERR_BUDGET = 6,         /* request exceeds the context's HBM budget  */
    GRMP_ERR_TIMEOUT = 7,        /* a bounded device-side wait gave up        */
    GRMP_ERR_NAN = 8,            /* non-finite value in an input or iterate   */
    GRMP_ERR_NO_DEVICE = 9       /* no CUDA device / library built without one */
} grmp_status;

typedef struct grmp_context_s *grmp_context;
typedef struct grmp_mesh_s *grmp_mesh;
typedef struct grmp_space_s *grmp_space;
typedef struct grmp_matrix_s *grmp_matrix;
typedef struct grmp_vector_s *grmp_vector;

/* --------------------------------------------------------------- context */

/* Library version as major*10000 + minor*100 + patch. */
int grmp_version(void);

/* Create a context on CUDA device `device`.  `hbm_budget_bytes` caps the
 * device memory the context may hold (0 = no cap); allocations beyond it fail
 * with GRMP_ERR_BUDGET.  No reference counterpart (the reference is CPU-only);
 * it is the state a LinearSolve algorithm cache holds (src/solvers.jl:89-101). */
int grmp_create_context(int device, size_t hbm_budget_bytes, grmp_context *out);
int grmp_destroy_context(grmp_context ctx);
const char *grmp_last_error(grmp_context ctx);
/* cudaStream_t of the context, as void*, for callers that time or order work. */
int grmp_context_stream(grmp_context ctx, void **stream);
int grmp_synchronize(grmp_context ctx);
/* Bytes of device memory currently held by the context's handles. */
int grmp_context_memory(grmp_context ctx, size_t *bytes_in_use);
/* Number of kernels this context has launched so far (instrumentation). */
int grmp_context_launches(grmp_context ctx, uint64_t *launches);
/* Polls (a grid-barrier poll is one L2 round trip, under a microsecond;
 * an mbarrier poll a few tens of ns) after which a bounded device-side wait of this
 * context's iterative solves gives up and the solve returns GRMP_ERR_TIMEOUT
 * (grid barriers of the persistent kernels, mbarrier waits of the staged
 * SpMV); 0 restores the default of 2^24.  No reference counterpart (the
 * reference has no device waits); it lets a caller bound how long a stalled
 * solve holds the GPU, and lets a test make a wait run out. */
int grmp_context_set_wait_limit(grmp_context ctx, int64_t polls);
/* Failure-detection check of the bounded waits: one cooperative launch in
 * which every block waits on a shared-memory mbarrier that nothing
 * completes, then block 0 leaves while the other blocks wait at a grid
 * barrier it never reaches.  Both waits give up after `polls` polls; the
 * statuses the waiting blocks recorded are returned in *grid_status and
 * *mbar_status (GRMP_ERR_TIMEOUT when the bounds work).  Nothing faults or
 * hangs and the context stays usable.  No reference counterpart. */
int grmp_selftest_wait_timeout(grmp_context ctx, int64_t polls, int32_t *grid_status, int32_t *mbar_status);
/* Device address of a vector's FP64 data (for coef_on_device inputs). */
int grmp_vector_device_ptr(grmp_vector v, void **dptr);

/* ------------------------------------------------------------------ mesh */

/* Upload a simplex mesh: coords [nverts][dim] (FP64), cell_verts
 * [ncells][dim+1].  Replaces the ExtendableGrids arrays Coordinates /
 * CellNodes read by L2GTransformer (src/feevaluator.jl:38). */
int grmp_mesh_upload(grmp_context ctx, int dim, int32_t nverts, const double *coords, int32_t ncells,
                     const int32_t *cell_verts, grmp_mesh *out);

/* Face data needed by the H1BR element and the RT0 / BDM1 reconstruction
 * (FaceNormals, FaceVolumes, CellFaces, CellFaceSigns of ExtendableGrids, read
 * in src/fedefs/h1v_br.jl:150-162 and src/reconstructions.jl:381-403):
 * cell_faces [ncells][dim+1], face_normals [nfaces][dim] (unit, globally
 * oriented), face_volumes [nfaces], cell_face_signs [ncells][dim+1] (+1/-1). */
int grmp_mesh_set_faces(grmp_mesh mesh, int32_t nfaces, const int32_t *cell_faces, const double *face_normals,
                        const double *face_volumes, const int8_t *cell_face_signs);
/* The same face data computed on the device from the mesh alone (faces
 * numbered in the lexicographic order of their sorted vertex triples / pairs,
 * the normal of a face the outward normal of the lowest-numbered cell that
 * has it, cell_face_signs +1 where a cell's outward normal agrees with it,
 * face_volumes the face areas / lengths), replacing a previous set. */
int grmp_mesh_build_faces(grmp_mesh mesh);
/* The mesh's face data into host arrays (any of them may be NULL):
 * cell_faces [ncells][dim+1], face_normals [nfaces][dim], face_volumes
 * [nfaces], cell_face_signs [ncells][dim+1]; *nfaces receives the count. */
int grmp_mesh_faces(grmp_mesh mesh, int32_t *nfaces, int32_t *cell_faces, double *face_normals, double *face_volumes,
                    int8_t *cell_face_signs);
int grmp_mesh_destroy(grmp_mesh mesh);

/* ----------------------------------------------------------------- space */

typedef enum {
    GRMP_FE_H1P1 = 1,     /* src/fedefs/h1_p1.jl                    */
    GRMP_FE_H1P2 = 2,     /* src/fedefs/h1_p2.jl                    */
    GRMP_FE_H1BR = 3,     /* src/fedefs/h1v_br.jl (2D and 3D)       */
    GRMP_FE_HDIVRT0 = 4,  /* reconstruction target only            */
    GRMP_FE_HDIVBDM1 = 5, /* reconstruction target only            */
    GRMP_FE_L2P0 = 6,     /* src/fedefs/l2_p0.jl                    */
    GRMP_FE_H1P2B = 7,    /* src/fedefs/h1_p2b.jl: H1P2B{2,2} (P2 + cell bubble, 2D vector);
                             reconstructed right-hand sides only    */
    GRMP_FE_HDIVRT1 = 8,  /* reconstruction target only (src/fedefs/hdiv_rt1.jl)  */
    GRMP_FE_HDIVBDM2 = 9  /* reconstruction target only (src/fedefs/hdiv_bdm2.jl) */
} grmp_fe_kind;

/* FESpace{FEType}(xgrid) (src/finiteelements.jl:72-119) with the cell DoF
 * map FES[CellDofs] (src/dofmaps.jl:201-330) supplied by the caller:
 * celldofs [ncells][ndofs4cell], component-major in the element's pattern
 * order. */
int grmp_space_create(grmp_mesh mesh, int fe_kind, int ncomponents, const int32_t *celldofs, int32_t ndofs,
                      grmp_space *out);
int grmp_space_destroy(grmp_space space);
/* FESpace{FEType}(xgrid) built on the device from the mesh alone: the dofmap
 * of src/dofmaps.jl:201-330 for H1P1 (pattern "N1"), H1P2 ("N1F1" in 2D,
 * "N1E1" in 3D, src/fedefs/h1_p2.jl:33-35) and H1BR{dim} ("N1f1",
 * src/fedefs/h1v_br.jl:33; its face data are built with
 * grmp_mesh_build_faces unless the mesh has some), components blocked.
 * Edges and faces are numbered in the lexicographic order of their sorted
 * vertex tuples (the host mesh module's numbering).  Replaces the host-side
 * dofmap build of a caller; ndofs_out (optional) receives the DoF count. */
int grmp_space_create_on_device(grmp_mesh mesh, int fe_kind, int ncomponents, grmp_space *out, int32_t *ndofs_out);
/* The space's CellDofs into a host array [ncells][ndofs4cell]. */
int grmp_space_celldofs(grmp_space space, int32_t *celldofs);
/* DoFs on the boundary faces (faces of exactly one cell) of any H1P1 / H1P2
 * / H1BR space, ascending: the BFaceDofs of the homogeneous Dirichlet branch
 * of boundarydata! (src/boundarydata.jl:200-260) over all boundary regions,
 * computed on the device.  fixed: host array of `capacity` entries, or NULL
 * to count only; *nfixed receives the count (GRMP_ERR_INVALID_ARG when it
 * exceeds a non-zero capacity). */
int grmp_space_boundary_dofs(grmp_space space, int32_t capacity, int32_t *fixed, int32_t *nfixed);
/* Number of local DoFs per cell for the space. */
int grmp_space_ndofs4cell(grmp_space space, int *out);

/* Reference tables of the space's element for the quadrature rule of `order`
 * (QuadratureRule{Float64,EG}(order), src/quadrature.jl:173-325, and the
 * reference basis / ForwardDiff derivative tables, src/feevaluator.jl:93-131,
 * :235-293).  Host-only query.  xref [nq][3], w [nq], vals [nq][nb],
 * derivs [nq][nb][dim] where nb = scalar basis size; pass NULL to only get
 * sizes.  Returns nq in *nq and nb in *nb. */
int grmp_reference_tables(int dim, int fe_kind, int order, int *nq, int *nb, double *xref, double *w, double *vals,
                          double *derivs);

/* ------------------------------------------------------- bilinear forms */

typedef enum {
    GRMP_OP_LAPLACE = 1,   /* (Gradient u, Gradient v): LaplaceOperator / BilinearForm([Gradient,Gradient])
                              src/pdeoperators.jl:154-169, :355-396                                     */
    GRMP_OP_MASS = 2,      /* (Identity u, Identity v): ReactionOperator, src/pdeoperators.jl:176-203     */
    GRMP_OP_HOOKE = 3,     /* (C eps(u), eps(v)) with SymmetricGradient{1}: HookStiffnessOperator2D/3D
                              src/pdeoperators.jl:256-315; param[0] = mu, param[1] = lambda            */
    GRMP_OP_RDIVRDIV = 4,  /* (div R u, div R v), R = BR -> RT0 reconstruction (ReconstructionDivergence,
                              src/feevaluator_h1.jl:409-437); iterated-penalty term.  In 3D the RT0
                              basis is mapped with A phi / |det A| (times the cell-face sign), so
                              div R u is the cell mean of div u on tetrahedra of either orientation */
    GRMP_OP_STRUCTURAL = 5, /* pattern only: couples every local pair of a cell (the Jacobian of a
                              NonlinearForm fills them all); contributes nothing to assembled values */
    GRMP_OP_JUMPGRAD = 6   /* BilinearForm([Jump(Gradient), Jump(Gradient)], Action(input |F|^param[0]);
                              AT = ON_IFACES) times factor: factor |F| |F|^p int_F [grad u].[grad v]
                              summed over interior faces (the interior-penalty stabilisation of
                              examples/Example203_ReactionConvectionDiffusion2D.jl:89-92; jumps as in
                              update_dii4op!, src/assemblypatterns.jl:103-153).  Scalar H1P1 / H1P2;
                              needs the mesh's faces; the pattern then holds the DoFs of face
                              neighbours; added after the cell terms, FP64 (FP32 values rounded) */
} grmp_op_kind;

/* One operator term.  Assembly of a list of terms adds them into one matrix,
 * as the reference adds several PDE operators into one FEMatrix block. */
typedef struct {
    int op_kind;             /* grmp_op_kind                                                        */
    int symmetric;           /* 1: APT_SymmetricBilinearForm, 0: APT_BilinearForm                   */
    double factor;           /* operator factor (e.g. kappa of LaplaceOperator(kappa))              */
    const double *cell_coef; /* optional [ncells] per-cell scalar (an Action with "I" dependency:
                                result = coef[cell] * input); NULL if absent                          */
    double param[4];         /* op-specific parameters (Hooke: mu, lambda)                           */
    int bonus_quadorder;     /* added to the quadrature order (src/assemblypatterns.jl:559-565)     */
    int coef_on_device;      /* 1: cell_coef is a device pointer of this context's GPU (e.g. the
                                data of a grmp_vector), read in place; 0: a host array, copied     */
} grmp_bilinear_term;

typedef enum {
    GRMP_FP64 = 0,
    GRMP_FP32 = 1,
    GRMP_FP64_FP32 = 2   /* assembly only: FP64 and FP32 values in one pass (each in its own arithmetic) */
} grmp_precision;

/* Build the sparsity pattern of the sum of `terms` on `space` x `space`:
 * the union of the nonzero local contributions, an entry being dropped when
 * every local contribution to it is exactly 0.0 in the reference's operation
 * order (_addnz, src/fematrix.jl:54-65).  Also builds the DoF->cell
 * incidence lists and the cell-to-CSR slot map used by assembly.  Replaces
 * FEMatrix{T}(FEs) + the ExtendableSparse LNK build (src/fematrix.jl:186-213). */
int grmp_pattern_build(grmp_space space, int nterms, const grmp_bilinear_term *terms, grmp_matrix *out);
int grmp_matrix_destroy(grmp_matrix A);
/* nrows, nnz and the maximum number of nonzeros of a row. */
int grmp_matrix_info(grmp_matrix A, int32_t *nrows, int64_t *nnz, int32_t *max_row_nnz);

/* Assemble the sum of `terms` into the matrix values in the given precision
 * (FP64 values and/or FP32 values are held separately in the handle;
 * GRMP_FP64_FP32 fills both from one walk of the incidence lists, the FP32
 * values computed in FP32 arithmetic exactly as a GRMP_FP32 assembly would;
 * an assembly in one precision leaves the other precision's values as they
 * were, so a MIXED solve after new coefficients wants GRMP_FP64_FP32).
 * Stands in for assemble!(A::FEMatrixBlock, AP::AssemblyPattern{<:APT_BilinearForm})
 * (src/assemblypatterns/bilinearform.jl:92-400).  Deterministic: each
 * nonzero is the sum of its cell contributions in ascending cell order. */
int grmp_assemble_bilinear(grmp_matrix A, int nterms, const grmp_bilinear_term *terms, int precision);

/* ---------------------------------------------------------- nonlinear forms */

/* NonlinearForm kernels (the reference takes a user kernel and differentiates
 * it with ForwardDiff; here a closed set with its Jacobian written out). */
typedef enum {
    GRMP_NL_DIFFUSION = 1,      /* ((kappa + beta u^2) grad u, grad v), scalar: NonlinearForm(Gradient,
                                   [Identity, Gradient], ...), examples/Example205_NonlinearPoisson2D.jl:114
                                   (kappa = beta = 1), Example206, ExampleA04, ExampleA05              */
    GRMP_NL_GRAD_DIFFUSION = 2, /* ((kappa + |grad u|^2) grad u, grad v), scalar: NonlinearForm(Gradient,
                                   [Gradient], ...), examples/Example205_NonlinearPoisson2D.jl:116       */
    GRMP_NL_CONVECTION = 3      /* ((u . grad) u, v), vector with ncomponents = dim: NonlinearForm(
                                   Identity, [Identity, Gradient], ...), the Navier-Stokes convection
                                   (examples/ExampleA11_NavierStokesFixpointIterations.jl:78,
                                   src/pdeoperators.jl:493)                                             */
} grmp_nl_kind;

typedef struct {
    int kind;                /* grmp_nl_kind                                          */
    double factor;           /* NonlinearForm factor                                  */
    double param[4];         /* DIFFUSION: kappa, beta; GRAD_DIFFUSION: kappa          */
    int bonus_quadorder;     /* added to the quadrature order                          */
} grmp_nonlinear_term;

/* Newton linearisation at the iterate u (full_assemble!,
 * src/assemblypatterns/nonlinearform.jl:44-240): with K the kernel, J its
 * Jacobian and input(.) the operator evaluations,
 *   A[j][i] (+)= vol factor sum_q w_q (J input(phi_i)) . test(phi_j)
 *   b[j]    (+)= vol factor sum_q w_q (J input(u) - K) . test(phi_j),
 * i.e. DG(u) into A and DG(u) u - G(u) into b, so that A x = b is the
 * Newton step's system for the next iterate x (the reference adds the same to
 * the PDE's matrix and right-hand side, src/solvers.jl:519-566).  add = 1
 * adds to A's values and b (after grmp_assemble_bilinear / _linear of the
 * linear operators), add = 0 overwrites them.  A's pattern must hold every
 * local pair: build it with a GRMP_OP_STRUCTURAL term (GRMP_ERR_INVALID_ARG
 * otherwise).  precision GRMP_FP64, or GRMP_FP64_FP32 (the FP32 values get
 * the FP64 contributions rounded).  The Jacobian is not symmetric: solve with
 * GRMP_SOLVE_BICGSTAB.  H1P1 / H1P2 spaces. */
int grmp_assemble_nonlinear(grmp_matrix A, grmp_vector b, grmp_vector u, const grmp_nonlinear_term *term,
                            int precision, int add);

/* A matrix from the caller's compressed sparse column arrays: the matrix
 * LinearSolve receives from solve_direct!, a SparseMatrixCSC{Float64,Int64}
 * (init(LinearProblem(A, b), alg), src/solvers.jl:89-101, :658-661;
 * FEMatrix entries, src/fematrix.jl:148-150).  colptr [n+1], rowval and
 * nzval [colptr[n] - index_base]; index_base 1 for Julia's arrays (0 for
 * C); row indices strictly increasing within a column.  symmetric = 1: the
 * matrix is symmetric and its CSC arrays are used as the CSR arrays (no
 * transpose); 0: the host transposes them once.  Rows whose diagonal is >=
 * penalty_threshold (> 0; e.g. 1e30 for the reference's 1e60 Dirichlet
 * penalty, src/solvers.jl:640-652) are penalty rows: the solvers work on the
 * matrix with those rows and columns eliminated (FP64, and rounded to FP32
 * for the mixed and FP32-factor solvers -- 1e60 overflows FP32), and
 * grmp_solve maps the caller's b accordingly (x_d = b_d / a_dd, b_i -= a_id
 * x_d), which reproduces the penalised system's solution up to O(1 / a_dd)
 * relative.  0 = no penalty rows.  The handle has no assembly space
 * (grmp_assemble_bilinear refuses it); its values are replaced with
 * grmp_matrix_update_values.  Iterative solves need a symmetric positive
 * definite matrix (after elimination). */
int grmp_matrix_from_csc(grmp_context ctx, int32_t n, const int64_t *colptr, const int64_t *rowval,
                         const double *nzval, int index_base, int symmetric, double penalty_threshold,
                         grmp_matrix *out);
/* New values for an imported matrix with the same pattern: nzval [nnz] in
 * the CSC order of the import (cache.A = A in the fixpoint loops,
 * src/solvers.jl:906-911, :1160-1165).  Penalty rows are detected again;
 * symbolic analyses and tuned SpMV configurations are kept. */
int grmp_matrix_update_values(grmp_matrix A, const double *nzval);
/* Number of penalty rows of an imported matrix's current values (0 for an
 * assembled matrix). */
int grmp_matrix_penalty_rows(grmp_matrix A, int32_t *count);

/* Copy the CSR arrays (rowptr [nrows+1] int64, cols [nnz], vals [nnz] FP64)
 * to host memory; any pointer may be NULL.  `precision` selects which values. */
int grmp_matrix_download(grmp_matrix A, int precision, int64_t *rowptr, int32_t *cols, double *vals);

/* --------------------------------------------------------- linear forms */

typedef enum {
    GRMP_RHS_CONST = 0,   /* f = const vector: params[ncomp]                                    */
    GRMP_RHS_CELL = 1,    /* f = per-cell vector: params[ncells][ncomp] ("I" dependency)         */
    GRMP_RHS_FOURIER = 2, /* f = sum_m a_m sin(pi k_m . x): params[nmodes][1+dim] = (a_m, k_m)   */
    GRMP_RHS_POLY = 3     /* f_c = sum_t coef_t x^e1 y^e2 z^e3: params[nterms][5]
                             = (component, coef, e1, e2, e3)                                   */
} grmp_rhs_kind;

typedef struct {
    int kind;               /* grmp_rhs_kind                                       */
    int ncomponents;        /* components of f                                     */
    const double *params;   /* see grmp_rhs_kind                                    */
    int64_t nparams;        /* number of doubles in params                           */
    double factor;          /* LinearForm factor                                     */
    int bonus_quadorder;    /* DataFunction bonus_quadorder                          */
    int test_operator;      /* 0 = Identity; 1 = ReconstructionIdentity{HDIVRT0{d}};
                               2 = ReconstructionIdentity{HDIVBDM1{d}} (1, 2: H1BR only;
                               3 = ReconstructionIdentity{HDIVRT1{2}},
                               4 = ReconstructionIdentity{HDIVBDM2{2}} (3, 4: H1P2B only,
                               src/reconstructions.jl:43-330, :405-469);
                               src/feevaluator_h1.jl:342-381, src/reconstructions.jl:351-535;
                               in 3D the BDM1 function matching the P1 normal-flux moments of
                               each face, which the reference's orientation-selected basis
                               spans)                                                     */
    const int32_t *cell_group; /* optional [ncells]: POLY data per cell group (one DataFunction
                                  per independent problem of a batch); params then hold
                                  [ngroups][nterms][5]                                 */
    int32_t ngroups;
} grmp_rhs;

/* b += LinearForm(test_operator, f) over the space (src/assemblypatterns/
 * linearform.jl:47-237).  FP64, deterministic (ascending cell order). */
int grmp_assemble_linear(grmp_space space, const grmp_rhs *rhs, grmp_vector b);

/* ------------------------------------------------------- item integrators */

typedef enum { GRMP_ITEM_IDENTITY = 0, GRMP_ITEM_GRADIENT = 1 } grmp_item_operator;

/* ItemIntegrator over all cells of an H1P1 / H1P2 space (scalar or vector),
 * replacing evaluate / evaluate! of src/assemblypatterns/itemintegrator.jl
 * (:173-330) for the three error/norm integrators of that file:
 *   L2ErrorIntegrator(data, op; factor)  (:40-94):  data != NULL, v == NULL
 *       integrand sum_j (data_j(x) - factor * (op u)_j)^2
 *   L2NormIntegrator(op)                 (:96-130): data == NULL, v == NULL
 *       integrand sum_j (factor * (op u)_j)^2
 *   L2DifferenceIntegrator(op)           (:132-158): v != NULL (data must be NULL)
 *       integrand sum_j ((op u)_j - (op v)_j)^2
 * op: GRMP_ITEM_IDENTITY (components u_c) or GRMP_ITEM_GRADIENT (component-major
 * [du_1/dx_1 .. du_1/dx_d, du_2/dx_1 ..]); data->ncomponents must equal the
 * operator's length (data->factor, test_operator and cell_group are ignored).
 * quadorder: the integrator's bonus order (>= 0), or -1 for the reference's
 * "auto" (2 * data->bonus_quadorder; 2 without data); the rule has order
 * polyorder - (op == GRADIENT) + bonus (src/assemblypatterns.jl:559-565).
 * cell_values (optional, host, [ncells]) receives the per-cell integrals, total
 * (optional, host) their sum; sqrt(total) is the error/norm.  FP64;
 * reproducible run to run (fixed summation order). */
int grmp_item_l2error(grmp_space space, grmp_vector u, grmp_vector v, int op, const grmp_rhs *data, double factor,
                      int quadorder, double *cell_values, double *total);

/* ItemIntegrator([Jump(Gradient)], action; AT = ON_IFACES): per interior face
 * factor |F| |F|^power int_F g, g = |[grad u]|^2 (kind 0) or ([grad u].n_F)^2
 * (kind 1, the jump term of examples/Example210_PoissonLshapeAdaptive2D.jl:58-75
 * with power 1); boundary faces give 0.  face_values [nfaces] (optional,
 * host) and their sum in ascending face order (optional).  Scalar H1P1 /
 * H1P2; needs the mesh's faces. */
int grmp_item_face_jumps(grmp_space space, grmp_vector u, int kind, double power, double factor, int bonus_quadorder,
                         double *face_values, double *total);

/* -------------------------------------------------------------- vectors */

int grmp_vector_create(grmp_context ctx, int32_t n, grmp_vector *out);
int grmp_vector_destroy(grmp_vector v);
int grmp_vector_upload(grmp_vector v, const double *host);
int grmp_vector_download(grmp_vector v, double *host);
int grmp_vector_fill(grmp_vector v, double value);

/* ------------------------------------------------------------- Dirichlet */

typedef enum { GRMP_DIRICHLET_PENALTY = 0, GRMP_DIRICHLET_ELIMINATE = 1 } grmp_dirichlet_mode;

/* Fix DoFs `fixed[nfixed]` to `values` (NULL = homogeneous).  PENALTY is the
 * reference's treatment: A[d,d] = penalty, b[d] = penalty * u_D[d]
 * (src/solvers.jl:640-652, src/fematrix.jl:349-355; default penalty 1e60).
 * ELIMINATE zeroes row and column d (b -= A[:,d] u_D), sets A[d,d] = 1 and
 * b[d] = u_D[d]; it gives the same free-DoF solution up to O(1/penalty) and is
 * the form the FP32 path needs (1e60 overflows FP32).  Applied to both the
 * FP64 and FP32 values present in A. */
int grmp_apply_dirichlet(grmp_matrix A, grmp_vector b, int32_t nfixed, const int32_t *fixed, const double *values,
                         int mode, double penalty);

/* ------------------------------------------------------------------ solve */

typedef enum {
    GRMP_SOLVE_FP64 = 0,   /* plain: FP64 Jacobi-PCG                                                 */
    GRMP_SOLVE_MIXED = 1,  /* FP32 Jacobi-PCG inside FP64 refinement (outer residual, update in FP64) */
    GRMP_SOLVE_DIRECT = 2, /* FP64 multifrontal Cholesky (nested-dissection order) + residual
                              refinement against the assembled FP64 matrix; in
                              grmp_stokes_batch_solve one factorisation per problem, reused by
                              every sweep.  SPD matrices (Dirichlet eliminated or penalised).     */
    GRMP_SOLVE_MIXED_DIRECT = 3, /* grmp_solve only: FP32 multifrontal Cholesky used as the
                              preconditioner of FP64 conjugate gradients on the FP64 matrix
                              (Dirichlet rows must be eliminated: 1e60 overflows FP32)           */
    GRMP_SOLVE_BICGSTAB = 4 /* grmp_solve only: FP64 Jacobi-preconditioned BiCGStab in one
                              persistent launch, for non-symmetric matrices (the Jacobian of a
                              NonlinearForm's Newton step, where the reference calls a sparse LU) */
} grmp_solve_mode;

typedef struct {
    double abstol;          /* stop when ||b - A x||_2 <= max(abstol, reltol*||b||_2)   */
    double reltol;
    int32_t maxiter;        /* cap on inner iterations                                   */
    int32_t mode;           /* grmp_solve_mode                                           */
    double inner_reltol;    /* MIXED: residual reduction per refinement (reliable update) */
    int32_t max_outer;      /* MIXED: cap on FP64 refinement steps                        */
    int32_t spmv_config;    /* SpMV lanes per row and loads in flight, coded 100*lanes + loads,
                               +10000 for the software-pipelined row loop: 208, 404, 408, 804,
                               1602, 10204, 10404, 10408, 10804, 10402, 10802; MIXED only,
                               rows streamed through shared memory in 32 KB windows by bulk
                               async copies: 20204, 20408, 20804 (512 threads, 3 stages per
                               block), 30408, 30804 (1024 threads, 6 stages); MIXED only,
                               the FP32 values with two-run 16-bit columns (two entries per
                               8-byte value load and 4-byte column load; rows whose columns
                               fall in two windows of 65536): 60404, 60208, 60802, 60408
                               (100*lanes + entry pairs in flight); MIXED only, the same
                               columns with the Jacobi-scaled FP32 values a_ij/sqrt(a_ii a_jj)
                               (unpreconditioned inner CG, no residual or inverse-diagonal
                               stream) and each row's A p kept in shared memory between the
                               SpMV and the vector phase: 64208, 64404 (r and p kept too),
                               65208, 65404, 66404 (A p only; 66xxx at 4 blocks per SM);
                               up to about 2.8 M rows; the whole solve in one
                               thread-block cluster of 8 or 16 blocks of 1024 threads
                               (hardware cluster barriers, reductions through distributed
                               shared memory; for systems that sit in L2): 70204, 70404,
                               70802 (pipelined row loop, both modes), 80204, 80404 (MIXED
                               only, two-run 16-bit columns); 0 = autotuned
                               per matrix and mode (timed trial solves); -1 = chosen from the
                               mean row length
                               (no timing, so the choice does not depend on concurrent GPU work) */
    int32_t grid_blocks;    /* persistent-kernel blocks: 0 = as many as fit, or, with
                               spmv_config 0, the autotuner's choice among that and one or
                               two blocks per SM (cheaper grid barriers on small systems) */
    int32_t use_initial_guess; /* 1: start from x, 0: start from 0                      */
} grmp_solve_params;

typedef struct {
    int32_t status;          /* grmp_status of the solve                     */
    int32_t iterations;      /* inner (or plain) iterations                  */
    int32_t outer_iterations;/* FP64 refinement steps (MIXED)                */
    int32_t spmv_config;     /* SpMV configuration used (100*lanes + loads)  */
    int32_t grid_blocks;
    double final_relres;     /* ||b - A x|| / ||b|| in FP64 at exit          */
    double solve_ms;         /* device time of the solve                     */
} grmp_solve_stats;

/* Fill params with defaults mirroring default_solver_kwargs
 * (src/solvers.jl:38-59): abstol = reltol = 1e-12. */
int grmp_solve_params_default(grmp_solve_params *p);

/* Solve A x = b.  Stands in for init(LinearProblem(A, b), alg; abstol, reltol)
 * + LinearSolve.solve(cache) (src/solvers.jl:89-101, :658-661).  `x` is
 * overwritten.  Returns GRMP_ERR_NOT_CONVERGED (with x = the last iterate)
 * when the caps are hit; device-side waits are bounded (GRMP_ERR_TIMEOUT). */
int grmp_solve(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *params,
               grmp_solve_stats *stats);

/* y = A x in the given precision (diagnostic / residual check,
 * src/solvers.jl:664-668). */
int grmp_spmv(grmp_matrix A, int precision, grmp_vector x, grmp_vector y);

/* Largest system grmp_solve_fp64_noalloc accepts (rows). */
#define GRMP_NOALLOC_MAX_ROWS 262144

/* FP64 Jacobi-PCG like grmp_solve with mode GRMP_SOLVE_FP64, but without
 * any device-memory allocation: its work arrays live in a fixed scratch
 * area of about 10.8 MB that is part of the loaded library on each device.
 * No counterpart in the reference (its solves allocate freely).
 *   - For callers that must not allocate during a solve: hosts whose own
 *     memory pool has taken the device's free memory, or time-stepping loops
 *     that cannot afford an allocation failing or stalling mid-step.
 *   - Systems up to GRMP_NOALLOC_MAX_ROWS rows; larger ones are rejected
 *     with GRMP_ERR_INVALID_ARG.  params->mode must be GRMP_SOLVE_FP64
 *     (GRMP_ERR_UNSUPPORTED otherwise).  spmv_config 0 uses the matrix's
 *     tuned configuration if grmp_solve has tuned it, else a heuristic; no
 *     tuning runs here.
 *   - The first call on a device looks up the scratch address (set-up);
 *     make it before any stream capture on that device begins.
 *   - The grid-barrier counters, the status word and the diagonal check flag
 *     in the scratch must start at zero; every call zeroes them itself.
 *   - Calls that overlap in time on the same device (e.g. from two host
 *     threads with two contexts) share the one scratch area and race: the
 *     caller must serialise them.
 *   - stats->solve_ms is host wall time of the whole call. */
int grmp_solve_fp64_noalloc(grmp_matrix A, grmp_vector b, grmp_vector x, const grmp_solve_params *params,
                            grmp_solve_stats *stats);

/* ------------------------------------------------- batched Stokes (BR/P0) */

typedef struct {
    int32_t nproblems;
    const int32_t *row_offsets;  /* [nproblems+1] velocity rows of each problem (contiguous, disjoint) */
    const int32_t *cell_offsets; /* [nproblems+1] cells (= P0 pressure DoFs) of each problem          */
    double lambda;               /* iterated-penalty parameter                                        */
    int32_t sweeps;              /* maximum iterated-penalty sweeps                                   */
    double sweep_tol;            /* stop a problem when ||p_new - p|| <= sweep_tol ||p_new|| (0: all)  */
    int32_t mode;                /* velocity solver: GRMP_SOLVE_FP64 / MIXED (block PCG), DIRECT (FP64
                                    multifrontal factor per problem, residual refinement) or
                                    MIXED_DIRECT (FP32 factor per problem preconditioning FP64 CG,
                                    FP64 factor as the per-problem fallback; maxiter bounds the CG
                                    iterations of a sweep with 4 maxiter + 200)                     */
    double reltol;               /* inner solve: ||rhs - A u|| <= reltol ||rhs|| per sweep             */
    double inner_reltol;         /* MIXED: refinement trigger                                          */
    int32_t maxiter;             /* inner iteration cap per sweep                                       */
    int32_t block_threads;       /* threads per problem (0 = 512)                                       */
    int32_t split_penalty;       /* MIXED: 0 = A's FP32 values hold the whole velocity operator;
                                    1 = they hold (nu grad u, grad v) alone and the inner FP32 operator
                                    applies lambda (div R u, div R v) per cell in factored form
                                    sum_T lambda/|T| (D_T.u)(D_T.v), D_T[I] = int_T div phi_I, which
                                    stays exact on divergence-free fields (needed when lambda/nu is
                                    large: FP32 rounding of the assembled penalty swamps the viscous
                                    term there)                                                      */
} grmp_stokes_batch_params;

typedef struct {
    int32_t status;
    int32_t max_iterations;      /* largest per-problem inner iteration total */
    int64_t total_iterations;
    int32_t max_sweeps;
    int32_t failed_problems;     /* problems that hit a cap                   */
    double max_relres;           /* worst final inner relative residual       */
    double solve_ms;
    int32_t fp64_fallbacks;      /* MIXED: inner solves that stalled in FP32 and
                                    were finished by FP64 PCG from the same iterate;
                                    MIXED_DIRECT: problems refactored in FP64 (a
                                    non-positive FP32 pivot or a stalled CG) */
} grmp_stokes_batch_stats;

/* Iterated-penalty Stokes solve of many independent Bernardi-Raugel / P0
 * problems assembled into one block-diagonal system (the reference's
 * solve_fixpoint_subiterations! with subiterations [[1],[2]],
 * src/solvers.jl:1018-1250, on the operators of
 * examples/Example221_StokesIterated2D.jl:80-90 without convection):
 *   velocity:  (nu grad u, grad v) + lambda (div R u, div R v) = (f, R v) + (p, div v)
 *   pressure:  p <- p - lambda * (1/|T|) int_T div u,  then mean(p) = 0
 *              (FixedIntegralMean, src/globalconstraints.jl:23-44).
 * A: the assembled velocity matrix over an H1BR{2} or H1BR{3} space (terms
 * LAPLACE and RDIVRDIV) with Dirichlet rows eliminated; bf: the reconstructed
 * right-hand side (f, R v) with the same rows zeroed.  u (velocity, per row)
 * and p (pressure, per cell) are overwritten.  One thread block owns one
 * problem for the whole solve, so a problem's result is bit-identical alone
 * and inside any batch.  iterations_per_problem (optional, [nproblems]). */
int grmp_stokes_batch_solve(grmp_matrix A, grmp_vector bf, grmp_vector u, grmp_vector p,
                            const grmp_stokes_batch_params *params, int32_t *iterations_per_problem,
                            grmp_stokes_batch_stats *stats);

/* ---------------------------------------------------------------- serving */

typedef struct grmp_server_s *grmp_server;

/* One assembly + solve request (a solve_direct! of a linear problem,
 * src/solvers.jl:622-686).  All arrays are host arrays, copied at submit;
 * term cell coefficients must be host arrays (coef_on_device = 0). */
typedef struct {
    int dim;
    int32_t nverts;
    const double *coords;       /* [nverts][dim]                                                  */
    int32_t ncells;
    const int32_t *cells;       /* [ncells][dim+1]                                                */
    int fe_kind;
    int ncomponents;
    int32_t ndofs;              /* 0 with celldofs == NULL: counted on the device                 */
    const int32_t *celldofs;    /* [ncells][ndofs4cell], or NULL: the DoF map is built on the
                                   device from the mesh (H1P1 / H1P2, grmp_space_create_on_device) */
    int nterms;
    const grmp_bilinear_term *terms;
    grmp_rhs rhs;               /* cell_group not allowed                                          */
    int32_t nfixed;             /* -1: every boundary DoF, found on the device                     */
    const int32_t *fixed;       /* homogeneous Dirichlet DoFs (eliminated)                         */
    grmp_solve_params solve;
    uint64_t mesh_key;          /* 0: nothing stays on the device after the request.  Otherwise the
                                   request's mesh, DoF map, sparsity pattern, solver workspace and
                                   vectors stay resident in the slot that ran it, and a later
                                   request with the same key and operator structure (term kinds,
                                   symmetry, quadrature bonus) reuses them: only its coefficients,
                                   right-hand side and solve run.  A resident pattern is built
                                   with unit factors and no cell coefficients, so that it holds
                                   every later coefficient field (as the reference's refill of a
                                   kept matrix, src/fematrix.jl:220-232); a one-off request's
                                   pattern drops its own exact zeros.  The caller promises the same
                                   mesh and element under one key (the reference reuses a solver
                                   cache the same way, src/solvers.jl:906-911).  Resident data
                                   count against the budget; the least recently used entries of
                                   idle slots are dropped when a request would not fit.           */
} grmp_request;

typedef struct {
    int32_t status;             /* grmp_status of the request               */
    int32_t slot;               /* worker that ran it                       */
    int32_t iterations, outer_iterations;
    double final_relres;
    double queue_ms;            /* submit -> admission                       */
    double run_ms;              /* admission -> result                       */
    double latency_ms;          /* submit -> result                          */
    double solve_ms;            /* device time of the solve                  */
    int32_t ndofs;              /* DoFs of the solution (x_out's length)     */
    int32_t resident;           /* 1: the request reused resident data       */
} grmp_request_stats;

/* A serving loop with `nslots` concurrent slots (one stream each) on device
 * `device`, admitting requests while their estimated device footprint fits in
 * `hbm_budget_bytes` (0 = unlimited).  No reference counterpart. */
int grmp_server_create(int device, size_t hbm_budget_bytes, int nslots, grmp_server *out);
/* Device bytes the server reserves against its budget while running request
 * q (its admission estimate: matrix in both precisions, pattern, slot map,
 * incidence, mesh, vectors and solver workspace, with 25% margin). */
int grmp_server_request_bytes(const grmp_request *q, size_t *bytes);

/* Queue a request (copied); returns its id at once.  GRMP_ERR_BUDGET if it
 * can never fit. */
int grmp_server_submit(grmp_server srv, const grmp_request *req, int64_t *id);
/* Wait for a request (timeout_s < 0: forever); x_out [ndofs] receives the
 * solution (with a device-built DoF map, query stats->ndofs first: x_out may
 * be NULL).  Returns the request's status (GRMP_ERR_TIMEOUT if still
 * running after timeout_s; it can be waited for again). */
int grmp_server_wait(grmp_server srv, int64_t id, double timeout_s, double *x_out, grmp_request_stats *stats);
/* Stop the workers (running requests finish first) and free the server. */
int grmp_server_destroy(grmp_server srv);

#ifdef __cplusplus
}
#endif

#endif /* GRMP_H */
