/*
 * nuto_gpu.h — C ABI of the GB300 (sm_103a) element-assembly path for NuTo.
 *
 * One context (nuto_gpu_ctx) holds one cell group on one GPU: the coordinate elements of a CellStorage, the
 * DOF types with their numbering, the Dirichlet constraints, the integrand and its history, the CSR pattern of
 * the global tangent and the solver workspace. Every call is stream-ordered on the context's stream; pointers
 * named d_* are device pointers owned by the caller, all others are host pointers borrowed for the duration of
 * the call. A context is externally synchronised (one host thread at a time). Every function returns a status
 * code; NUTO_GPU_OK is 0 and nuto_gpu_last_error() gives the message of the last failure. No C++ exception
 * crosses this boundary.
 *
 * Reference interfaces replaced (paths relative to the NuTo project root):
 *   nuto_gpu_set_cells          CellStorage::AddCells                    nuto/mechanics/tools/CellStorage.cpp:6-16
 *                               IntegrationTypeTensorProduct<D>(n, GAUSS) nuto/mechanics/integrationtypes/IntegrationTypeTensorProduct.cpp:15-39
 *   nuto_gpu_add_dof_type       ElementFem::GetDofNumbering              nuto/mechanics/elements/ElementFem.h:58-70
 *                               DofNumbering::Build / DofInfo            nuto/mechanics/dofs/DofNumbering.cpp:32-58
 *   nuto_gpu_set_dirichlet      Constraint::Component + RhsRamp          nuto/mechanics/constraints/ConstraintCompanion.cpp:12-53
 *                               Constraints::GetSparseGlobalRhs          nuto/mechanics/constraints/Constraints.cpp:37-50
 *   nuto_gpu_build_pattern      pattern of SimpleAssembler::BuildMatrix + ToEigen
 *                                                                        nuto/mechanics/cell/SimpleAssembler.cpp:100-156
 *                                                                        nuto/mechanics/dofs/DofMatrixSparseConvertEigen.h:40-67
 *   nuto_gpu_set_integrand      MomentumBalance<D> + LinearElastic<D>     nuto/mechanics/integrands/MomentumBalance.h:14-53
 *                               MomentumBalance<D> + LocalIsotropicDamage nuto/mechanics/constitutive/LocalIsotropicDamage.h:33-143
 *                               GradientDamage<D, Constant|Decreasing>   nuto/mechanics/integrands/GradientDamage.h:25-186
 *   nuto_gpu_set_history        GradientDamage::mKappas / EvolutionImplicit::mKappas (public members)
 *   nuto_gpu_build_vector       SimpleAssembler::BuildVector(cells, dofs, Bind(integrand, &Gradient))
 *                                                                        nuto/mechanics/cell/SimpleAssembler.cpp:38-65
 *   nuto_gpu_build_matrix       SimpleAssembler::BuildMatrix(cells, dofs, Bind(integrand, &Hessian0)) + ToEigen
 *                                                                        nuto/mechanics/cell/SimpleAssembler.cpp:100-156
 *   nuto_gpu_update_history     TimeDependentProblem::UpdateHistory      nuto/mechanics/tools/TimeDependentProblem.cpp:78-85
 *   nuto_gpu_build_lumped_mass  SimpleAssembler::BuildDiagonallyLumpedMatrix + DynamicMomentumBalance::Hessian2
 *                                                                        nuto/mechanics/cell/SimpleAssembler.cpp:67-98
 *   nuto_gpu_add_boundary_cells / nuto_gpu_build_external_load
 *                               NeumannBc::ExternalLoad on boundary cells nuto/mechanics/integrands/NeumannBc.h:28-36
 *   nuto_gpu_set_constant_gradient  a constant gradient function          nuto/mechanics/tools/TimeDependentProblem.cpp:56-66
 *   nuto_gpu_eval_ip            Cell::Eval (post-processing of kappa, damage, strain, stress) nuto/mechanics/cell/Cell.h:80-93
 *   nuto_gpu_assemble_cell_vectors / _matrices
 *                               the scatter half of SimpleAssembler::BuildVector/BuildMatrix for caller-given cell
 *                               results (any CellInterface::VectorFunction/MatrixFunction)
 *   nuto_gpu_solve              Solve (C^T K C u = C^T f) + EigenSparseSolve nuto/mechanics/solver/Solve.cpp:8-34,
 *                                                                        nuto/math/EigenSparseSolve.cpp:22-73
 *   nuto_gpu_set_preconditioner (none: the reference factorises the matrix)
 *   nuto_gpu_do_step            QuasistaticSolver::DoStep (trial state, NewtonRaphson::Solve with LineSearch,
 *                               UpdateHistory)                           nuto/mechanics/tools/QuasistaticSolver.cpp:51-147,
 *                                                                        nuto/math/NewtonRaphson.h:62-94, nuto/math/LineSearch.h:38-63
 *   nuto_gpu_do_step_host       the same with the state vector and history in host memory (NuTo keeps mX on the host)
 */
#ifndef NUTO_GPU_H
#define NUTO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NUTO_GPU_OK 0
#define NUTO_GPU_EINVAL 1   /* invalid argument or unsupported combination */
#define NUTO_GPU_ENOMEM 2   /* device allocation failed */
#define NUTO_GPU_ENOCONV 3  /* Newton or Krylov did not converge (NewtonRaphson::NoConvergence) */
#define NUTO_GPU_ENAN 4     /* NaN/Inf in a residual or a Krylov scalar */
#define NUTO_GPU_ETIMEOUT 5 /* a bounded device wait gave up */
#define NUTO_GPU_ECUDA 6    /* CUDA runtime error */
#define NUTO_GPU_ESTATE 7   /* call out of order (e.g. build_matrix before build_pattern) */

/* interpolations: InterpolationQuadLinear, InterpolationBrickLinear, InterpolationBrickQuadratic */
#define NUTO_GPU_QUAD4 0
#define NUTO_GPU_HEX8 1
#define NUTO_GPU_HEX20 2

/* integrands */
#define NUTO_GPU_MB_LINEAR_ELASTIC 0 /* MomentumBalance<D> with LinearElastic<D> */
#define NUTO_GPU_MB_LOCAL_DAMAGE 1   /* MomentumBalance<D> with LocalIsotropicDamage<D> (EvolutionImplicit) */
#define NUTO_GPU_GRADIENT_DAMAGE 2   /* GradientDamage<D, interaction, DamageLawExponential> */

#define NUTO_GPU_PLANE_STRESS 0
#define NUTO_GPU_PLANE_STRAIN 1
#define NUTO_GPU_DAMAGE_FULL 0
#define NUTO_GPU_DAMAGE_UNILATERAL 1
#define NUTO_GPU_INTERACTION_CONSTANT 0
#define NUTO_GPU_INTERACTION_DECREASING 1

/* arithmetic of the tangent values and of the Krylov iteration */
#define NUTO_GPU_FP32 32
#define NUTO_GPU_FP64 64
#define NUTO_GPU_MIXED 48 /* nuto_gpu_do_step only: FP32 tangent and preconditioner, FP64 Krylov vectors */
/* nuto_gpu_build_matrix only: FP64 values with the law in FP64 and the node-pair products in double-float FP32
   arithmetic (about 1e-14 relative; Hex8 and Quad4, plain FP64 otherwise): the tangent of the exact final phase */
#define NUTO_GPU_FP64X 65

/* Krylov methods */
#define NUTO_GPU_SOLVER_AUTO 0     /* PCG for the symmetric integrands, GMRES otherwise */
#define NUTO_GPU_SOLVER_PCG 1      /* preconditioned CG */
#define NUTO_GPU_SOLVER_BICGSTAB 2 /* Jacobi-preconditioned BiCGStab (always Jacobi) */
#define NUTO_GPU_SOLVER_GMRES 3    /* restarted GMRES(80), right-preconditioned (flexible form) */

/* preconditioners of PCG and GMRES (nuto_gpu_set_preconditioner) */
#define NUTO_GPU_PRECOND_JACOBI 1 /* diagonal */
#define NUTO_GPU_PRECOND_AMG 2    /* aggregation multigrid V-cycle in FP32 (default) */

typedef struct nuto_gpu_ctx nuto_gpu_ctx;

/* Integrand and law parameters. The plane state applies to every 2D law of the integrand. */
typedef struct nuto_gpu_integrand
{
    int kind;               /* NUTO_GPU_MB_LINEAR_ELASTIC | NUTO_GPU_MB_LOCAL_DAMAGE | NUTO_GPU_GRADIENT_DAMAGE */
    int dim;                /* 2 or 3 */
    double E, nu;           /* LinearElastic / LinearElasticDamage */
    int plane_state;        /* NUTO_GPU_PLANE_STRESS | NUTO_GPU_PLANE_STRAIN */
    int damage_application; /* NUTO_GPU_DAMAGE_FULL | NUTO_GPU_DAMAGE_UNILATERAL */
    double kappa0, beta, alpha; /* DamageLawExponential(kappa0, beta, alpha) */
    double k;               /* ModifiedMisesStrainNorm(nu, k) */
    double c;               /* GradientDamage nonlocal parameter */
    int interaction;        /* NUTO_GPU_INTERACTION_CONSTANT | NUTO_GPU_INTERACTION_DECREASING */
    double R, eta;          /* NonlocalInteraction::Decreasing(R, eta) */
    int disp_slot;          /* DOF slot of the displacements */
    int eeq_slot;           /* DOF slot of the nonlocal equivalent strains (GRADIENT_DAMAGE only), else -1 */
} nuto_gpu_integrand;

/* Newton / Krylov options of nuto_gpu_do_step */
typedef struct nuto_gpu_step_options
{
    int precision;      /* NUTO_GPU_FP32: FP32 tangent + FP32 Krylov, FP64 residual and refinement;
                           NUTO_GPU_MIXED: FP32 tangent + preconditioner, FP64 Krylov vectors and accumulation;
                           NUTO_GPU_FP64: everything FP64 */
    int method;         /* NUTO_GPU_SOLVER_* */
    double newton_rtol; /* converged when |C^T r| <= max(newton_atol, newton_rtol * |C^T (r + K db)|_trial) */
    double newton_atol;
    int max_newton;     /* NewtonRaphson::Solve maxIterations (the reference uses 6) */
    int line_search;    /* 1: NuTo::NewtonRaphson::LineSearch (6 halvings), 0: plain Newton */
    double krylov_rtol; /* inner Krylov tolerance relative to |rhs| (the lower bound with forcing = 1) */
    int max_krylov;
    int forcing;        /* 0: every solve to krylov_rtol; 1: Eisenstat-Walker forcing terms (choice 1) */
    double exact_tangent_below; /* NUTO_GPU_FP32 only; > 0: once |C^T r| < exact_tangent_below * tolerance, the
                                   tangent of the remaining Newton iterations is assembled in FP64 and every
                                   solve refines against it (FP32 Krylov and preconditioner on its FP32
                                   rounding inside an FP64 refinement), so that the last Newton steps use the
                                   exact Jacobian; 0: off. Default 1e4: with the FP32 tangent alone the
                                   near-singular modes of a damaged zone converge only linearly, and a state
                                   at the 1e-8 residual can lie 1e-5 from the converged FP64 solution; with the
                                   exact last iterations it lies as close as the FP64 path's (below 1e-6) */
    double forcing_floor; /* forcing = 1 only: the forcing term is never below forcing_floor * tolerance / |C^T r|,
                             so the solve of the last Newton iteration leaves a linear residual of about
                             forcing_floor times the Newton tolerance. Default 0.5. Smaller values solve the last
                             system more tightly: the converged state then sits further below the tolerance, and
                             its distance to the exactly converged solution shrinks in proportion (the residual
                             test weighs the near-singular modes of a damaged zone only weakly) */
} nuto_gpu_step_options;

/* statistics of the last nuto_gpu_do_step / nuto_gpu_solve */
typedef struct nuto_gpu_stats
{
    int newton_iterations;
    int krylov_iterations;   /* summed over the step */
    int residual_evaluations;
    int matrix_assemblies;
    double final_residual;   /* |C^T r| at exit */
    double reference_residual;
    double ms_assemble_matrix;
    double ms_assemble_vector;
    double ms_krylov;
    double ms_total;
    double ms_spmv;          /* device time of the Krylov sparse matrix-vector products (CUDA events) */
    int64_t spmv_launches;
    int64_t kernel_launches; /* kernels launched by the step */
} nuto_gpu_stats;

/* ---- context ----------------------------------------------------------------------------------------- */
int nuto_gpu_create(nuto_gpu_ctx** ctx, int device, void* cuda_stream /* cudaStream_t or NULL */);
int nuto_gpu_destroy(nuto_gpu_ctx* ctx);
/* message of the last failure of ctx; with ctx == NULL the last failed nuto_gpu_create of this thread */
const char* nuto_gpu_last_error(const nuto_gpu_ctx* ctx);
int nuto_gpu_synchronize(nuto_gpu_ctx* ctx);
int nuto_gpu_version(void);

/* ---- cells, DOF types, constraints --------------------------------------------------------------------- */
/* Coordinate elements of the cells, cell id = row of coord_conn (CellStorage::AddCells). coords are
   n_coord_nodes x dim, coord_conn is n_cells x nodes-per-element (local node order of the interpolation). */
int nuto_gpu_set_cells(nuto_gpu_ctx* ctx, int dim, int geo_interp, int64_t n_coord_nodes, const double* coords,
                       int64_t n_cells, const int32_t* coord_conn, int gauss_points_per_direction);

/* A DOF type. dof_conn is n_cells x nodes-per-element of DOF-node ids, dof_numbers is n_dof_nodes x ncomp and
   holds NodeSimple::GetDofNumber(component) (components of a node must be consecutive numbers, which
   DofNumbering::Build guarantees). n_independent + n_dependent = n_dof_nodes * ncomp. The slot index returned
   is the position in the combined (ToEigen) order. */
int nuto_gpu_add_dof_type(nuto_gpu_ctx* ctx, int ncomp, int interp, int64_t n_dof_nodes, const int32_t* dof_conn,
                          const int32_t* dof_numbers, int64_t n_independent, int64_t n_dependent, int* slot);

/* Dirichlet (unit) constraints of one slot: dependent DOF numbers with rhs(t) = rhs_const + rhs_slope * t
   (RhsConstant / RhsRamp); the value is rounded through float like Constraints::GetSparseGlobalRhs. */
int nuto_gpu_set_dirichlet(nuto_gpu_ctx* ctx, int slot, int64_t n_equations, const int32_t* dependent_dofs,
                           const double* rhs_const, const double* rhs_slope);

/* Builds the CSR pattern of the combined matrix and the cell-to-CSR maps. Outputs the combined size and nnz. */
int nuto_gpu_build_pattern(nuto_gpu_ctx* ctx, int64_t* n_dofs, int64_t* nnz);
/* Copies the pattern to host arrays (row_ptr: n_dofs + 1, col_idx: nnz). The pattern is structurally
   symmetric, so these are also the column pointers / row indices of NuTo's column-major matrix. */
int nuto_gpu_copy_pattern(nuto_gpu_ctx* ctx, int64_t* row_ptr, int32_t* col_idx);
/* Device pointers of the pattern (valid until the context is destroyed). */
int nuto_gpu_pattern_device(nuto_gpu_ctx* ctx, const int64_t** d_row_ptr, const int32_t** d_col_idx);
/* Sizes of the solver's copy of the tangent (no counterpart in the reference): values of the padded pair layout
   the Krylov products stream (node row segments per slot pair padded to multiples of 4) and entries of the
   neighbour lists that drive the gathers; for traffic accounting. */
int nuto_gpu_solver_layout(const nuto_gpu_ctx* ctx, int64_t* padded_values, int64_t* neighbour_entries);
/* State of the multigrid preconditioner after the last solve (no counterpart in the reference): levels of the
   first DOF slot's hierarchy (0: not built) and whether the sweep ran as a CUDA graph (1) or kernel by kernel (0). */
int nuto_gpu_multigrid_info(const nuto_gpu_ctx* ctx, int* levels, int* graph_active);

/* Launch shapes chosen by the autotuner (no counterpart in the reference). The first FP32 tangent of a context
   times its node-row kernel with 2, 4 and 8 warps per block, the double-buffered variant (a grid of resident
   blocks) with 2 and 4 and the element-matrix form (cell matrices, then a row gather) with 2 and 4, and the first
   Krylov product per (value, vector) type pair times the padded-layout kernel with 4, 8 and 16 lanes per node; each
   keeps the fastest (environment NUTO_GPU_AUTOTUNE=0 keeps the defaults: 4 warps, node rows, 8 lanes). choices
   (6 ints): tangent warps per block, the tangent's form (0 node rows, 1 double-buffered, 2 element matrices), then
   the lanes per node for (FP32 values, FP32 vectors), (FP32, FP64), (FP64, FP32), (FP64, FP64); 0 = not tuned yet.
   times_ms (19 floats): the tangent with 2 / 4 / 8 warps, double-buffered with 2 / 4 warps, then per type pair the
   product with 4 / 8 / 16 lanes (one launch each), then the element-matrix form with 2 / 4 warps. */
int nuto_gpu_autotune_info(const nuto_gpu_ctx* ctx, int* choices, float* times_ms);
/* Iteration limit of every bounded device wait (no counterpart in the reference; default 4,194,304): the tensor-core
   tangent of Hex20 cells waits on its MMA completion barrier. A wait that runs out sets NUTO_GPU_ETIMEOUT in the
   context's status word, the kernel drains its work in flight (with a fixed limit), releases its tensor memory and
   returns; nuto_gpu_synchronize and nuto_gpu_do_step then return NUTO_GPU_ETIMEOUT and clear the word. A small limit
   makes the waits run out on purpose (tests). */
int nuto_gpu_set_spin_limit(nuto_gpu_ctx* ctx, long long iterations);

int nuto_gpu_set_integrand(nuto_gpu_ctx* ctx, const nuto_gpu_integrand* params);
int nuto_gpu_num_integration_points(const nuto_gpu_ctx* ctx);
/* history kappa: n_cells x n_ip doubles (host pointers) */
int nuto_gpu_set_history(nuto_gpu_ctx* ctx, const double* kappa);
int nuto_gpu_get_history(nuto_gpu_ctx* ctx, double* kappa);
/* Per-cell factor of the integrand's Young's modulus (host pointer, n_cells values > 0; NULL: 1 everywhere): cell e
   integrates with E_e = scale[e] * E, which scales its stress, material tangent and dsigma/domega, i.e. the
   displacement rows of its cell vector and matrix (the eeq rows do not depend on E). A heterogeneous modulus field,
   the parameter of the adjoint workload; NuTo gives each cell group one law, so the reference counterpart is one
   integrand per cell (nuto/mechanics/integrands/GradientDamage.h:25-60 with its own LinearElasticDamage). */
int nuto_gpu_set_cell_scale(nuto_gpu_ctx* ctx, const double* scale);

/* ---- hot path: device pointers, stream-ordered ---------------------------------------------------------- */
/* f = sum over cells of the integrand's Gradient (combined layout, all DOFs incl. dependent ones) */
int nuto_gpu_build_vector(nuto_gpu_ctx* ctx, const double* d_u, double* d_f);
/* CSR values of sum over cells of the integrand's Hessian0; d_values is nnz floats (FP32) or doubles (FP64) */
int nuto_gpu_build_matrix(nuto_gpu_ctx* ctx, const double* d_u, int precision, void* d_values);
/* Both at one state: the values of nuto_gpu_build_matrix(ctx, d_u, precision, d_values) and the vector of
   nuto_gpu_build_vector(ctx, d_u, d_f), bitwise the same as the two calls. NewtonRaphson::Solve needs the residual
   and the derivative at the same x (nuto/math/NewtonRaphson.h:62-94, through TimeDependentProblem::Gradient and
   Hessian0, nuto/mechanics/tools/TimeDependentProblem.cpp:56-76). The FP64 residual runs on a second stream of the
   context as a few resident blocks per SM beside the tangent's kernels (its work sits on the FP64 pipe, the
   tangent's on FP32 issue); both are complete, in the context's stream order, when the call's work is. precision
   NUTO_GPU_FP32 or NUTO_GPU_FP64. The first call of a context runs the two in sequence. */
int nuto_gpu_build_system(nuto_gpu_ctx* ctx, const double* d_u, int precision, void* d_values, double* d_f);
/* nuto_gpu_build_system with host buffers, the form SimpleAssembler::BuildVector/BuildMatrix return their results in
   (host Eigen objects, nuto/mechanics/cell/SimpleAssembler.cpp:38-156): h_u (n_dofs doubles) is copied in, the CSR
   values (nnz floats or doubles) and f (n_dofs doubles) are copied back, and the call returns when they are in host
   memory. The copy of the values starts as soon as the tangent is done, while the residual still runs. The state and
   results pass through device buffers of the context (allocated on the first call). Pass page-locked host memory for
   the copies to run asynchronously; pageable memory works, through the driver's staging. */
int nuto_gpu_build_system_host(nuto_gpu_ctx* ctx, const double* h_u, int precision, void* h_values, double* h_f);
/* The FP32 values of nuto_gpu_build_matrix(ctx, d_u, NUTO_GPU_FP32, d_values), computed without allocating any
   memory: the integration-point records go to a fixed 16 MiB device array inside the library instead of a buffer
   of the context. For callers that must not allocate device memory once set up. Limit: cells x integration points
   x record size <= 4,194,304 floats (12,192 Hex8 gradient-damage cells, 2,099 Hex20 local-damage cells); larger
   meshes get NUTO_GPU_EINVAL. Call nuto_gpu_build_matrix with NUTO_GPU_FP32 once first: it completes the set-up
   that allocates (NUTO_GPU_ESTATE otherwise). The first call on each device also looks up the array's address,
   so make it before any stream capture. The array is shared by all contexts on a device: calls that can overlap
   (other streams, other host threads) race and must be serialised by the caller. No counterpart in the
   reference. */
int nuto_gpu_build_matrix_noalloc(nuto_gpu_ctx* ctx, const double* d_u, float* d_values);
/* kappa <- max(kappa, kappa(u)) at every integration point */
int nuto_gpu_update_history(nuto_gpu_ctx* ctx, const double* d_u);
/* Lumped mass: SimpleAssembler::BuildDiagonallyLumpedMatrix (nuto/mechanics/cell/SimpleAssembler.cpp:67-98) of
   DynamicMomentumBalance<D>::Hessian2 (nuto/mechanics/integrands/DynamicMomentumBalance.h:22-30) with density rho:
   per cell the diagonal of rho N^T N det J w, scaled by (sum of all entries / sum of the diagonal) / components,
   summed into d_m (combined layout; the displacement rows, zero elsewhere). */
int nuto_gpu_build_lumped_mass(nuto_gpu_ctx* ctx, double rho, double* d_m);
/* Boundary cells for NeumannBc<D>::ExternalLoad (nuto/mechanics/integrands/NeumannBc.h:28-36): Line2 faces in 2D
   or Quad4 faces in 3D on the context's coordinate nodes (coord_conn, n_faces x nodes_per_face) and on the DOF
   nodes of a displacement slot (dof_conn), integrated with the codimension-1 Jacobian of
   nuto/mechanics/cell/Jacobian.h:51-88 and a tensor Gauss rule. *group receives the group index. */
int nuto_gpu_add_boundary_cells(nuto_gpu_ctx* ctx, int slot, int64_t n_faces, int nodes_per_face,
                                const int32_t* coord_conn, const int32_t* dof_conn, int gauss_points_per_direction,
                                int* group);
/* f = sum over the group's cells of ExternalLoad = N^T p det J w (SimpleAssembler::BuildVector over boundary cells,
   nuto/mechanics/cell/SimpleAssembler.cpp:38-65); traction p has dim entries (host), d_f combined layout. */
int nuto_gpu_build_external_load(nuto_gpu_ctx* ctx, int group, const double* traction, double* d_f);
/* A constant vector added to the residual of nuto_gpu_do_step, R = f_int(u) + g, as a u-independent gradient
   function of TimeDependentProblem::AddGradientFunction (nuto/mechanics/tools/TimeDependentProblem.cpp:56-66)
   would add it (e.g. g = -external load for force-driven steps). d_g == NULL removes it. */
int nuto_gpu_set_constant_gradient(nuto_gpu_ctx* ctx, const double* d_g);
/* Values at every integration point for post-processing: Cell::Eval (nuto/mechanics/cell/Cell.h:80-93) with
   GradientDamage::Kappa (nuto/mechanics/integrands/GradientDamage.h:127-130), the damage law, Nabla::Strain and the
   law's stress. d_out is n_cells x n_ip x width doubles (width: Voigt size for strain and stress, else 1). */
#define NUTO_GPU_IP_KAPPA 0  /* max(kappa history, eeq) / max(kappa history, local equivalent strain) */
#define NUTO_GPU_IP_DAMAGE 1 /* omega(kappa) of DamageLawExponential, 0 for linear elasticity */
#define NUTO_GPU_IP_STRAIN 2 /* engineering strain, Voigt order */
#define NUTO_GPU_IP_STRESS 3 /* stress of the law (LinearElastic, LinearElasticDamage with omega) */
#define NUTO_GPU_IP_EEQ 4    /* nonlocal eeq (gradient damage), else the local modified-Mises equivalent strain */
int nuto_gpu_eval_ip(nuto_gpu_ctx* ctx, const double* d_u, int quantity, double* d_out);
/* scatter of caller-given cell vectors (n_cells x n_local doubles, slot-major, node, component) */
int nuto_gpu_assemble_cell_vectors(nuto_gpu_ctx* ctx, const double* d_cell_vectors, double* d_f);
/* scatter of caller-given cell matrices (n_cells x n_local x n_local doubles, row-major) into CSR values */
int nuto_gpu_assemble_cell_matrices(nuto_gpu_ctx* ctx, const double* d_cell_matrices, int precision,
                                    void* d_values);

/* Solves C^T K C y = C^T b for the constrained system of the CSR values d_values (Dirichlet C: the constrained
   rows and columns are eliminated) and writes x = C y (zero at dependent DOFs). */
int nuto_gpu_solve(nuto_gpu_ctx* ctx, int precision, int method, const void* d_values, const double* d_b,
                   double* d_x, double rtol, int max_iterations, int* iterations, double* relative_residual);
/* y = K x for the CSR values d_values (FP32 or FP64) and FP64 device vectors, the product of the Krylov solvers
   and the Newton refinement (padded pair layout, 16-byte value loads); no counterpart in the reference, where
   Eigen's SparseMatrix * VectorXd does it. compensated = 1 (FP32 values only) forms the sums in compensated FP32
   (about 1e-14 relative to sum |K x|) instead of FP64 arithmetic. */
int nuto_gpu_spmv(nuto_gpu_ctx* ctx, int precision, const void* d_values, const double* d_x, double* d_y,
                  int compensated);
/* Preconditioner of the PCG and GMRES solves of nuto_gpu_solve and nuto_gpu_do_step (NUTO_GPU_PRECOND_*). The
   multigrid hierarchy (spatial aggregates of the DOF nodes, piecewise-constant transfer per component) is built
   on the first solve after build_pattern; its coarse operators are rebuilt once per tangent. No counterpart in
   the reference, which factorises the matrix (EigenSparseSolve.cpp:22-73). */
int nuto_gpu_set_preconditioner(nuto_gpu_ctx* ctx, int preconditioner);

/* ---- discrete adjoint of the load path (no counterpart in the reference) -------------------------------- */
/* The reverse sweep of the gradient-damage load path, one load step at a time, for a loss L(u_N) after N load steps
   and the parameters p = (per-cell Young's modulus E_e = scale[e] * E, kappa0, beta). For load step n, with the
   context's history set to kappa_{n-1} (nuto_gpu_history_device) and the step's converged state u_n:
     1. nuto_gpu_adjoint_history_load(u_n, kbar, ubar): ubar += sum over the loading points (eeq >= kappa_{n-1}) of
        kbar N on the eeq rows (kbar: n_cells x n_ip, the history adjoint carried from step n + 1; zero at n = N,
        where ubar = dL/du_N);
     2. assemble K(u_n) (nuto_gpu_build_matrix, FP64), transpose it (nuto_gpu_transpose_values) and solve
        K^T lambda = ubar on the independent DOFs (nuto_gpu_solve);
     3. nuto_gpu_adjoint_step(u_n, lambda, kbar, kbar_prev, grad_e, grad_params): grad_e[e] += dL/dE_e,
        grad_params[0..1] += dL/dkappa0, dL/dbeta of the step, and kbar_prev = the history adjoint for step n - 1.
   The forward it differentiates: QuasistaticSolver::DoStep (nuto/mechanics/tools/QuasistaticSolver.cpp:116-147)
   with GradientDamage::Gradient/Hessian0/Update (nuto/mechanics/integrands/GradientDamage.h:70-125). Gradient
   damage on Quad4 / Hex8 cells. All sums run in a fixed order (bitwise reproducible). */
/* K^T on the same (structurally symmetric) pattern: d_transposed[p] = d_values[position of the transposed entry]. */
int nuto_gpu_transpose_values(nuto_gpu_ctx* ctx, int precision, const void* d_values, void* d_transposed);
/* Device pointer of the context's history kappa (n_cells x n_ip doubles), e.g. to restore a checkpoint. */
int nuto_gpu_history_device(nuto_gpu_ctx* ctx, double** d_kappa);
int nuto_gpu_adjoint_history_load(nuto_gpu_ctx* ctx, const double* d_u, const double* d_kbar, double* d_ubar);
int nuto_gpu_adjoint_step(nuto_gpu_ctx* ctx, const double* d_u, const double* d_lambda, const double* d_kbar,
                          double* d_kbar_prev, double* d_grad_e, double* d_grad_params);

/* ---- quasistatic driver ------------------------------------------------------------------------------ */
int nuto_gpu_default_step_options(nuto_gpu_step_options* opts);
/* state x (combined layout, host) and the global time; resets the history to zero when reset_history != 0 */
int nuto_gpu_set_state(nuto_gpu_ctx* ctx, const double* x, double global_time, int reset_history);
int nuto_gpu_get_state(nuto_gpu_ctx* ctx, double* x, double* global_time);
/* Device pointer of the resident state vector (n_dofs doubles). */
int nuto_gpu_state_device(nuto_gpu_ctx* ctx, double** d_x);
/* QuasistaticSolver::DoStep(newGlobalTime) on the resident state; on success the state and history advance
   and *newton_iterations holds the iteration count. NUTO_GPU_ENOCONV leaves state and history unchanged. */
int nuto_gpu_do_step(nuto_gpu_ctx* ctx, double new_global_time, const nuto_gpu_step_options* opts,
                     int* newton_iterations);
/* The same with host buffers: x_in/kappa_in are uploaded, the step runs, x_out/kappa_out are downloaded
   (kappa pointers may be NULL to keep the resident history). */
int nuto_gpu_do_step_host(nuto_gpu_ctx* ctx, double new_global_time, const nuto_gpu_step_options* opts,
                          const double* x_in, const double* kappa_in, double* x_out, double* kappa_out,
                          int* newton_iterations);
int nuto_gpu_get_stats(const nuto_gpu_ctx* ctx, nuto_gpu_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* NUTO_GPU_H */
