/*
 * nlgpu: GB300 (sm_103a) implementation of NonLocFEM's nonlocal thermal hot
 * path behind a plain C ABI.
 *
 * Every entry point takes plain host pointers and sizes (no C++ or CUDA types
 * in the signatures) and returns an nlgpu_status.  A context (nlgpu_ctx) owns
 * the device copies of one problem: mesh, neighbour lists, matrices,
 * preconditioner and solver vectors.  One context per host thread; calls on
 * one context are serialised on the context's CUDA stream.
 *
 * Index conventions follow the reference application: node and element
 * numbers are int64 on the boundary (mesh_2d<T, I> with I = int64_t in the
 * reference's tests), matrix row pointers and column indices are int64
 * (Eigen::SparseMatrix<T, RowMajor, J> with J = int64_t, NonLocFEM/main.cpp:15).
 * Matrices cross the boundary in the reference's storage: the upper triangle
 * of the symmetric "inner" part, full rows of the "bound" part, CSR with
 * sorted columns (conductivity_matrix_2d.hpp:39-72).
 */
#ifndef NLGPU_H
#define NLGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nlgpu_ctx nlgpu_ctx;

/* Status codes.  The reference throws std::domain_error / std::logic_error;
 * across the C ABI those become NLGPU_ERR_ARG / NLGPU_ERR_STATE. */
enum {
    NLGPU_OK = 0,
    NLGPU_ERR_ARG = 1,          /* invalid argument (sizes, indices, kinds) */
    NLGPU_ERR_CUDA = 2,         /* a CUDA runtime call failed (no device, launch error, ...) */
    NLGPU_ERR_UNSUPPORTED = 3,  /* valid input outside what this build implements */
    NLGPU_ERR_STATE = 4,        /* call order violated (e.g. solve before assembly) */
    NLGPU_ERR_NUMERICAL = 5,    /* factorisation breakdown after all diagonal shifts */
    NLGPU_ERR_NO_CONVERGENCE = 6, /* iteration limit reached before the tolerance */
    NLGPU_ERR_OUT_OF_MEMORY = 7,
    NLGPU_ERR_TIMEOUT = 8       /* a bounded device-side wait gave up */
};

/* element_2d_t numbering (libraries/mesh/mesh_2d/elements_set.hpp:22-28) */
enum { NLGPU_BILINEAR = 2, NLGPU_QUADRATIC_SERENDIPITY = 3 };

/* influence kinds (libraries/solvers/solver_2d/influence_functions_2d.hpp:39-148) */
enum { NLGPU_INFLUENCE_CONSTANT = 0, NLGPU_INFLUENCE_POLYNOMIAL = 1,
       NLGPU_INFLUENCE_EXPONENTIAL = 2, NLGPU_INFLUENCE_FAST_POLYNOMIAL = 3 };

/* conductivity kinds (libraries/solvers/solver_2d/thermal/thermal_parameters_2d.hpp:8-23);
 * anisotropic components are ordered XX, YY, XY (libraries/constants/nonlocal_constants.hpp:9) */
enum { NLGPU_CONDUCTIVITY_ISOTROPIC = 0, NLGPU_CONDUCTIVITY_ORTHOTROPIC = 1, NLGPU_CONDUCTIVITY_ANISOTROPIC = 2 };

/* diameter_expanding_strategy (libraries/mesh/mesh_2d/find_neighbours.hpp:7) */
enum { NLGPU_EXPAND_NO = 0, NLGPU_EXPAND_MAX = 1, NLGPU_EXPAND_MIN = 2, NLGPU_EXPAND_MEAN = 3 };

/* assemble_part (libraries/solvers/solver_2d/base/matrix_assembler_2d.hpp:15-19) */
enum { NLGPU_PART_LOCAL = 0, NLGPU_PART_FULL = 2 };

/* boundary condition kinds (thermal_boundary_conditions_2d.hpp:9-98): temperature_2d,
 * flux_2d, convection_2d, radiation_2d, combined_flux_2d */
enum { NLGPU_BC_TEMPERATURE = 0, NLGPU_BC_FLUX = 1, NLGPU_BC_CONVECTION = 2, NLGPU_BC_RADIATION = 3,
       NLGPU_BC_COMBINED_FLUX = 4 };

/* matrices that can be copied out */
enum { NLGPU_MATRIX_INNER = 0, NLGPU_MATRIX_BOUND = 1, NLGPU_MATRIX_LOCAL = 2 };

/* preconditioners of the conjugate gradient */
/* ILLT_LEARNED: ILLT plus the learned correction (see nlgpu_mpnn_*); it always
 * runs in the mixed-precision flexible CG */
enum { NLGPU_PRECONDITIONER_IDENTITY = 0, NLGPU_PRECONDITIONER_ILLT = 1, NLGPU_PRECONDITIONER_ILLT_LEARNED = 2 };

/* precision of the solve */
enum { NLGPU_PRECISION_FP64 = 0, NLGPU_PRECISION_MIXED = 1 };

/* MIXED: how the FP32 ILLT application solves its two triangular systems.
 * k > 0: k Jacobi sweeps per triangle (the first k + 1 terms of the Neumann
 * series of each triangular inverse; fully parallel passes); < 0: exact
 * level-scheduled substitution, as the FP64 path.  0 in the options selects
 * the default below. */
#define NLGPU_DEFAULT_TRIANGULAR_SWEEPS 6
#define NLGPU_EXACT_TRIANGULAR_SWEEPS (-1)

/* Nonlocal model of one material: model_parameters<2, T> (equation_parameters.hpp:18-24)
 * plus its influence function and constant conductivity (parameter_2d). */
typedef struct nlgpu_model_2d {
    int influence;            /* NLGPU_INFLUENCE_* */
    int n;                    /* powered-distance exponent (2 = Euclidean) */
    int p;                    /* polynomial / exponential exponent */
    double q;                 /* polynomial power or exponential rate */
    double radius[2];         /* nonlocal radii r1, r2 */
    double local_weight;      /* p1; the model is nonlocal when p1 < 0.999 */
    int conductivity_kind;    /* NLGPU_CONDUCTIVITY_* */
    double conductivity[3];   /* lambda | (lx, ly) | (xx, yy, xy) */
} nlgpu_model_2d;

typedef struct nlgpu_solve_options {
    double tolerance;         /* relative residual target (|b - Ax| / |b|) */
    int64_t max_iterations;
    int preconditioner;       /* NLGPU_PRECONDITIONER_* */
    int precision;            /* NLGPU_PRECISION_* */
    double inner_tolerance;   /* MIXED: relative reduction of each FP32 inner solve (<= 0: 1e-2) */
    int triangular_sweeps;    /* MIXED: see NLGPU_DEFAULT_TRIANGULAR_SWEEPS (0: the default) */
    int coarse_aggregates;    /* MIXED with ILLT: 0 none; > 0 adds a coarse-space correction over about
                                 that many node aggregates (no counterpart in the reference, whose
                                 preconditioner is ILLT alone) */
    double coarse_aspect;     /* width / height of the aggregates' grid cells; <= 0: (lambda_x /
                                 lambda_y)^0.7 for an orthotropic conductivity, 1 otherwise */
} nlgpu_solve_options;

typedef struct nlgpu_solve_report {
    int64_t iterations;       /* CG iterations */
    double residual;          /* final |b - Ax| / |b| (FP64, recomputed) */
    double reference_residual;/* sqrt(r.z) / |b|, the reference's stopping measure */
    int preconditioner_ok;    /* 0 if ILLT failed and identity was used */
    int preconditioner_shifts;/* diagonal-shift attempts used by the factorisation */
    int64_t nnz_inner;        /* stored entries of the upper inner matrix */
    int64_t nnz_solver;       /* stored entries of the matrix the SpMV reads */
    int64_t element_pairs;    /* sum over elements of the neighbour count */
    double seconds_neighbours, seconds_pattern, seconds_assembly, seconds_boundary,
           seconds_preconditioner, seconds_solve, seconds_total;
    int64_t outer_iterations; /* MIXED: FP64 refinement steps (iterations counts the inner ones) */
    int learned_fallback;     /* ILLT_LEARNED: 1 when the correction was gated off or stalled */
    int column_bytes;         /* MIXED: bytes per column index the FP32 SpMV reads (2: 16-bit row offsets) */
    int64_t nonlinear_iterations; /* radiation: fixed-point steps (0 for a linear problem) */
    int neumann;              /* 1 for a pure Neumann problem (integral condition) */
    int64_t nnz_fp32;         /* MIXED: entries the FP32 SpMV reads (the strictly upper part with
                                 NLGPU_OPTION_FP32_SYMMETRIC, else nnz_solver) */
    int fp32_symmetric;       /* MIXED: 1 when the FP32 SpMV reads the strictly upper part */
} nlgpu_solve_report;

/* ---- library ------------------------------------------------------------ */
const char* nlgpu_status_string(int status);
/* Message of the last failed call on the calling thread ("" if none). */
const char* nlgpu_last_error(void);
/* Device count seen by the CUDA runtime (0 when no GPU is visible). */
int nlgpu_device_count(int* count);
/* Number of kernels this library launched in the calling process so far. */
int64_t nlgpu_kernel_launches(void);
/* Selects the CUDA device of the calling thread for contexts created after it. */
int nlgpu_set_device(int device);

/* ---- context ------------------------------------------------------------ */
/* Creates a context on the current device.  `stream` is a cudaStream_t to run
 * on, or NULL for a stream the context creates and owns. */
int nlgpu_create(nlgpu_ctx** ctx, void* stream);
int nlgpu_destroy(nlgpu_ctx* ctx);
int nlgpu_synchronize(nlgpu_ctx* ctx);

/* ---- mesh: mesh_2d<T, I>::mesh_2d + init (libraries/mesh/mesh_2d/mesh_2d.hpp:83-108)
 * nodes: n_nodes x 2 (x, y); elements: n_elements x nodes_per_element in the
 * reference's local node order; one element type per mesh. */
int nlgpu_mesh_2d(nlgpu_ctx* ctx, int element_type, int64_t n_nodes, const double* nodes,
                  int64_t n_elements, const int64_t* elements);
/* Quadrature data as mesh_2d stores it: coordinates [e][q][2], |J| [e][q],
 * derivatives dN.adj(J) [e][i][q][2] (mesh_container_2d_utils.hpp:101-123).
 * Any pointer may be NULL. */
int nlgpu_get_quadrature(nlgpu_ctx* ctx, double* qcoords, double* jacobians, double* derivatives);
/* Element basis tables: qN, qNxi, qNeta [i][q], weights [q], N_i(0,0) [i]
 * (element_2d_integrate.hpp:69-106).  sizes: nodes_per_element, qnodes. */
int nlgpu_get_basis(nlgpu_ctx* ctx, int* nodes_per_element, int* qnodes, double* qN, double* qNxi,
                    double* qNeta, double* weights, double* centre);

/* ---- mesh files: mesh_parser<T, I, mesh_format::SU2>::parse (su2_parser.hpp:165-195)
 * Reads an SU2 file into the reference's mesh_container_2d numbering: the
 * element lines pass through the same hashed containers as in the reference,
 * so 2D elements, boundary (1D) elements and groups come out in the
 * reference's order for the same file.  2D elements listed in no 2D marker
 * form the group "DEFAULT".  Host code; needs no GPU. */
typedef struct nlgpu_su2 nlgpu_su2;
int nlgpu_su2_read(const char* path, nlgpu_su2** mesh);
int nlgpu_su2_free(nlgpu_su2* mesh);
/* Message of the last failed nlgpu_su2_read on the calling thread. */
const char* nlgpu_su2_last_error(void);
/* Any output may be NULL.  element_type: NLGPU_BILINEAR or
 * NLGPU_QUADRATIC_SERENDIPITY when every 2D element has that type, else -1
 * (nodes_per_element 0 when the 2D types differ). */
int nlgpu_su2_info(const nlgpu_su2* mesh, int64_t* n_nodes, int64_t* n_elements_2d, int* nodes_per_element,
                   int* element_type, int* n_groups);
/* nodes [n_nodes][2] */
int nlgpu_su2_nodes(const nlgpu_su2* mesh, double* nodes);
/* 2D elements [n_elements_2d][nodes_per_element], local node order, the
 * container's element numbering (ready for nlgpu_mesh_2d). */
int nlgpu_su2_elements_2d(const nlgpu_su2* mesh, int64_t* elements);
/* Group g (0 <= g < n_groups) in the container's group order: its name
 * (NUL-terminated; name_capacity bytes available), dimension (1: boundary
 * line elements, 2: area elements), first element and count in the
 * container's numbering (1D elements are numbered after the 2D ones), nodes
 * per element, and the elements' nodes [count][nodes_per_element] in local
 * order (end, [middle,] end for line elements: ready for
 * nlgpu_add_boundary_2d).  Any output may be NULL. */
int nlgpu_su2_group(const nlgpu_su2* mesh, int g, char* name, int64_t name_capacity, int* dimension,
                    int64_t* first, int64_t* count, int* nodes_per_element, int64_t* nodes);

/* ---- node renumbering ------------------------------------------------------
 * mesh::utils::cuthill_mckee (cuthill_mckee.hpp:166-171): the Cuthill-McKee
 * order of the node graph (nodes coupled through an element when only_local
 * or the model is local, else through an element and its neighbours, as the
 * assembled matrix couples them), started from the first node of smallest
 * degree.  permutation [n_nodes]: permutation[old] = new.  reverse != 0
 * returns the inverse permutation, as the reference does.  The nonlocal graph
 * needs the neighbour search (run here if it has not run).  A graph that is
 * not connected is rejected (NLGPU_ERR_UNSUPPORTED). */
int nlgpu_cuthill_mckee(nlgpu_ctx* ctx, int only_local, int reverse, int64_t* permutation);
/* mesh_2d::renumbering (mesh_2d.hpp:258-262, mesh_container_2d.hpp:333-350):
 * node i becomes node permutation[i]: coordinates, element connectivity,
 * boundary groups and per-node Dirichlet values move with it; neighbour lists
 * (per element) stay; matrices are assembled afresh on the next call. */
int nlgpu_renumbering(nlgpu_ctx* ctx, const int64_t* permutation);

/* ---- model ---------------------------------------------------------------- */
int nlgpu_set_model_2d(nlgpu_ctx* ctx, const nlgpu_model_2d* model);
/* Spatially varying isotropic conductivity, one value per quadrature point
 * [e][q] (evaluate_conductivity.hpp:9-48).  With a nonlocal model this makes
 * the problem non-symmetric (problem_settings.hpp:32-34). */
int nlgpu_set_conductivity_field(nlgpu_ctx* ctx, const double* values);
/* Heat capacity and density for the nonstationary solver (parameter_2d). */
int nlgpu_set_capacity(nlgpu_ctx* ctx, double capacity, double density);

/* ---- neighbours: mesh::find_neighbours (find_neighbours.hpp:120-160) ------- */
/* Runs the bucketed centre-distance search with the widened radius.  Outputs
 * (may be NULL): the widened radii [2] and the total number of pairs. */
int nlgpu_find_neighbours(nlgpu_ctx* ctx, int strategy, double* search_radius, int64_t* pairs);
/* Neighbour lists in the reference's order: offsets [n_elements + 1], list [pairs]. */
int nlgpu_get_neighbours(nlgpu_ctx* ctx, int64_t* offsets, int64_t* list);

/* ---- boundary conditions and right-hand side ------------------------------- */
/* One boundary group: n_edges line elements of nodes_per_edge (2 or 3) nodes,
 * local order (end, [middle,] end).  kind NLGPU_BC_TEMPERATURE with a constant
 * value (node_values may give one value per listed node instead), or
 * NLGPU_BC_FLUX with a constant flux (thermal_boundary_conditions_2d.hpp:25-39).
 * Groups apply in the order added; a node in two temperature groups keeps the
 * first non-zero value (boundary_condition_first_kind_2d.hpp:16-26). */
int nlgpu_add_boundary_2d(nlgpu_ctx* ctx, int kind, int64_t n_edges, int nodes_per_edge,
                          const int64_t* edges, double value, const double* node_values);
/* A second-kind group of any flux kind (thermal_boundary_conditions_2d.hpp:25-98):
 *   NLGPU_BC_FLUX           flux q;
 *   NLGPU_BC_CONVECTION     heat transfer alpha and ambient temperature T_a: the
 *                           flux alpha T_a, and alpha int N_i N_j on the edges in
 *                           the matrix (convection_condition_2d.hpp:11-31);
 *   NLGPU_BC_RADIATION      emissivity eps: sigma eps T^4 leaves through the edges,
 *                           solved by the reference's fixed-point loop
 *                           (radiation_condition_2d.hpp:59-104,
 *                           stationary_heat_equation_solver_2d.hpp:66-116);
 *   NLGPU_BC_COMBINED_FLUX  all three (combined_flux_2d).
 * A stationary problem whose groups are all NLGPU_BC_FLUX (or that has none) is
 * a pure Neumann problem: the temperature is fixed by the integral condition
 * int T = energy (conductivity_matrix_2d.hpp:83-104), after the check that the
 * fluxes balance (|sum f| <= 1e-10, stationary_heat_equation_solver_2d.hpp:38-41).
 * A convection or radiation edge that shares a node with a temperature group is
 * rejected (NLGPU_ERR_UNSUPPORTED) when the solve starts: the reference then
 * inserts couplings into the Dirichlet rows and columns that this library does
 * not reproduce. */
int nlgpu_add_flux_boundary_2d(nlgpu_ctx* ctx, int kind, int64_t n_edges, int nodes_per_edge, const int64_t* edges,
                               double flux, double heat_transfer, double ambient_temperature, double emissivity);
/* stationary_equation_parameters_2d (stationary_heat_equation_solver_2d.hpp:19-26):
 * the radiation loop stops after max_iterations or when the relative change of
 * the temperature or the norm of the residual falls to tolerance (defaults
 * 1e-8, 100); energy is int T for a pure Neumann problem (default 0);
 * initial_temperature [n_nodes] (may be NULL: zero) starts the radiation loop. */
int nlgpu_set_stationary_parameters(nlgpu_ctx* ctx, double tolerance, int64_t max_iterations, double energy,
                                    const double* initial_temperature);
/* Rows of the stationary system: n_nodes, or n_nodes + 1 for a pure Neumann
 * problem (the reference's Lagrange row; nlgpu_get_matrix and nlgpu_get_rhs then
 * return n_nodes + 1 rows).  Valid after assembly. */
int nlgpu_get_system_rows(nlgpu_ctx* ctx, int64_t* rows);
/* Volume source: constant value, or one value per quadrature point [e][q] when
 * per_qnode is not NULL (right_part_2d.hpp:10-35). */
int nlgpu_set_source(nlgpu_ctx* ctx, double value, const double* per_qnode);
/* Overrides the Dirichlet value of each Dirichlet node (values [n_nodes]). */
int nlgpu_set_dirichlet_values(nlgpu_ctx* ctx, const double* values);
int nlgpu_clear_boundaries(nlgpu_ctx* ctx);

/* ---- assembly: conductivity_matrix_2d::compute (conductivity_matrix_2d.hpp:166-193)
 * part NLGPU_PART_FULL assembles p1*K_local + (1-p1)*K_nonlocal into the
 * inner/bound pair; NLGPU_PART_LOCAL assembles p1*K_local (the matrix the
 * ILLT preconditioner is built from).  Dirichlet rows get a unit diagonal. */
int nlgpu_conductivity_matrix_2d(nlgpu_ctx* ctx, int part, int64_t* nnz_inner, int64_t* nnz_bound);
/* Copies a matrix out in the reference's CSR storage (see top of file). */
int nlgpu_get_matrix(nlgpu_ctx* ctx, int which, int64_t* rowptr, int64_t* col, double* val);
/* Right-hand side after boundary conditions: flux and source integrals,
 * f -= K_bound x_D, f[D] = x_D (boundary_condition_first_kind_2d.hpp:50-59).
 * rhs_init (may be NULL) receives the vector before the first-kind step. */
int nlgpu_get_rhs(nlgpu_ctx* ctx, double* rhs, double* rhs_init);

/* ---- heat_equation_solution_2d::calc_flux (heat_equation_solution_2d.hpp:99-137)
 * Nodal heat flux of a temperature field [n_nodes] on the context's mesh and
 * model: -Lambda grad T at the quadrature points, for a nonlocal model mixed
 * p1 local + (1 - p1) influence-weighted average over the neighbours'
 * quadrature points, then averaged to the nodes from the Gauss point nearest
 * to each node, weighted by element area (mesh_2d_utils.hpp:82-101).
 * Runs the neighbour search first if the model is nonlocal and it has not
 * run.  flux_x, flux_y: [n_nodes]. */
int nlgpu_calc_flux(nlgpu_ctx* ctx, const double* temperature, double* flux_x, double* flux_y);

/* ---- solve: stationary_heat_equation_solver_2d (stationary_heat_equation_solver_2d.hpp:46-120)
 * Runs neighbours (if not yet run), both assemblies, boundary conditions,
 * ILLT(p1 K_local) and preconditioned CG; writes the nodal temperature
 * [n_nodes].  report may be NULL. */
int nlgpu_stationary_2d(nlgpu_ctx* ctx, const nlgpu_solve_options* options, double* temperature,
                        nlgpu_solve_report* report);
/* Only the solve stage on the already assembled system (for timing it alone). */
int nlgpu_solve_assembled(nlgpu_ctx* ctx, const nlgpu_solve_options* options, double* temperature,
                          nlgpu_solve_report* report);
/* The solve stage of many contexts at once, each with its system assembled
 * (nlgpu_conductivity_matrix_2d(FULL)).  The non-symmetric systems (a
 * conductivity field with a nonlocal model; the reference solves each with
 * Jacobi-preconditioned BiCGSTAB, stationary_heat_equation_solver_2d.hpp:105-108)
 * run as one block-diagonal BiCGSTAB, every instance with its own scalars
 * and stop test |b - A x| <= tolerance |b|; an instance whose recurrence
 * breaks down or drifts starts again from its x.  precision FP64: the
 * reference's diagonal preconditioner; MIXED: the ILLT of every instance's
 * p1 K_local applied in FP32 (products and vectors stay FP64; the same
 * choice applies to a single non-symmetric nlgpu_solve_assembled /
 * nlgpu_stationary_2d).  Symmetric instances are solved one after another as
 * by nlgpu_solve_assembled.  temperatures[k]: [n_nodes of
 * instance k]; reports may be NULL, else [count].  Returns
 * NLGPU_ERR_NO_CONVERGENCE when an instance did not converge (every output is
 * still written). */
int nlgpu_solve_assembled_batch(int64_t count, nlgpu_ctx* const* instances, const nlgpu_solve_options* options,
                                double* const* temperatures, nlgpu_solve_report* reports);

/* ---- slae::conjugate_gradient on caller matrices (conjugate_gradient.hpp:15-79)
 * A: upper CSR of a symmetric matrix with the diagonal first in each row;
 * optional ILLT preconditioner built from P (upper CSR, same size), the
 * eigen_ILLT_preconditioner of eigen_preconditioner.hpp:57.
 * x0 may be NULL (zero start).  Stops when |b - Ax| / |b| <= tolerance. */
int nlgpu_cg_solve(nlgpu_ctx* ctx, int64_t n, const int64_t* a_rowptr, const int64_t* a_col,
                   const double* a_val, const int64_t* p_rowptr, const int64_t* p_col,
                   const double* p_val, const double* b, const double* x0, double tolerance,
                   int64_t max_iterations, double* x, nlgpu_solve_report* report);

/* ---- ILLT behind slae::preconditioner_base (preconditioner_base.hpp:8-15),
 * the GPU counterpart of eigen_preconditioner<T, I, Eigen::IncompleteCholesky<
 * T, Eigen::Upper, Eigen::NaturalOrdering<I>>> (eigen_preconditioner.hpp:9-57).
 * compute: factorises an upper-stored symmetric CSR (row pointers [n + 1],
 * sorted columns with the diagonal first, values; the reference's RowMajor
 * int64 storage) and writes computation_info as Eigen::ComputationInfo
 * (0 Success, 1 NumericalIssue when every diagonal shift failed; the
 * reference then falls back to the identity).  The factor stays in the
 * context until the next compute.  solve: y = M^-1 x for host vectors [n]. */
int nlgpu_illt_compute(nlgpu_ctx* ctx, int64_t n, const int64_t* rowptr, const int64_t* col, const double* val,
                       int* computation_info);
int nlgpu_illt_solve(nlgpu_ctx* ctx, int64_t n, const double* x, double* y);
/* The same factor applied in FP32 as the mixed-precision solve applies it:
 * sweeps > 0 Jacobi sweeps per triangle, < 0 exact level-scheduled sweeps
 * (no counterpart in the reference). */
int nlgpu_illt_solve_f32(nlgpu_ctx* ctx, int64_t n, int sweeps, const float* x, float* y);

/* ---- learned correction on top of ILLT (no counterpart in the reference) ----
 * A 4-layer message-passing network (width 64, tanh, no biases) over the
 * graph of the local stiffness pattern, A_hat = D^-1/2 |offdiag K_local| D^-1/2:
 *   X0 = [r / rms(r), z / rms(z)] with z = ILLT^-1 r,  U0 = [X0, A_hat X0],
 *   H1 = tanh(U0 W1), H2 = tanh([H1, A_hat H1] W2), H3 = tanh([H2, A_hat H2] W3),
 *   P(r) = z + rms(z) [H3, A_hat H3] w4.
 * W2, W3 run as BF16 tensor-core GEMMs with FP32 accumulation.  Parameters
 * are NLGPU_MPNN_PARAMS floats packed [W1 4x64 | W2 128x64 | W3 128x64 | w4 128]
 * (row-major, input x output).  The correction is used by the solves with
 * NLGPU_PRECONDITIONER_ILLT_LEARNED (inside the mixed-precision flexible CG,
 * switched off for the rest of a solve when it stalls).
 * train: on the context's assembled system (after nlgpu_conductivity_matrix_2d
 * and boundary conditions): harvests (r, e) pairs from plain FP64 ILLT-CG runs
 * on the system's right-hand side and random ones (x_k every 16 iterations,
 * e = x* - x_k, r = A e), then minimises (P(r) - e)^T A (P(r) - e) / e^T A e
 * with Adam.  loss_grad: one pair on the assembled system; writes z, P(r), the
 * loss and its gradient (packed like the parameters); the weights do not change. */
#define NLGPU_MPNN_PARAMS 16768
typedef struct nlgpu_train_options {
    int right_hand_sides;     /* solves harvested (the first uses the system's own right-hand side) */
    int epochs;
    int batch;                /* pairs per Adam step */
    double learning_rate;
    unsigned seed;
} nlgpu_train_options;
typedef struct nlgpu_train_report {
    int64_t samples, steps;
    double loss_illt;         /* mean loss of ILLT alone on the pairs */
    double loss_first, loss_last;   /* mean loss after the first / last epoch */
    double seconds_harvest, seconds_train;
    /* validation gate: the system's own right-hand side solved to 1e-10 with and
     * without the correction; it stays enabled only when it was faster */
    int64_t validation_iterations_learned, validation_iterations_illt;
    double validation_seconds_learned, validation_seconds_illt;
    int learned_enabled;
} nlgpu_train_report;
int nlgpu_mpnn_set_weights(nlgpu_ctx* ctx, const float* params);
/* The validation gate's decision, to carry it with the weights to another
 * context (1: the correction is used; 0: ILLT alone).  Setting weights enables it. */
int nlgpu_mpnn_set_enabled(nlgpu_ctx* ctx, int enabled);
int nlgpu_mpnn_get_weights(nlgpu_ctx* ctx, float* params);
int nlgpu_mpnn_train(nlgpu_ctx* ctx, const nlgpu_train_options* options, nlgpu_train_report* report);
int nlgpu_mpnn_loss_grad(nlgpu_ctx* ctx, const float* r, const float* e, float* z, float* p, double* loss,
                         float* grad);

/* ---- conjugate gradient that allocates nothing (no counterpart in the reference)
 * For callers that cannot allocate device memory when they solve (an external
 * memory budget or pool, a loop that must not touch the allocator, buffers
 * owned by another framework): identity-preconditioned CG on a symmetric
 * matrix already in device memory, full-row CSR (row pointers int64 [n + 1],
 * columns int32, values double), right-hand side d_b [n] and solution d_x [n]
 * (initial guess on entry) also in device memory.  Its work vectors live in
 * a fixed scratch array inside the library, sized for at most
 * NLGPU_NOALLOC_MAX_ROWS rows (about 1.6 MB, held on every GPU that loads the
 * library until the process exits); no cudaMalloc or cudaFree is called, and
 * n above NLGPU_NOALLOC_MAX_ROWS is rejected with NLGPU_ERR_ARG.  The first
 * call on a device looks the array's device address up (make it before any
 * stream capture).  The call zeroes its own counters in the array; d_x must
 * hold the starting guess (zeros for a zero start).  All calls share the
 * array: calls that overlap on the GPU race.  Stops when |r| <= tolerance |b|
 * (|r| of the CG recurrence) or after max_iterations; reports the iterations
 * and |b - A x| / |b| recomputed from x (also when the starting guess already
 * meets the tolerance: 0 iterations).  b = 0 sets x = 0.  Returns
 * NLGPU_ERR_NO_CONVERGENCE, with x, iterations and residual filled, when the
 * iteration cap is reached and |b - A x| > tolerance |b|.
 * `stream` is a cudaStream_t or NULL; the call returns after the stream has
 * finished its work. */
#define NLGPU_NOALLOC_MAX_ROWS 65536
int nlgpu_cg_solve_noalloc(void* stream, int64_t n, const int64_t* d_rowptr, const int32_t* d_col,
                           const double* d_val, const double* d_b, double* d_x, double tolerance,
                           int64_t max_iterations, int64_t* iterations, double* residual);

/* ---- equilibrium_equation (mechanical/equilibrium_equation_2d.hpp:19-60):
 * nonlocal plane elasticity, two degrees of freedom per node.  The mesh,
 * neighbours and the nonlocal model (influence, radii, p1 of
 * nlgpu_set_model_2d; its conductivity is not used) are the context's.
 * Rows and columns of the stiffness matrices are 2 node + component
 * (component 0 = x, 1 = y), as matrix_assembler_2d<T, I, J, 2> numbers them.
 *
 * nlgpu_set_elastic_2d replaces raw_mechanical_parameters' elastic part with
 * constant parameters and forms the Hooke matrix as elastic_parameters.hpp's
 * hooke() does: NLGPU_ELASTIC_ISOTROPIC {E, nu}; NLGPU_ELASTIC_ORTHOTROPIC
 * {E_x, E_y, nu_x, nu_y, G}; NLGPU_ELASTIC_ANISOTROPIC {E_x, E_y, nu_x, nu_y,
 * G, angle} (the orthotropic matrix rotated by `angle`).  hooke_out (6
 * values or NULL) receives h11, h12, h66, h22, h16, h26. */
enum { NLGPU_ELASTIC_ISOTROPIC = 0, NLGPU_ELASTIC_ORTHOTROPIC = 1, NLGPU_ELASTIC_ANISOTROPIC = 2 };
int nlgpu_set_elastic_2d(nlgpu_ctx* ctx, int kind, const double* parameters, double* hooke_out);
/* mechanical_boundaries_conditions_2d: one boundary group (line elements as in
 * nlgpu_add_boundary_2d) with a condition per component: NLGPU_MECH_NONE,
 * NLGPU_MECH_DISPLACEMENT (displacement_2d, first kind) or
 * NLGPU_MECH_PRESSURE (pressure_2d, second kind) with its constant value. */
enum { NLGPU_MECH_NONE = 0, NLGPU_MECH_DISPLACEMENT = 1, NLGPU_MECH_PRESSURE = 2 };
int nlgpu_add_mechanical_boundary_2d(nlgpu_ctx* ctx, int64_t n_edges, int nodes_per_edge, const int64_t* edges,
                                     int kind_x, double value_x, int kind_y, double value_y);
int nlgpu_clear_mechanical_boundaries(nlgpu_ctx* ctx);
/* stiffness_matrix::compute (stiffness_matrix_2d.hpp:176-197) of NLGPU_PART_FULL
 * (inner and bound, with the right-hand side: pressure integrals, then
 * f -= K_bound u_D, f[D] = u_D) or NLGPU_PART_LOCAL (p1 x the local
 * stiffness, the ILLT's matrix). */
int nlgpu_stiffness_matrix_2d(nlgpu_ctx* ctx, int part, int64_t* nnz_inner, int64_t* nnz_bound);
/* CSR of NLGPU_MATRIX_INNER / _BOUND / _LOCAL of the stiffness (2 n rows;
 * rowptr [2n + 1], then col / val of rowptr[2n] entries; pass NULL for what is
 * not wanted) and the right-hand side [2n] after / before the first kind. */
int nlgpu_get_stiffness_matrix(nlgpu_ctx* ctx, int which, int64_t* rowptr, int64_t* col, double* val);
int nlgpu_get_mechanical_rhs(nlgpu_ctx* ctx, double* rhs, double* rhs_init);
/* equilibrium_equation: assembles (FULL), then solves with CG and the ILLT of
 * the LOCAL stiffness (options->preconditioner NLGPU_PRECONDITIONER_ILLT; the
 * reference uses it for a nonlocal model and the identity otherwise; an ILLT
 * that fails falls back to the identity) in FP64 or the mixed precision of
 * the thermal solve.  displacement [2 n]: u_x, u_y per node. */
int nlgpu_equilibrium_equation_2d(nlgpu_ctx* ctx, const nlgpu_solve_options* options, double* displacement,
                                  nlgpu_solve_report* report);

/* ---- nonstationary_heat_equation_solver_2d (nonstationary_heat_equation_solver_2d.hpp:16-106)
 * compute: assembles dt*K + C (unit Dirichlet diagonal) for the current mesh,
 * model and boundary groups; initial temperature [n_nodes] or NULL (zero).
 * step: one implicit Euler step with the Dirichlet nodes set to
 * dirichlet_value (or per-node dirichlet_values when not NULL), CG with the
 * identity preconditioner and x0 = previous temperature. */
int nlgpu_nonstationary_2d_compute(nlgpu_ctx* ctx, double time_step, const double* initial);
int nlgpu_nonstationary_2d_step(nlgpu_ctx* ctx, double dirichlet_value, const double* dirichlet_values,
                                double tolerance, int64_t max_iterations, double* temperature,
                                int64_t* iterations);

/* ---- batched nonstationary stepping (no counterpart in the reference: it
 * batches calls of nonstationary_heat_equation_solver_2d::calc_step)
 * create: instances already set up by nlgpu_nonstationary_2d_compute (each with
 * its own mesh, model, time step and boundaries; their sizes may differ); the
 * batch copies their matrices and current temperatures and releases the
 * contexts' upper-storage copies of dt K + C and their full -> upper maps, which
 * only a radiation update reads (batches take no radiation edges); the
 * contexts still step on their own.  step: one implicit-Euler step of every instance, the
 * Dirichlet nodes of instance k set to dirichlet_values[k]; CG with the
 * identity preconditioner from the previous temperature, as calc_step, on the
 * block-diagonal system of all instances (one launch per stage for all of
 * them, CUDA-graph replayed iteration chunks, each instance stopping on its
 * own |r| <= tolerance |b|); iterations[k] (or NULL) receives each count.
 * temperature: copies instance `index`'s current temperature out. */
typedef struct nlgpu_batch nlgpu_batch;
int nlgpu_batch_create(nlgpu_batch** batch, int64_t count, nlgpu_ctx* const* instances);
int nlgpu_batch_destroy(nlgpu_batch* batch);
int nlgpu_batch_step(nlgpu_batch* batch, const double* dirichlet_values, double tolerance, int64_t max_iterations,
                     int64_t* iterations);
int nlgpu_batch_temperature(nlgpu_batch* batch, int64_t index, double* temperature);
/* Per instance: rows and the entries the batched step's SpMV reads (the
 * system matrix C + dt K in full padded rows), arrays of `count` values. */
int nlgpu_batch_sizes(nlgpu_batch* batch, int64_t* rows, int64_t* system_entries);
/* The batched step's solver: NLGPU_BATCH_IDENTITY_FP64 (default; the
 * reference's identity-preconditioned FP64 CG per instance, each with its own
 * scalars and stop) or NLGPU_BATCH_MIXED_ILLT (mixed-precision FCG on the whole
 * block-diagonal system with the ILLT of every instance's C + dt p1 K_local,
 * FP64 reliable updates, every instance held to |b_k - A_k x_k| <= tol |b_k|,
 * FP64 ILLT-CG as its fallback; the iteration counts it reports are those of
 * the whole system). */
enum { NLGPU_BATCH_IDENTITY_FP64 = 0, NLGPU_BATCH_MIXED_ILLT = 1 };
int nlgpu_batch_set_method(nlgpu_batch* batch, int method);
/* NLGPU_BATCH_MIXED_ILLT: the last step's FCG iterations, FP64 refinement
 * steps and whether the FP64 ILLT-CG fallback ran (zeros for the identity CG). */
int nlgpu_batch_last_solve(nlgpu_batch* batch, int64_t* inner_iterations, int64_t* outer_iterations, int* fallback);

/* ---- stationary_heat_equation_solver_1d (stationary_heat_equation_solver_1d.hpp:43-122)
 * One segment [0, length] of `elements` Lagrange elements of `order` 1
 * (Gauss-2) or 2 (Gauss-3), constant conductivity, influence kind
 * 0 = polynomial_1d<2,1>, 1 = polynomial_1d<1,1>, 2 = normal, 3 = constant
 * (influence_functions_1d.hpp:10-75), temperature t_left at x = 0, flux
 * q_right at x = length, source sin(pi x) when sin_source != 0.  Writes the
 * nodal temperature [elements * order + 1]. */
int nlgpu_stationary_1d(nlgpu_ctx* ctx, int64_t elements, int order, double length, double radius,
                        double local_weight, int influence, double conductivity, double t_left,
                        double q_right, int sin_source, double* temperature);

/* ---- nonstationary_heat_equation_solver_1d (nonstationary_heat_equation_solver_1d.hpp:24-259)
 * compute: one segment [0, length] as nlgpu_stationary_1d, constant capacity
 * and density, implicit Euler step time_step; left_kind / right_kind
 * NLGPU_BC_TEMPERATURE, NLGPU_BC_FLUX or NLGPU_BC_CONVECTION (convection_1d,
 * thermal_boundary_conditions_1d.hpp:36-55: its heat transfer coefficient set
 * before by nlgpu_nonstationary_1d_convection); initial_temperature [n] or
 * NULL (zero), n = elements * order + 1.  Assembles dt K + C (C the capacity
 * matrix; a temperature end's row and column routed out with a unit
 * diagonal, a convection end's diagonal + dt h, as the reference) and factors
 * it once.
 * step: calc_step with the ends' values (temperature, flux, or a convection
 * end's ambient temperature, as set at compute) and the sin(pi x) source when
 * sin_source; f = dt (flux or h T_ambient + source) + C T_prev, first kind,
 * solve; temperature [n] receives the new temperature (or NULL).
 * temperature: the current temperature. */
int nlgpu_nonstationary_1d_convection(nlgpu_ctx* ctx, double heat_transfer_left, double heat_transfer_right);
int nlgpu_nonstationary_1d_compute(nlgpu_ctx* ctx, int64_t elements, int order, double length, double radius,
                                   double local_weight, int influence, double conductivity, double capacity,
                                   double density, double time_step, int left_kind, int right_kind,
                                   const double* initial_temperature, int64_t* nodes);
int nlgpu_nonstationary_1d_step(nlgpu_ctx* ctx, double left_value, double right_value, int sin_source,
                                double* temperature);
int nlgpu_nonstationary_1d_temperature(nlgpu_ctx* ctx, double* temperature);

/* ---- measurement utilities (no counterpart in the reference) ---------------
 * Events recorded on the context's stream (slots 0..63) and the device time
 * between two of them; an L2 flush (writes `bytes` of scratch memory); and the
 * average device time of one kernel stage over `reps` launches on the current
 * problem: 0 SpMV of the solver matrix, 1 pair assembly (FULL part),
 * 2 ILLT application (both triangular sweeps), 3 neighbour search, 4 FP32
 * SpMV of the solver matrix, 5 FP32 ILLT application with exact level-scheduled
 * sweeps, 6 FP32 ILLT application with the Jacobi sweeps of the last mixed
 * solve (NLGPU_DEFAULT_TRIANGULAR_SWEEPS before any), 7 pair assembly in
 * float-float (stage 1 is the FP64 one), 8 nodal flux of the last solution. */
/* Options of a context: NLGPU_OPTION_GLOBAL_SWEEPS = 1 makes the ILLT
 * triangular sweeps read and write their values in global memory instead of
 * the TMA-fed shared-memory ring (same arithmetic); NLGPU_OPTION_ORDERED_PAIRS
 * = 1 makes a symmetric assembly evaluate every ordered element pair instead
 * of each unordered pair once (both for comparison).
 * NLGPU_OPTION_ASSEMBLY_PRECISION selects how the nonlocal pair blocks are
 * computed: NLGPU_ASSEMBLY_AUTO (default) in float-float on the FP32 pipes for
 * a mixed-precision stationary solve and in FP64 otherwise, NLGPU_ASSEMBLY_FF
 * always in float-float, NLGPU_ASSEMBLY_FP64 always in FP64.  Float-float
 * (about 48 significant bits) applies to the fast-polynomial, polynomial and
 * exponential influence with constant conductivity; other models use FP64.
 * NLGPU_OPTION_FP32_SYMMETRIC = 1 makes the mixed solve's FP32 SpMV read only
 * the strictly upper part of a symmetric solver matrix (half the entries,
 * transposed contributions added with shared-memory atomics) instead of its
 * full rows (the default; for comparison).
 * NLGPU_OPTION_ASSEMBLY_WARPS sets the warps per CTA of the float-float pair
 * assembly: 16 or 32, or 0 (default) to time both on a sample of elements at
 * the first float-float assembly of each (element type, influence kind, pair
 * mode) and keep the faster; nlgpu_assembly_tuning reports the choice. */
enum { NLGPU_OPTION_GLOBAL_SWEEPS = 0, NLGPU_OPTION_ORDERED_PAIRS = 1, NLGPU_OPTION_ASSEMBLY_PRECISION = 2,
       NLGPU_OPTION_FP32_SYMMETRIC = 3, NLGPU_OPTION_ASSEMBLY_WARPS = 4 };
enum { NLGPU_ASSEMBLY_AUTO = 0, NLGPU_ASSEMBLY_FF = 1, NLGPU_ASSEMBLY_FP64 = 2 };
int nlgpu_set_option(nlgpu_ctx* ctx, int option, int value);
/* Warps per CTA of the last float-float pair assembly (0 before any) and the
 * sample times (ms) of the last tuning with 16 and 32 warps (0 when none ran). */
int nlgpu_assembly_tuning(nlgpu_ctx* ctx, int* warps, double* sample_ms);
int nlgpu_event_record(nlgpu_ctx* ctx, int slot);
int nlgpu_event_elapsed(nlgpu_ctx* ctx, int start_slot, int stop_slot, double* milliseconds);
int nlgpu_flush_l2(nlgpu_ctx* ctx, int64_t bytes);
int nlgpu_time_stage(nlgpu_ctx* ctx, int stage, int reps, double* milliseconds);
/* The learned correction's tensor-core GEMM on its own (for checking it):
 * C[M x N] = A[M x K] . B[N x K]^T with A, B BF16 bit patterns (K contiguous,
 * K a multiple of 8), N 64 or 128, FP32 accumulation and output; splits > 1
 * splits K over CTAs that add with FP32 atomics. */
int nlgpu_gemm_bf16(int64_t M, int N, int64_t K, int splits, const uint16_t* A, const uint16_t* B, float* C);

#ifdef __cplusplus
}
#endif

#endif /* NLGPU_H */
