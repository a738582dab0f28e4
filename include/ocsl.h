/*
 * ocsl.h -- C ABI of the GB300 (sm_103a) linear-solve library that replaces
 * OpenCSLSolver's CMatrix_solver hot path (cmatrix_solver.h:27-95,
 * cmatrix_solver.cpp:233-780).
 *
 * Data layout is the reference's own, so a caller hands over the members of
 * CMatrix_solver unchanged:
 *   row_ptr       size_t[n+1]      CCSR::row_ptr      (cmatrix_solver.h:40)
 *   column_index  size_t[nnz]      CCSR::column_index (cmatrix_solver.h:41),
 *                                  boundary rows carry a phantom column
 *                                  (size_t)-1 with value 0 (cfvm.cpp:89-94);
 *                                  it is accepted and skipped.
 *   value         double[nnz]      CCSR::value        (cmatrix_solver.h:39)
 *   b, x          double[n]        b_vector / x_vector (cmatrix_solver.h:88-89)
 *
 * Every function returns an ocsl_status.  Nothing falls back to the CPU: a
 * process without a usable GPU gets OCSL_NO_DEVICE.  One context owns one
 * CUDA stream on one device and is not re-entrant (like the reference's
 * CMatrix_solver, which is driven from one thread, cflow_solver.cpp:289).
 */
#ifndef OCSL_H
#define OCSL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ocsl_ctx ocsl_ctx;

typedef enum {
    OCSL_OK = 0,
    OCSL_NOT_CONVERGED = 1, /* tolerance mode hit maxit (x holds the last iterate) */
    OCSL_ZERO_PIVOT = 2,    /* a zero or infinite pivot in the factor: mode R
                               still computes exactly as the reference (which has
                               no check) and reports it; mode T runs no iteration
                               and leaves x unchanged                               */
    OCSL_NONFINITE = 3,     /* NaN/Inf met in the iteration                       */
    OCSL_BAD_PATTERN = 4,   /* pattern rejected by ocsl_set_pattern               */
    OCSL_TIMEOUT = 5,       /* a bounded device wait gave up (triangular sweep)   */
    OCSL_CUDA_ERROR = 6,
    OCSL_BAD_ARGUMENT = 7,
    OCSL_NO_PATTERN = 8,    /* ocsl_set_pattern has not been called               */
    OCSL_NO_DEVICE = 9,
    OCSL_BREAKDOWN = 10     /* Krylov breakdown (rho, sigma or omega became 0)    */
} ocsl_status;

typedef enum {
    /* Reference-faithful ("mode R"): the reference's own algorithms, fixed
     * iteration counts, exits and return values.  Bit-identical to the
     * restatement in oracle/ocsl_oracle.c.                                      */
    OCSL_CG_REF = 0,            /* CMatrix_solver::CG_solve, cmatrix_solver.cpp:635-680          */
    OCSL_BICGSTAB_REF = 1,      /* CMatrix_solver::ILU_BICGSTAB_solve, cmatrix_solver.cpp:682-762 */
    /* Tolerance mode ("mode T"): run to ||b - A x||_2 / ||b||_2 <= tol.        */
    OCSL_PCG = 2,               /* Jacobi-preconditioned CG, FP64 (symmetric systems)            */
    OCSL_ILU_BICGSTAB = 3,      /* ILU(0)-BiCGSTAB, FP64, the reference's ILU factor             */
    OCSL_ILU_BICGSTAB_IR32 = 4  /* FP32 ILU-BiCGSTAB inside FP64 iterative refinement            */
} ocsl_method;

typedef struct {
    double tol;         /* relative residual target (mode T), default 1e-10            */
    int maxit;          /* total Krylov iterations allowed (mode T), default 5000     */
    int ilu_sweeps;     /* fixed-point ILU sweeps, default 3 (cmatrix_solver.cpp:521) */
    double inner_tol;   /* IR32: inner relative reduction per refinement step, default
                           1e-5; the last step asks only for what is still missing    */
    int inner_maxit;    /* IR32: iterations per inner solve, default 500              */
} ocsl_opts;

typedef struct {
    double residual;    /* mode R: the value the reference function returns;
                           mode T: final true relative residual (FP64)               */
    int iterations;     /* iterations that updated x (mode T: total inner iterations) */
    int outer_iterations; /* IR32 refinement steps                                   */
    int status;         /* same as the return value                                 */
    double solve_ms;    /* device time of the solve (CUDA events)                   */
} ocsl_result;

/* Fill *opts with the defaults above. */
void ocsl_default_opts(ocsl_opts* opts);
const char* ocsl_status_string(int status);
/* Last error message of a context (or of creation when ctx is NULL). */
const char* ocsl_last_error(const ocsl_ctx* ctx);
/* Library version string. */
const char* ocsl_version(void);

/* Context.  Replaces the construction of CMatrix_solver
 * (cmatrix_solver.cpp:30-34, called by cfvm.cpp:84). */
int ocsl_create(ocsl_ctx** ctx, int device);
int ocsl_destroy(ocsl_ctx* ctx);
/* Use a caller-owned cudaStream_t (NULL restores the context's own stream). */
int ocsl_set_stream(ocsl_ctx* ctx, void* stream);
int ocsl_synchronize(ocsl_ctx* ctx);

/* Fix the sparsity pattern once per run, as CFVM::define_matrix_structure
 * does (cfvm.cpp:74-98) followed by extract_diag_indexes
 * (cmatrix_solver.cpp:455-469).  Host pointers.  Builds the int32 device
 * CSR, the diagonal map, the ILU product table and the level schedules of the
 * triangular sweeps.  Rejects (OCSL_BAD_PATTERN) rows without a diagonal,
 * columns >= n other than the phantom, and rows whose entries before / after
 * the diagonal are not below / above it. */
int ocsl_set_pattern(ocsl_ctx* ctx, size_t n, const size_t* row_ptr, const size_t* column_index);
/* Host-only check of a pattern (no device needed): the same validation and
 * level analysis as ocsl_set_pattern.  Writes the real nnz, the forward /
 * backward level counts and the detected 7-point box dims (nx, ny, nz; zeros
 * when the pattern is not a box); on OCSL_BAD_PATTERN writes the reason into
 * err.  Any output pointer may be NULL. */
int ocsl_check_pattern(size_t n, const size_t* row_ptr, const size_t* column_index,
                       int64_t* nnz_real, int32_t* fw_levels, int32_t* bw_levels,
                       int32_t* box_dims, char* err, size_t err_len);
/* Build the reference's pattern from the mesh's face connectivity in
 * O(n + faces), host-only: row i = i and its face neighbours ascending, plus
 * one phantom column (size_t)-1 when cell i has a boundary face -- the matrix
 * structure CFVM::define_matrix_structure (cfvm.cpp:74-98) builds with
 * quadratic insert_element calls.  Call with row_ptr = NULL to get *nnz, then
 * with row_ptr[n+1] and column_index[*nnz]. */
int ocsl_build_pattern(size_t n, int64_t n_faces, const int32_t* left, const int32_t* right,
                       int64_t n_bc, const int32_t* bc_left, size_t* row_ptr,
                       size_t* column_index, size_t* nnz);
/* Pattern facts: n, stored nnz (with phantoms), real nnz, forward and
 * backward level counts. */
int ocsl_pattern_info(const ocsl_ctx* ctx, int64_t* n, int64_t* nnz, int64_t* nnz_real,
                      int32_t* fw_levels, int32_t* bw_levels);

/* One solve with HOST buffers: the drop-in for CMatrix_solver::solve()
 * (cmatrix_solver.cpp:764-780) and, with OCSL_CG_REF / OCSL_BICGSTAB_REF, for
 * CG_solve() / ILU_BICGSTAB_solve().  value and b are read, x is the initial
 * guess on entry and the solution on return (x_vector is overwritten in
 * place, as in the reference).  opts may be NULL (defaults). */
int ocsl_solve(ocsl_ctx* ctx, int method, const double* value, const double* b, double* x,
               const ocsl_opts* opts, ocsl_result* result);
/* Same with DEVICE pointers (resident data, no host copies). */
int ocsl_solve_device(ocsl_ctx* ctx, int method, const double* d_value, const double* d_b,
                      double* d_x, const ocsl_opts* opts, ocsl_result* result);

/* Several right-hand sides that share one matrix (the three momentum
 * components of an inviscid or slip case, cflow_solver.cpp:258-290):
 * d_b and d_x are [nrhs][n]; the factor is built once and reused by every
 * right-hand side; with OCSL_ILU_BICGSTAB_IR32 they are solved in lockstep
 * groups of up to four (ocsl_set_col_batching).  result[nrhs].  No reference
 * counterpart (the reference assembles and solves each component
 * separately). */
int ocsl_solve_multi_device(ocsl_ctx* ctx, int method, const double* d_value, int nrhs,
                            const double* d_b, double* d_x, const ocsl_opts* opts,
                            ocsl_result* result);

/* Batched solves of many independent systems (no reference counterpart).
 * A batch owns one context per system (pattern analysed once, device memory
 * reused) and `workers` host threads, each driving its own CUDA stream, which
 * take systems largest first; the systems' solves overlap on the GPU.
 * Systems are given in the reference's CSR layout, each with nrhs >= 1
 * right-hand sides sharing its matrix. */
typedef struct ocsl_batch ocsl_batch;
typedef struct {
    size_t n;
    const size_t* row_ptr;
    const size_t* column_index;
    int nrhs;
} ocsl_batch_system;
int ocsl_batch_create(ocsl_batch** batch, int device, int count, const ocsl_batch_system* systems,
                      int workers);
int ocsl_batch_destroy(ocsl_batch* batch);
/* d_value[i] (nnz_i), d_b[i] and d_x[i] ([nrhs_i][n_i]) are DEVICE pointers;
 * result holds sum(nrhs_i) entries, system by system.  Returns the first
 * non-OK status of any solve (every solve still runs). */
int ocsl_batch_solve_device(ocsl_batch* batch, int method, const double* const* d_value,
                            const double* const* d_b, double* const* d_x, const ocsl_opts* opts,
                            ocsl_result* result);
const char* ocsl_batch_last_error(const ocsl_batch* batch);
/* One-graph mode of ocsl_batch_solve_device for OCSL_ILU_BICGSTAB_IR32: the
 * host factors every system (as above), then ONE graph launch runs every
 * solve of every system -- each system's right-hand sides one after another,
 * the systems side by side, every refinement and inner loop on the device
 * (conditional WHILE nodes with bounded control kernels, as
 * ocsl_set_device_loop) -- with no host round trip until all are done.  The
 * graph is instantiated on the first call and replayed while the method, the
 * options and the value, b and x pointers stay the same.  Results are
 * bit-identical to the host-driven batch.  Other methods keep the host-driven
 * batch.  enable = 0 (default) turns it off.  No reference counterpart. */
int ocsl_batch_set_graph(ocsl_batch* batch, int enable);

/* Kernel-level entry points on DEVICE pointers, one per reference routine. */
/* y = A x (mode 0); y = z - A x (mode 1); y = fma(a, A x, z) (mode 2).
 * cmatrix_solver.cpp:338-453 gemv. */
int ocsl_gemv_device(ocsl_ctx* ctx, int mode, double a, const double* d_value, const double* d_x,
                     const double* d_z, double* d_y);
/* <x, y> in the library's fixed tile order; cmatrix_solver.cpp:233 norm. */
int ocsl_dot_device(ocsl_ctx* ctx, size_t n, const double* d_x, const double* d_y,
                    double* result);
/* sum (absolute = 0, cmatrix_solver.cpp:244-252 sum) or sum of |x|
 * (absolute = 1, :255-263 ABSsum) of n elements, in the tile order. */
int ocsl_sum_device(ocsl_ctx* ctx, size_t n, const double* d_x, int absolute, double* result);
/* out = x * y element by element; :266-272 product. */
int ocsl_product_device(ocsl_ctx* ctx, size_t n, const double* d_x, const double* d_y,
                        double* d_out);
/* out = a x + b y with the reference's special cases for b = +-1 and a = +-1
 * (:284-335); d_y = NULL gives out = a x (:275-281). */
int ocsl_axpy_device(ocsl_ctx* ctx, size_t n, double a, const double* d_x, double b,
                     const double* d_y, double* d_out);
/* M = `sweeps` fixed-point ILU sweeps of A; cmatrix_solver.cpp:472-552.
 * M is always written; OCSL_ZERO_PIVOT reports a zero or infinite diagonal
 * of it (the reference's commented-out check, :495-500). */
int ocsl_ilu_device(ocsl_ctx* ctx, const double* d_A, double* d_M, int sweeps);
/* y = L^-1 b, cmatrix_solver.cpp:555-572 ILU_forsub. */
int ocsl_forsub_device(ocsl_ctx* ctx, const double* d_M, const double* d_b, double* d_y);
/* x = U^-1 y, cmatrix_solver.cpp:595-611 ILU_backsub. */
int ocsl_backsub_device(ocsl_ctx* ctx, const double* d_M, const double* d_y, double* d_x);

/* Adjoint solve.  No counterpart in the reference (it has no adjoint); it
 * serves gradients of a loss L(x) of the solution x = A^-1 b:
 *   A^T lambda = g (g = dL/dx)  gives  dL/db = lambda,  dL/dA_ij = -lambda_i x_j.
 * Solves A^T lambda = g for the context's pattern and the values of A in A's
 * own CSR order (the transpose is formed on the device through a slot map
 * built once per pattern, on the first call).  Any method of ocsl_solve;
 * lambda is in/out (initial guess, then the solution). */
int ocsl_solve_transpose(ocsl_ctx* ctx, int method, const double* value, const double* g,
                         double* lambda, const ocsl_opts* opts, ocsl_result* result);
int ocsl_solve_transpose_device(ocsl_ctx* ctx, int method, const double* d_value,
                                const double* d_g, double* d_lambda, const ocsl_opts* opts,
                                ocsl_result* result);
/* d_out[k] = (alpha * u_i) * v_j for every stored entry k = (i, j) of the
 * pattern, 0 on phantom entries: with alpha = -1, u = lambda, v = x this is
 * dL/dA on A's sparsity pattern.  No reference counterpart. */
int ocsl_pattern_outer_device(ocsl_ctx* ctx, double alpha, const double* d_u, const double* d_v,
                              double* d_out);

/* ------------------------------------------------------------------------
 * Face-loop coefficient assembly of the flow solver
 * (cflow_solver_cell_face_loops.cpp:37-446 with solvers_common.h:32-151):
 * fills the context's CSR values, b and x0 of one momentum component, the
 * pressure correction or the enthalpy equation from the cell / face state,
 * as the reference's face loop, boundary-face loop and cell loop do between
 * `clear()` and `solve()` (cflow_solver.cpp:258-290, 319-349, 431-460).
 * One GPU thread per cell gathers its faces in face order, so there are no
 * atomics and every entry is summed in the order of the reference's
 * single-thread loops.  Viscosity is Sutherland's law written
 * C1 * T * sqrt(T) / (T + C2) (the reference's pow(T, 1.5) differs by at most
 * an ulp).  The viscous stress part of the momentum faces,
 * CFlow_face::stress_explicit_part (cflow_solver_cell_face_loops.cpp:25-35),
 * is an input.
 * ---------------------------------------------------------------------- */
typedef enum {
    OCSL_EQ_MOMENTUM = 0, OCSL_EQ_PRESSURE = 1, OCSL_EQ_ENTHALPY = 2,
    OCSL_EQ_HEAT = 3  /* heat conduction, cheat_solver.cpp:32-65 */
} ocsl_equation;
/* Boundary kinds: the values of enums::Eflow_BC_type and Ewall_BC_type (enums.h:39-41). */
typedef enum {
    OCSL_BC_EMPTY = 0, OCSL_BC_SYMMETRY = 1, OCSL_BC_WALL = 2, OCSL_BC_VELOCITY_INLET = 3,
    OCSL_BC_SUPERSONIC_INLET = 4, OCSL_BC_PRESSURE_OUTLET = 5
} ocsl_bc_type;
typedef enum { OCSL_WALL_NO_SLIP = 0, OCSL_WALL_SLIP = 1 } ocsl_wall_type;
/* enums::Ethermal_BC_type */
typedef enum { OCSL_THERMAL_CONSTANT_TEMPERATURE = 0, OCSL_THERMAL_ADIABATIC = 1 } ocsl_thermal_type;

typedef struct {
    int equation;       /* ocsl_equation                                          */
    int dimension;      /* momentum component 0, 1, 2                             */
    int viscous;        /* Eflow_type_visc::Viscous (else inviscid)               */
    int blended;        /* Econv_flux_type::Blended_central (else first-order upwind) */
    int transient;      /* Etimestepping_type::Transient (else steady)            */
    double implicit_underrelaxation;  /* CFlow_solver::implicit_underrelaxation  */
    double R_specific, gamma, sutherland[2], prandtl;  /* Cfluid_properties      */
    double thermal_diffusivity;  /* Cconfiguration::thermal_diffusivity (heat)    */
} ocsl_assembly;

/* Per-assembly state, DEVICE pointers.  Face arrays follow the order given to
 * ocsl_set_faces; vector quantities are [3][count] (component-major). */
typedef struct {
    /* interior faces (CFVM_face, CFlow_face) */
    const double* geo_aver;
    const double* ksi_A;          /* diffusion_ksi_A                              */
    const double* mdot;
    const double* density;        /* face density                                 */
    const double* qy;
    const double* stress;         /* [3][n_faces]; viscous momentum only          */
    /* boundary faces (CFVM_BC_face, CFlow_BC_face) */
    const int32_t* bc_type;       /* ocsl_bc_type                                 */
    const int32_t* bc_wall;       /* ocsl_wall_type                               */
    const int32_t* bc_supersonic; /* supersonic_flag                              */
    const double* bc_area;
    const double* bc_area_vector; /* [3][n_bc]                                    */
    const double* bc_perp_dist;
    const double* bc_ksi_A;
    const double* bc_mdot;
    const double* bc_density;
    const double* bc_qy;
    const double* bc_temperature;
    const double* bc_enthalpy;
    const double* bc_velocity;    /* [3][n_bc]                                    */
    const double* bc_value;       /* Dirichlet value of the pressure-correction
                                     boundary terms; NULL = 0, as the reference  */
    /* cells (CFVM_cell, CFlow_cell) */
    const double* volume;
    const double* delta_t;
    const double* velocity;       /* [3][n]                                       */
    const double* velocity_last;  /* [3][n]                                       */
    const double* pressure_grad;  /* [3][n]                                       */
    const double* density_c;
    const double* density_last;
    const double* pressure;
    const double* pressure_last;
    const double* pressure_corr;
    const double* temperature;
    const double* enthalpy;
    const double* enthalpy_last;
    const int32_t* bc_thermal;    /* ocsl_thermal_type (heat conduction)          */
} ocsl_flow_state;

/* The mesh's face-to-cell connectivity (host arrays, once per mesh, after
 * ocsl_set_pattern): interior face f joins cells left[f] and right[f],
 * boundary face g belongs to cell bc_left[g].  Every (left, right) and
 * (right, left) pair must be stored in the pattern (OCSL_BAD_ARGUMENT
 * otherwise).  No reference counterpart (the reference walks pointers). */
int ocsl_set_faces(ocsl_ctx* ctx, int64_t n_faces, const int32_t* left, const int32_t* right,
                   int64_t n_bc, const int32_t* bc_left);
/* Assemble one equation into d_value (nnz, phantoms 0), d_b and d_x0 (n);
 * optional outputs (NULL to skip): d_ap (n) the final diagonal (ap_vec of a
 * momentum component, cflow_solver_cell_face_loops.cpp:168-169) and
 * d_total_mdot (n) the cell mass balance of the pressure equation (:180-183). */
int ocsl_assemble_device(ocsl_ctx* ctx, const ocsl_assembly* eq, const ocsl_flow_state* state,
                         double* d_value, double* d_b, double* d_x0, double* d_ap,
                         double* d_total_mdot);
/* Adjoint of the pressure-correction boundary values: for a loss with
 * dL/db = lambda, d_grad[g] = lambda[bc_left[g]] * D_g where D_g multiplies
 * bc_value[g] in b (the Dirichlet terms of supersonic inlets and subsonic
 * outlets, solvers_common.h:56-67), 0 for other faces.  No reference
 * counterpart. */
int ocsl_bc_value_grad_device(ocsl_ctx* ctx, const ocsl_assembly* eq,
                              const ocsl_flow_state* state, const double* d_lambda,
                              double* d_grad);

/* ------------------------------------------------------------------------
 * The SIMPLE inner iteration on the device: CFlow_solver::iterate
 * (cflow_solver.cpp:229-476) -- boundary conditions, the pressure gradient,
 * the explicit viscous stress (viscous flows), the three momentum assemblies
 * and solves, face mass fluxes, the pressure-correction assembly and solve,
 * the corrections of pressure, mass fluxes, densities and velocities, and the
 * enthalpy assembly and solve with the temperature and Mach updates -- all on
 * the context's stream, with no host round trip between the stages.  Every
 * boundary kind of ocsl_bc_type, inviscid or viscous, transient or steady
 * (eq->transient, eq->implicit_underrelaxation).  The state of
 * ocsl_flow_state is read AND WRITTEN in place: cells (pressure, velocity,
 * density_c, temperature, enthalpy, pressure_corr, pressure_grad), interior
 * faces (mdot, density, qy, stress for viscous flows) and boundary faces
 * (bc_mdot, bc_density, bc_qy, bc_enthalpy, bc_supersonic, and on pressure
 * outlets bc_temperature, bc_velocity).  ocsl_set_faces must have been
 * called.
 * ---------------------------------------------------------------------- */
typedef struct {
    /* interior-face metrics (CFVM_face), [3][n_faces] for vectors */
    const double* face_area_vector;
    const double* face_alpha;
    const double* face_distance;   /* cell_center_distance                     */
    const double* face_unit;       /* cell_center_unit_vector                  */
    /* boundary-face metrics (CFVM_BC_face), [3][n_bc] for vectors */
    const double* bc_distance;
    const double* bc_unit;
    const double* bc_alpha;
    const double* bc_out_pressure; /* CFlow_BC_face::Out_Pressure (outlets)     */
    /* per-iteration fields the iteration writes (DEVICE pointers) */
    double* bc_pressure;           /* CFlow_BC_face::Pressure (n_bc)             */
    double* pressure_corr_grad;    /* [3][n]                                     */
    double* ap;                    /* CFlow_cell::ap (n)                         */
    double* ap_vec;                /* [3][n]                                     */
    double* mach;                  /* n                                          */
    double* total_mdot;            /* n                                          */
    /* Cfluid_properties and CFlow_solver constants */
    double cp, Tref, H_formation;
    double relax_p, relax_u;       /* explicit_underrelaxation_P / _u            */
} ocsl_flow_iteration;

typedef struct {
    /* Momentum_global_residual[0..2], Pressure_global_residual (sum |b| of the
     * pressure-correction system), Enthalpy_global_residual */
    double residual[5];
    int iterations[5];             /* of the five solves, in solve order       */
    int status[5];                 /* ocsl_status of each solve                */
} ocsl_flow_report;

/* One inner iteration.  methods[0] solves the three momentum components,
 * methods[1] the pressure correction, methods[2] the enthalpy (the reference
 * has one switch for all, cconfiguration.cpp:213-228; CG_REF / BICGSTAB_REF
 * are the reference's CG_solve / ILU_BICGSTAB_solve).  opts applies to the
 * tolerance-mode methods (NULL = defaults).  Returns the first failing solve's
 * status (the iteration still runs to the end, as the reference's does), or
 * OCSL_OK; report (may be NULL) receives the residuals and per-solve results.
 * The residual sums are taken in the library's tile order, so they may differ
 * from the reference's serial sums in the last bits. */
int ocsl_flow_iterate_device(ocsl_ctx* ctx, const ocsl_assembly* eq,
                             const ocsl_flow_state* state, const ocsl_flow_iteration* it,
                             const int* methods, const ocsl_opts* opts,
                             ocsl_flow_report* report);
/* CFlow_solver::update_timestep for a transient run (cflow_solver.cpp:503-512):
 * velocity, density, pressure and enthalpy are copied to their *_last fields. */
int ocsl_flow_end_step_device(ocsl_ctx* ctx, const ocsl_flow_state* state);

/* ------------------------------------------------------------------------
 * Mesh input: an SU2 ASCII mesh (tetrahedra, hexahedra, wedges; triangle and
 * quadrilateral boundary markers), read and turned into the finite-volume
 * arrays the reference builds in Read_SU2_mesh (cgeometry_supply.h:201-433),
 * Cgeometry (cgeometry.cpp) and CFVM::create_FVM_from_geometry
 * (cfvm.cpp:100-175), with the reference's face and boundary-face numbering,
 * in O(cells + faces) on the host (the reference's connectivity search is
 * quadratic around every node).  Vectors are [3][count].  The arrays feed
 * ocsl_build_pattern / ocsl_set_faces and the state structs above; they stay
 * owned by the mesh object.
 * ---------------------------------------------------------------------- */
typedef struct ocsl_mesh ocsl_mesh;
typedef struct {
    int64_t n_cells, n_faces, n_bc;
    int32_t n_markers;
    /* interior faces (CFVM_face) */
    const int32_t* face_left;
    const int32_t* face_right;
    const double* face_geo_aver;
    const double* face_ksi_A;        /* diffusion_ksi_A                         */
    const double* face_area_vector;
    const double* face_alpha;
    const double* face_distance;     /* cell_center_distance                    */
    const double* face_unit;         /* cell_center_unit_vector                 */
    /* boundary faces (CFVM_BC_face), marker by marker in file order */
    const int32_t* bc_left;
    const int32_t* bc_marker;        /* marker index (the configuration's BC)   */
    const double* bc_area;
    const double* bc_area_vector;
    const double* bc_alpha;
    const double* bc_distance;
    const double* bc_unit;
    const double* bc_perp_dist;
    const double* bc_ksi_A;
    /* cells (CFVM_cell, Cgeo_cell) */
    const double* cell_volume;
    const double* cell_center;
} ocsl_mesh_arrays;
/* OCSL_BAD_ARGUMENT with the reason in err (may be NULL) on a file the reader
 * cannot take. */
int ocsl_mesh_read_su2(const char* path, ocsl_mesh** mesh, char* err, size_t err_len);
int ocsl_mesh_view(const ocsl_mesh* mesh, ocsl_mesh_arrays* arrays);
const char* ocsl_mesh_marker_name(const ocsl_mesh* mesh, int marker);
int ocsl_mesh_destroy(ocsl_mesh* mesh);

/* ------------------------------------------------------------------------
 * VTK output of a solution on a mesh read by ocsl_mesh_read_su2: the two
 * legacy-ASCII files of Cpost_processing::write_VTK_file and
 * write_boundary_VTK_file (cpost_processing.cpp:26-187, 238-401; written by
 * Croot::start_solver at the end of a run and every VTK_file_frequency steps,
 * croot.cpp:226-240) with the same sections, names, node orders and number
 * format -- byte-identical to the reference's files for the same state at
 * the default 6 significant digits (its std::ostream default); digits up to
 * 17 give a round-trip exact file.  Field pointers may be DEVICE memory (the
 * ocsl_flow_state arrays the device SIMPLE iteration writes, streamed to the
 * host in chunks while the previous chunk is formatted) or host memory
 * (no GPU needed then).  Vectors are [3][count].  Either path may be NULL to
 * skip that file.  OCSL_BAD_ARGUMENT with the reason in err on a missing field
 * or an unwritable file.
 * ---------------------------------------------------------------------- */
typedef struct {
    int heat;        /* 1: heat conduction (Temperature only), 0: fluid flow            */
    int digits;      /* significant digits, 0 = 6 (the reference's), at most 17         */
    /* cells (n_cells; vectors [3][n_cells]) */
    const double* density;        /* flow: CFlow_cell::Density                           */
    const double* pressure;       /* flow                                                */
    const double* temperature;    /* flow and heat                                       */
    const double* mach;           /* flow                                                */
    const double* velocity;       /* flow                                                */
    const double* pressure_grad;  /* flow                                                */
    /* boundary faces (n_bc), in the mesh's boundary-face order */
    const double* bc_temperature; /* heat: CHeat_BC_face::Temperature                     */
    const int32_t* bc_type;       /* flow: ocsl_bc_type, for the wall stress             */
    const int32_t* bc_wall;       /* flow: ocsl_wall_type                                */
    int viscous;                  /* flow: Eflow_type_visc::Viscous (wall stress != 0)   */
    double sutherland[2];         /* flow: viscosity C1 T^1.5 / (T + C2)                 */
} ocsl_vtk_fields;
int ocsl_vtk_write(const ocsl_mesh* mesh, const ocsl_vtk_fields* fields, const char* cells_path,
                   const char* boundary_path, char* err, size_t err_len);

/* Tolerance-mode solves with their control flow on the device: the loops of
 * OCSL_ILU_BICGSTAB_IR32 (refinement and inner FP32 loop), OCSL_ILU_BICGSTAB
 * and OCSL_PCG (restarts and Krylov loop) run as conditional WHILE graph
 * nodes with single-thread control kernels taking the decisions the host
 * takes otherwise (residual checks, the next inner tolerance, budgets,
 * restarts, statuses), so one graph launch runs the whole solve with no host
 * round trip; every loop continues only below a device iteration bound (the
 * inner budget, 1000 refinement steps or 64 restarts, maxit).  The graph is
 * kept and replayed while its pointers and options hold.  Results are
 * bit-identical to the host-driven loop.  Applies to single-right-hand-side
 * solves on a stream that can be captured (not the legacy default stream),
 * without profiling; otherwise the host drives the loop.  enable = 0
 * (default) keeps the host loop.  No reference counterpart. */
int ocsl_set_device_loop(ocsl_ctx* ctx, int enable);

/* CSR SpMV shape (the SpMV of every non-box pattern, e.g. tetrahedral
 * meshes; box patterns use stencil records): lanes per row 1 (one thread per
 * row, 32 rows per warp; the default), 4 (8 rows per warp) or 16 (2 rows per
 * warp), where a row's lanes load its entries side by side and its first
 * lane runs the fma chain in CSR order -- results are identical for every
 * shape.  0 = default.  Reset by ocsl_set_pattern.  No reference
 * counterpart (the reference's gemv is one thread per row,
 * cmatrix_solver.cpp:338-453). */
int ocsl_set_spmv_lanes(ocsl_ctx* ctx, int lanes);
int ocsl_spmv_lanes(const ocsl_ctx* ctx, int* lanes);
/* Autotuner of the CSR SpMV's lanes per row (rows per warp) for this pattern
 * and matrix: times y = A x with its fused dot for each shape with CUDA
 * events, in the precision a solve of `method` computes its inner SpMVs in
 * (FP32 for OCSL_ILU_BICGSTAB_IR32, else FP64), keeps the fastest and reports
 * it with its time in microseconds. */
int ocsl_autotune_spmv_device(ocsl_ctx* ctx, int method, const double* d_value, int* lanes,
                              double* spmv_us);

/* Triangular-sweep kernel: 0 automatic (structured when the pattern is a
 * natural-order 7-point box stencil, level-scheduled otherwise), 1 always the
 * level-scheduled kernel, 2 the structured CTA kernel, 3 the structured
 * warp-pipelined kernel (2 and 3: OCSL_BAD_ARGUMENT if the pattern is not a
 * box).  With kind 2, tile_a / tile_b set the CTA kernel's column tile, one
 * thread per column, at most 256 (0 = default 16 x 8).  With kind 3 they set
 * the warp-pipelined kernel's warps per CTA (1..8, 0 = default 4) and its
 * start lag behind an upstream CTA in rows (0 = default 6).  In automatic
 * mode a single right-hand side uses the warp-pipelined kernel (or, after
 * ocsl_autotune_device, whichever structured kernel timed faster for that
 * precision); column-batched solves use the CTA kernel.  All kernels give
 * bit-identical results. */
int ocsl_set_sweep_kernel(ocsl_ctx* ctx, int kind, int tile_a, int tile_b);
/* Thread-block clusters of the structured sweep: cx x cy neighbouring column
 * tiles (cx * cy <= 16; 1 x 1 = none; 0 x 0 = automatic, the default: 2 x 4
 * when the box has at least 64 column tiles, none below; batch contexts use
 * 1 x 1) run as one cluster and
 * pass their face values through distributed shared memory instead of global
 * memory.  Clipped to the tile grid; a shape the device cannot schedule, or
 * whose face buffers (columns x s-extent x (TA + TB) values) do not fit the
 * shared memory, runs as single tiles.  Results are bit-identical for every
 * shape.  No reference counterpart (the reference sweeps serially,
 * cmatrix_solver.cpp:555-611). */
int ocsl_set_sweep_cluster(ocsl_ctx* ctx, int cx, int cy);
/* Whether single-right-hand-side sweeps of the FP64 (fp32 = 0) or FP32
 * (fp32 = 1) solvers run the warp-pipelined kernel (*on), and its warps per
 * CTA and start lag; zeros when they do not. */
int ocsl_wave_geometry(const ocsl_ctx* ctx, int fp32, int* on, int* warps, int* lag);
/* The structured-sweep geometry of the FP64 (fp32 = 0) or FP32 (fp32 = 1)
 * sweeps: tiles[2] = (TA, TB), cluster[2] = (cx, cy) after clipping; zeros
 * when no structured sweep applies.  ocsl_set_sweep_kernel and
 * ocsl_set_sweep_cluster set both precisions, ocsl_autotune_device the one
 * its method sweeps in. */
int ocsl_sweep_geometry(const ocsl_ctx* ctx, int fp32, int* tiles, int* cluster);
/* The sweep kernel in use (1 level-scheduled, 2 structured CTA kernel, 3
 * structured warp-pipelined, 4 the one-warp serial sweep that automatic mode
 * gives tiny systems whose schedule is at least a quarter as deep as they are
 * long, such as 1D meshes: n * sizeof(double) <= 40 KB, 5 one launch per
 * level, for schedules of at most 16 levels that are each a contiguous row
 * range, such as multicolour-ordered patterns), the detected box
 * dims (nx, ny, nz; zeros when not a box) and the structured tile (TA, TB)
 * of the FP64 sweeps (ocsl_sweep_geometry: either precision). */
int ocsl_sweep_info(const ocsl_ctx* ctx, int* kind, int* dims, int* tiles);
/* Autotuner of the structured sweep's column tile (block shape) for this
 * pattern and matrix: factors d_value as a solve of `method` would, times a
 * forward + backward sweep for each candidate tile (16x8, 16x16, 32x4, 32x8,
 * 8x16, 8x8, 64x2, 64x4, 128x1, 128x2, as clipped to the box), each alone
 * and in clusters of 2x2, 4x2, 2x4 and 4x4 tiles, with CUDA events, and
 * keeps the fastest for later solves of the same precision: the FP32
 * geometry for OCSL_ILU_BICGSTAB_IR32, the FP64 one for the FP64 methods
 * (ocsl_sweep_geometry reports both, with the cluster shape).
 * Reports the tile and its sweep-pair time in microseconds; zeros,
 * and no change, when the structured kernel does not apply.  The tile does
 * not change any result. */
int ocsl_autotune_device(ocsl_ctx* ctx, int method, const double* d_value, int* tile_a,
                         int* tile_b, double* sweep_us);

/* Allocation-free dot product.  This entry point has no counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc -- programs
 * whose device memory is reserved up front by another allocator (a
 * framework's caching pool, a fixed budget taken at start-up), so that a
 * cudaMalloc would fail, and hosts whose plugins may not allocate or free
 * device memory while they run, because cudaMalloc and cudaFree can
 * synchronise the device and stall the host's other streams.
 * It needs no context and allocates nothing: its scratch is a fixed
 * 32,832-byte device array that every GPU loading this library keeps until
 * exit.  Computes <x, y> over n <= 8,388,608 elements (larger n:
 * OCSL_BAD_ARGUMENT) in the same fixed tile order as ocsl_dot_device, writing
 * the result to the device double *d_result, asynchronously on `stream`
 * (a cudaStream_t, NULL for the legacy default stream).  The first call on a
 * device resolves the scratch address with cudaGetSymbolAddress, so make it
 * before any stream capture.  That address belongs to the device's primary
 * context and is kept for the life of the process: it is not valid after a
 * cudaDeviceReset, nor under another driver context made current on that
 * device.  All calls share the scratch: calls that overlap on the GPU
 * (concurrent streams) race and must be serialised by the caller.  A null
 * pointer, or one not aligned to 8 bytes, is OCSL_BAD_ARGUMENT before any
 * CUDA call. */
int ocsl_dot_noalloc(size_t n, const double* d_x, const double* d_y, double* d_result,
                     void* stream);
/* Message of the last failed ocsl_dot_noalloc on this thread. */
const char* ocsl_noalloc_last_error(void);

/* Failure injection for tests of the bounded waits (no reference
 * counterpart: the reference's sweeps are serial and never wait).  With
 * OCSL_FAULT_SKIP_FIRST_TILE the next triangular sweep this context launches
 * leaves out the first unit of its schedule -- tile (or cluster of tiles) 0
 * of the structured sweep, chunk 0 of the level-scheduled one -- by starting
 * its work dispenser at 1 with one unit fewer in the grid.  Nothing computes
 * those rows, every wait on them runs out after its bound (about a second),
 * the waiting rows store NaN and the call reports OCSL_TIMEOUT; no kernel
 * faults or traps, and the context solves normally afterwards.  The
 * injection is consumed by that one sweep; OCSL_FAULT_NONE cancels it. */
#define OCSL_FAULT_NONE 0
#define OCSL_FAULT_SKIP_FIRST_TILE 1
int ocsl_inject_fault(ocsl_ctx* ctx, int kind);

/* Row ordering of the tolerance-mode solves (OCSL_PCG, OCSL_ILU_BICGSTAB,
 * OCSL_ILU_BICGSTAB_IR32; no reference counterpart: the reference factors
 * and sweeps in natural order, cmatrix_solver.cpp:682-762).
 *   OCSL_ORDER_NATURAL (default): the system as given.
 *   OCSL_ORDER_MULTICOLOUR: the rows are coloured greedily in natural order
 *     (each row the smallest colour none of its lower neighbours has: the
 *     red-black parity colouring of a box stencil) and renumbered colour by
 *     colour, ascending within a colour; the solve runs on P A P^T, P b,
 *     P x0 and scatters x back.  Every triangular sweep then has one level
 *     per colour, so its rows are independent within a level, at the price
 *     of a weaker ILU(0) (more Krylov iterations); Jacobi PCG is unchanged
 *     up to the summation order.  The permuted pattern is built by the
 *     first solve after the pattern is set (OCSL_BAD_PATTERN when two
 *     neighbouring rows could share a colour: a pattern that is not
 *     structurally symmetric).  The reference-faithful methods ignore the
 *     setting; ocsl_solve_multi_device solves its right-hand sides one after
 *     another (no column batching), each through the permuted system; the
 *     transposed solves (ocsl_solve_transpose*) follow the setting too.
 * The sweep-kernel settings (ocsl_set_sweep_kernel and the structured
 * geometry) apply to the natural order only: the permuted pattern is swept by
 * the level-scheduled kernel. */
#define OCSL_ORDER_NATURAL 0
#define OCSL_ORDER_MULTICOLOUR 1
int ocsl_set_ordering(ocsl_ctx* ctx, int ordering);
/* The ordering in use, and the colour count and sweep levels (forward,
 * backward) of the permuted pattern: zeros while it is not built.  *stencil
 * is 1 when the permuted pattern is the red-black ordering of a 7-point box
 * with an even x extent: SpMV and preconditioner then read stencil records
 * (neighbour rows computed, no column indices), bit-identical to the CSR
 * kernels. */
int ocsl_ordering_info(const ocsl_ctx* ctx, int* ordering, int* colours, int32_t* levels,
                       int* stencil);
/* perm[new row] = original row of the multicolour ordering (n entries,
 * host memory); builds the permuted pattern if needed. */
int ocsl_ordering_permutation(ocsl_ctx* ctx, int32_t* perm, size_t n);
/* Host-only (no device needed): the multicolour ordering of a pattern, as
 * ocsl_set_ordering builds it -- perm[n] (perm[new row] = original row) and
 * the colour count; OCSL_BAD_PATTERN with the reason in err (may be NULL) for
 * a pattern ocsl_set_pattern rejects or one that cannot be coloured. */
int ocsl_colour_pattern(size_t n, const size_t* row_ptr, const size_t* column_index,
                        int32_t* perm, int32_t* colours, char* err, size_t err_len);

/* Tolerance-mode solves replay each batch of Krylov iterations after the
 * first from a CUDA graph captured on the context's stream (not on the legacy
 * default stream, not while profiling).  enable = 0 launches every kernel
 * directly; results are identical either way. */
int ocsl_set_graphs(ocsl_ctx* ctx, int enable);

/* ocsl_solve_multi_device with OCSL_ILU_BICGSTAB_IR32 runs its right-hand
 * sides in lockstep, up to four per pass: every SpMV, vector and sweep launch
 * serves all of them, and each keeps its own scalars, inner tolerance and
 * stopping test, so every column's result is bit-identical to solving it
 * alone with the same factor.  enable = 0 solves them one after another;
 * enable = 2 runs the lockstep with an SpMM-style SpMV on box patterns (one
 * CTA per row tile reads each stencil record once for all columns, same
 * bits; measured no faster than the default one CTA per tile and column,
 * whose repeated record reads L2 serves). */
int ocsl_set_col_batching(ocsl_ctx* ctx, int enable);

/* Kernel timing.  While enabled, every kernel the context launches is
 * bracketed by CUDA events on its stream and accounted to a category:
 *   0 spmv_f64  1 spmv_f32  2 fw_sweep_f64  3 bw_sweep_f64  4 fw_sweep_f32
 *   5 bw_sweep_f32  6 ilu_factor  7 vector_f64  8 vector_f32  9 sweep_fill
 * ocsl_profile_read synchronises, writes per-category milliseconds and launch
 * counts (arrays of OCSL_PROFILE_CATEGORIES) and clears the record. */
#define OCSL_PROFILE_CATEGORIES 10
int ocsl_profile_enable(ocsl_ctx* ctx, int enable);
int ocsl_profile_read(ocsl_ctx* ctx, double* ms, int64_t* launches);
const char* ocsl_profile_category_name(int category);

#ifdef __cplusplus
}
#endif

#endif /* OCSL_H */
