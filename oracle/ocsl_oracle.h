/* TEST INFRASTRUCTURE ONLY -- the CPU oracle.  Never linked into, loaded by
 * or called from the product path (opencslsolver_gb300/).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and only as
 * the checker or the timed CPU baseline.
 *
 * A plain-C restatement of OpenCSLSolver's linear-solve path
 * (cmatrix_solver.cpp), on the reference's own data layout:
 *   row_ptr   uint64[n+1], column_index uint64[nnz] (a boundary row carries
 *             a phantom column UINT64_MAX with value 0, cfvm.cpp:89-94),
 *   value     double[nnz], vectors double[n].
 *
 * Rounding is explicit.  Where the reference's expression is `a*x + y`
 * (compiled with -ffast-math and FMA contraction on), the oracle calls fma();
 * everything else is a separately rounded operation.  Dot products use the
 * "tile order" below, which the CUDA kernels reproduce exactly, so the GPU
 * results are bit-identical to this oracle; orc_dot_seq gives the
 * single-thread order of the reference's OpenMP loop (cmatrix_solver.cpp:233)
 * for pinning against the reference binary.
 *
 * Tile order: a vector is cut into tiles of 2048 elements; inside a tile,
 * lane t (0..255) accumulates elements t, t+256, ..., t+1792 with fma from
 * 0.0; each group of 32 lanes is combined by a xor butterfly (offsets 16, 8,
 * 4, 2, 1); the 8 group sums are added in order.  The tile sums are reduced
 * the same way: lane t adds tiles t, t+256, ... in order, then butterfly,
 * then the 8 group sums in order.
 *
 * Parity status: pinned.  tests/test_oracle.py checks every function against
 * the reference's own unit-test system (cmatrix_solver_supply.h:29-114) and
 * against the reference binary built from its sources (oracle/_ref).
 */
#ifndef OCSL_ORACLE_H
#define OCSL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "ocsl.h" /* data layout of the assembly inputs (ocsl_assembly, ocsl_flow_state) */

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_TILE 2048
#define ORC_LANES 256

/* Set the OpenMP thread count used by every oracle routine. */
void orc_set_threads(int threads);

/* Dot products (cmatrix_solver.cpp:233-241 norm). */
double orc_dot(size_t n, const double* x, const double* y);      /* tile order */
double orc_dot_seq(size_t n, const double* x, const double* y);  /* sequential */

/* cmatrix_solver.cpp:244-263 sum / ABSsum (tile order), :266-272 product,
 * :275-335 axpy (y == NULL: out = a x). */
double orc_sum(size_t n, const double* x, int absolute);
void orc_product(size_t n, const double* x, const double* y, double* out);
void orc_axpy(size_t n, double a, const double* x, double b, const double* y, double* out);

/* y = A x (mode 0), y = z - A x (mode 1), y = fma(a, A x, z) (mode 2);
 * cmatrix_solver.cpp:338-453 gemv.  Phantom columns (>= n) are skipped. */
void orc_gemv(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
              const double* x, int mode, double a, const double* z, double* y);

/* cmatrix_solver.cpp:455-469.  Returns 0, or -1 if a row has no diagonal. */
int orc_extract_diag(size_t n, const uint64_t* rp, const uint64_t* col, int32_t* diag);

/* cmatrix_solver.cpp:472-552: `sweeps` Jacobi fixed-point ILU sweeps, M
 * starting as a copy of A (:702).  M is the output (nnz). */
void orc_ilu_fixed_point(size_t n, const uint64_t* rp, const uint64_t* col, const double* A,
                         const int32_t* diag, int sweeps, double* M);

/* cmatrix_solver.cpp:555-572 and :595-611. */
void orc_forsub(size_t n, const uint64_t* rp, const uint64_t* col, const double* M,
                const int32_t* diag, const double* b, double* y);
void orc_backsub(size_t n, const uint64_t* rp, const uint64_t* col, const double* M,
                 const int32_t* diag, const double* y, double* x);

/* cmatrix_solver.cpp:635-680 CG_solve and :682-762 ILU_BICGSTAB_solve, with
 * the reference's fixed iteration counts, exits and return values.  x is in/out;
 * *iters receives the iterations that updated x. */
double orc_cg_ref(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                  const double* b, double* x, int* iters);
double orc_bicgstab_ref(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                        const double* b, double* x, int* iters);

/* Tolerance mode (textbook algorithms run to ||b - A x|| / ||b|| <= tol).
 * Return 0 when converged, 1 when maxit was reached.  *relres receives the
 * final true relative residual computed from scratch. */
int orc_bicgstab_tol(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                     const double* b, double* x, double tol, int maxit, int ilu_sweeps,
                     int* iters, double* relres);
int orc_pcg_tol(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                const double* b, double* x, double tol, int maxit, int* iters, double* relres);
/* FP32 inner ILU-BiCGSTAB inside an FP64 iterative-refinement loop. */
int orc_bicgstab_ir32(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                      const double* b, double* x, double tol, int maxit, double inner_tol,
                      int inner_maxit, int ilu_sweeps, int* iters, int* outer, double* relres);

/* Face-loop coefficient assembly (ocsl_oracle_assembly.c): the reference's
 * single-thread loop order; `st` holds HOST pointers.  ap / total_mdot may be
 * NULL. */
void orc_assemble(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                  const int32_t* left, const int32_t* right, int64_t nb, const int32_t* bc_left,
                  const ocsl_assembly* q, const ocsl_flow_state* st, double* value, double* b,
                  double* x0, double* ap, double* total_mdot);
void orc_bc_value_grad(size_t n, const uint64_t* rp, int64_t nb, const int32_t* bc_left,
                       const ocsl_assembly* q, const ocsl_flow_state* st, const double* lambda,
                       double* grad);

/* The SIMPLE inner iteration around the assembly and the solves
 * (ocsl_oracle_flow.c): `st` and `it` hold HOST pointers and are updated in
 * place as ocsl_flow_iterate_device updates its device arrays.  methods[3]
 * as there (OCSL_CG_REF, OCSL_BICGSTAB_REF, and with opts OCSL_PCG and
 * OCSL_ILU_BICGSTAB, whose tol, maxit, ilu_sweeps are read); given_x (may be NULL)
 * replaces solve e's result by given_x[e]; sys_* (may be NULL) receive the
 * five assembled systems (5 x nnz, 5 x n) before each solve.  Returns 0, or -1
 * for an unsupported method. */
void orc_flow_set_bc(size_t n, int64_t nb, const int32_t* bc_left, const ocsl_assembly* q,
                     const ocsl_flow_state* st, const ocsl_flow_iteration* it);
void orc_flow_stress(size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                     const ocsl_assembly* q, const ocsl_flow_state* st,
                     const ocsl_flow_iteration* it);
void orc_flow_bc_mdot(size_t n, int64_t nb, const int32_t* bc_left, const ocsl_assembly* q,
                      const ocsl_flow_state* st, const ocsl_flow_iteration* it);
void orc_flow_bc_pcorr(int64_t nb, const int32_t* bc_left, const ocsl_flow_state* st,
                       const ocsl_flow_iteration* it);
void orc_flow_grad(int corr, size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                   int64_t nb, const int32_t* bc_left, const ocsl_flow_state* st,
                   const ocsl_flow_iteration* it);
void orc_flow_velocity_update(size_t n, int d, const double* x, const ocsl_flow_state* st,
                              const ocsl_flow_iteration* it, double* res);
void orc_flow_face_mdot(size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                        int blended, const ocsl_flow_state* st, const ocsl_flow_iteration* it);
void orc_flow_pcorr(size_t n, const double* x, const ocsl_flow_state* st,
                    const ocsl_flow_iteration* it);
void orc_flow_correct(size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                      int64_t nb, const int32_t* bc_left, const ocsl_assembly* q,
                      const ocsl_flow_state* st, const ocsl_flow_iteration* it);
void orc_flow_enthalpy_update(size_t n, const double* x, const ocsl_assembly* q,
                              const ocsl_flow_state* st, const ocsl_flow_iteration* it,
                              double* res);
void orc_flow_end_step(size_t n, const ocsl_flow_state* st);
int orc_flow_iterate(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                     const int32_t* left, const int32_t* right, int64_t nb,
                     const int32_t* bc_left, const ocsl_assembly* q, const ocsl_flow_state* st,
                     const ocsl_flow_iteration* it, const int* methods, const ocsl_opts* opts,
                     const double* const* given_x, double* sys_value, double* sys_b,
                     double* sys_x0, double* residual, int* iterations);
/* The same iteration with every solve handed to `solve` instead (slot 0-2
 * momentum x/y/z, 3 pressure correction, 4 enthalpy; method = methods[] of
 * that equation): x holds x0 on entry and the solution on return, nonzero
 * return = failure.  Lets a host program put an external solver -- the C++
 * drop-in over the GPU library -- under the oracle's SIMPLE loop. */
typedef int (*orc_solve_fn)(void* user, int slot, int method, size_t n, const double* val,
                            const double* b, double* x);
int orc_flow_iterate_with(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                          const int32_t* left, const int32_t* right, int64_t nb,
                          const int32_t* bc_left, const ocsl_assembly* q,
                          const ocsl_flow_state* st, const ocsl_flow_iteration* it,
                          const int* methods, orc_solve_fn solve, void* user,
                          double* residual);

/* Exact relative residual ||b - A x||_2 / ||b||_2 in long double. */
double orc_true_relres(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                       const double* b, const double* x);

#ifdef __cplusplus
}
#endif

#endif /* OCSL_ORACLE_H */
