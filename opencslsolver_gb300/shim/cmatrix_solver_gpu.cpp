// Drop-in for OpenCSLSolver's linear solves: routes CMatrix_solver::solve(),
// CG_solve() and ILU_BICGSTAB_solve() (cmatrix_solver.h:82-84) to the GB300
// library through its C ABI (include/ocsl.h).  The reference's flow and heat
// solvers keep calling the same member functions on the same data
// (matrix.value / row_ptr / column_index, b_vector, x_vector).
//
// Link recipe (the reference's own objects unchanged, this file added):
//   g++ ... cmatrix_solver_gpu.cpp -I<reference dir> -I<repo>/include
//       -Wl,--wrap=_ZN14CMatrix_solver5solveEv
//       -Wl,--wrap=_ZN14CMatrix_solver8CG_solveEv
//       -Wl,--wrap=_ZN14CMatrix_solver18ILU_BICGSTAB_solveEv
//       -L<repo>/opencslsolver_gb300/_lib -locsl_gb300
// With --wrap, every call of these members from another object file
// (cflow_solver.cpp:289,349,460; cheat_solver.cpp:141; the unit tests in
// cmatrix_solver_supply.h) lands in the __wrap_ functions below.
//
// Semantics kept from the reference:
//   * solve() dispatches on root.configuration->ematrix_solver_type and adds
//     its elapsed microseconds to root.total_elapsed_matrix_solution_time
//     (cmatrix_solver.cpp:764-780);
//   * CG_solve() / ILU_BICGSTAB_solve() run the reference's algorithms with
//     their fixed iteration counts and return the same residual definitions
//     (cmatrix_solver.cpp:635-762); x_vector is overwritten in place.
// The environment variable OCSL_SOLVER selects a tolerance-mode method for
// solve() instead ("pcg", "ilu_bicgstab", "ilu_bicgstab_ir32"), OCSL_TOL its
// tolerance, OCSL_DEVICE the GPU.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

#include "croot.h"
#include "ocsl.h"

namespace {

struct GpuSolver {
    ocsl_ctx* ctx = nullptr;
    size_t n = 0, nnz = 0;
    const size_t* rp = nullptr;
    const size_t* col = nullptr;
};

std::unordered_map<const CMatrix_solver*, GpuSolver> g_solvers;

[[noreturn]] void die(const char* what, int status, const ocsl_ctx* ctx)
{
    // The reference has no error path in its solvers; like its file errors
    // (cconfiguration.cpp:81-84) a failure ends the run with a message.
    std::fprintf(stderr, "ocsl: %s failed: %s (%s)\n", what, ocsl_status_string(status),
                 ocsl_last_error(ctx));
    std::exit(1);
}

GpuSolver& gpu_for(CMatrix_solver* s)
{
    GpuSolver& g = g_solvers[s];
    if (!g.ctx) {
        const char* dev = std::getenv("OCSL_DEVICE");
        const int rc = ocsl_create(&g.ctx, dev ? std::atoi(dev) : 0);
        if (rc != OCSL_OK) die("ocsl_create", rc, nullptr);
        // an OCSL_SOLVER=ilu_bicgstab_ir32 solve runs as one graph launch with
        // its loops on the device (same results, no host round trip per batch
        // of iterations; the other methods are unaffected)
        ocsl_set_device_loop(g.ctx, 1);
    }
    // The pattern is fixed once per run (cfvm.cpp:84-97); upload it again only
    // if the vectors were replaced or resized.
    const size_t n = s->matrix.row_ptr.size() - 1, nnz = s->matrix.column_index.size();
    if (g.n != n || g.nnz != nnz || g.rp != s->matrix.row_ptr.data() ||
        g.col != s->matrix.column_index.data()) {
        const int rc = ocsl_set_pattern(g.ctx, n, s->matrix.row_ptr.data(),
                                        s->matrix.column_index.data());
        if (rc != OCSL_OK) die("ocsl_set_pattern", rc, g.ctx);
        g.n = n;
        g.nnz = nnz;
        g.rp = s->matrix.row_ptr.data();
        g.col = s->matrix.column_index.data();
    }
    return g;
}

double run(CMatrix_solver* s, int method)
{
    GpuSolver& g = gpu_for(s);
    ocsl_opts opts;
    ocsl_default_opts(&opts);
    if (const char* t = std::getenv("OCSL_TOL")) opts.tol = std::atof(t);
    ocsl_result r;
    const int rc = ocsl_solve(g.ctx, method, s->matrix.value.data(), s->b_vector.value.data(),
                              s->x_vector.value.data(), &opts, &r);
    if (rc == OCSL_ZERO_PIVOT && (method == OCSL_CG_REF || method == OCSL_BICGSTAB_REF)) {
        // The reference's solvers carry on through a zero pivot (their check
        // is commented out, cmatrix_solver.cpp:495-500) and x_vector holds
        // exactly what they would compute; say so once and continue.
        static bool warned = false;
        if (!warned) std::fprintf(stderr, "ocsl: warning: %s\n", ocsl_last_error(g.ctx));
        warned = true;
        return r.residual;
    }
    if (rc != OCSL_OK && rc != OCSL_NOT_CONVERGED) die("ocsl_solve", rc, g.ctx);
    return r.residual;
}

int tolerance_method()
{
    const char* m = std::getenv("OCSL_SOLVER");
    if (!m) return -1;
    if (!std::strcmp(m, "pcg")) return OCSL_PCG;
    if (!std::strcmp(m, "ilu_bicgstab")) return OCSL_ILU_BICGSTAB;
    if (!std::strcmp(m, "ilu_bicgstab_ir32")) return OCSL_ILU_BICGSTAB_IR32;
    return -1;
}

}  // namespace

extern "C" {

// CMatrix_solver::CG_solve (cmatrix_solver.cpp:635-680)
double __wrap__ZN14CMatrix_solver8CG_solveEv(CMatrix_solver* self)
{
    return run(self, OCSL_CG_REF);
}

// CMatrix_solver::ILU_BICGSTAB_solve (cmatrix_solver.cpp:682-762)
double __wrap__ZN14CMatrix_solver18ILU_BICGSTAB_solveEv(CMatrix_solver* self)
{
    return run(self, OCSL_BICGSTAB_REF);
}

// CMatrix_solver::solve (cmatrix_solver.cpp:764-780)
void __wrap__ZN14CMatrix_solver5solveEv(CMatrix_solver* self)
{
    const auto begin = std::chrono::steady_clock::now();
    const int tol_method = tolerance_method();
    if (tol_method >= 0)
        run(self, tol_method);
    else if (root.configuration->ematrix_solver_type == enums::Ematrix_solver_type::CG)
        run(self, OCSL_CG_REF);
    else if (root.configuration->ematrix_solver_type == enums::Ematrix_solver_type::ILU_BICSTAB)
        run(self, OCSL_BICGSTAB_REF);
    const auto end = std::chrono::steady_clock::now();
    root.total_elapsed_matrix_solution_time +=
        std::chrono::duration_cast<std::chrono::microseconds>(end - begin).count();
}

}  // extern "C"
