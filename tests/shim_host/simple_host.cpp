// The solve side of a SIMPLE loop as the reference's flow solver runs it, as a
// small shared library: one CMatrix_solver object for every equation whose
// pattern is set once (cfvm.cpp:84-97), and per solve the caller's protocol
// (cflow_solver.cpp:258-298, 316-356, 428-469): fill matrix.value, b_vector
// and x_vector (x0 = the current field), pick the method through
// root.configuration->ematrix_solver_type, call solve(), read x_vector.
// Linked with -Wl,--wrap into the C++ drop-in
// (opencslsolver_gb300/shim/cmatrix_solver_gpu.cpp), so solve() runs on the
// GPU through libocsl_gb300.so.  Test infrastructure
// (tests/test_gpu_dropin.py): simple_host_solve has the signature of the
// oracle's orc_solve_fn, so the oracle's host-side SIMPLE stages drive it.
#include <cstdint>
#include <cstring>

#include "croot.h"
#include "ocsl.h"

Croot root;

namespace {
CMatrix_solver g_solver;
size_t g_n = 0;
}  // namespace

extern "C" {

int simple_host_set_pattern(size_t n, const uint64_t* row_ptr, const uint64_t* column_index)
{
    const size_t nnz = row_ptr[n];
    g_solver.matrix.row_ptr.assign(row_ptr, row_ptr + n + 1);
    g_solver.matrix.column_index.assign(column_index, column_index + nnz);
    g_solver.matrix.value.assign(nnz, 0.0);
    g_solver.b_vector.value.assign(n, 0.0);
    g_solver.x_vector.value.assign(n, 0.0);
    g_n = n;
    return 0;
}

// orc_solve_fn: slot 0-2 momentum, 3 pressure correction, 4 enthalpy.
int simple_host_solve(void*, int, int method, size_t n, const double* val, const double* b,
                      double* x)
{
    if (n != g_n) return -1;
    if (method == OCSL_CG_REF)
        root.configuration->ematrix_solver_type = enums::Ematrix_solver_type::CG;
    else if (method == OCSL_BICGSTAB_REF)
        root.configuration->ematrix_solver_type = enums::Ematrix_solver_type::ILU_BICSTAB;
    else
        return -1;
    std::memcpy(g_solver.matrix.value.data(), val, g_solver.matrix.value.size() * sizeof(double));
    std::memcpy(g_solver.b_vector.value.data(), b, n * sizeof(double));
    std::memcpy(g_solver.x_vector.value.data(), x, n * sizeof(double));
    g_solver.solve();
    std::memcpy(x, g_solver.x_vector.value.data(), n * sizeof(double));
    return 0;
}

unsigned long long simple_host_elapsed_us(void)
{
    return root.total_elapsed_matrix_solution_time;
}

}  // extern "C"
