// Test infrastructure only: drives the UNMODIFIED reference through the two
// routes by which it reaches its linear solver, and is linked by
// oracle/Makefile three ways -- with the reference's own solver
// (ref_driver_cpu), with the C++ drop-in
// opencslsolver_gb300/shim/cmatrix_solver_gpu.cpp over an oracle-backed fake
// of the C ABI (ref_driver_fake), and with the drop-in over the GPU library
// (ref_driver_gpu).
//
//   ref_driver_* shocktube <fields.txt> <threads> <steps> <inner>
//       The reference SIMPLE loop (Croot::run_config, croot.cpp:35-49) on the
//       1000-cell shock tube with the reference's single solver switch
//       (ILU-BiCGSTAB for every equation, cconfiguration.cpp:213-228), through
//       CMatrix_solver::solve() (cflow_solver.cpp:289,349,460); writes the
//       final fields.
//   ref_driver_* unit
//       The reference's own solver unit tests (cmatrix_solver_supply.h:29-114),
//       which call CG_solve() and ILU_BICGSTAB_solve() directly and print the
//       residuals they return.
#include "croot.h"
#include "cmatrix_solver_supply.h"
#include "shocktube_config.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

int main(int argc, char** argv)
{
    if (argc >= 2 && !std::strcmp(argv[1], "unit")) {
        std::cout.precision(17);
        unit_tests::test_matrix_solver_cg();
        unit_tests::test_matrix_solver_ILU_BICGSTAB();
        return 0;
    }
    if (argc < 6 || std::strcmp(argv[1], "shocktube")) {
        std::fprintf(stderr, "usage: %s shocktube fields.txt threads steps inner | unit\n",
                     argv[0]);
        return 1;
    }
    Cconfiguration config;
    make_shocktube_config(config, std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]));
    root.run_config(config);
    return write_shocktube_fields(argv[2]);
}
