// Test stand-in for the reference program's headers, used to build the C++
// drop-in (opencslsolver_gb300/shim/cmatrix_solver_gpu.cpp) where the
// reference's own sources are absent -- the GPU host.  It declares, under the
// reference's names, only what the drop-in reads or writes:
//   CMatrix_solver::matrix.{value,row_ptr,column_index}, b_vector.value,
//   x_vector.value and the three solver members (cmatrix_solver.h:27-95);
//   root.configuration->ematrix_solver_type (croot.h:53, enums.h:46) and
//   root.total_elapsed_matrix_solution_time (croot.h:67).
// Names and member types follow the reference so that the drop-in compiles
// unchanged and its member functions get the reference's mangled names
// (e.g. _ZN14CMatrix_solver5solveEv); nothing else of the reference is here.
#pragma once
#include <cstddef>
#include <memory>
#include <vector>

namespace enums {
enum class Ematrix_solver_type { CG, ILU_BICSTAB };
}

class CMatrix_solver {
public:
    struct CCSR {
        std::vector<double> value;
        std::vector<size_t> row_ptr;
        std::vector<size_t> column_index;
    };
    struct Cvector {
        std::vector<double> value;
    };
    double CG_solve();
    double ILU_BICGSTAB_solve();
    void solve();
    CCSR matrix;
    Cvector b_vector;
    Cvector x_vector;
};

struct Cconfiguration {
    enums::Ematrix_solver_type ematrix_solver_type = enums::Ematrix_solver_type::ILU_BICSTAB;
};

struct Croot {
    std::shared_ptr<Cconfiguration> configuration = std::make_shared<Cconfiguration>();
    unsigned long long int total_elapsed_matrix_solution_time = 0;
};

extern Croot root;
