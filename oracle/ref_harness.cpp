// Test infrastructure only: a C-ABI harness around the UNMODIFIED reference
// solver (OpenCSLSolver's CMatrix_solver, cmatrix_solver.h:27-95), compiled
// together with the reference's own sources by oracle/Makefile into
// oracle/_ref/liboracle_ref.so.  It lets the Python tests pin the oracle
// restatement (oracle/ocsl_oracle.c) and generate golden vectors.
//
// Every function fills the reference's public CSR / vector members directly
// (the reference's pattern builder CCSR::insert_element,
// cmatrix_solver.cpp:57-103, is quadratic) and then calls the reference's own
// member function.  Column indices use the reference's size_t layout, so a
// boundary row's phantom column (size_t)-1 (cfvm.cpp:89-94) is passed through
// unchanged.
#include "croot.h"

#include <cstdint>
#include <cstring>
#include <omp.h>

namespace {

CMatrix_solver make_solver(size_t n, size_t nnz, const uint64_t* rp,
                           const uint64_t* col, const double* val)
{
    CMatrix_solver s(n, n, nnz);
    s.matrix.row_ptr.assign(rp, rp + n + 1);
    s.matrix.column_index.assign(col, col + nnz);
    s.matrix.value.assign(val, val + nnz);
    // Same preparation as CFVM::define_matrix_structure (cfvm.cpp:96-97).
    s.M = s.matrix;
    s.extract_diag_indexes();
    return s;
}

void load_vec(CMatrix_solver::Cvector& v, size_t n, const double* src)
{
    v.value.assign(src, src + n);
    v.n_values = n;
}

}  // namespace

extern "C" {

void refh_set_threads(int t)
{
    omp_set_dynamic(0);
    omp_set_num_threads(t);
}

// cmatrix_solver.cpp:635 CG_solve: returns the reference's residual, x in/out.
double refh_cg_solve(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
                     const double* val, const double* b, double* x)
{
    CMatrix_solver s = make_solver(n, nnz, rp, col, val);
    load_vec(s.b_vector, n, b);
    load_vec(s.x_vector, n, x);
    double res = s.CG_solve();
    std::memcpy(x, s.x_vector.value.data(), n * sizeof(double));
    return res;
}

// cmatrix_solver.cpp:682 ILU_BICGSTAB_solve.
double refh_bicgstab_solve(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
                           const double* val, const double* b, double* x)
{
    CMatrix_solver s = make_solver(n, nnz, rp, col, val);
    load_vec(s.b_vector, n, b);
    load_vec(s.x_vector, n, x);
    double res = s.ILU_BICGSTAB_solve();
    std::memcpy(x, s.x_vector.value.data(), n * sizeof(double));
    return res;
}

// cmatrix_solver.cpp:338 / :369 gemv.  z == nullptr selects the 4-argument form.
void refh_gemv(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
               const double* val, double a, const double* x, double bcoef,
               const double* z, double* y)
{
    CMatrix_solver s = make_solver(n, nnz, rp, col, val);
    CMatrix_solver::Cvector vx(n), vz(n), vy(n);
    load_vec(vx, n, x);
    if (z) {
        load_vec(vz, n, z);
        s.gemv(a, s.matrix, vx, bcoef, vz, vy);
    } else {
        s.gemv(a, s.matrix, vx, vy);
    }
    std::memcpy(y, vy.value.data(), n * sizeof(double));
}

// cmatrix_solver.cpp:233 norm (a dot product).
// cmatrix_solver.cpp:244-263 (static members)
double refh_sum(size_t n, const double* x, int absolute)
{
    CMatrix_solver::Cvector vx(n);
    load_vec(vx, n, x);
    return absolute ? CMatrix_solver::ABSsum(vx) : CMatrix_solver::sum(vx);
}

// :266-272 product
void refh_product(size_t n, const double* x, const double* y, double* out)
{
    CMatrix_solver s(n, n, 0);
    CMatrix_solver::Cvector vx(n), vy(n), vo(n);
    load_vec(vx, n, x);
    load_vec(vy, n, y);
    s.product(vx, vy, vo);
    std::memcpy(out, vo.value.data(), n * sizeof(double));
}

// :275-335 axpy (y == NULL: the one-vector overload)
void refh_axpy(size_t n, double a, const double* x, double b, const double* y, double* out)
{
    CMatrix_solver s(n, n, 0);
    CMatrix_solver::Cvector vx(n), vy(n), vo(n);
    load_vec(vx, n, x);
    if (y) {
        load_vec(vy, n, y);
        s.axpy(a, vx, b, vy, vo);
    } else {
        s.axpy(a, vx, vo);
    }
    std::memcpy(out, vo.value.data(), n * sizeof(double));
}

double refh_norm(size_t n, const double* x, const double* y)
{
    CMatrix_solver s(n, n, 0);
    CMatrix_solver::Cvector vx(n), vy(n);
    load_vec(vx, n, x);
    load_vec(vy, n, y);
    return s.norm(vx, vy);
}

// cmatrix_solver.cpp:455 extract_diag_indexes.
void refh_extract_diag(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
                       int32_t* diag)
{
    std::vector<double> zeros(nnz, 0.0);
    CMatrix_solver s = make_solver(n, nnz, rp, col, zeros.data());
    for (size_t i = 0; i < n; ++i) diag[i] = s.diag_index[i];
}

// cmatrix_solver.cpp:472 ILU_decompose, prepared the way ILU_BICGSTAB_solve
// prepares it (:702-704): M starts as a copy of A.
void refh_ilu_decompose(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
                        const double* A, double* M_out)
{
    CMatrix_solver s = make_solver(n, nnz, rp, col, A);
    s.M.copy_same_structure(s.matrix);
    s.ILU_decompose(s.matrix, s.M, s.diag_index);
    std::memcpy(M_out, s.M.value.data(), nnz * sizeof(double));
}

// cmatrix_solver.cpp:555 ILU_forsub with a given factor M.
void refh_forsub(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
                 const double* M, const double* b, double* y)
{
    CMatrix_solver s = make_solver(n, nnz, rp, col, M);
    CMatrix_solver::Cvector vb(n), vy(n);
    load_vec(vb, n, b);
    s.ILU_forsub(s.M, s.diag_index, vb, vy);
    std::memcpy(y, vy.value.data(), n * sizeof(double));
}

// cmatrix_solver.cpp:595 ILU_backsub with a given factor M.
void refh_backsub(size_t n, size_t nnz, const uint64_t* rp, const uint64_t* col,
                  const double* M, const double* y, double* x)
{
    CMatrix_solver s = make_solver(n, nnz, rp, col, M);
    CMatrix_solver::Cvector vy(n), vx(n);
    load_vec(vy, n, y);
    s.ILU_backsub(s.M, s.diag_index, vy, vx);
    std::memcpy(x, vx.value.data(), n * sizeof(double));
}

}  // extern "C"
