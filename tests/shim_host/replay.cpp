// Replays recorded CMatrix_solver calls through the C++ drop-in on the GPU:
// the calls a SIMPLE loop makes (fill matrix / b_vector / x_vector of ONE
// solver object, pick the method through root.configuration, call solve(),
// read x_vector), linked with -Wl,--wrap so that solve(), CG_solve() and
// ILU_BICGSTAB_solve() land in the drop-in and from there in
// libocsl_gb300.so.  Test infrastructure (tests/test_gpu_dropin.py).
//
//   replay <calls.bin> <out.bin>
// calls.bin: u64 n, u64 nnz, u64 ncalls, row_ptr[n+1], column_index[nnz], then
// per call: i32 method (0 CG, 1 ILU_BICSTAB, 2 direct CG_solve(), 3 direct
// ILU_BICGSTAB_solve()), value[nnz], b[n], x0[n].
// out.bin: per call x[n] and the returned residual (0 for solve()), then the
// accumulated root.total_elapsed_matrix_solution_time (u64, microseconds).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "croot.h"

Croot root;

template <typename T>
static bool rd(FILE* f, T* p, size_t n)
{
    return std::fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char** argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: replay calls.bin out.bin\n");
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    FILE* o = std::fopen(argv[2], "wb");
    if (!f || !o) {
        std::perror("open");
        return 2;
    }
    uint64_t hdr[3];
    if (!rd(f, hdr, 3)) return 3;
    const size_t n = hdr[0], nnz = hdr[1], ncalls = hdr[2];
    CMatrix_solver s;  // one object for every equation, as the reference has
    s.matrix.row_ptr.resize(n + 1);
    s.matrix.column_index.resize(nnz);
    s.matrix.value.resize(nnz);
    s.b_vector.value.resize(n);
    s.x_vector.value.resize(n);
    if (!rd(f, s.matrix.row_ptr.data(), n + 1) || !rd(f, s.matrix.column_index.data(), nnz))
        return 3;
    for (size_t k = 0; k < ncalls; ++k) {
        int32_t method = 0;
        if (!rd(f, &method, 1) || !rd(f, s.matrix.value.data(), nnz) ||
            !rd(f, s.b_vector.value.data(), n) || !rd(f, s.x_vector.value.data(), n))
            return 3;
        double res = 0.0;
        if (method == 0 || method == 1) {
            root.configuration->ematrix_solver_type =
                method == 0 ? enums::Ematrix_solver_type::CG : enums::Ematrix_solver_type::ILU_BICSTAB;
            s.solve();
        } else if (method == 2) {
            res = s.CG_solve();
        } else {
            res = s.ILU_BICGSTAB_solve();
        }
        std::fwrite(s.x_vector.value.data(), sizeof(double), n, o);
        std::fwrite(&res, sizeof(double), 1, o);
    }
    const uint64_t us = root.total_elapsed_matrix_solution_time;
    std::fwrite(&us, sizeof(us), 1, o);
    std::fclose(o);
    std::fclose(f);
    return 0;
}
