// Test infrastructure only: runs the UNMODIFIED reference SIMPLE loop
// (Croot::run_config, croot.cpp:35-49) on the 1000-cell 1D shock tube and
// records selected linear-solve calls plus the final fields, so that golden
// fixtures can be made from the reference itself.
//
// Linked by oracle/Makefile with -Wl,--wrap=_ZN14CMatrix_solver5solveEv: every
// call of CMatrix_solver::solve() made by the flow solver
// (cflow_solver.cpp:289,349,460) lands in the wrapper below, which
//   * picks the solver per equation: the reference only has one global
//     switch (cconfiguration.cpp:213-228), the workload wants CG for the
//     three momentum solves and ILU-BiCGSTAB for p' and enthalpy;
//   * for a recorded call, saves (values, b, x0) before and x after the
//     reference's own solve(), and the residual the reference's solver
//     returns on an identical copy of the solver object.
//
// Usage: ref_shocktube <out_dir> <threads> <steps> <inner> <record spec...>
// A record spec "s:i" records every equation of inner iteration i of step s.
#include "croot.h"
#include "shocktube_config.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <set>
#include <string>
#include <utility>

extern "C" void __real__ZN14CMatrix_solver5solveEv(CMatrix_solver* self);

namespace {

std::string g_out;
long g_call = 0;
bool g_pattern_written = false;
std::set<std::pair<int, int>> g_record;

void write_block(FILE* f, const void* p, size_t bytes)
{
    if (bytes && std::fwrite(p, 1, bytes, f) != bytes) {
        std::perror("fwrite");
        std::exit(2);
    }
}

void dump_pattern(CMatrix_solver* s)
{
    std::string path = g_out + "/pattern.bin";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    uint64_t n = s->matrix.n_rows, nnz = s->matrix.value.size();
    write_block(f, &n, 8);
    write_block(f, &nnz, 8);
    for (size_t v : s->matrix.row_ptr) { uint64_t u = v; write_block(f, &u, 8); }
    for (size_t v : s->matrix.column_index) { uint64_t u = v; write_block(f, &u, 8); }
    std::fclose(f);
}

}  // namespace

extern "C" void __wrap__ZN14CMatrix_solver5solveEv(CMatrix_solver* self)
{
    const int eq = int(g_call % 5);  // x, y, z momentum, p', enthalpy
    root.configuration->ematrix_solver_type =
        eq < 3 ? enums::Ematrix_solver_type::CG : enums::Ematrix_solver_type::ILU_BICSTAB;

    const bool rec = g_record.count({root.i_iteration, root.i_inner_iter}) != 0;
    if (!rec) {
        __real__ZN14CMatrix_solver5solveEv(self);
        ++g_call;
        return;
    }
    if (!g_pattern_written) {
        dump_pattern(self);
        g_pattern_written = true;
    }

    CMatrix_solver copy = *self;  // identical inputs for the residual probe
    const size_t n = self->b_vector.value.size();
    const size_t nnz = self->matrix.value.size();
    std::vector<double> x0 = self->x_vector.value;

    __real__ZN14CMatrix_solver5solveEv(self);
    const double res = eq < 3 ? copy.CG_solve() : copy.ILU_BICGSTAB_solve();

    char name[256];
    std::snprintf(name, sizeof name, "%s/call_%05ld.bin", g_out.c_str(), g_call);
    FILE* f = std::fopen(name, "wb");
    if (!f) { std::perror(name); std::exit(2); }
    int32_t hdr[4] = {root.i_iteration, root.i_inner_iter, eq, eq < 3 ? 0 : 1};
    uint64_t sizes[2] = {n, nnz};
    write_block(f, hdr, sizeof hdr);
    write_block(f, sizes, sizeof sizes);
    write_block(f, &res, 8);
    write_block(f, self->matrix.value.data(), nnz * 8);
    write_block(f, self->b_vector.value.data(), n * 8);
    write_block(f, x0.data(), n * 8);
    write_block(f, self->x_vector.value.data(), n * 8);
    // The copy's x must equal the original's: same inputs, same thread count.
    write_block(f, copy.x_vector.value.data(), n * 8);
    std::fclose(f);
    ++g_call;
}

int main(int argc, char** argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s out_dir threads steps inner [s:i ...]\n", argv[0]);
        return 1;
    }
    g_out = argv[1];
    const int threads = std::atoi(argv[2]);
    const int steps = std::atoi(argv[3]);
    const int inner = std::atoi(argv[4]);
    for (int a = 5; a < argc; ++a) {
        int s = 0, i = 0;
        if (std::sscanf(argv[a], "%d:%d", &s, &i) == 2) g_record.insert({s, i});
    }

    Cconfiguration config;
    make_shocktube_config(config, threads, steps, inner);
    root.run_config(config);

    if (int rc = write_shocktube_fields(g_out + "/fields.txt")) return rc;
    std::printf("solve calls: %ld\n", g_call);
    return 0;
}
