// Test infrastructure only: runs the UNMODIFIED reference SIMPLE loop one
// inner iteration at a time -- CFlow_solver::iterate (cflow_solver.cpp:229-476)
// and update_timestep (:503-519), the calls Croot::start_solver makes
// (croot.cpp:119-252) -- on the 1000-cell 1D shock tube (shocktube_config.h),
// the 200-cell viscous channel / steady cases or a 3D viscous channel on a mesh
// read from an SU2 file (flow_configs.h), and writes
// the whole flow state at chosen points, so that the device SIMPLE iteration
// and its oracle restatement can be checked against the reference's own
// arithmetic.
//
// Linked by oracle/Makefile with -Wl,--wrap=_ZN14CMatrix_solver5solveEv: the
// wrapper picks the linear solver per equation (the reference has one global
// switch, cconfiguration.cpp:213-228) and, inside a recorded inner iteration,
// writes the flow state and the assembled system right before each of the
// five solves.
//
// Usage: ref_flow <out_dir> <shocktube|channel|steady|box3d=<mesh.su2>> <bicg|cg> <steps>
//                 <inner> <record spec...>
//   bicg: every equation through ILU_BICGSTAB_solve; cg: the three momentum
//   equations through CG_solve, p' and enthalpy through ILU_BICGSTAB_solve.
//   A record spec "s:i" records inner iteration i of step s: the state before
//   each solve (pre_s_i_e.bin, e = 0..4) and after the iteration (post_s_i.bin).
// Also written: setup.bin (mesh metrics, fluid constants, initial state),
// final.bin (the state after the last step) and the reference's VTK files of
// that state, solution.vtk and solution_BC.vtk (Cpost_processing).
// File format: repeated [u32 name length][name][u8 kind 'd'|'i'|'u'][u64 count][data].
#include "croot.h"
#include "flow_configs.h"
#include "shocktube_config.h"

#include <omp.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <utility>
#include <vector>

extern "C" void __real__ZN14CMatrix_solver5solveEv(CMatrix_solver* self);

namespace {

std::string g_out;
bool g_cg = false;
long g_call = 0;
std::set<std::pair<int, int>> g_record;

struct Writer {
    FILE* f;
    explicit Writer(const std::string& path) : f(std::fopen(path.c_str(), "wb"))
    {
        if (!f) { std::perror(path.c_str()); std::exit(2); }
    }
    ~Writer() { std::fclose(f); }
    void raw(const void* p, size_t bytes)
    {
        if (bytes && std::fwrite(p, 1, bytes, f) != bytes) { std::perror("fwrite"); std::exit(2); }
    }
    void put(const char* name, char kind, const void* data, uint64_t count, size_t elem)
    {
        uint32_t len = (uint32_t)std::strlen(name);
        raw(&len, 4);
        raw(name, len);
        raw(&kind, 1);
        raw(&count, 8);
        raw(data, count * elem);
    }
    void d(const char* name, const std::vector<double>& v) { put(name, 'd', v.data(), v.size(), 8); }
    void i(const char* name, const std::vector<int32_t>& v) { put(name, 'i', v.data(), v.size(), 4); }
    void u(const char* name, const std::vector<uint64_t>& v) { put(name, 'u', v.data(), v.size(), 8); }
};

template <class C, class F>
std::vector<double> col(const C& items, F f)
{
    std::vector<double> v;
    v.reserve(items.size());
    for (const auto& it : items) v.push_back(f(it));
    return v;
}

template <class C, class F>
std::vector<double> col3(const C& items, F f)  // [3][count], component-major
{
    std::vector<double> v(3 * items.size());
    for (size_t k = 0; k < items.size(); ++k) {
        const Svector s = f(items[k]);
        for (int d = 0; d < 3; ++d) v[d * items.size() + k] = s.val[d];
    }
    return v;
}

template <class C, class F>
std::vector<int32_t> coli(const C& items, F f)
{
    std::vector<int32_t> v;
    v.reserve(items.size());
    for (const auto& it : items) v.push_back((int32_t)f(it));
    return v;
}

using Fc = CFlow_solver::CFlow_cell;
using Ff = CFlow_solver::CFlow_face;
using Fb = CFlow_solver::CFlow_BC_face;
using Vf = CFVM::CFVM_face;
using Vb = CFVM::CFVM_BC_face;

// Every field of the flow state that the SIMPLE iteration reads or writes.
void write_state(Writer& w)
{
    const auto& fl = *root.Flow_solver;
    w.d("cell_velocity", col3(fl.cells, [](const Fc& c) { return c.Velocity; }));
    w.d("cell_velocity_last", col3(fl.cells, [](const Fc& c) { return c.Velocity_last_t; }));
    w.d("cell_density", col(fl.cells, [](const Fc& c) { return c.Density; }));
    w.d("cell_density_last", col(fl.cells, [](const Fc& c) { return c.Density_last_t; }));
    w.d("cell_pressure", col(fl.cells, [](const Fc& c) { return c.Pressure; }));
    w.d("cell_pressure_last", col(fl.cells, [](const Fc& c) { return c.Pressure_last_t; }));
    w.d("cell_pressure_grad", col3(fl.cells, [](const Fc& c) { return c.Pressure_grad; }));
    w.d("cell_pressure_corr", col(fl.cells, [](const Fc& c) { return c.Pressure_corr; }));
    w.d("cell_pressure_corr_grad", col3(fl.cells, [](const Fc& c) { return c.Pressure_corr_grad; }));
    w.d("cell_enthalpy", col(fl.cells, [](const Fc& c) { return c.Enthalpy; }));
    w.d("cell_enthalpy_last", col(fl.cells, [](const Fc& c) { return c.Enthalpy_last_t; }));
    w.d("cell_ap", col(fl.cells, [](const Fc& c) { return c.ap; }));
    w.d("cell_ap_vec", col3(fl.cells, [](const Fc& c) { return c.ap_vec; }));
    w.d("cell_delta_t", col(fl.cells, [](const Fc& c) { return c.delta_t; }));
    w.d("cell_temperature", col(fl.cells, [](const Fc& c) { return c.Temperature; }));
    w.d("cell_total_mdot", col(fl.cells, [](const Fc& c) { return c.total_mdot; }));
    w.d("cell_mach", col(fl.cells, [](const Fc& c) { return c.Mach; }));
    w.d("face_mdot", col(fl.faces, [](const Ff& f) { return f.Mdot; }));
    w.d("face_density", col(fl.faces, [](const Ff& f) { return f.Density; }));
    w.d("face_qy", col(fl.faces, [](const Ff& f) { return f.Qy; }));
    w.d("face_stress", col3(fl.faces, [](const Ff& f) { return f.stress_explicit_part; }));
    w.i("bc_type", coli(fl.BC_faces, [](const Fb& f) { return (int)f.eflow_BC_type; }));
    w.i("bc_wall", coli(fl.BC_faces, [](const Fb& f) { return (int)f.ewall_BC_type; }));
    w.i("bc_thermal", coli(fl.BC_faces, [](const Fb& f) { return (int)f.eThermal_BC_type; }));
    w.i("bc_supersonic", coli(fl.BC_faces, [](const Fb& f) { return f.supersonic_flag ? 1 : 0; }));
    w.d("bc_pressure", col(fl.BC_faces, [](const Fb& f) { return f.Pressure; }));
    w.d("bc_out_pressure", col(fl.BC_faces, [](const Fb& f) { return f.Out_Pressure; }));
    w.d("bc_mdot", col(fl.BC_faces, [](const Fb& f) { return f.Mdot; }));
    w.d("bc_density", col(fl.BC_faces, [](const Fb& f) { return f.Density; }));
    w.d("bc_qy", col(fl.BC_faces, [](const Fb& f) { return f.Qy; }));
    w.d("bc_temperature", col(fl.BC_faces, [](const Fb& f) { return f.Temperature; }));
    w.d("bc_enthalpy", col(fl.BC_faces, [](const Fb& f) { return f.Enthalpy; }));
    w.d("bc_velocity", col3(fl.BC_faces, [](const Fb& f) { return f.Velocity; }));
    w.d("residuals", {fl.Momentum_global_residual.val[0], fl.Momentum_global_residual.val[1],
                      fl.Momentum_global_residual.val[2], fl.Pressure_global_residual,
                      fl.Enthalpy_global_residual});
    w.d("implicit_underrelaxation", {fl.implicit_underrelaxation});
}

// CFlow_solver::iterate for the configuration's three switches (croot.cpp:139-213).
template <enums::Etimestepping_type T, enums::Eflow_type_visc V>
void iterate_flux()
{
    auto& fl = *root.Flow_solver;
    if (root.configuration->econv_flux_type == enums::Econv_flux_type::Blended_central)
        fl.iterate<T, V, enums::Econv_flux_type::Blended_central>(root.FVM, root.Matrix_solver,
                                                                  root.Fluid_properties);
    else
        fl.iterate<T, V, enums::Econv_flux_type::First_order_upwind>(root.FVM, root.Matrix_solver,
                                                                     root.Fluid_properties);
}

template <enums::Etimestepping_type T>
void iterate_visc()
{
    if (root.configuration->eflow_type_visc == enums::Eflow_type_visc::Viscous)
        iterate_flux<T, enums::Eflow_type_visc::Viscous>();
    else
        iterate_flux<T, enums::Eflow_type_visc::Inviscid>();
}

void iterate_once()
{
    if (root.configuration->etimestepping_type == enums::Etimestepping_type::Transient)
        iterate_visc<enums::Etimestepping_type::Transient>();
    else
        iterate_visc<enums::Etimestepping_type::Steady>();
}

void write_setup()
{
    const auto& fvm = *root.FVM;
    const auto& fl = *root.Flow_solver;
    const auto& fp = *root.Fluid_properties;
    Writer w(g_out + "/setup.bin");
    const auto& cfg = *root.configuration;
    w.i("switches", {cfg.eflow_type_visc == enums::Eflow_type_visc::Viscous ? 1 : 0,
                     cfg.econv_flux_type == enums::Econv_flux_type::Blended_central ? 1 : 0,
                     cfg.etimestepping_type == enums::Etimestepping_type::Transient ? 1 : 0});
    w.d("relax_ramp", {cfg.implicit_underrelax, cfg.implicit_underrelax_max,
                       (double)cfg.underrelax_ramp_iteration});
    w.d("fluid", {fp.R_specific, fp.gamma, fp.Sutherland_coefs[0], fp.Sutherland_coefs[1],
                  fp.Prandlt_number, fl.implicit_underrelaxation, fp.cp, fp.Tref,
                  fp.H_formation, fl.explicit_underrelaxation_P, fl.explicit_underrelaxation_u});
    w.i("face_left", coli(fvm.faces, [](const Vf& f) { return f.left_cell_index; }));
    w.i("face_right", coli(fvm.faces, [](const Vf& f) { return f.right_cell_index; }));
    w.d("face_geo_aver", col(fvm.faces, [](const Vf& f) { return f.geo_aver; }));
    w.d("face_ksi_A", col(fvm.faces, [](const Vf& f) { return f.diffusion_ksi_A; }));
    w.d("face_area_vector", col3(fvm.faces, [](const Vf& f) { return f.area_vector; }));
    w.d("face_alpha", col3(fvm.faces, [](const Vf& f) { return f.alpha; }));
    w.d("face_distance", col(fvm.faces, [](const Vf& f) { return f.cell_center_distance; }));
    w.d("face_unit", col3(fvm.faces, [](const Vf& f) { return f.cell_center_unit_vector; }));
    w.i("bc_left", coli(fvm.BC_faces, [](const Vb& f) { return f.left_cell_index; }));
    w.i("bc_marker", coli(fvm.BC_faces, [](const Vb& f) {
            return root.geometry->faces[f.global_face_index].boundary_marker;
        }));
    w.d("bc_area", col(fvm.BC_faces, [](const Vb& f) { return f.area; }));
    w.d("bc_area_vector", col3(fvm.BC_faces, [](const Vb& f) { return f.area_vector; }));
    w.d("bc_alpha", col3(fvm.BC_faces, [](const Vb& f) { return f.alpha; }));
    w.d("bc_distance", col(fvm.BC_faces, [](const Vb& f) { return f.cell_center_distance; }));
    w.d("bc_unit", col3(fvm.BC_faces, [](const Vb& f) { return f.cell_center_unit_vector; }));
    w.d("bc_perp_dist", col(fvm.BC_faces, [](const Vb& f) { return f.perp_dist; }));
    w.d("bc_ksi_A", col(fvm.BC_faces, [](const Vb& f) { return f.diffusion_ksi_A; }));
    w.d("cell_volume", col(fvm.cells, [](const CFVM::CFVM_cell& c) { return c.volume; }));
    const auto& m = root.Matrix_solver->matrix;
    w.u("row_ptr", std::vector<uint64_t>(m.row_ptr.begin(), m.row_ptr.end()));
    w.u("column_index", std::vector<uint64_t>(m.column_index.begin(), m.column_index.end()));
    write_state(w);
}

}  // namespace

extern "C" void __wrap__ZN14CMatrix_solver5solveEv(CMatrix_solver* self)
{
    const int eq = int(g_call % 5);  // x, y, z momentum, p', enthalpy
    root.configuration->ematrix_solver_type = (g_cg && eq < 3)
                                                  ? enums::Ematrix_solver_type::CG
                                                  : enums::Ematrix_solver_type::ILU_BICSTAB;
    if (g_record.count({root.i_iteration, root.i_inner_iter})) {
        char name[512];
        std::snprintf(name, sizeof name, "%s/pre_%d_%d_%d.bin", g_out.c_str(), root.i_iteration,
                      root.i_inner_iter, eq);
        Writer w(name);
        write_state(w);
        w.d("value", self->matrix.value);
        w.d("b", self->b_vector.value);
        w.d("x0", self->x_vector.value);
        __real__ZN14CMatrix_solver5solveEv(self);
        w.d("x", self->x_vector.value);
    } else {
        __real__ZN14CMatrix_solver5solveEv(self);
    }
    ++g_call;
}

int main(int argc, char** argv)
{
    if (argc < 6) {
        std::fprintf(stderr, "usage: ref_flow <out_dir> <shocktube|channel|steady> <bicg|cg> "
                             "<steps> <inner> [s:i ...]\n");
        return 2;
    }
    g_out = argv[1];
    const std::string kase = argv[2];
    g_cg = std::strcmp(argv[3], "cg") == 0;
    const int steps = std::atoi(argv[4]), inner = std::atoi(argv[5]);
    for (int k = 6; k < argc; ++k) {
        int s = 0, i = 0;
        if (std::sscanf(argv[k], "%d:%d", &s, &i) == 2) g_record.insert({s, i});
    }
    Cconfiguration config;
    if (kase == "shocktube") {
        make_shocktube_config(config, 1, steps, inner);
    } else if (kase == "channel" || kase == "steady") {
        make_viscous_config(config, kase == "steady", steps, inner);
    } else if (kase.rfind("box3d=", 0) == 0) {
        make_box3d_config(config, kase.substr(6), steps, inner);
    } else {
        std::fprintf(stderr, "unknown case %s\n", kase.c_str());
        return 2;
    }
    root.configuration = std::make_shared<Cconfiguration>(config);
    omp_set_dynamic(0);
    omp_set_num_threads(1);
    root.create_geometry();
    root.initialize_solver();
    write_setup();
    auto& fl = *root.Flow_solver;
    for (int s = 0; s < steps; ++s) {
        for (int i = 0; i < inner; ++i) {
            root.i_iteration = s;
            root.i_inner_iter = i;
            iterate_once();
            if (g_record.count({s, i})) {
                char name[512];
                std::snprintf(name, sizeof name, "%s/post_%d_%d.bin", g_out.c_str(), s, i);
                Writer w(name);
                write_state(w);
            }
        }
        fl.update_timestep();
    }
    {
        Writer w(g_out + "/final.bin");
        write_state(w);
    }
    // the reference's own VTK output of the final state (croot.cpp:239-240)
    root.post_processing = std::make_shared<Cpost_processing>();
    root.post_processing->write_VTK_file(g_out + "/solution.vtk");
    root.post_processing->write_boundary_VTK_file(g_out + "/solution_BC.vtk");
    return 0;
}
