// Test infrastructure only: records the inputs and outputs of the reference's
// face-loop coefficient assembly (cflow_solver_cell_face_loops.cpp:25-446,
// solvers_common.h:32-151) from the UNMODIFIED reference SIMPLE loop, so the
// GPU assembly can be checked against it on CPU-free fixtures.
//
// Linked by oracle/Makefile with -Wl,--wrap=_ZN14CMatrix_solver5solveEv.  The
// flow solver assembles one equation and calls CMatrix_solver::solve()
// (cflow_solver.cpp:289,349,460) right after; at that moment the solver's
// matrix, b and x hold the assembled system, and the cell / face state holds
// exactly the inputs the assembly read (the assembly writes only ap, ap_vec
// and total_mdot, recorded as side outputs).  For every recorded call the
// wrapper writes one file of named arrays, then runs the reference's solve.
//
// Usage: ref_assembly <out_dir> <case> <first_call> <n_calls>
//   cases: shocktube  1000-cell shock tube, inviscid, blended, transient
//          channel    200 cells, viscous, upwind, transient, velocity inlet,
//                     no-slip side walls, pressure outlet
//          steady     200 cells, viscous, blended, steady with implicit
//                     under-relaxation, supersonic inlet, slip walls, outlet
//          heat       100-cell heat conduction (cheat_solver.cpp), fixed
//                     temperatures at both ends, adiabatic sides
//          heat3d=<mesh.su2>  heat conduction on a mesh read from an SU2 file
//                     (markers inlet, walls, outlet: 250 K, adiabatic, 450 K),
//                     6 steps; run from <out_dir> as the working directory, the
//                     reference's own run writes solution.vtk / solution_BC.vtk
//                     there (croot.cpp:239-240), and final_heat.bin holds the
//                     state they were written from
// File format: repeated [u32 name length][name][u8 kind 'd'|'i'|'u'][u64 count][data].
#include "croot.h"
#include "flow_configs.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

extern "C" void __real__ZN14CMatrix_solver5solveEv(CMatrix_solver* self);

namespace {

std::string g_out;
long g_call = 0, g_first = 0, g_count = 0;

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

void record(CMatrix_solver* s, int eq)
{
    const auto& fvm = *root.FVM;
    const auto& fl = *root.Flow_solver;
    const auto& fp = *root.Fluid_properties;
    const auto& cfg = *root.configuration;
    char name[512];
    std::snprintf(name, sizeof name, "%s/call_%05ld.bin", g_out.c_str(), g_call);
    Writer w(name);
    w.i("meta", {eq, cfg.eflow_type_visc == enums::Eflow_type_visc::Viscous ? 1 : 0,
                 cfg.econv_flux_type == enums::Econv_flux_type::Blended_central ? 1 : 0,
                 cfg.etimestepping_type == enums::Etimestepping_type::Transient ? 1 : 0});
    w.d("fluid", {fp.R_specific, fp.gamma, fp.Sutherland_coefs[0], fp.Sutherland_coefs[1],
                  fp.Prandlt_number, fl.implicit_underrelaxation});
    // mesh: interior faces, boundary faces, cells
    w.i("face_left", coli(fvm.faces, [](const CFVM::CFVM_face& f) { return f.left_cell_index; }));
    w.i("face_right", coli(fvm.faces, [](const CFVM::CFVM_face& f) { return f.right_cell_index; }));
    w.d("face_geo_aver", col(fvm.faces, [](const CFVM::CFVM_face& f) { return f.geo_aver; }));
    w.d("face_ksi_A", col(fvm.faces, [](const CFVM::CFVM_face& f) { return f.diffusion_ksi_A; }));
    w.i("bc_left", coli(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.left_cell_index; }));
    w.d("bc_area", col(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.area; }));
    w.d("bc_area_vector", col3(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.area_vector; }));
    w.d("bc_perp_dist", col(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.perp_dist; }));
    w.d("bc_ksi_A", col(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.diffusion_ksi_A; }));
    w.d("cell_volume", col(fvm.cells, [](const CFVM::CFVM_cell& c) { return c.volume; }));
    // flow state
    using Fc = CFlow_solver::CFlow_cell;
    using Ff = CFlow_solver::CFlow_face;
    using Fb = CFlow_solver::CFlow_BC_face;
    w.d("face_mdot", col(fl.faces, [](const Ff& f) { return f.Mdot; }));
    w.d("face_density", col(fl.faces, [](const Ff& f) { return f.Density; }));
    w.d("face_qy", col(fl.faces, [](const Ff& f) { return f.Qy; }));
    w.d("face_stress", col3(fl.faces, [](const Ff& f) { return f.stress_explicit_part; }));
    w.i("bc_type", coli(fl.BC_faces, [](const Fb& f) { return (int)f.eflow_BC_type; }));
    w.i("bc_wall", coli(fl.BC_faces, [](const Fb& f) { return (int)f.ewall_BC_type; }));
    w.i("bc_thermal", coli(fl.BC_faces, [](const Fb& f) { return (int)f.eThermal_BC_type; }));
    w.i("bc_supersonic", coli(fl.BC_faces, [](const Fb& f) { return f.supersonic_flag ? 1 : 0; }));
    w.d("bc_mdot", col(fl.BC_faces, [](const Fb& f) { return f.Mdot; }));
    w.d("bc_density", col(fl.BC_faces, [](const Fb& f) { return f.Density; }));
    w.d("bc_qy", col(fl.BC_faces, [](const Fb& f) { return f.Qy; }));
    w.d("bc_temperature", col(fl.BC_faces, [](const Fb& f) { return f.Temperature; }));
    w.d("bc_enthalpy", col(fl.BC_faces, [](const Fb& f) { return f.Enthalpy; }));
    w.d("bc_velocity", col3(fl.BC_faces, [](const Fb& f) { return f.Velocity; }));
    w.d("cell_velocity", col3(fl.cells, [](const Fc& c) { return c.Velocity; }));
    w.d("cell_velocity_last", col3(fl.cells, [](const Fc& c) { return c.Velocity_last_t; }));
    w.d("cell_pressure_grad", col3(fl.cells, [](const Fc& c) { return c.Pressure_grad; }));
    w.d("cell_density", col(fl.cells, [](const Fc& c) { return c.Density; }));
    w.d("cell_density_last", col(fl.cells, [](const Fc& c) { return c.Density_last_t; }));
    w.d("cell_pressure", col(fl.cells, [](const Fc& c) { return c.Pressure; }));
    w.d("cell_pressure_last", col(fl.cells, [](const Fc& c) { return c.Pressure_last_t; }));
    w.d("cell_pressure_corr", col(fl.cells, [](const Fc& c) { return c.Pressure_corr; }));
    w.d("cell_temperature", col(fl.cells, [](const Fc& c) { return c.Temperature; }));
    w.d("cell_enthalpy", col(fl.cells, [](const Fc& c) { return c.Enthalpy; }));
    w.d("cell_enthalpy_last", col(fl.cells, [](const Fc& c) { return c.Enthalpy_last_t; }));
    w.d("cell_delta_t", col(fl.cells, [](const Fc& c) { return c.delta_t; }));
    // the assembled system and side outputs
    std::vector<uint64_t> rp(s->matrix.row_ptr.begin(), s->matrix.row_ptr.end());
    std::vector<uint64_t> ci(s->matrix.column_index.begin(), s->matrix.column_index.end());
    w.u("row_ptr", rp);
    w.u("column_index", ci);
    w.d("value", s->matrix.value);
    w.d("b", s->b_vector.value);
    w.d("x0", s->x_vector.value);
    w.d("cell_ap_vec", col3(fl.cells, [](const Fc& c) { return c.ap_vec; }));
    w.d("cell_total_mdot", col(fl.cells, [](const Fc& c) { return c.total_mdot; }));
}

// Heat conduction (cheat_solver.cpp:32-65): the equation's inputs are the
// cell temperatures, the boundary faces' thermal kind and temperature, the
// diffusivity and the global time step.
void record_heat(CMatrix_solver* s)
{
    const auto& fvm = *root.FVM;
    const auto& hs = *root.Heat_solver;
    const auto& cfg = *root.configuration;
    char name[512];
    std::snprintf(name, sizeof name, "%s/call_%05ld.bin", g_out.c_str(), g_call);
    Writer w(name);
    w.i("meta", {5, 0, 0, 1});
    w.d("fluid", {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, cfg.thermal_diffusivity, cfg.global_delta_t});
    w.i("face_left", coli(fvm.faces, [](const CFVM::CFVM_face& f) { return f.left_cell_index; }));
    w.i("face_right", coli(fvm.faces, [](const CFVM::CFVM_face& f) { return f.right_cell_index; }));
    w.d("face_ksi_A", col(fvm.faces, [](const CFVM::CFVM_face& f) { return f.diffusion_ksi_A; }));
    w.i("bc_left", coli(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.left_cell_index; }));
    w.d("bc_ksi_A", col(fvm.BC_faces, [](const CFVM::CFVM_BC_face& f) { return f.diffusion_ksi_A; }));
    w.d("cell_volume", col(fvm.cells, [](const CFVM::CFVM_cell& c) { return c.volume; }));
    using Hc = CHeat_solver::CHeat_cell;
    using Hb = CHeat_solver::CHeat_BC_face;
    w.i("bc_thermal", coli(hs.BC_faces, [](const Hb& f) { return (int)f.ethermal_BC_type; }));
    w.d("bc_temperature", col(hs.BC_faces, [](const Hb& f) { return f.Temperature; }));
    w.d("cell_temperature", col(hs.cells, [](const Hc& c) { return c.Temperature; }));
    std::vector<uint64_t> rp(s->matrix.row_ptr.begin(), s->matrix.row_ptr.end());
    std::vector<uint64_t> ci(s->matrix.column_index.begin(), s->matrix.column_index.end());
    w.u("row_ptr", rp);
    w.u("column_index", ci);
    w.d("value", s->matrix.value);
    w.d("b", s->b_vector.value);
    w.d("x0", s->x_vector.value);
}

}  // namespace

extern "C" void __wrap__ZN14CMatrix_solver5solveEv(CMatrix_solver* self)
{
    const bool heat = root.configuration->eproblem_type == enums::Eproblem_type::Heat_conduction;
    const int eq = int(g_call % 5);  // x, y, z momentum, p', enthalpy (cflow_solver.cpp)
    if (g_call >= g_first && g_call < g_first + g_count) {
        if (heat)
            record_heat(self);
        else
            record(self, eq);
    }
    __real__ZN14CMatrix_solver5solveEv(self);
    ++g_call;
}

int main(int argc, char** argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s out_dir case first_call n_calls\n", argv[0]);
        return 1;
    }
    g_out = argv[1];
    const std::string kase = argv[2];
    g_first = std::atol(argv[3]);
    g_count = std::atol(argv[4]);
    Cconfiguration c;
    auto& ic = *c.inital_condition;
    if (kase == "shocktube") {
        base_1d(c, 1000);
        c.eflow_type_visc = enums::Eflow_type_visc::Inviscid;
        c.econv_flux_type = enums::Econv_flux_type::Blended_central;
        c.etimestepping_type = enums::Etimestepping_type::Transient;
        c.global_delta_t = 1.0e-6;
        ic.einitial_condition_type = enums::Einitial_condition_type::Shock_tube;
        ic.Pressure = 1.0e5;
        ic.Temperature = 348.4;
        ic.Pressure2 = 1.0e4;
        ic.Temperature2 = 278.7;
        ic.Velocity.val[0] = ic.Velocity.val[1] = ic.Velocity.val[2] = 0.0;
        c.boundary_conditions[0].eflow_BC_type = enums::Eflow_BC_type::wall;
        c.boundary_conditions[0].ewall_BC_type = enums::Ewall_BC_type::slip;
        c.boundary_conditions[1].eflow_BC_type = enums::Eflow_BC_type::empty;
        c.boundary_conditions[2].eflow_BC_type = enums::Eflow_BC_type::wall;
        c.boundary_conditions[2].ewall_BC_type = enums::Ewall_BC_type::slip;
        c.max_iteration = 2;
        c.max_inner_iteration = 3;
    } else if (kase == "channel" || kase == "steady") {
        const bool steady = kase == "steady";
        make_viscous_config(c, steady, steady ? 4 : 2, steady ? 1 : 3);
    } else if (kase == "heat") {
        base_1d(c, 100);
        c.eproblem_type = enums::Eproblem_type::Heat_conduction;
        c.global_delta_t = 50.0;
        c.thermal_diffusivity = 2.0e-3;
        ic.Temperature = 300.0;
        c.boundary_conditions[0].ethermal_BC_type = enums::Ethermal_BC_type::constant_temperature;
        c.boundary_conditions[0].Temperature = 250.0;
        c.boundary_conditions[1].ethermal_BC_type = enums::Ethermal_BC_type::adiabatic;
        c.boundary_conditions[2].ethermal_BC_type = enums::Ethermal_BC_type::constant_temperature;
        c.boundary_conditions[2].Temperature = 450.0;
        c.max_iteration = 6;
        c.max_inner_iteration = 1;
    } else if (kase.rfind("heat3d=", 0) == 0) {
        c.openmp_number_of_threads = 1;
        c.eproblem_type = enums::Eproblem_type::Heat_conduction;
        c.ematrix_solver_type = enums::Ematrix_solver_type::ILU_BICSTAB;
        c.emesh_source = enums::Emesh_source::from_file;
        c.mesh_filename = kase.substr(7);
        c.set_BC_number(3);
        c.global_delta_t = 0.5;
        c.thermal_diffusivity = 2.0e-3;
        ic.Temperature = 300.0;
        c.boundary_conditions[0].ethermal_BC_type = enums::Ethermal_BC_type::constant_temperature;
        c.boundary_conditions[0].Temperature = 250.0;
        c.boundary_conditions[1].ethermal_BC_type = enums::Ethermal_BC_type::adiabatic;
        c.boundary_conditions[2].ethermal_BC_type = enums::Ethermal_BC_type::constant_temperature;
        c.boundary_conditions[2].Temperature = 450.0;
        c.max_iteration = 6;
        c.max_inner_iteration = 1;
    } else {
        std::fprintf(stderr, "unknown case %s\n", kase.c_str());
        return 1;
    }
    root.run_config(c);
    std::printf("solve calls: %ld\n", g_call);
    if (kase.rfind("heat3d=", 0) == 0) {
        using Hc = CHeat_solver::CHeat_cell;
        using Hb = CHeat_solver::CHeat_BC_face;
        const auto& hs = *root.Heat_solver;
        Writer w(g_out + "/final_heat.bin");
        w.d("cell_temperature", col(hs.cells, [](const Hc& x) { return x.Temperature; }));
        w.d("bc_temperature", col(hs.BC_faces, [](const Hb& f) { return f.Temperature; }));
        w.i("bc_thermal", coli(hs.BC_faces, [](const Hb& f) { return (int)f.ethermal_BC_type; }));
    }
    return 0;
}
