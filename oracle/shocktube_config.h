// Test infrastructure only: the 1000-cell shock-tube configuration shared by
// the reference harnesses (ref_shocktube.cpp records solve calls of the
// reference's CPU solver; shim_driver.cpp runs the same case with the GPU
// drop-in linked in).  Built through the reference's in-memory configuration
// the way tests.h:69-107 builds its own shock tube.
#pragma once
#include "croot.h"

// 1000-cell shock tube over [0, 1] m: walls at both ends, empty sides, left
// p=1e5 Pa T=348.4 K, right p=1e4 Pa T=278.7 K, dt=1e-6 s.
inline void make_shocktube_config(Cconfiguration& config, int threads, int steps, int inner)
{
    config.openmp_number_of_threads = threads;
    config.eproblem_type = enums::Eproblem_type::Fluid_flow;
    config.eflow_type_visc = enums::Eflow_type_visc::Inviscid;
    config.etimestepping_type = enums::Etimestepping_type::Transient;
    config.ematrix_solver_type = enums::Ematrix_solver_type::ILU_BICSTAB;
    config.econv_flux_type = enums::Econv_flux_type::Blended_central;
    config.emesh_source = enums::Emesh_source::generate_1D;
    config.geo_parameters_1D[0] = 1.0;
    config.geo_parameters_1D[1] = 0.01;
    config.geo_parameters_1D[2] = 0.01;
    config.geo_parameters_1D[3] = 1000;
    config.global_delta_t = 1.0e-6;
    config.inital_condition->einitial_condition_type = enums::Einitial_condition_type::Shock_tube;
    config.inital_condition->Pressure = 1.0e5;
    config.inital_condition->Temperature = 348.4;
    config.inital_condition->Pressure2 = 1.0e4;
    config.inital_condition->Temperature2 = 278.7;
    config.inital_condition->Velocity.val[0] = 0.0;
    config.inital_condition->Velocity.val[1] = 0.0;
    config.inital_condition->Velocity.val[2] = 0.0;
    config.set_BC_number(3);
    config.boundary_conditions[0].eflow_BC_type = enums::Eflow_BC_type::wall;
    config.boundary_conditions[0].ewall_BC_type = enums::Ewall_BC_type::slip;
    config.boundary_conditions[1].eflow_BC_type = enums::Eflow_BC_type::empty;
    config.boundary_conditions[2].eflow_BC_type = enums::Eflow_BC_type::wall;
    config.boundary_conditions[2].ewall_BC_type = enums::Ewall_BC_type::slip;
    config.max_iteration = steps;
    config.max_inner_iteration = inner;
}

// Final fields at full precision (the reference's VTK writer keeps 6 digits).
inline int write_shocktube_fields(const std::string& path)
{
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) { std::perror(path.c_str()); return 2; }
    for (const auto& c : root.Flow_solver->cells)
        std::fprintf(f, "%.17g %.17g %.17g %.17g\n", c.Pressure, c.Velocity.val[0],
                     c.Temperature, c.Density);
    std::fclose(f);
    return 0;
}
