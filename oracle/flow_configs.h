// Test infrastructure only: the 200-cell viscous flow cases shared by the
// reference recorders (ref_assembly.cpp records their assembled systems,
// ref_flow.cpp their SIMPLE-iteration states).  Built through the
// reference's in-memory configuration, as tests.h:69-107 builds its own cases.
#pragma once
#include "croot.h"

#include <string>

// A 1D mesh over [0, 1] m with 0.01 x 0.01 m sides; boundary condition 0 is
// the x = 0 end, 1 the sides, 2 the x = 1 end.
inline void base_1d(Cconfiguration& c, int cells)
{
    c.openmp_number_of_threads = 1;
    c.eproblem_type = enums::Eproblem_type::Fluid_flow;
    c.ematrix_solver_type = enums::Ematrix_solver_type::ILU_BICSTAB;
    c.emesh_source = enums::Emesh_source::generate_1D;
    c.geo_parameters_1D[0] = 1.0;
    c.geo_parameters_1D[1] = 0.01;
    c.geo_parameters_1D[2] = 0.01;
    c.geo_parameters_1D[3] = cells;
    c.set_BC_number(3);
}

// channel: 200 cells, viscous, first-order upwind, transient (dt 1e-5 s),
//          velocity inlet (20 m/s, 300 K), no-slip side walls, pressure outlet
//          (1e5 Pa);
// steady:  200 cells, viscous, blended, steady with implicit under-relaxation
//          ramping 0.5 -> 0.8 over 10 steps, supersonic inlet (700 m/s, 300 K,
//          1e5 Pa), slip side walls, pressure outlet (1e5 Pa).
inline void make_viscous_config(Cconfiguration& c, bool steady, int steps, int inner)
{
    auto& ic = *c.inital_condition;
    base_1d(c, 200);
    c.eflow_type_visc = enums::Eflow_type_visc::Viscous;
    c.econv_flux_type = steady ? enums::Econv_flux_type::Blended_central
                               : enums::Econv_flux_type::First_order_upwind;
    c.etimestepping_type = steady ? enums::Etimestepping_type::Steady
                                  : enums::Etimestepping_type::Transient;
    c.global_delta_t = 1.0e-5;
    c.implicit_underrelax = 0.5;
    c.implicit_underrelax_max = 0.8;
    c.underrelax_ramp_iteration = 10;
    const double u = steady ? 700.0 : 20.0;
    ic.einitial_condition_type = enums::Einitial_condition_type::Uniform;
    ic.Pressure = 1.0e5;
    ic.Temperature = 300.0;
    ic.Velocity.val[0] = u;
    ic.Velocity.val[1] = 0.0;
    ic.Velocity.val[2] = 0.0;
    auto& in = c.boundary_conditions[0];
    in.eflow_BC_type = steady ? enums::Eflow_BC_type::supersonic_velocity_inlet
                              : enums::Eflow_BC_type::velocity_inlet;
    in.Velocity.val[0] = u;
    in.Velocity.val[1] = 0.0;
    in.Velocity.val[2] = 0.0;
    in.Temperature = 300.0;
    in.Pressure = 1.0e5;
    c.boundary_conditions[1].eflow_BC_type = enums::Eflow_BC_type::wall;
    c.boundary_conditions[1].ewall_BC_type =
        steady ? enums::Ewall_BC_type::slip : enums::Ewall_BC_type::no_slip;
    c.boundary_conditions[2].eflow_BC_type = enums::Eflow_BC_type::pressure_outlet;
    c.boundary_conditions[2].Pressure = 1.0e5;
    c.max_iteration = steps;
    c.max_inner_iteration = inner;
}

// box3d:   a mesh read from an SU2 file (markers: inlet, walls, outlet, in this
//          order), viscous, blended, transient (dt 2e-6 s): velocity inlet
//          (20, 3, 2) m/s at 300 K, no-slip walls, pressure outlet (1e5 Pa);
//          uniform start (20, 0, 0) m/s, 300 K, 1e5 Pa.
inline void make_box3d_config(Cconfiguration& c, const std::string& mesh, int steps, int inner)
{
    auto& ic = *c.inital_condition;
    c.openmp_number_of_threads = 1;
    c.eproblem_type = enums::Eproblem_type::Fluid_flow;
    c.ematrix_solver_type = enums::Ematrix_solver_type::ILU_BICSTAB;
    c.emesh_source = enums::Emesh_source::from_file;
    c.mesh_filename = mesh;
    c.set_BC_number(3);
    c.eflow_type_visc = enums::Eflow_type_visc::Viscous;
    c.econv_flux_type = enums::Econv_flux_type::Blended_central;
    c.etimestepping_type = enums::Etimestepping_type::Transient;
    c.global_delta_t = 2.0e-6;
    c.implicit_underrelax = 0.5;
    c.implicit_underrelax_max = 0.8;
    c.underrelax_ramp_iteration = 10;
    ic.einitial_condition_type = enums::Einitial_condition_type::Uniform;
    ic.Pressure = 1.0e5;
    ic.Temperature = 300.0;
    ic.Velocity.val[0] = 20.0;
    ic.Velocity.val[1] = 0.0;
    ic.Velocity.val[2] = 0.0;
    auto& in = c.boundary_conditions[0];
    in.eflow_BC_type = enums::Eflow_BC_type::velocity_inlet;
    in.Velocity.val[0] = 20.0;
    in.Velocity.val[1] = 3.0;
    in.Velocity.val[2] = 2.0;
    in.Temperature = 300.0;
    in.Pressure = 1.0e5;
    c.boundary_conditions[1].eflow_BC_type = enums::Eflow_BC_type::wall;
    c.boundary_conditions[1].ewall_BC_type = enums::Ewall_BC_type::no_slip;
    c.boundary_conditions[2].eflow_BC_type = enums::Eflow_BC_type::pressure_outlet;
    c.boundary_conditions[2].Pressure = 1.0e5;
    c.max_iteration = steps;
    c.max_inner_iteration = inner;
}
