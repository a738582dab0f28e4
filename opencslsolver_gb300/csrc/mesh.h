// The mesh object behind ocsl_mesh_* (mesh.cpp) and ocsl_vtk_write (vtk.cpp).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

struct ocsl_mesh {
    int64_t n_cells = 0, n_faces = 0, n_bc = 0;
    std::vector<std::string> markers;
    std::vector<int32_t> face_left, face_right, bc_left, bc_marker;
    std::vector<double> face_geo_aver, face_ksi_A, face_area_vector, face_alpha, face_distance,
        face_unit, bc_area, bc_area_vector, bc_alpha, bc_distance, bc_unit, bc_perp_dist,
        bc_ksi_A, cell_volume, cell_center;
    // what the VTK writer needs besides the finite-volume arrays:
    std::vector<double> nodes;          // x, y, z per node, file order (Cgeometry::nodes)
    std::vector<int8_t> cell_kind;      // 10 tetrahedron, 12 hexahedron, 13 wedge
    std::vector<int32_t> cell_nodes;    // 8 per cell, the reference's Cgeo_cell::i_nodes order
    std::vector<int32_t> bc_nodes;      // 4 per boundary face (-1 in slot 3 for a triangle),
                                        // the owning cell's local face order (Cgeo_face::i_nodes)
    std::vector<double> bc_normal;      // [3][n_bc] unit normal (Cgeo_face::normal)
    std::vector<double> bc_center;      // [3][n_bc] (Cgeo_face::center)
};
