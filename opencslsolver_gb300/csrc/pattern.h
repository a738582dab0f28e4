// Host-side pattern analysis (see pattern.cpp).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace ocsl {

constexpr int kChunkRows = 256;  // rows per chunk of a sweep level (one CTA)
// Schedules of at most this many levels, each a contiguous ascending row
// range (multicolour orderings), are swept one launch per level.
constexpr int kRangeMaxLevels = 16;

// A pattern that is exactly the 7-point stencil of an nx * ny * nz box in
// natural order (row = i + nx * (j + ny * k)), with optional phantom columns
// after the real ones.  Such rows can be swept by the structured kernel.
struct BoxShape {
    bool ok = false;
    int dim[3] = {0, 0, 0};     // nx, ny, nz
};

struct HostPattern {
    BoxShape box;
    int n = 0;
    int nnz = 0;
    long long nnz_real = 0;
    int fw_levels = 0;
    int bw_levels = 0;
    std::vector<int> rp, col, diag;
    std::vector<int> pair_ptr, pair_k, pair_slot;
    std::vector<int> fw_order, fw_chunk, bw_order, bw_chunk;
    // (first row, end row) of each level in schedule order when every level is
    // a contiguous row range and there are at most kRangeMaxLevels; else empty
    std::vector<int> fw_range, bw_range;
};

// Recognise the 7-point box stencil (see BoxShape); O(nnz).
BoxShape detect_box(int n, const std::vector<int>& rp, const std::vector<int>& col);

// Validate the reference-layout pattern and build the device tables.
// Returns false with a message on a rejected pattern.
bool analyse_pattern(size_t n, const size_t* row_ptr, const size_t* column_index, HostPattern& hp,
                     std::string& err);

// Per-cell incidence lists of the mesh's faces for the gather assembly: the
// interior faces of each cell in ascending face order, each with its side
// (bit 0: 1 when the cell is the face's right cell) and the CSR slot of the
// off-diagonal entry (cell, other cell); the boundary faces of each cell in
// ascending order.  Returns false with a message if a face names a cell out
// of range or its pair is not stored in the pattern.
struct FaceTables {
    std::vector<int> cell_ptr, cell_ent, cell_slot, bc_ptr, bc_ent;
};
bool build_face_tables(int n, const std::vector<int>& rp, const std::vector<int>& col,
                       long long nf, const int32_t* left, const int32_t* right, long long nb,
                       const int32_t* bc_left, FaceTables& ft, std::string& err);

// The reference's CSR pattern built from the mesh's face connectivity in
// O(n + faces): row i holds i, its face neighbours in ascending order, and one
// phantom column (SIZE_MAX) when the cell has a boundary face -- what
// CFVM::define_matrix_structure (cfvm.cpp:74-98) builds with repeated
// insert_element calls (cmatrix_solver.cpp:57-103, quadratic).  Returns false
// with a message on a face naming a cell out of range.
bool build_pattern_from_faces(size_t n, long long nf, const int32_t* left, const int32_t* right,
                              long long nb, const int32_t* bc_left, std::vector<size_t>& row_ptr,
                              std::vector<size_t>& column_index, std::string& err);

// A multicolour ordering of a structurally symmetric pattern: rows coloured
// greedily in natural order (the smallest colour none of the row's
// already-coloured neighbours has; the parity colouring of a box stencil),
// then numbered colour by colour, ascending within a colour.  In the
// permuted pattern a row's lower entries are rows of lower colours only, so
// a triangular sweep has one level per colour.  perm[new] = old row;
// rp / col: the permuted pattern in the reference's layout (phantom column
// SIZE_MAX kept last); slot[new slot] = the original slot of the entry.
struct ColouredPattern {
    int colours = 0;
    std::vector<int> start;  // [colours + 1]: colour c holds new rows [start[c], start[c+1])
    std::vector<int> perm, slot;
    std::vector<size_t> rp, col;
};
bool colour_pattern(int n, const std::vector<int>& rp, const std::vector<int>& col,
                    ColouredPattern& cp, std::string& err);

}  // namespace ocsl
