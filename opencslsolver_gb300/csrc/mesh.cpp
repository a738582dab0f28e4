// SU2 mesh reader and finite-volume metrics in O(cells + faces) (ocsl_mesh_*,
// include/ocsl.h): the data the reference builds in Read_SU2_mesh
// (cgeometry_supply.h:201-433), Cgeometry (cgeometry.cpp:23-680) and
// CFVM::create_FVM_from_geometry (cfvm.cpp:100-175), in the same order, so that
// the face and boundary-face numbering -- and with it the matrix pattern and
// every face array the assembly and the SIMPLE iteration read -- is the
// reference's.
//
// The reference pairs faces by visiting, for every node, every pair of cells
// around it and comparing their faces (quadratic per node) and finds each
// boundary element's cell by intersecting node-to-cell lists.  Here every
// cell face is hashed once by its sorted node ids: a key seen twice is an
// interior face, once a boundary face.  The reference creates an interior
// face the first time it meets it, which is at its lowest node id, with the
// lower cell index as the left cell and that cell's local node order; sorting
// the pairs by (lowest node, left cell, right cell) gives the same sequence.
// Boundary faces follow in marker order, element order within a marker, with
// their cell's local node order.
//
// Arithmetic follows the reference's expressions term by term (it is compiled
// with -ffast-math, so its last bits may differ).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/ocsl.h"
#include "mesh.h"

namespace {

struct V3 {
    double x = 0, y = 0, z = 0;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 cross(V3 a, V3 b)  // tensor.h:117-123
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double mag(V3 a) { return std::sqrt(dot(a, a)); }

enum CellKind { TET = 10, HEX = 12, WEDGE = 13 };

struct Cell {
    int kind;
    int node[8];
    int nnodes() const { return kind == TET ? 4 : kind == WEDGE ? 6 : 8; }
    int nfaces() const { return kind == TET ? 4 : kind == WEDGE ? 5 : 6; }
};

// Local faces of each cell kind (cgeometry.cpp:80-228), node slots of the cell.
const int kTetFaces[4][4] = {{1, 0, 2, -1}, {0, 1, 3, -1}, {1, 2, 3, -1}, {2, 0, 3, -1}};
const int kWedgeFaces[5][4] = {{0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {0, 2, 1, -1},
                               {3, 4, 5, -1}};
const int kHexFaces[6][4] = {{0, 1, 5, 4}, {1, 3, 7, 5}, {3, 2, 6, 7},
                             {2, 0, 4, 6}, {1, 0, 2, 3}, {4, 5, 7, 6}};

// Node ids of local face f of cell c (-1 in slot 3 for a triangle).
void face_nodes(const Cell& c, int f, int out[4])
{
    const int(*t)[4] = c.kind == TET ? kTetFaces : c.kind == WEDGE ? kWedgeFaces : kHexFaces;
    for (int k = 0; k < 4; ++k) out[k] = t[f][k] < 0 ? -1 : c.node[t[f][k]];
}

struct Key {
    int n[4];  // sorted node ids, -1 first for a triangle
    bool operator==(const Key& o) const { return !std::memcmp(n, o.n, sizeof n); }
};
struct KeyHash {
    size_t operator()(const Key& k) const
    {
        uint64_t h = 1469598103934665603ull;
        for (int v : k.n) h = (h ^ (uint64_t)(uint32_t)v) * 1099511628211ull;
        return (size_t)h;
    }
};
Key make_key(const int nodes[4])
{
    Key k;
    std::memcpy(k.n, nodes, sizeof k.n);
    std::sort(k.n, k.n + 4);
    return k;
}

// Face area, unit normal and centre (cgeometry.cpp:330-373): the normal and
// the first half of the area come from the triangle (0, 1, 2); a quad adds
// the triangle (0, 2, 3) and area-weights the two triangle centres.
void face_geometry(const std::vector<V3>& X, const int nd[4], double& area, V3& normal, V3& centre)
{
    V3 v0 = X[nd[1]] - X[nd[0]], v1 = X[nd[2]] - X[nd[0]];
    normal = cross(v0, v1);
    double length = mag(normal);
    normal = (1.0 / length) * normal;
    area = 0.5 * length;
    centre = X[nd[0]] + X[nd[1]] + X[nd[2]];
    centre = (1.0 / 3.0) * centre;
    if (nd[3] >= 0) {
        centre = area * centre;
        v0 = X[nd[2]] - X[nd[0]];
        v1 = X[nd[3]] - X[nd[0]];
        length = mag(cross(v0, v1));
        area = area + 0.5 * length;
        centre = centre + ((0.5 * length / 3.0) * (X[nd[0]] + X[nd[2]] + X[nd[3]]));
        centre = (1.0 / area) * centre;
    }
}

double tet_volume(V3 a, V3 b, V3 c, V3 d)  // cgeometry.cpp:72-78
{
    return (1.0 / 6.0) * dot(b - a, cross(c - a, d - a));
}

// Cell volume and centre (cgeometry.cpp:377-541): a tet directly, a wedge as
// 3 and a hex as 6 tets around node 0, centres weighted by the tet volumes.
void cell_geometry(const std::vector<V3>& X, const Cell& c, double& vol, V3& centre)
{
    static const int kWedgeTets[3][4] = {{0, 4, 5, 3}, {0, 4, 1, 5}, {0, 1, 2, 5}};
    static const int kHexTets[6][4] = {{0, 2, 7, 3}, {0, 2, 6, 7}, {0, 7, 1, 3},
                                       {0, 7, 5, 1}, {0, 7, 4, 5}, {0, 7, 6, 4}};
    auto P = [&](int slot) { return X[c.node[slot]]; };
    if (c.kind == TET) {
        vol = tet_volume(P(0), P(1), P(2), P(3));
        centre = (1.0 / 4.0) * (P(0) + P(1) + P(2) + P(3));
        return;
    }
    const int(*t)[4] = c.kind == WEDGE ? kWedgeTets : kHexTets;
    const int nt = c.kind == WEDGE ? 3 : 6;
    vol = 0.0;
    for (int k = 0; k < nt; ++k) {
        const double dv = tet_volume(P(t[k][0]), P(t[k][1]), P(t[k][2]), P(t[k][3]));
        const V3 s = P(t[k][0]) + P(t[k][1]) + P(t[k][2]) + P(t[k][3]);
        if (k == 0) {
            vol = dv;
            centre = (dv / 4.0) * s;
        } else {
            vol += dv;
            centre = centre + (dv / 4.0) * s;
        }
    }
    centre = (1.0 / vol) * centre;
}

void set_err(char* err, size_t len, const std::string& msg)
{
    if (err && len) std::snprintf(err, len, "%s", msg.c_str());
}

// "NAME= value" header lines, as the reference scans them (getline up to '=').
bool seek(std::istream& in, const char* name, std::string& value)
{
    std::string line;
    while (std::getline(in, line)) {
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        if (line.compare(0, eq, name) == 0) {
            value = line.substr(eq + 1);
            return true;
        }
    }
    return false;
}

std::string trim(std::string s)
{
    s.erase(std::remove(s.begin(), s.end(), ' '), s.end());
    s.erase(std::remove(s.begin(), s.end(), '\r'), s.end());
    return s;
}

}  // namespace

extern "C" {

int ocsl_mesh_read_su2(const char* path, ocsl_mesh** out, char* err, size_t err_len)
{
    if (!path || !out) {
        set_err(err, err_len, "null path or output");
        return OCSL_BAD_ARGUMENT;
    }
    *out = nullptr;
    std::ifstream in(path);
    if (!in) {
        set_err(err, err_len, std::string("cannot open ") + path);
        return OCSL_BAD_ARGUMENT;
    }
    std::string value;
    // cells (types 10 tetrahedron, 12 hexahedron, 13 wedge), each followed by its index
    if (!seek(in, "NELEM", value)) {
        set_err(err, err_len, "no NELEM section");
        return OCSL_BAD_ARGUMENT;
    }
    const long ncell = std::atol(value.c_str());
    std::vector<Cell> cells((size_t)std::max(0L, ncell));
    for (long i = 0; i < ncell; ++i) {
        Cell& c = cells[i];
        int idx;
        if (!(in >> c.kind)) {
            set_err(err, err_len, "truncated element list");
            return OCSL_BAD_ARGUMENT;
        }
        if (c.kind == HEX) {  // SU2 order to the reference's node slots (cgeometry_supply.h:268-277)
            static const int slot[8] = {0, 1, 3, 2, 4, 5, 7, 6};
            for (int k = 0; k < 8; ++k) in >> c.node[slot[k]];
        } else if (c.kind == TET || c.kind == WEDGE) {
            for (int k = 0; k < c.nnodes(); ++k) in >> c.node[k];
        } else {
            set_err(err, err_len, "element type " + std::to_string(c.kind) +
                                      " (only 10 tetrahedron, 12 hexahedron, 13 wedge)");
            return OCSL_BAD_ARGUMENT;
        }
        in >> idx;
    }
    if (!seek(in, "NPOIN", value)) {
        set_err(err, err_len, "no NPOIN section");
        return OCSL_BAD_ARGUMENT;
    }
    const long npoin = std::atol(value.c_str());
    std::vector<V3> X((size_t)std::max(0L, npoin));
    for (long i = 0; i < npoin; ++i) {
        int idx;
        if (!(in >> X[i].x >> X[i].y >> X[i].z >> idx)) {
            set_err(err, err_len, "truncated point list");
            return OCSL_BAD_ARGUMENT;
        }
    }
    for (const Cell& c : cells)
        for (int k = 0; k < c.nnodes(); ++k)
            if (c.node[k] < 0 || c.node[k] >= npoin) {
                set_err(err, err_len, "element node out of range");
                return OCSL_BAD_ARGUMENT;
            }

    // interior faces: every cell face hashed once by its sorted nodes
    struct Seen {
        int cell, face;
        bool paired;
    };
    std::unordered_map<Key, Seen, KeyHash> first;
    first.reserve(cells.size() * 6);
    struct Pair {
        int minnode, L, R, lface;
    };
    std::vector<Pair> pairs;
    pairs.reserve(cells.size() * 3);
    for (int ci = 0; ci < (int)cells.size(); ++ci) {
        for (int f = 0; f < cells[ci].nfaces(); ++f) {
            int nd[4];
            face_nodes(cells[ci], f, nd);
            const Key k = make_key(nd);
            auto it = first.find(k);
            if (it == first.end()) {
                first.emplace(k, Seen{ci, f, false});
            } else if (!it->second.paired) {
                it->second.paired = true;
                const int a = it->second.cell, af = it->second.face;
                const int L = std::min(a, ci), R = std::max(a, ci);
                const int lface = L == a ? af : f;
                const int mn = k.n[0] < 0 ? k.n[1] : k.n[0];  // a triangle's key starts with -1
                pairs.push_back({mn, L, R, lface});
            } else {
                set_err(err, err_len, "a face shared by more than two cells");
                return OCSL_BAD_ARGUMENT;
            }
        }
    }
    std::sort(pairs.begin(), pairs.end(), [](const Pair& a, const Pair& b) {
        if (a.minnode != b.minnode) return a.minnode < b.minnode;
        if (a.L != b.L) return a.L < b.L;
        return a.R < b.R;
    });

    // boundary faces, marker by marker (element type 5 triangle, 9 quadrilateral)
    if (!seek(in, "NMARK", value)) {
        set_err(err, err_len, "no NMARK section");
        return OCSL_BAD_ARGUMENT;
    }
    auto* m = new ocsl_mesh();
    const long nmark = std::atol(value.c_str());
    std::vector<std::pair<int, int>> bcf;  // (cell, local face), in file order
    for (long im = 0; im < nmark; ++im) {
        bool ok = seek(in, "MARKER_TAG", value);
        if (ok) {
            m->markers.push_back(trim(value));
            ok = seek(in, "MARKER_ELEMS", value);
        }
        if (!ok) {
            delete m;
            set_err(err, err_len, "marker " + std::to_string(im) + " incomplete");
            return OCSL_BAD_ARGUMENT;
        }
        const long ne = std::atol(value.c_str());
        for (long e = 0; e < ne; ++e) {
            int t, nd[4] = {-1, -1, -1, -1};
            in >> t;
            const int cnt = t == 5 ? 3 : t == 9 ? 4 : 0;
            if (!cnt) {
                delete m;
                set_err(err, err_len, "boundary element type " + std::to_string(t));
                return OCSL_BAD_ARGUMENT;
            }
            for (int k = 0; k < cnt; ++k) in >> nd[k];
            auto it = first.find(make_key(nd));
            if (!in || it == first.end() || it->second.paired) {
                delete m;
                set_err(err, err_len, "a boundary element that is not a free cell face");
                return OCSL_BAD_ARGUMENT;
            }
            bcf.push_back({it->second.cell, it->second.face});
            m->bc_marker.push_back((int32_t)im);
        }
    }

    // geometry (cgeometry.cpp:662-670), then the finite-volume metrics (cfvm.cpp:100-175)
    const int64_t n = (int64_t)cells.size(), nf = (int64_t)pairs.size(), nb = (int64_t)bcf.size();
    m->n_cells = n;
    m->n_faces = nf;
    m->n_bc = nb;
    std::vector<V3> cc(n);
    m->cell_volume.resize(n);
    m->cell_center.resize(3 * n);
    for (int64_t i = 0; i < n; ++i) {
        cell_geometry(X, cells[i], m->cell_volume[i], cc[i]);
        m->cell_center[i] = cc[i].x;
        m->cell_center[n + i] = cc[i].y;
        m->cell_center[2 * n + i] = cc[i].z;
    }
    auto put3 = [](std::vector<double>& a, int64_t count, int64_t k, V3 v) {
        a[k] = v.x;
        a[count + k] = v.y;
        a[2 * count + k] = v.z;
    };
    m->face_left.resize(nf);
    m->face_right.resize(nf);
    m->face_geo_aver.resize(nf);
    m->face_ksi_A.resize(nf);
    m->face_distance.resize(nf);
    m->face_area_vector.resize(3 * nf);
    m->face_alpha.resize(3 * nf);
    m->face_unit.resize(3 * nf);
    for (int64_t k = 0; k < nf; ++k) {
        const Pair& p = pairs[k];
        int nd[4];
        face_nodes(cells[p.L], p.lface, nd);
        double area;
        V3 normal, fc;
        face_geometry(X, nd, area, normal, fc);
        const V3 A = area * normal;
        V3 d = cc[p.R] - cc[p.L];
        const V3 alpha = (1.0 / dot(A, d)) * A;  // with the unnormalised cell-to-cell vector
        const double dist = mag(d);
        d = (1.0 / dist) * d;
        m->face_left[k] = p.L;
        m->face_right[k] = p.R;
        put3(m->face_area_vector, nf, k, A);
        put3(m->face_alpha, nf, k, alpha);
        put3(m->face_unit, nf, k, d);
        m->face_distance[k] = dist;
        m->face_ksi_A[k] = dot(alpha, A);
        m->face_geo_aver[k] = mag(cc[p.R] - fc) / dist;
    }
    m->nodes.resize(3 * X.size());
    for (size_t i = 0; i < X.size(); ++i) {
        m->nodes[3 * i] = X[i].x;
        m->nodes[3 * i + 1] = X[i].y;
        m->nodes[3 * i + 2] = X[i].z;
    }
    m->cell_kind.resize(n);
    m->cell_nodes.assign(8 * n, -1);
    for (int64_t i = 0; i < n; ++i) {
        m->cell_kind[i] = (int8_t)cells[i].kind;
        for (int k = 0; k < cells[i].nnodes(); ++k) m->cell_nodes[8 * i + k] = cells[i].node[k];
    }
    m->bc_nodes.resize(4 * nb);
    m->bc_normal.resize(3 * nb);
    m->bc_center.resize(3 * nb);
    m->bc_left.resize(nb);
    m->bc_area.resize(nb);
    m->bc_distance.resize(nb);
    m->bc_perp_dist.resize(nb);
    m->bc_ksi_A.resize(nb);
    m->bc_area_vector.resize(3 * nb);
    m->bc_alpha.resize(3 * nb);
    m->bc_unit.resize(3 * nb);
    for (int64_t g = 0; g < nb; ++g) {
        const int c = bcf[g].first;
        int nd[4];
        face_nodes(cells[c], bcf[g].second, nd);
        double area;
        V3 normal, fc;
        face_geometry(X, nd, area, normal, fc);
        const V3 A = area * normal;
        std::memcpy(&m->bc_nodes[4 * g], nd, sizeof nd);
        put3(m->bc_normal, nb, g, normal);
        put3(m->bc_center, nb, g, fc);
        const V3 d = fc - cc[c];
        const double dist = mag(fc - cc[c]);
        const V3 alpha = (1.0 / dot(A, d)) * A;
        const V3 u = (1.0 / dist) * d;
        m->bc_left[g] = c;
        m->bc_area[g] = area;
        put3(m->bc_area_vector, nb, g, A);
        put3(m->bc_alpha, nb, g, alpha);
        put3(m->bc_unit, nb, g, u);
        m->bc_distance[g] = dist;
        m->bc_ksi_A[g] = dot(alpha, A);
        m->bc_perp_dist[g] = dot(dist * u, (1.0 / area) * A);
    }
    *out = m;
    return OCSL_OK;
}

int ocsl_mesh_view(const ocsl_mesh* m, ocsl_mesh_arrays* v)
{
    if (!m || !v) return OCSL_BAD_ARGUMENT;
    v->n_cells = m->n_cells;
    v->n_faces = m->n_faces;
    v->n_bc = m->n_bc;
    v->n_markers = (int32_t)m->markers.size();
    v->face_left = m->face_left.data();
    v->face_right = m->face_right.data();
    v->face_geo_aver = m->face_geo_aver.data();
    v->face_ksi_A = m->face_ksi_A.data();
    v->face_area_vector = m->face_area_vector.data();
    v->face_alpha = m->face_alpha.data();
    v->face_distance = m->face_distance.data();
    v->face_unit = m->face_unit.data();
    v->bc_left = m->bc_left.data();
    v->bc_marker = m->bc_marker.data();
    v->bc_area = m->bc_area.data();
    v->bc_area_vector = m->bc_area_vector.data();
    v->bc_alpha = m->bc_alpha.data();
    v->bc_distance = m->bc_distance.data();
    v->bc_unit = m->bc_unit.data();
    v->bc_perp_dist = m->bc_perp_dist.data();
    v->bc_ksi_A = m->bc_ksi_A.data();
    v->cell_volume = m->cell_volume.data();
    v->cell_center = m->cell_center.data();
    return OCSL_OK;
}

const char* ocsl_mesh_marker_name(const ocsl_mesh* m, int marker)
{
    if (!m || marker < 0 || marker >= (int)m->markers.size()) return nullptr;
    return m->markers[marker].c_str();
}

int ocsl_mesh_destroy(ocsl_mesh* m)
{
    delete m;
    return OCSL_OK;
}

}  // extern "C"
