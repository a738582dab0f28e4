// VTK output of a solution straight from the device (ocsl_vtk_write,
// include/ocsl.h): the two legacy-ASCII files the reference's post-processing
// writes at the end of a run and every VTK_file_frequency steps
// (Cpost_processing::write_VTK_file / write_boundary_VTK_file and their data
// sections, cpost_processing.cpp:26-187, 238-401, called from
// croot.cpp:226-240) -- same sections, names, order, cell-node orders and
// number formatting, so the files are byte-identical to the reference's for
// the same mesh and state.
//
// The reference streams every number through std::ostream with its default
// format, i.e. printf's "%.6g"; here the digits are selectable (6 by default,
// up to 17 for a round-trip exact file).  Fields may sit in device memory (the
// state the device SIMPLE iteration keeps, ocsl_flow_state) or in host
// memory.  Device fields are copied in chunks through two pinned staging
// buffers on a private stream, the next chunk in flight while the current one
// is formatted; each chunk is formatted by all host threads in parallel, one
// contiguous slice of lines per thread, and written in order.
#include <cuda_runtime.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ocsl.h"
#include "mesh.h"

namespace {

constexpr size_t kChunk = size_t(1) << 20;  // lines per staged chunk

struct Fail {
    int status;
    std::string msg;
};

bool on_device(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // no GPU, or not a CUDA pointer: host memory
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw Fail{OCSL_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e)};
}

// One line of output per index: up to three numbers, separated by spaces.
struct LineFormat {
    int digits;
    int width;  // numbers per line
};

// std::to_chars with a precision formats exactly as printf's "%.*g" does
// (C locale), several times faster than snprintf.
int put_number(char* out, double v, int digits)
{
    const auto r = std::to_chars(out, out + 32, v, std::chars_format::general, digits);
    return (int)(r.ptr - out);
}

int put_int(char* out, long long v)
{
    const auto r = std::to_chars(out, out + 24, v);
    return (int)(r.ptr - out);
}

// Lines [0, count) of integers: line i = ints(i, out) written into out
// (returns the characters written, at most max_line), in parallel slices.
template <typename F>
void format_int_lines(size_t count, size_t max_line, F ints, std::string& text, unsigned threads)
{
    const unsigned t = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, count / 4096 + 1));
    std::vector<std::vector<char>> parts(t);
    std::vector<size_t> used(t, 0);
    auto work = [&](unsigned k) {
        const size_t lo = count * k / t, hi = count * (k + 1) / t;
        std::vector<char>& buf = parts[k];
        buf.resize((hi - lo) * max_line + 1);
        char* p = buf.data();
        for (size_t i = lo; i < hi; ++i) p += ints(i, p);
        used[k] = (size_t)(p - buf.data());
    };
    if (t == 1) {
        work(0);
    } else {
        std::vector<std::thread> pool;
        for (unsigned k = 0; k < t; ++k) pool.emplace_back(work, k);
        for (auto& th : pool) th.join();
    }
    for (unsigned k = 0; k < t; ++k) text.append(parts[k].data(), used[k]);
}

// Formats lines [0, count) whose numbers are cols[c][i] into `text`, in
// parallel slices, and appends the slices in order.
void format_lines(const double* const* cols, size_t count, LineFormat f, std::string& text,
                  unsigned threads)
{
    const size_t per_line = (size_t)f.width * 32;
    const unsigned t = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, count / 4096 + 1));
    std::vector<std::vector<char>> parts(t);
    std::vector<size_t> used(t, 0);
    auto work = [&](unsigned k) {
        const size_t lo = count * k / t, hi = count * (k + 1) / t;
        std::vector<char>& buf = parts[k];
        buf.resize((hi - lo) * per_line + 1);
        char* p = buf.data();
        for (size_t i = lo; i < hi; ++i) {
            for (int c = 0; c < f.width; ++c) {
                if (c) *p++ = ' ';
                p += put_number(p, cols[c][i], f.digits);
            }
            *p++ = '\n';
        }
        used[k] = (size_t)(p - buf.data());
    };
    if (t == 1) {
        work(0);
    } else {
        std::vector<std::thread> pool;
        for (unsigned k = 0; k < t; ++k) pool.emplace_back(work, k);
        for (auto& th : pool) th.join();
    }
    for (unsigned k = 0; k < t; ++k) text.append(parts[k].data(), used[k]);
}

class Writer {
public:
    Writer(const char* path, int digits) : digits_(digits)
    {
        f_ = std::fopen(path, "wb");
        if (!f_) throw Fail{OCSL_BAD_ARGUMENT, std::string("cannot open ") + path};
        threads_ = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    }
    ~Writer()
    {
        if (f_) std::fclose(f_);
        if (stream_) cudaStreamDestroy(stream_);
        for (int k = 0; k < 2; ++k) {
            if (stage_[k]) cudaFreeHost(stage_[k]);
            if (done_[k]) cudaEventDestroy(done_[k]);
        }
    }
    void close()
    {
        flush();
        const bool bad = std::fclose(f_) != 0;
        f_ = nullptr;
        if (bad) throw Fail{OCSL_BAD_ARGUMENT, "write failed"};
    }
    void text(const std::string& s)
    {
        buf_ += s;
        if (buf_.size() > (size_t(8) << 20)) flush();
    }
    int digits() const { return digits_; }
    unsigned threads() const { return threads_; }

    // Lines of `width` numbers: component c of line i is cols[c][i]; cols
    // point to device or host memory (each column decided on its own).
    void columns(const double* const* cols, int width, size_t count)
    {
        bool dev[3] = {false, false, false};
        bool any = false;
        for (int c = 0; c < width; ++c) any |= dev[c] = on_device(cols[c]);
        const LineFormat f{digits_, width};
        if (!any) {
            format_lines(cols, count, f, buf_, threads_);
            if (buf_.size() > (size_t(8) << 20)) flush();
            return;
        }
        staging();
        auto issue = [&](size_t chunk, int slot) {
            const size_t lo = chunk * kChunk, len = std::min(kChunk, count - lo);
            for (int c = 0; c < width; ++c)
                if (dev[c])
                    check(cudaMemcpyAsync(stage_[slot] + (size_t)c * kChunk, cols[c] + lo,
                                          len * sizeof(double), cudaMemcpyDeviceToHost, stream_),
                          "cudaMemcpyAsync");
            check(cudaEventRecord(done_[slot], stream_), "cudaEventRecord");
        };
        const size_t chunks = (count + kChunk - 1) / kChunk;
        if (chunks) issue(0, 0);
        for (size_t k = 0; k < chunks; ++k) {
            const int slot = (int)(k & 1);
            check(cudaEventSynchronize(done_[slot]), "cudaEventSynchronize");
            if (k + 1 < chunks) issue(k + 1, slot ^ 1);  // overlaps the formatting below
            const size_t lo = k * kChunk, len = std::min(kChunk, count - lo);
            const double* part[3];
            for (int c = 0; c < width; ++c)
                part[c] = dev[c] ? stage_[slot] + (size_t)c * kChunk : cols[c] + lo;
            format_lines(part, len, f, buf_, threads_);
            flush();
        }
    }

private:
    void flush()
    {
        if (!buf_.empty() && std::fwrite(buf_.data(), 1, buf_.size(), f_) != buf_.size())
            throw Fail{OCSL_BAD_ARGUMENT, "write failed"};
        buf_.clear();
    }
    void staging()
    {
        if (stream_) return;
        check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        for (int k = 0; k < 2; ++k) {
            check(cudaMallocHost((void**)&stage_[k], 3 * kChunk * sizeof(double)),
                  "cudaMallocHost");
            check(cudaEventCreateWithFlags(&done_[k], cudaEventDisableTiming), "cudaEventCreate");
        }
    }

    FILE* f_ = nullptr;
    int digits_;
    unsigned threads_ = 1;
    std::string buf_;
    cudaStream_t stream_ = nullptr;
    double* stage_[2] = {nullptr, nullptr};
    cudaEvent_t done_[2] = {nullptr, nullptr};
};

// A whole field in host memory (device fields copied once): the boundary
// file reads cell values through bc_left, a gather over few faces.
std::vector<double> host_copy(const double* p, size_t count)
{
    std::vector<double> h(count);
    if (!count) return h;
    if (on_device(p))
        check(cudaMemcpy(h.data(), p, count * sizeof(double), cudaMemcpyDeviceToHost),
              "cudaMemcpy");
    else
        std::memcpy(h.data(), p, count * sizeof(double));
    return h;
}

std::vector<int32_t> host_copy_i(const int32_t* p, size_t count)
{
    std::vector<int32_t> h(count);
    if (!count) return h;
    if (on_device(p))
        check(cudaMemcpy(h.data(), p, count * sizeof(int32_t), cudaMemcpyDeviceToHost),
              "cudaMemcpy");
    else
        std::memcpy(h.data(), p, count * sizeof(int32_t));
    return h;
}

void header(Writer& w, const ocsl_mesh& m)  // cpost_processing.cpp:254-266, 333-345
{
    w.text("# vtk DataFile Version 1.0\nSolver Data File\nASCII\nDATASET UNSTRUCTURED_GRID\n"
           "POINTS " + std::to_string(m.nodes.size() / 3) + " double\n");
    const size_t np = m.nodes.size() / 3;
    std::vector<double> xyz[3];
    for (int c = 0; c < 3; ++c) {
        xyz[c].resize(np);
        for (size_t i = 0; i < np; ++i) xyz[c][i] = m.nodes[3 * i + c];
    }
    const double* cols[3] = {xyz[0].data(), xyz[1].data(), xyz[2].data()};
    w.columns(cols, 3, np);
}

void scalar(Writer& w, const char* name, const double* v, size_t count)
{
    w.text(std::string("SCALARS ") + name + " double 1\nLOOKUP_TABLE default\n");
    w.columns(&v, 1, count);
}

void vector3(Writer& w, const char* keyword, const char* name, const double* v, size_t count)
{
    w.text(std::string(keyword) + " " + name + " double\n");
    const double* cols[3] = {v, v + count, v + 2 * count};
    w.columns(cols, 3, count);
}

void write_cells(const ocsl_mesh& m, const ocsl_vtk_fields& f, const char* path, int digits)
{
    Writer w(path, digits);
    header(w, m);
    const size_t n = (size_t)m.n_cells;
    size_t list = 0;  // cpost_processing.cpp:268-275
    for (size_t i = 0; i < n; ++i)
        list += m.cell_kind[i] == 10 ? 5 : m.cell_kind[i] == 13 ? 7 : 9;
    w.text("CELLS " + std::to_string(n) + " " + std::to_string(list) + "\n");
    // node orders of VTK_TETRA / VTK_WEDGE / VTK_HEXAHEDRON from the
    // reference's i_nodes (cpost_processing.cpp:279-302)
    static const int kTet[4] = {0, 1, 2, 3}, kWedge[6] = {0, 2, 1, 3, 5, 4},
                     kHex[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    std::string s;
    for (size_t lo = 0; lo < n; lo += kChunk) {
        const size_t len = std::min(kChunk, n - lo);
        format_int_lines(len, 9 * 12, [&](size_t i, char* p) {
            const size_t c = lo + i;
            const int kind = m.cell_kind[c];
            const int* order = kind == 10 ? kTet : kind == 13 ? kWedge : kHex;
            const int cnt = kind == 10 ? 4 : kind == 13 ? 6 : 8;
            char* q = p + put_int(p, cnt);
            for (int k = 0; k < cnt; ++k) {
                *q++ = ' ';
                q += put_int(q, m.cell_nodes[8 * c + order[k]]);
            }
            *q++ = '\n';
            return (int)(q - p);
        }, s, w.threads());
        w.text(s);
        s.clear();
    }
    s = "CELL_TYPES " + std::to_string(n) + "\n";
    for (size_t lo = 0; lo < n; lo += kChunk) {
        const size_t len = std::min(kChunk, n - lo);
        format_int_lines(len, 4, [&](size_t i, char* p) {
            char* q = p + put_int(p, m.cell_kind[lo + i]);
            *q++ = '\n';
            return (int)(q - p);
        }, s, w.threads());
        w.text(s);
        s.clear();
    }
    s = "CELL_DATA " + std::to_string(n) + "\n";
    w.text(s);
    // write_VTK_data (cpost_processing.cpp:26-127)
    scalar(w, "Volume[m3]", m.cell_volume.data(), n);
    vector3(w, "VECTORS", "Center", m.cell_center.data(), n);
    if (f.heat) {
        scalar(w, "Temperature[K]", f.temperature, n);
    } else {
        scalar(w, "Density[Kg/m^3]", f.density, n);
        scalar(w, "Pressure[Pa]", f.pressure, n);
        scalar(w, "Temperature[K]", f.temperature, n);
        // Cfluid_properties::get_viscosity (cfluid_properties.cpp:123-128)
        std::vector<double> T = host_copy(f.temperature, n), mu(n);
        for (size_t i = 0; i < n; ++i)
            mu[i] = f.sutherland[0] * std::pow(T[i], 1.5) / (T[i] + f.sutherland[1]);
        scalar(w, "viscosity", mu.data(), n);
        scalar(w, "MACH", f.mach, n);
        vector3(w, "VECTORS", "Velocity[m/s]", f.velocity, n);
        vector3(w, "VECTORS", "Pres_grad", f.pressure_grad, n);
    }
    w.close();
}

void write_boundary(const ocsl_mesh& m, const ocsl_vtk_fields& f, const char* path, int digits)
{
    Writer w(path, digits);
    header(w, m);
    const size_t nb = (size_t)m.n_bc, n = (size_t)m.n_cells;
    size_t list = 0;  // cpost_processing.cpp:347-354
    for (size_t g = 0; g < nb; ++g) list += m.bc_nodes[4 * g + 3] < 0 ? 4 : 5;
    std::string s = "CELLS " + std::to_string(nb) + " " + std::to_string(list) + "\n";
    for (size_t g = 0; g < nb; ++g) {  // :358-372
        const int cnt = m.bc_nodes[4 * g + 3] < 0 ? 3 : 4;
        s += std::to_string(cnt);
        for (int k = 0; k < cnt; ++k) {
            s += ' ';
            s += std::to_string(m.bc_nodes[4 * g + k]);
        }
        s += '\n';
    }
    s += "CELL_TYPES " + std::to_string(nb) + "\n";
    for (size_t g = 0; g < nb; ++g) s += m.bc_nodes[4 * g + 3] < 0 ? "5\n" : "9\n";
    s += "CELL_DATA " + std::to_string(nb) + "\n";
    w.text(s);
    // write_boundary_VTK_data (cpost_processing.cpp:129-187)
    scalar(w, "Area[m2]", m.bc_area.data(), nb);
    vector3(w, "VECTORS", "normal", m.bc_normal.data(), nb);
    s = "SCALARS Marker double 1\nLOOKUP_TABLE default\n";
    for (size_t g = 0; g < nb; ++g) s += std::to_string(m.bc_marker[g]) + "\n";
    w.text(s);
    vector3(w, "Vectors", "area_vector", m.bc_area_vector.data(), nb);
    vector3(w, "Vectors", "center", m.bc_center.data(), nb);
    if (f.heat) {
        scalar(w, "Temperature[K]", f.bc_temperature, nb);
    } else {
        const std::vector<double> mach = host_copy(f.mach, n), T = host_copy(f.temperature, n),
                                  u = host_copy(f.velocity, 3 * n);
        const std::vector<int32_t> type = host_copy_i(f.bc_type, nb),
                                   wall = host_copy_i(f.bc_wall, nb);
        std::vector<double> bm(nb), st(3 * nb, 0.0);
        for (size_t g = 0; g < nb; ++g) {
            const size_t c = (size_t)m.bc_left[g];
            bm[g] = mach[c];
            // CFlow_solver::calc_wall_stress (cflow_solver_supply.cpp:223-239)
            if (type[g] == OCSL_BC_WALL && f.viscous && wall[g] == OCSL_WALL_NO_SLIP) {
                const double a = m.bc_area[g];
                double nrm[3], v[3];
                for (int d = 0; d < 3; ++d) {
                    nrm[d] = (1.0 / a) * m.bc_area_vector[d * nb + g];
                    v[d] = u[d * n + c];
                }
                // the reference's build contracts dot() into two fmas and
                // v - (v.n) n into one per component
                const double vn = std::fma(v[2], nrm[2], std::fma(v[1], nrm[1], v[0] * nrm[0]));
                const double mu =
                    f.sutherland[0] * std::pow(T[c], 1.5) / (T[c] + f.sutherland[1]);
                const double k = mu / m.bc_perp_dist[g];
                for (int d = 0; d < 3; ++d) st[d * nb + g] = k * std::fma(-vn, nrm[d], v[d]);
            }
        }
        scalar(w, "MACH", bm.data(), nb);
        vector3(w, "Vectors", "Stress_vector", st.data(), nb);
    }
    w.close();
}

void set_err(char* err, size_t len, const std::string& msg)
{
    if (err && len) std::snprintf(err, len, "%s", msg.c_str());
}

}  // namespace

extern "C" int ocsl_vtk_write(const ocsl_mesh* mesh, const ocsl_vtk_fields* f,
                              const char* cells_path, const char* boundary_path, char* err,
                              size_t err_len)
{
    if (!mesh || !f) {
        set_err(err, err_len, "null mesh or fields");
        return OCSL_BAD_ARGUMENT;
    }
    const int digits = f->digits ? f->digits : 6;
    if (digits < 1 || digits > 17) {
        set_err(err, err_len, "digits must be 0 (the reference's 6) or 1..17");
        return OCSL_BAD_ARGUMENT;
    }
    const bool cells_need = cells_path && mesh->n_cells > 0;
    if (cells_need && !f->temperature) {
        set_err(err, err_len, "temperature is required");
        return OCSL_BAD_ARGUMENT;
    }
    if (!f->heat && (cells_need || (boundary_path && mesh->n_bc > 0)) &&
        (!f->density || !f->pressure || !f->temperature || !f->mach || !f->velocity ||
         !f->pressure_grad || (mesh->n_bc > 0 && (!f->bc_type || !f->bc_wall)))) {
        set_err(err, err_len, "a flow field is missing (density, pressure, temperature, mach, "
                              "velocity, pressure_grad, bc_type, bc_wall)");
        return OCSL_BAD_ARGUMENT;
    }
    if (f->heat && boundary_path && mesh->n_bc > 0 && !f->bc_temperature) {
        set_err(err, err_len, "bc_temperature is required");
        return OCSL_BAD_ARGUMENT;
    }
    try {
        if (cells_path) write_cells(*mesh, *f, cells_path, digits);
        if (boundary_path) write_boundary(*mesh, *f, boundary_path, digits);
    } catch (const Fail& e) {
        set_err(err, err_len, e.msg);
        return e.status;
    } catch (const std::exception& e) {
        set_err(err, err_len, e.what());
        return OCSL_BAD_ARGUMENT;
    }
    return OCSL_OK;
}
