// Internal declarations shared by the library's translation units.
//
// Device layout (one context, one pattern, sizes for the 128^3 hex case in
// brackets):
//   rp    int32[n+1]  row pointers            [8.4 MB]
//   col   int32[nnz]  columns, phantom -> -1  [58.7 MB]
//   diag  int32[n]    position of (i, i)      [8.4 MB]
//   pair_ptr/k/slot   ILU product table: for stored entry j of row i, the
//                     positions (k, slot) of the products M_ik * M_(col k, col j)
//                     the reference's fixed-point sweep adds, in its order
//   fw_order/fw_chunk, bw_order/bw_chunk: level schedules of the sweeps
//   values double[nnz] (and float[nnz] copies for the FP32 inner solver)
//   vectors double[n] / float[n]
//
// Reductions follow the "tile order" (see tile_reduce below), which the CPU
// oracle restates exactly, so reduced scalars are bit-identical to it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ocsl.h"
#include "pattern.h"

namespace ocsl {

constexpr int kThreads = 256;          // threads per CTA of every tile kernel
constexpr int kRowsPerThread = 8;      // rows / elements per thread per tile
constexpr int kTile = kThreads * kRowsPerThread;  // 2048 rows per tile
constexpr int kMaxDots = 3;
constexpr int kMaxCols = 4;            // right-hand sides of one column-batched launch

// Scalars of one Krylov iteration, resident on the device.  Reduction
// epilogues write them, vector kernels read them; the host reads the block
// only to decide whether to stop.
struct Scalars {
    double rr, bb, rho, rhon, alpha, omega, beta, ss, res, rnorm, tol2, sigma;
    double sum[4];   // raw results of the last reduction
    int done;        // set -> every later kernel of the solve returns at once
    int half;        // tolerance mode: converged at the half step, x += alpha p^ pending
    int iters;       // iterations that updated x
    int breakdown;   // Krylov breakdown seen
    int status;      // ocsl_status of the device side
    int pad[3];
};

// Epilogue applied by the last CTA of a reduction to the reduced sums.
enum EpiOp : int {
    EP_STORE = 0,
    // reference CG (cmatrix_solver.cpp:635-680)
    EP_RC_INIT, EP_RC_ALPHA, EP_RC_RES,
    // reference ILU-BiCGSTAB (cmatrix_solver.cpp:682-762)
    EP_RB_INIT, EP_RB_ALPHA, EP_RB_OMEGA, EP_RB_RUPD,
    // tolerance-mode BiCGSTAB
    EP_TB_INIT, EP_TB_SIGMA, EP_TB_S, EP_TB_OMEGA, EP_TB_RUPD, EP_TRUE_RES,
    // tolerance-mode PCG
    EP_PC_INIT, EP_PC_ALPHA, EP_PC_RUPD,
    // FP32 inner solve of the refinement loop: s0 = <r32, r32>
    EP_IR_INNER_INIT,
};

// Dot-product selection of a fused kernel (bit mask, slots in this order).
enum DotSel : int { DOT_YY = 1, DOT_ZZ = 2, DOT_WY = 4 };

struct ReduceState {
    double* partials;    // [kMaxCols][kMaxDots][max_tiles]
    unsigned* counter;   // [kMaxCols] CTAs finished (reset by the last one)
    int max_tiles;
};

// Column batching of the tile kernels: `n` right-hand sides (columns) whose
// vectors lie `ld` elements apart run in one launch of ntiles * n CTAs.  CTA
// b works on column b % n and tile b / n, so the CTAs reading the same rows
// of A run together and A comes from DRAM once; column c uses scalars block
// sc + c and its own reduction partials and counter.  `shared` marks the
// vector arguments (bit i = pointer i) that all columns share (dinv).
struct Cols {
    int n = 1;
    long long ld = 0;
    unsigned shared = 0;
    int spmm = 0;  // box SpMV: one CTA per tile serves every column (box_spmm_kernel)
};

// Geometry of the structured sweep (7-point box patterns): canonical dims
// (a, b, s) with s the dimension a CTA spans, (a, b) cut into TA x TB tiles.
struct BoxGeom {
    int D[3];      // extents of a, b, s
    int S[3];      // row strides of a, b, s
    int order[3];  // dims by descending stride = CSR order of the lower entries
    int span;      // which of x (0), y (1), z (2) is the spanned dimension s
    int TA, TB, nta, ntb;
    // Thread-block clusters of CX x CY neighbouring tiles (1 x 1: none).  A
    // tile hands its face values to a downstream tile of the same cluster
    // through distributed shared memory; nca x ncb clusters cover the tiles.
    int CX, CY, nca, ncb;
};

struct DevPattern {
    int spmv_lanes = 1;  // CSR SpMV lanes per row (1, 4, 16; ocsl_set_spmv_lanes / autotuner)
    bool box_ok;
    BoxGeom box;    // geometry of the FP64 structured sweeps
    BoxGeom box32;  // and of the FP32 ones (tuned separately)
    int n;
    int nnz;
    const int* rp;
    const int* col;
    const int* diag;
    const int* pair_ptr;
    const int* pair_k;
    const int* pair_slot;
    const int* fw_order;
    const int* fw_chunk;
    int fw_nchunks;
    const int* bw_order;
    const int* bw_chunk;
    int bw_nchunks;
    // levels that are contiguous row ranges (HostPattern::fw_range / bw_range):
    // count (0 = not applicable) and (first row, end row) per level
    int fw_nrange, bw_nrange;
    int fw_range[2 * kRangeMaxLevels], bw_range[2 * kRangeMaxLevels];
    // the ranges are the colours of a multicolour ordering (fw ascending, bw
    // descending): a row's lower entries lie in lower colours, its upper ones
    // in higher colours, so the last colour's rows have no upper entries
    bool coloured;
};

// Face-to-cell incidence of the mesh (ocsl_set_faces), for the assembly.
struct DevFaces {
    int nf = 0, nb = 0;
    const int* left = nullptr;      // [nf]
    const int* right = nullptr;     // [nf]
    const int* bc_left = nullptr;   // [nb]
    const int* cell_ptr = nullptr;  // [n+1] interior-face entries of each cell
    const int* cell_ent = nullptr;  // face << 1 | (1 if the cell is the face's right cell)
    const int* cell_slot = nullptr; // CSR slot of the entry (cell, other cell) in the cell's row
    const int* bc_ptr = nullptr;    // [n+1] boundary-face entries of each cell
    const int* bc_ent = nullptr;    // boundary face index
};

struct SweepSync {
    unsigned* ticket;    // chunk dispenser (reset by the last CTA)
    unsigned* finished;
    int* err;            // ocsl_status of a bounded wait that gave up
    // Host side only (ocsl_inject_fault): the launcher starts the dispenser at
    // 1 and launches one tile / cluster / chunk fewer, so the first unit of
    // the schedule is never computed and the waits on it run out.
    int skip_first;
};

// Sets the dispenser to 1 on `st` (its only word is 0 between launches: the
// last CTA of every sweep resets it).
void preset_ticket_one(cudaStream_t st, unsigned* ticket);

// ------------------------------------------------------------------ host-side launchers
// All launchers enqueue on `st` and never synchronise.

template <typename T>
void launch_spmv(cudaStream_t st, const DevPattern& P, const T* val, const T* x, T* y,
                 int mode, const double* scal_a, double a_const, const T* z, T* y_copy,
                 const T* w, int dots, const ReduceState& R, Scalars* sc, int epi, int it,
                 int maxit, const Cols& cols = Cols{});

// SpMV on packed stencil records ([2][n][4], the structured sweeps' layout, of A
// itself) for natural-order 7-point box patterns; dims = (nx, ny, nz).
template <typename T>
void launch_box_spmv(cudaStream_t st, int n, const int* dims, const T* rec, const T* x, T* y,
                     int mode, double a_const, const T* z, T* y_copy, const T* w, int dots,
                     const ReduceState& R, Scalars* sc, int epi, int it, int maxit,
                     const Cols& cols = Cols{});

// Vector kernels: the op decides which pointers it uses.
enum VecOp : int {
    V_RB_P = 0,   // dum = fma(-w, v, p); p = fma(w, dum, r)
    V_RB_HS,      // h = fma(a, y, x); s = fma(-a, v, r)
    V_RB_XR,      // x = fma(w, z, h); r = fma(-w, t, s); dots <r0,r>, <r,r>
    V_DOT2,       // dots <a,b>, <a,a>
    V_DOT1,       // dot <a,b>
    V_RC_XR,      // x = fma(a, p, x); rn = fma(-a, q, r); dot <rn,rn>
    V_RC_P,       // p = fma(beta, p, rn)
    V_TB_S,       // s = fma(-a, v, r); dot <s,s>
    V_TB_XR,      // x = fma(w, sh, fma(a, ph, x)); r = fma(-w, t, s); dots <r,r>, <rh,r>
    V_TB_P,       // p = fma(beta, fma(-w, v, p), r)
    V_TB_HALF,    // if half: x = fma(a, ph, x)
    V_COPY2,      // u = r; v = r
    V_PC_INIT,    // z = r * dinv; p = z; dot <r,z>
    V_PC_XRZ,     // x = fma(a,p,x); r = fma(-a,q,r); z = r*dinv; dots <r,r>, <r,z>
    V_PC_P,       // p = fma(beta, p, z)
    V_IR_SCALE,   // f0 = float(r * (1/rnorm)); f1 = f0; f2 = f0; f3 = 0; dot <f0,f0>
    V_IR_UPDATE,  // x = fma(double(f0), rnorm, x)
    V_SUM,        // dot-free sum: s = s + x (cmatrix_solver.cpp:244-252)
    V_ABSSUM,     // s = s + |x| (:255-263)
    V_PRODUCT,    // out = x * y (:266-272)
    V_AXPY,       // out = a x + b y with the reference's special cases (:275-335)
    V_SCALE,      // out = a x (:275-281)
};

struct VecPtrs {
    void* v[8];
};

template <typename T>
void launch_vec(cudaStream_t st, int op, int n, const VecPtrs& p, const ReduceState& R,
                Scalars* sc, const Scalars* sc_outer, int epi, int it, int maxit,
                const Cols& cols = Cols{});

// pivot_err (last sweep only): set to OCSL_ZERO_PIVOT when a diagonal of the
// factor is zero or infinite (or its FP32 reciprocal is infinite)
template <typename T>
void launch_ilu_sweep(cudaStream_t st, const DevPattern& P, const T* A, const T* Mold, T* Mnew,
                      double* dinv, float* M32, float* dinv32, float* A32, const int* done,
                      int* pivot_err = nullptr);

template <typename T>
void launch_fw_sweep(cudaStream_t st, const DevPattern& P, const T* M, const T* rhs, T* out,
                     const SweepSync& S, const int* done);
// divmode 0: divide by M_ii (reference); 1: multiply by dinv
template <typename T>
void launch_bw_sweep(cudaStream_t st, const DevPattern& P, const T* M, const T* dinv,
                     const T* rhs, T* out, int divmode, const SweepSync& S, const int* done);
// One-warp sweep in natural (forward) or reverse (backward) row order for
// tiny systems with a deep schedule; the solution is staged in n * sizeof(T)
// bytes of shared memory (at most kSerialMaxBytes, which leaves the kernel's
// row staging room under the 48 KB a launch may take without opting in).
constexpr int kSerialMaxBytes = 40 * 1024;
// A natural-order nx x ny x nz 7-point box with even nx in its red-black
// (multicolour) ordering: colour 0 = cells with i + j + k even, numbered
// first, each colour in natural order.  Since nx is even, every pair of cells
// (2m, 2m + 1) of an x-line holds one of each colour, so natural cell p has
// rank p / 2 in its colour: row t (colour c = t >= n0, rank r = t - c n0) is
// cell p = 2r + b with j = (r / hx) % ny, k = r / (hx ny), b = (c + j + k) & 1,
// i = 2 (r % hx) + b, hx = nx / 2.  Its neighbours lie in the other colour at
// ranks r - 1 + b (x-), r + b (x+), r -+ hx (y-+), r -+ hx ny (z-+), and its CSR
// row holds them in the order z-, y-, x-, x+, y+, z+ with the diagonal last
// (colour 1: every neighbour has a smaller index) or first (colour 0).
// Stencil records [2][n][4]: (z-, y-, x-, x+) and (y+, z+, diagonal, unused).
struct RbGeom {
    int n, n0, nx, ny, nz, hx;
    // per row: bits 0-5 which neighbours exist, bit 6 the parity b (saves
    // the kernels four integer divisions a row; built and checked on the host)
    const unsigned char* info;
};
struct RbRow {
    int c;        // colour
    int nb[6];    // neighbour rows z-, y-, x-, x+, y+, z+ (valid where has)
    bool has[6];
};
// The row's neighbours from its info byte.
__device__ __forceinline__ RbRow rb_row_info(const RbGeom& g, int t)
{
    RbRow o;
    o.c = t >= g.n0 ? 1 : 0;
    const int r = t - o.c * g.n0;
    const unsigned f = __ldg(g.info + t);
    const int b = (int)(f >> 6) & 1;
    const int ob = (1 - o.c) * g.n0;
    const int sz = g.hx * g.ny;
    const int off[6] = {-sz, -g.hx, b - 1, b, g.hx, sz};
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        o.has[s] = (f >> s) & 1u;
        o.nb[s] = o.has[s] ? ob + r + off[s] : t;
    }
    return o;
}
__host__ __device__ __forceinline__ RbRow rb_row(const RbGeom& g, int t)
{
    RbRow o;
    o.c = t >= g.n0 ? 1 : 0;
    const int r = t - o.c * g.n0;
    const int rx = r % g.hx, rjk = r / g.hx;
    const int j = rjk % g.ny, k = rjk / g.ny;
    const int b = (o.c + j + k) & 1;
    const int i = 2 * rx + b;
    const int ob = (1 - o.c) * g.n0;  // the other colour's first row
    const int sz = g.hx * g.ny;
    o.has[0] = k > 0;
    o.has[1] = j > 0;
    o.has[2] = i > 0;
    o.has[3] = i < g.nx - 1;
    o.has[4] = j < g.ny - 1;
    o.has[5] = k < g.nz - 1;
    o.nb[0] = ob + r - sz;
    o.nb[1] = ob + r - g.hx;
    o.nb[2] = ob + r - 1 + b;
    o.nb[3] = ob + r + b;
    o.nb[4] = ob + r + g.hx;
    o.nb[5] = ob + r + sz;
#pragma unroll
    for (int s = 0; s < 6; ++s)
        if (!o.has[s]) o.nb[s] = t;  // never read; an address inside the vector
    return o;
}
// CSR (FP64) -> red-black stencil records in TO, through the host-built
// slot of every entry (0-5 neighbours, 6 diagonal, -1 phantom).
template <typename TO>
void launch_rb_records(cudaStream_t st, const RbGeom& g, const int* rp, const signed char* slot,
                       const double* M, TO* rec);
// y = A x and its fused dots / epilogues on the records (spmv_kernel's
// contract, bit-identical to it on the same matrix).
template <typename T>
void launch_rb_spmv(cudaStream_t st, const RbGeom& g, const T* rec, const T* x, T* y, int mode,
                    double a_const, const T* z, T* y_copy, const T* w, int dots,
                    const ReduceState& R, Scalars* sc, int epi, int it, int maxit);
// out = U^-1 L^-1 rhs on the factor's records: colour 1 (forward then
// backward: no upper entries), then colour 0 (backward; its y is rhs) --
// launch_coloured_precond's arithmetic, two launches, no column indices.
template <typename T>
void launch_rb_precond(cudaStream_t st, const RbGeom& g, const T* rec, const T* dinv,
                       const T* rhs, T* out, int divmode, const int* done);

// One sweep over a pattern whose levels are contiguous row ranges: one launch
// per level, rows of a level independent, plain loads (no waits, no prefill).
template <typename T>
void launch_range_sweep(cudaStream_t st, const DevPattern& P, bool forward, const T* M,
                        const T* dinv, const T* rhs, T* out, int divmode, const int* done);
// Both sweeps of the ILU preconditioner, out = U^-1 L^-1 rhs, on a
// colour-ordered pattern (DevPattern::coloured: fw_range holds the colours in
// ascending order): 2 colours - 2 launches, tmp holds y of the middle colours.
template <typename T>
void launch_coloured_precond(cudaStream_t st, const DevPattern& P, const T* M, const T* dinv,
                             const T* rhs, T* tmp, T* out, int divmode, const int* done);
template <typename T>
void launch_serial_sweep(cudaStream_t st, const DevPattern& P, bool forward, const T* M,
                         const T* dinv, const T* rhs, T* out, int divmode, const int* done);

void launch_convert_f64_f32(cudaStream_t st, int n, const double* in, float* out);

// Structured sweep on the packed stencil factor ([2][n][4]: (z-, y-, x-, 0),
// (x+, y+, z+, diagonal term)); divmode 0 divides by the diagonal term, 1
// multiplies by it.
// Column-batched form: cols.n (<= kMaxCols) right-hand sides cols.ld apart in
// one wavefront pass; `done` then points at column 0's flag, the others
// follow every done_stride ints, and the launch is skipped once all are set.
template <typename T>
void launch_box_sweep(cudaStream_t st, const BoxGeom& g, int n, const T* soa, const T* rhs, T* out,
                      bool forward, int divmode, const SweepSync& S, const int* done,
                      const Cols& cols = Cols{}, int done_stride = 0);
// Dynamic shared memory of one structured-sweep CTA of `threads` threads
// (records and rhs staged kPF wavefronts ahead, a two-slot ring per column);
// a launch needs it <= kBoxSmemLimit.
size_t box_sweep_smem(int threads, int elem_size, int ncols);
constexpr size_t kBoxSmemOptin = 227 * 1024;            // per-block opt-in maximum
constexpr size_t kBoxSmemLimit = kBoxSmemOptin - 1024;   // dynamic part, static kept below 1 KB
// The same for geometry g, including a clustered tile's two face buffers
// (ncols x s-extent x (TA + TB) values).
size_t box_sweep_smem(const BoxGeom& g, int elem_size, int ncols);
constexpr int kMaxClusterTiles = 16;
// g with clusters of cx x cy tiles (clipped to the tile grid and to 16
// tiles; 1 x 1 = no clusters).
BoxGeom box_with_cluster(BoxGeom g, int cx, int cy);
// Warp-pipelined structured sweep (kernels_wave.cu), one right-hand side.
// Canonical coordinates a = x, s = the longer of y and z, b = the other; a
// warp solves a tile of 32 (along a, one lane each) x K (along b) columns,
// K = 4 in FP32 and 2 in FP64; a CTA holds WB warps stacked along b.  The
// factor's records are stored per direction in the sweep's step order
// ([nwb][nwa][T][K][32] records, T = Ds + K - 1 + 31), which depends on the
// box and K only, not on WB or the lag.
constexpr int kWaveMaxWarps = 8;
struct WaveGeom {
    int D[3];      // extents of a, b, s
    int S[3];      // physical row strides of a, b, s
    int span;      // 2: s = z (b = y); 1: s = y (b = z)
    int K;         // columns per warp along b
    int nwa, nwb;  // warp tiles along a and b
    int T;         // steps of a warp tile
    int WB;        // warps per CTA
    int nta, ntb;  // CTA tiles along a and b
    int lag;       // start lag behind an upstream CTA (rows)
    int lag_sh;    // start lag behind the warp below (rows)
};
int wave_cols_per_warp(int elem_size);
// Dynamic shared memory of one CTA (cp.async rings and the face buffers
// between its warps).
size_t wave_sweep_smem(const WaveGeom& g, int elem_size);
// Geometry of an nx * ny * nz box for `warps` warps per CTA (0 = default 4;
// clipped to the box and to the shared-memory limit); lag 0 = default.
WaveGeom make_wave_geom(const int* dims, int elem_size, int warps, int lag = 0);
// Records (of 4 elements) in one direction's step-order layout.
size_t wave_layout_elems(const WaveGeom& g);
// face_a: [nwa * nwb][T][K], face_b: [nwa * nwb][T][32] elements of the
// sweep's type, all-ones between launches.
template <typename T>
void launch_wave_sweep(cudaStream_t st, const WaveGeom& g, const T* rec, const T* rhs, T* out,
                       void* face_a, void* face_b, bool forward, int divmode, const SweepSync& S,
                       const int* done);
// CSR factor (FP64) -> the forward and backward step-order record layouts of g.
template <typename TO>
void launch_box_to_wave(cudaStream_t st, const int* dims, int n, const int* rp, const double* M,
                        const WaveGeom& g, TO* fw, TO* bw, int recip);

// CSR factor (FP64) -> packed stencil records in TO; diagonal term =
// diagonal, or 1/diagonal with recip.
template <typename TO>
void launch_box_to_soa(cudaStream_t st, const int* dims, int n, const int* rp, const double* M,
                       TO* soa, int recip);

// All-ones fill of a sweep output, skipped once the solve is done: once all
// of the ndone flags done[q * done_stride] are set.
void launch_fill_ones(cudaStream_t st, void* out, size_t bytes, const int* done, int ndone = 1,
                      int done_stride = 0);

// Factor side outputs without a sweep: dinv = 1 / M_ii and FP32 copies.
void launch_factor_outputs(cudaStream_t st, const DevPattern& P, const double* M, const double* A,
                           double* dinv, float* M32, float* dinv32, float* A32,
                           int* pivot_err = nullptr);

// assembly.cu
// face_mu / face_pdum (FlowDev): per-face values computed once per iteration
// (bit-identical to evaluating them per face side); null: evaluated here.
void launch_assemble(cudaStream_t st, const DevPattern& P, const DevFaces& F,
                     const ocsl_assembly& q, const ocsl_flow_state& s, double* value, double* b,
                     double* x0, double* ap, double* total_mdot, const double* face_mu = nullptr,
                     const double* face_pdum = nullptr);
void launch_bc_value_grad(cudaStream_t st, const DevFaces& F, const ocsl_assembly& q,
                          const ocsl_flow_state& s, const double* lambda, double* grad);

// flow.cu: the SIMPLE inner iteration around the assembly and the solves.
// Cell arrays [n] ([3][n] for vectors), face arrays [nf] ([3][nf]), boundary
// arrays [nb] ([3][nb]); the state is updated in place.
struct FlowDev {
    // cells
    double* pressure;
    double* velocity;           // [3][n]
    double* velocity_last;      // [3][n]
    double* density_c;
    double* density_last;
    double* pressure_last;
    double* temperature;
    double* enthalpy;
    double* enthalpy_last;
    double* pressure_corr;
    double* pressure_grad;       // [3][n]
    double* pressure_corr_grad;  // [3][n]
    double* ap;
    double* ap_vec;              // [3][n]
    double* mach;
    const double* volume;
    // interior faces
    const int* left;
    const int* right;
    const double* geo_aver;
    const double* area_vector;   // [3][nf]
    const double* alpha;         // [3][nf]
    const double* distance;
    const double* unit;          // [3][nf]
    double* mdot;
    double* face_density;
    double* qy;
    double* stress;              // [3][nf], viscous flows
    // per-face values the iteration's assemblies share (library buffers [nf]):
    // mu(T_f) of the face-loop translation unit (momentum and enthalpy) and
    // the pressure equation's convective coefficient drho/dp(T_f) / rho_f * m
    double* face_mu;
    double* face_pdum;
    double* vol_ap;  // [n] volume / ap after the momentum components (library buffer)
    // boundary faces
    const int* bc_type;
    const int* bc_left;
    const double* bc_area;
    const double* bc_area_vector;  // [3][nb]
    const double* bc_unit;         // [3][nb]
    const double* bc_alpha;        // [3][nb]
    const double* bc_distance;
    const double* bc_out_pressure;
    double* bc_pressure;
    double* bc_mdot;
    double* bc_density;
    double* bc_qy;
    double* bc_enthalpy;
    double* bc_temperature;
    double* bc_velocity;           // [3][nb]
    int* bc_supersonic;
    // constants
    double relax_p, relax_u, cp, Tref, H_formation;
    double R, gamma, suth0, suth1;
};
// The stages of one inner iteration (flow.cu); each launch is skipped when
// its loop is empty.
void launch_flow_set_bc(cudaStream_t st, int n, int nb, const FlowDev& f);
void launch_flow_grad(cudaStream_t st, bool corr, int n, int nf, int nb, const FlowDev& f,
                      const DevFaces& F);
// stress (viscous) and face_mu; face_mu alone when !viscous
void launch_flow_stress(cudaStream_t st, int n, int nf, const FlowDev& f, bool viscous);
void launch_flow_velocity_update(cudaStream_t st, int n, int d, const double* x, const FlowDev& f,
                                 double* res);
void launch_flow_face_mdot(cudaStream_t st, int n, int nf, int nb, const FlowDev& f, int blended);
void launch_flow_pcorr(cudaStream_t st, int n, int nb, const double* x, const FlowDev& f);
void launch_flow_correct(cudaStream_t st, int n, int nf, int nb, const FlowDev& f, int blended);
void launch_flow_enthalpy_update(cudaStream_t st, int n, const double* x, const FlowDev& f,
                                 double* res);
void launch_flow_end_step(cudaStream_t st, int n, const FlowDev& f);
void launch_take_sum(cudaStream_t st, const Scalars* sc, double* out);

// adjoint.cu: out[k] = val[perm[k]] (gather) and out[perm[k]] = in[k] (scatter)
void launch_gather_values(cudaStream_t st, long long nnz, const int* perm, const double* val,
                          double* out);
void launch_scatter_values(cudaStream_t st, long long n, const int* perm, const double* in,
                           double* out);
void launch_pattern_outer(cudaStream_t st, const DevPattern& P, double alpha, const double* u,
                          const double* v, double* out);

}  // namespace ocsl
