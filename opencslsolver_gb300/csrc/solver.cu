// Context, pattern upload, Krylov drivers and the extern "C" boundary
// (include/ocsl.h).
//
// Drivers enqueue every kernel of a solve on the context's stream; the Krylov
// scalars live on the device (Scalars) and every kernel returns at once when
// `done` is set, so the reference-faithful solvers (at most 4 / 3 iterations)
// run without a single host round trip, and the tolerance-mode solvers look at
// the scalars only between batches of iterations, one batch ahead.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ocsl_internal.cuh"
#include "ir32_graph.h"
#include "pattern.h"

using namespace ocsl;

namespace {

thread_local std::string g_create_error;

const char* kVersion = "ocsl-gb300 0.1 (sm_103a)";

struct CudaError {
    cudaError_t code;
    const char* what;
};

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) throw CudaError{e_, #call};    \
    } while (0)

template <typename T>
T* dalloc(size_t count)
{
    void* p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc(&p, count * sizeof(T)));
    return static_cast<T*>(p);
}

template <typename T>
T* upload(const std::vector<T>& v)
{
    T* d = dalloc<T>(v.size());
    if (!v.empty()) CK(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return d;
}

// Fixed-iteration counts and exits of the reference (cmatrix_solver.cpp:637,684).
constexpr int kRefCgIters = 4;
constexpr int kRefBicgIters = 3;

enum Vec64 { R, P, Q, RN, V, R0, S, DUM, H, T, Y, Z, DUM2, PH, SH, RH, TMP, NVEC64 };
enum Vec32 { F_RI, F_RH, F_P, F_PH, F_V, F_S, F_SH, F_T, F_TMP, F_D, NVEC32 };

// Scalars blocks on the device: 0 main / outer, 1 inner, 2 utility; the
// column-batched solve uses kMaxCols outer blocks from kScOuterCols and
// kMaxCols inner blocks from kScInnerCols.
constexpr int kScOuterCols = 3;
constexpr int kScInnerCols = kScOuterCols + kMaxCols;
constexpr int kScFlow = kScInnerCols + kMaxCols;  // residual sums of the SIMPLE iteration
constexpr int kScBlocks = kScFlow + 1;
// Pinned host mirrors: read copies [0, 16), upload staging [16, 32),
// two inspection slots of kMaxCols blocks from 32.
constexpr int kHostStage = 16;
constexpr int kHostInspect = 32;
constexpr int kHostSlots = kHostInspect + 2 * kMaxCols;
static_assert(kScBlocks <= kHostStage, "host mirror layout");

}  // namespace

namespace {
BoxGeom make_box_geom(const BoxShape& bs, int TA_req, int TB_req);
}

constexpr int kAutoClusterTiles = 64;  // tiles from which clusters pay by default

struct ocsl_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;

    bool has_pattern = false;
    HostPattern hp;  // kept for ocsl_pattern_info
    DevPattern P{};
    int* d_pat[10] = {};

    double* d_A = nullptr;  // values of host-buffer solves
    double* d_b = nullptr;
    double* d_x = nullptr;
    double* d_Ma = nullptr;
    double* d_Mb = nullptr;
    double* d_dinv = nullptr;
    double* v64[NVEC64] = {};
    float* d_A32 = nullptr;
    float* d_M32 = nullptr;
    float* d_dinv32 = nullptr;
    float* v32[NVEC32] = {};
    // column-batched solves: [kMaxCols][n] work vectors (allocated on first use)
    double* v64c = nullptr;           // FP64 residuals
    float* v32c[NVEC32] = {};         // FP32 inner vectors
    double* d_soa64 = nullptr;  // stencil-SoA factor copies (7-point box patterns)
    float* d_soa32 = nullptr;
    double* d_recA64 = nullptr;  // stencil records of A itself, for the box SpMV
    float* d_recA32 = nullptr;

    ReduceState R{};
    Scalars* d_sc = nullptr;  // [kScBlocks]: main / outer, inner, utility, column blocks
    Scalars* h_sc = nullptr;  // [kHostSlots] pinned mirrors
    SweepSync S{};
    unsigned* d_sync = nullptr;
    int* d_err = nullptr;
    int* h_err = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    cudaEvent_t ev_batch[2] = {nullptr, nullptr};

    // sweep kernel choice (ocsl_set_sweep_kernel): 0 auto, 1 level-scheduled, 2 structured
    int sweep_kernel = 0;
    // ocsl_inject_fault: the next sweep leaves out the first unit of its schedule
    bool fault_skip_pending = false;
    // the sync block of the next sweep launch (consumes a pending injection)
    SweepSync next_sync()
    {
        SweepSync s = S;
        s.skip_first = fault_skip_pending ? 1 : 0;
        fault_skip_pending = false;
        return s;
    }
    // structured-sweep geometry requests per precision ([0] FP64, [1] FP32):
    // TA, TB (0 = heuristic) and tiles per thread-block cluster
    int box_tile[2][2] = {{0, 0}, {0, 0}};
    // 0 x 0 = automatic: 2 x 4 tiles per cluster on a grid of at least
    // kAutoClusterTiles tiles, single tiles below (few tile hops to save)
    int box_cluster[2][2] = {{0, 0}, {0, 0}};
    // Warp-pipelined sweep (kernels_wave.cu) for single right-hand sides, per
    // precision ([0] FP64, [1] FP32): on / off, warps per CTA and start lag
    // requests (0 = automatic), and the geometry built from them.
    // Off by default: on the boxes measured (64^3, 128^3) the CTA kernel's
    // wavefront is shorter; ocsl_autotune_device switches it on per precision
    // where it times faster, ocsl_set_sweep_kernel(3, ...) forces it.
    bool wave_on[2] = {false, false};
    bool wave_tuning = false;  // the autotuner is timing it: keep its layouts
    int wave_req[2][2] = {{0, 0}, {0, 0}};
    WaveGeom wave[2] = {};
    // its step-order record layouts ([0] forward, [1] backward) and face
    // buffers (all-ones between launches; refilled after a wait ran out)
    double* d_wrec64[2] = {nullptr, nullptr};
    float* d_wrec32[2] = {nullptr, nullptr};
    void* d_wface[2] = {nullptr, nullptr};
    size_t wface_bytes[2] = {0, 0};
    bool wave_faces_dirty = false;
    // the warp-pipelined kernel applies to this box (its layout stays within
    // 16 n records: boxes much thinner than a warp in x are left to the CTA kernel)
    bool wave_fits[2] = {false, false};
    // P.box / P.box32 and the wave geometries from the requests (box patterns only)
    void rebuild_box_geoms()
    {
        if (!hp.box.ok) return;
        for (int k = 0; k < 2; ++k) {
            const int elem = k == 0 ? 8 : 4;
            wave[k] = make_wave_geom(hp.box.dim, elem, wave_req[k][0], wave_req[k][1]);
            wave_fits[k] = wave_layout_elems(wave[k]) <= 16 * (size_t)std::max(P.n, 1);
        }
        BoxGeom* geo[2] = {&P.box, &P.box32};
        for (int k = 0; k < 2; ++k) {
            const BoxGeom g = make_box_geom(hp.box, box_tile[k][0], box_tile[k][1]);
            int cx = box_cluster[k][0], cy = box_cluster[k][1];
            if (cx == 0) {
                const bool big = g.nta * g.ntb >= kAutoClusterTiles;
                cx = big ? 2 : 1;
                cy = big ? 4 : 1;
            }
            *geo[k] = box_with_cluster(g, cx, cy);
        }
    }

    // CUDA graph of one batch of Krylov iterations, reused while its key
    // (method and the pointers the iterations read) stays the same
    cudaGraphExec_t graph_exec = nullptr;
    bool graphs_on = true;
    int graph_kind = 0;
    // FP32-refined solves run their refinement and inner loops on the device
    // (conditional graph nodes, ocsl_set_device_loop); its control block
    bool device_loop = false;
    void* d_irctl = nullptr;
    int n_irctl = 0;
    cudaStream_t capture_stream = nullptr;  // loop bodies captured inside another capture
    // the instantiated graph of the last device-driven solve and its key
    cudaGraphExec_t ir_exec = nullptr;
    std::vector<unsigned char> ir_key;
    // several right-hand sides of the FP32-inner solver in lockstep (else one by one)
    int col_batching = 1;  // 0 one after another, 1 lockstep, 2 lockstep with the SpMM box SpMV
    const void* graph_ptr[6] = {};

    // factor of the last solve (buffer and SoA copies), for solves that reuse it
    const double* fac_M = nullptr;
    const double* fac_soa64 = nullptr;
    const float* fac_soa32 = nullptr;
    bool fac_checked = false;  // fac_status holds the pivot check of fac_M
    int fac_status = OCSL_OK;

    // the pattern qualifies for the one-warp serial sweep ([0] FP64, [1] FP32)
    bool serial_ok[2] = {false, false};
    // the pattern is the red-black ordering of an even-nx box (a multicolour
    // child): SpMV and preconditioner on stencil records (d_recA*, d_soa*)
    // built through the slot of every CSR entry
    bool rb_ok = false;
    RbGeom rb{};
    signed char* d_rbslot = nullptr;

    // SIMPLE iteration on the device (ocsl_flow_iterate_device): the system
    // of the equation being solved, a residual work vector, the per-call
    // outputs (device and pinned host), and the boundary-kind check of the
    // last state seen
    struct FlowOut {
        double residual[5];
        int iterations[5];
        int err[5];
    };
    double* d_fval = nullptr;
    double* d_fb = nullptr;
    double* d_fx = nullptr;
    double* d_ftmp = nullptr;
    double* d_fmu = nullptr;    // [nf] FlowDev::face_mu
    double* d_fpdum = nullptr;  // [nf] FlowDev::face_pdum
    double* d_fvolap = nullptr;  // [n] FlowDev::vol_ap
    FlowOut* d_fout = nullptr;
    FlowOut* h_fout = nullptr;
    const void* flow_bc_checked = nullptr;
    // the captured inner iteration (reference-faithful solves), replayed while
    // its key -- every argument of the call and the stream -- stays the same;
    // the first call with a key runs directly (it allocates), the next captures
    cudaGraphExec_t flow_exec = nullptr;
    std::vector<unsigned char> flow_key;
    int flow_seen = 0;
    Scalars* d_sc_ref = nullptr;  // the scalars block a reference-faithful solve starts from
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    void drop_flow_graph()
    {
        if (flow_exec) cudaGraphExecDestroy(flow_exec);
        flow_exec = nullptr;
        flow_key.clear();
        flow_seen = 0;
    }

    // face-loop assembly: the mesh's face incidence (ocsl_set_faces)
    DevFaces F{};
    int* d_faces[8] = {};
    bool has_faces = false;

    // adjoint: a child context holding the transposed pattern, and the map
    // from its CSR slots to this pattern's slots (built on first use)
    ocsl_ctx* tctx = nullptr;
    int* d_tperm = nullptr;
    long long nnzT = 0;

    // multicolour ordering of the tolerance-mode solves (ocsl_set_ordering):
    // a child context holding the permuted pattern P A P^T, the permutation
    // (perm[new row] = original row) and the map from its CSR slots to this
    // pattern's slots (built by the first solve that needs them)
    int ordering = OCSL_ORDER_NATURAL;
    ocsl_ctx* cctx = nullptr;
    int* d_cperm = nullptr;
    int* d_cslot = nullptr;
    int colours = 0;

    // kernel timing (ocsl_profile_*)
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_ev;  // pairs
    std::vector<int> prof_cat;
    size_t prof_used = 0;

    void free_pattern();
    void free_all();
    // Forget the captured iteration graph: its kernels and launch shapes belong
    // to the pattern, sweep kernel and geometry it was captured with.
    void drop_graph()
    {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
        graph_kind = 0;
        drop_flow_graph();
        if (ir_exec) cudaGraphExecDestroy(ir_exec);
        ir_exec = nullptr;
        ir_key.clear();
    }
    void ensure_reduce(int ntiles);
    void ensure_fp32();
    void ensure_cols();
    // step-order records and face buffers of the warp-pipelined sweep (k: 0 FP64, 1 FP32)
    void ensure_wave(int k);
};

void ocsl_ctx::free_pattern()
{
    drop_graph();
    fac_M = nullptr;
    fac_soa64 = nullptr;
    fac_soa32 = nullptr;
    if (tctx) ocsl_destroy(tctx);
    tctx = nullptr;
    if (d_tperm) cudaFree(d_tperm);
    d_tperm = nullptr;
    nnzT = 0;
    if (cctx) ocsl_destroy(cctx);
    cctx = nullptr;
    if (d_rbslot) cudaFree(d_rbslot);
    d_rbslot = nullptr;
    rb_ok = false;
    for (int** pp : {&d_cperm, &d_cslot}) { if (*pp) cudaFree(*pp); *pp = nullptr; }
    colours = 0;
    for (auto& p : d_faces) { if (p) cudaFree(p); p = nullptr; }
    F = DevFaces{};
    has_faces = false;
    double** dflow[] = {&d_fval, &d_fb, &d_fx, &d_ftmp, &d_fmu, &d_fpdum, &d_fvolap};
    for (auto pp : dflow) { if (*pp) cudaFree(*pp); *pp = nullptr; }
    flow_bc_checked = nullptr;
    for (auto& p : d_pat) { if (p) cudaFree(p); p = nullptr; }
    double** d64[] = {&d_A, &d_b, &d_x, &d_Ma, &d_Mb, &d_dinv};
    for (auto pp : d64) { if (*pp) cudaFree(*pp); *pp = nullptr; }
    for (auto& v : v64) { if (v) cudaFree(v); v = nullptr; }
    float** d32[] = {&d_A32, &d_M32, &d_dinv32, &d_soa32, &d_recA32};
    if (d_recA64) cudaFree(d_recA64);
    d_recA64 = nullptr;
    if (d_soa64) cudaFree(d_soa64);
    d_soa64 = nullptr;
    for (auto pp : d32) { if (*pp) cudaFree(*pp); *pp = nullptr; }
    for (auto& v : v32) { if (v) cudaFree(v); v = nullptr; }
    if (v64c) cudaFree(v64c);
    v64c = nullptr;
    for (auto& v : v32c) { if (v) cudaFree(v); v = nullptr; }
    for (int k = 0; k < 2; ++k) {
        if (d_wrec64[k]) cudaFree(d_wrec64[k]);
        if (d_wrec32[k]) cudaFree(d_wrec32[k]);
        if (d_wface[k]) cudaFree(d_wface[k]);
        d_wrec64[k] = nullptr;
        d_wrec32[k] = nullptr;
        d_wface[k] = nullptr;
        wface_bytes[k] = 0;
        wave_fits[k] = false;
    }
    wave_faces_dirty = false;
    has_pattern = false;
    P = DevPattern{};
}

void ocsl_ctx::free_all()
{
    free_pattern();
    if (R.partials) cudaFree(R.partials);
    if (R.counter) cudaFree(R.counter);
    R = ReduceState{};
    if (d_sc) cudaFree(d_sc);
    if (h_sc) cudaFreeHost(h_sc);
    if (d_sync) cudaFree(d_sync);
    if (d_err) cudaFree(d_err);
    if (h_err) cudaFreeHost(h_err);
    d_sc = nullptr; h_sc = nullptr; d_sync = nullptr; d_err = nullptr; h_err = nullptr;
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
    for (auto& e : ev_batch) { if (e) cudaEventDestroy(e); e = nullptr; }
    for (auto& e : prof_ev) cudaEventDestroy(e);
    prof_ev.clear();
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    if (d_fout) cudaFree(d_fout);
    if (h_fout) cudaFreeHost(h_fout);
    if (d_sc_ref) cudaFree(d_sc_ref);
    if (d_irctl) cudaFree(d_irctl);
    d_irctl = nullptr;
    n_irctl = 0;
    if (capture_stream) cudaStreamDestroy(capture_stream);
    capture_stream = nullptr;
    if (ir_exec) cudaGraphExecDestroy(ir_exec);
    ir_exec = nullptr;
    ir_key.clear();
    d_fout = nullptr;
    h_fout = nullptr;
    d_sc_ref = nullptr;
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    ev_fork = ev_join = nullptr;
    if (own_stream) cudaStreamDestroy(own_stream);
    own_stream = stream = nullptr;
}

void ocsl_ctx::ensure_reduce(int ntiles)
{
    ntiles = std::max(ntiles, 1);
    if (R.partials && R.max_tiles >= ntiles) return;
    if (R.partials) CK(cudaFree(R.partials));
    R.partials = dalloc<double>((size_t)kMaxCols * kMaxDots * ntiles);
    R.max_tiles = ntiles;
    if (!R.counter) {
        R.counter = dalloc<unsigned>(kMaxCols);
        CK(cudaMemset(R.counter, 0, sizeof(unsigned) * kMaxCols));
    }
}

void ocsl_ctx::ensure_fp32()
{
    if (d_A32) return;
    const size_t n = (size_t)P.n, nnz = (size_t)P.nnz;
    d_A32 = dalloc<float>(nnz);
    d_M32 = dalloc<float>(nnz);
    d_dinv32 = dalloc<float>(n);
    for (auto& v : v32) v = dalloc<float>(n);
    if (hp.box.ok) d_soa32 = dalloc<float>(8 * n);
}

void ocsl_ctx::ensure_wave(int k)
{
    const WaveGeom& g = wave[k];
    const size_t recs = wave_layout_elems(g);
    const size_t face = (size_t)g.nwa * g.nwb * g.T * (g.K + 32) * (k == 0 ? 8 : 4);
    if (k == 0 && !d_wrec64[0]) {
        d_wrec64[0] = dalloc<double>(4 * recs);
        d_wrec64[1] = dalloc<double>(4 * recs);
    }
    if (k == 1 && !d_wrec32[0]) {
        d_wrec32[0] = dalloc<float>(4 * recs);
        d_wrec32[1] = dalloc<float>(4 * recs);
    }
    if (!d_wface[k]) {
        CK(cudaMalloc(&d_wface[k], face));
        CK(cudaMemset(d_wface[k], 0xFF, face));
        wface_bytes[k] = face;
    }
}

void ocsl_ctx::ensure_cols()
{
    if (v64c) return;
    const size_t n = (size_t)P.n;
    v64c = dalloc<double>(kMaxCols * n);
    for (auto& v : v32c) v = dalloc<float>(kMaxCols * n);
}

namespace {

int fail(ocsl_ctx* c, int status, const std::string& msg)
{
    if (c) c->last_error = msg;
    return status;
}

int from_cuda(ocsl_ctx* c, const CudaError& e)
{
    std::string msg = std::string(e.what) + ": " + cudaGetErrorString(e.code);
    return fail(c, OCSL_CUDA_ERROR, msg);
}

ocsl_opts resolve(const ocsl_opts* o)
{
    ocsl_opts d;
    ocsl_default_opts(&d);
    if (!o) return d;
    ocsl_opts r = *o;
    if (!(r.tol > 0.0)) r.tol = d.tol;
    if (r.maxit <= 0) r.maxit = d.maxit;
    if (r.ilu_sweeps < 0) r.ilu_sweeps = d.ilu_sweeps;
    if (!(r.inner_tol > 0.0)) r.inner_tol = d.inner_tol;
    if (r.inner_maxit <= 0) r.inner_maxit = d.inner_maxit;
    return r;
}

// ------------------------------------------------------------------ helpers

enum ProfCat { PC_SPMV64, PC_SPMV32, PC_FW64, PC_BW64, PC_FW32, PC_BW32, PC_ILU, PC_VEC64, PC_VEC32,
               PC_FILL, PC_COUNT };
const char* kProfNames[PC_COUNT] = {"spmv_f64", "spmv_f32", "fw_sweep_f64", "bw_sweep_f64",
                                    "fw_sweep_f32", "bw_sweep_f32", "ilu_factor", "vector_f64",
                                    "vector_f32", "sweep_fill"};
constexpr size_t kProfMaxPairs = 1 << 18;

// Brackets one launch with events when profiling is on.
struct ProfScope {
    ocsl_ctx* c;
    cudaStream_t st;
    size_t slot = ~size_t(0);
    ProfScope(ocsl_ctx* c_, cudaStream_t st_, int cat) : c(c_), st(st_)
    {
        if (!c->prof_on || c->prof_used >= kProfMaxPairs) return;
        if (2 * c->prof_used + 2 > c->prof_ev.size()) {
            for (int k = 0; k < 2; ++k) {
                cudaEvent_t e;
                CK(cudaEventCreate(&e));
                c->prof_ev.push_back(e);
            }
        }
        slot = c->prof_used++;
        c->prof_cat.push_back(cat);
        CK(cudaEventRecord(c->prof_ev[2 * slot], st));
    }
    ~ProfScope()
    {
        if (slot != ~size_t(0)) cudaEventRecord(c->prof_ev[2 * slot + 1], st);
    }
};

template <typename TT>
constexpr bool is_f64() { return sizeof(TT) == 8; }

// Canonical geometry of the structured sweep: the longest dimension is spanned
// by each CTA (ties to the larger stride), the other two are tiled.
BoxGeom make_box_geom(const BoxShape& bs, int TA_req, int TB_req)
{
    const int E[3] = {bs.dim[0], bs.dim[1], bs.dim[2]};
    const int St[3] = {1, bs.dim[0], bs.dim[0] * bs.dim[1]};
    int span = 2;
    for (int d = 1; d >= 0; --d)
        if (E[d] > E[span]) span = d;
    int rest[2], m = 0;
    for (int d = 0; d < 3; ++d)
        if (d != span) rest[m++] = d;  // ascending stride
    BoxGeom g{};
    g.span = span;
    const int dims[3] = {rest[0], rest[1], span};
    for (int k = 0; k < 3; ++k) {
        g.D[k] = E[dims[k]];
        g.S[k] = St[dims[k]];
    }
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int x, int y) { return g.S[x] > g.S[y]; });
    for (int k = 0; k < 3; ++k) g.order[k] = ord[k];
    // one CTA per tile, TA x TB <= 256 threads (16 x 8 by default)
    int ta_ = TA_req > 0 ? TA_req : (g.D[1] == 1 ? 128 : 16);
    int tb_ = TB_req > 0 ? TB_req : (g.D[1] == 1 ? 1 : 8);
    ta_ = std::max(1, std::min(ta_, 256));
    tb_ = std::max(1, std::min(tb_, 256 / ta_));
    g.TA = std::min(ta_, std::max(1, g.D[0]));
    g.TB = std::min(tb_, std::max(1, g.D[1]));
    g.nta = (g.D[0] + g.TA - 1) / g.TA;
    g.ntb = (g.D[1] + g.TB - 1) / g.TB;
    return box_with_cluster(g, 1, 1);
}

struct Solve {
    ocsl_ctx* c;
    cudaStream_t st;
    const DevPattern& P;
    int n;
    const double* soa64 = nullptr;  // stencil-SoA copy of the current factor
    const float* soa32 = nullptr;
    bool reuse = false;  // the factor of the previous solve on the same values is still valid
    // SpMV through the stencil records of A (box patterns), for the matrix
    // the records were built from
    const double* matA64 = nullptr;
    const double* recA64 = nullptr;
    const float* recA32 = nullptr;
    // Column batching: every spmv / vec / sweep of this solve serves cols.n
    // right-hand sides n elements apart, column q with scalars block k + q;
    // outer_k is the scalars block the refinement-loop vector ops read.
    Cols cols{};
    int outer_k = 0;

    Scalars* sc(int k) const { return c->d_sc + k; }

    // Blocks k .. k + count - 1 from the host: tol2[q] (one value when
    // tol2 has one entry) and the done flag done[q] (none when null).
    void reset_scalars_n(int k, int count, const double* tol2, const int* done_q,
                         double omega0 = 1.0)
    {
        CK(cudaStreamSynchronize(st));  // the staging slots may still be in flight
        for (int q = 0; q < count; ++q) {
            Scalars& s = c->h_sc[kHostStage + k + q];
            std::memset(&s, 0, sizeof s);
            s.tol2 = tol2[q];
            s.alpha = 1.0;
            s.omega = omega0;
            s.rhon = 1.0;
            s.rho = 1.0;
            s.done = done_q ? done_q[q] : 0;
        }
        CK(cudaMemcpyAsync(c->d_sc + k, c->h_sc + kHostStage + k, count * sizeof(Scalars),
                           cudaMemcpyHostToDevice, st));
    }
    void reset_scalars(int k, double tol2, double omega0 = 1.0)
    {
        reset_scalars_n(k, 1, &tol2, nullptr, omega0);
    }
    const Scalars* read_scalars_n(int k, int count)
    {
        CK(cudaMemcpyAsync(c->h_sc + k, c->d_sc + k, count * sizeof(Scalars),
                           cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return c->h_sc + k;
    }
    Scalars read_scalars(int k) { return *read_scalars_n(k, 1); }
    // Set block k's done flag alone.
    void mark_done(int k)
    {
        CK(cudaStreamSynchronize(st));  // the staging slot may still be in flight
        Scalars& stage = c->h_sc[kHostStage + k];
        stage.done = 1;
        CK(cudaMemcpyAsync(&c->d_sc[k].done, &stage.done, sizeof(int), cudaMemcpyHostToDevice,
                           st));
    }
    const int* done(int k) const { return &c->d_sc[k].done; }
    static constexpr int kDoneStride = (int)(sizeof(Scalars) / sizeof(int));

    template <typename TT>
    void spmv(const TT* val, const TT* x, TT* y, int mode, const TT* z, TT* ycopy, const TT* w,
              int dots, int k, int epi, int it = 0, int maxit = 0)
    {
        ProfScope ps(c, st, is_f64<TT>() ? PC_SPMV64 : PC_SPMV32);
        const TT* rec = nullptr;
        if constexpr (sizeof(TT) == 8) {
            if (recA64 && val == matA64) rec = recA64;
        } else {
            if (recA32 && val == c->d_A32) rec = recA32;
        }
        if (rec && c->rb_ok)
            launch_rb_spmv<TT>(st, c->rb, rec, x, y, mode, 0.0, z, ycopy, w, dots, c->R,
                               k >= 0 ? sc(k) : nullptr, epi, it, maxit);
        else if (rec)
            launch_box_spmv<TT>(st, P.n, c->hp.box.dim, rec, x, y, mode, 0.0, z, ycopy, w, dots,
                                c->R, k >= 0 ? sc(k) : nullptr, epi, it, maxit, cols);
        else
            launch_spmv<TT>(st, P, val, x, y, mode, nullptr, 0.0, z, ycopy, w, dots, c->R,
                            k >= 0 ? sc(k) : nullptr, epi, it, maxit, cols);
    }
    // Stencil records of A for the box SpMV (7-point box patterns); built
    // from the FP64 values, so the FP32 records equal (float)A like A32.
    void prepare_spmv(const double* A, bool want64, bool want32)
    {
        matA64 = A;
        recA64 = nullptr;
        recA32 = nullptr;
        if (c->rb_ok && cols.n == 1) {  // red-black records (single right-hand side)
            // the FP32-inner solver's few FP64 residuals read the CSR: building
            // FP64 records for them would cost more than it saves
            if (want32) want64 = false;
            if (want64 && !c->d_recA64) c->d_recA64 = dalloc<double>(8 * (size_t)P.n);
            if (want32 && !c->d_recA32) c->d_recA32 = dalloc<float>(8 * (size_t)P.n);
            const bool have = reuse && c->fac_M;
            ProfScope ps(c, st, PC_ILU);
            if (want64) {
                if (!have) launch_rb_records<double>(st, c->rb, P.rp, c->d_rbslot, A, c->d_recA64);
                recA64 = c->d_recA64;
            }
            if (want32) {
                if (!have) launch_rb_records<float>(st, c->rb, P.rp, c->d_rbslot, A, c->d_recA32);
                recA32 = c->d_recA32;
            }
            return;
        }
        if (!c->hp.box.ok) return;
        if (want64 && !c->d_recA64) c->d_recA64 = dalloc<double>(8 * (size_t)P.n);
        if (want32 && !c->d_recA32) c->d_recA32 = dalloc<float>(8 * (size_t)P.n);
        const bool have = reuse && c->fac_M;  // same values as the previous solve
        ProfScope ps(c, st, PC_ILU);
        if (want64) {
            if (!have) launch_box_to_soa<double>(st, c->hp.box.dim, P.n, P.rp, A, c->d_recA64, 0);
            recA64 = c->d_recA64;
        }
        if (want32) {
            if (!have) launch_box_to_soa<float>(st, c->hp.box.dim, P.n, P.rp, A, c->d_recA32, 0);
            recA32 = c->d_recA32;
        }
    }
    template <typename TT>
    void vec(int op, std::initializer_list<const void*> ptrs, int k, int epi, int it = 0,
             int maxit = 0)
    {
        VecPtrs vp{};
        int i = 0;
        for (const void* p : ptrs) vp.v[i++] = const_cast<void*>(p);
        ProfScope ps(c, st, is_f64<TT>() ? PC_VEC64 : PC_VEC32);
        launch_vec<TT>(st, op, n, vp, c->R, k >= 0 ? sc(k) : nullptr, sc(outer_k), epi, it, maxit,
                       cols);
    }
    // Fixed-point ILU factor (cmatrix_solver.cpp:702-704): M starts as A,
    // `sweeps` Jacobi sweeps; returns the buffer holding the factor.  The
    // last sweep also writes the reciprocal diagonal and the FP32 copies
    // when asked; with zero sweeps the factor is A itself.
    const double* factor(const double* A, int sweeps, bool want_dinv, bool want_fp32, int k)
    {
        const int* dn = k >= 0 ? done(k) : nullptr;
        double* dinv = want_dinv ? c->d_dinv : nullptr;
        float* M32 = want_fp32 ? c->d_M32 : nullptr;
        float* dinv32 = want_fp32 ? c->d_dinv32 : nullptr;
        float* A32 = want_fp32 ? c->d_A32 : nullptr;
        // every factor's diagonal is checked on the device (OCSL_ZERO_PIVOT
        // into the context's error word, read by pivot_status / at the end)
        if (sweeps == 0) {
            ProfScope ps(c, st, PC_ILU);
            launch_factor_outputs(st, P, A, A, dinv, M32, dinv32, A32, c->d_err);
            return A;
        }
        const double* src = A;
        double* bufs[2] = {c->d_Ma, c->d_Mb};
        for (int s = 0; s < sweeps; ++s) {
            double* dst = bufs[s & 1];
            const bool last = s == sweeps - 1;
            ProfScope ps(c, st, PC_ILU);
            launch_ilu_sweep<double>(st, P, A, src, dst, last ? dinv : nullptr,
                                     last ? M32 : nullptr, last ? dinv32 : nullptr,
                                     last ? A32 : nullptr, dn, last ? c->d_err : nullptr);
            src = dst;
        }
        return src;
    }
    // The last tolerance-mode iteration's V_TB_P left tmp and p^ filled with
    // the sweep sentinel (single column only; reset by run_batches).
    bool tb_prefilled = false;
    // prefilled: `out` already holds the sentinel (a fused fill upstream).
    template <typename TT>
    void fw(const TT* M, const TT* rhs, TT* out, int k, bool prefilled = false)
    {
        if (use_serial<TT>() || use_range()) {
            ProfScope ps(c, st, is_f64<TT>() ? PC_FW64 : PC_FW32);
            for (int q = 0; q < cols.n; ++q) {
                const int* dn = k >= 0 ? done(k + q) : nullptr;
                if (!use_serial<TT>())
                    launch_range_sweep<TT>(st, P, true, M, nullptr, rhs + q * cols.ld,
                                           out + q * cols.ld, 0, dn);
                else
                    launch_serial_sweep<TT>(st, P, true, M, nullptr, rhs + q * cols.ld,
                                            out + q * cols.ld, 0, dn);
            }
            return;
        }
        const bool wave = use_box() && soa<TT>() && use_wave<TT>();
        if (!prefilled && !wave) {  // the warp-pipelined sweep keeps its faces apart
            ProfScope ps(c, st, PC_FILL);
            fill_sentinel(out, k);
        }
        ProfScope ps(c, st, is_f64<TT>() ? PC_FW64 : PC_FW32);
        if (wave)
            wave_sweep<TT>(rhs, out, true, 0, k);
        else if (use_box() && soa<TT>())
            launch_box_sweep<TT>(st, sweep_geom<TT>(), P.n, soa<TT>(), rhs, out, true, 0,
                                 c->next_sync(), k >= 0 ? done(k) : nullptr, cols, kDoneStride);
        else
            for (int q = 0; q < cols.n; ++q)  // level-scheduled: one launch per column
                launch_fw_sweep<TT>(st, P, M, rhs + q * cols.ld, out + q * cols.ld,
                                    c->next_sync(), k >= 0 ? done(k + q) : nullptr);
    }
    // out = U^-1 L^-1 rhs through tmp (dead afterwards): one fused pass per
    // colour on a colour-ordered pattern, else the two sweeps
    template <typename TT>
    void precond(const TT* M, const TT* dinv, const TT* rhs, TT* tmp, TT* out, int divmode, int k,
                 bool prefilled)
    {
        if (c->rb_ok && cols.n == 1 && soa<TT>() && use_range()) {
            ProfScope ps(c, st, is_f64<TT>() ? PC_FW64 : PC_FW32);
            launch_rb_precond<TT>(st, c->rb, soa<TT>(), dinv, rhs, out, divmode,
                                  k >= 0 ? done(k) : nullptr);
            return;
        }
        if (P.coloured && use_range() && !use_serial<TT>()) {
            ProfScope ps(c, st, is_f64<TT>() ? PC_FW64 : PC_FW32);
            for (int q = 0; q < cols.n; ++q)
                launch_coloured_precond<TT>(st, P, M, dinv, rhs + q * cols.ld, tmp + q * cols.ld,
                                            out + q * cols.ld, divmode,
                                            k >= 0 ? done(k + q) : nullptr);
            return;
        }
        fw<TT>(M, rhs, tmp, k, prefilled);
        bw<TT>(M, dinv, tmp, out, divmode, k, prefilled);
    }
    // the sweeps write every row without a prefilled output
    template <typename TT>
    bool sweeps_need_fill() const
    {
        return !use_serial<TT>() && !use_range() && !(use_box() && use_wave<TT>());
    }
    // The box geometry, narrowed while a CTA's staging for cols.n columns
    // exceeds the shared-memory limit.
    template <typename TT>
    BoxGeom sweep_geom() const
    {
        BoxGeom g = is_f64<TT>() ? P.box : P.box32;
        if (box_sweep_smem(g, (int)sizeof(TT), cols.n) > kBoxSmemLimit)
            g = box_with_cluster(g, 1, 1);  // face buffers first
        while (box_sweep_smem(g.TA * g.TB, (int)sizeof(TT), cols.n) > kBoxSmemLimit &&
               g.TA * g.TB > 32)
            g = g.TB > 1 ? make_box_geom(c->hp.box, g.TA, (g.TB + 1) / 2)
                         : make_box_geom(c->hp.box, (g.TA + 1) / 2, 1);
        return g;
    }
    bool use_box() const { return P.box_ok && c->sweep_kernel != 1; }
    // one launch per level: few levels, each a contiguous row range (not a
    // box; a pending fault injection exercises the waits of the other kernels)
    bool use_range() const
    {
        return P.fw_nrange > 0 && P.bw_nrange > 0 && !P.box_ok && c->sweep_kernel <= 1 &&
               !c->fault_skip_pending;
    }
    // the one-warp serial sweep (automatic mode, tiny deep patterns; a
    // pending fault injection exercises the waits of the other kernels)
    template <typename TT>
    bool use_serial() const
    {
        return c->sweep_kernel == 0 && c->serial_ok[is_f64<TT>() ? 0 : 1] && !c->fault_skip_pending;
    }
    // the warp-pipelined kernel serves one right-hand side at a time; kind 2
    // forces the CTA kernel, kind 3 the warp-pipelined one
    template <typename TT>
    bool use_wave() const
    {
        const int k = is_f64<TT>() ? 0 : 1;
        if (cols.n != 1 || !wave_possible(k)) return false;
        return c->sweep_kernel == 3 || c->wave_on[k];
    }
    // the step-order records are kept for this precision (the CTA kernel is
    // not forced and the box is not too thin for the warp tiles)
    bool wave_possible(int k) const
    {
        return P.box_ok && c->sweep_kernel != 2 && c->sweep_kernel != 1 && c->wave_fits[k] &&
               (c->sweep_kernel == 3 || c->wave_on[k] || c->wave_tuning);
    }
    template <typename TT>
    const TT* wave_rec(bool forward) const
    {
        if constexpr (sizeof(TT) == 8) return c->d_wrec64[forward ? 0 : 1];
        else return c->d_wrec32[forward ? 0 : 1];
    }
    template <typename TT>
    void wave_sweep(const TT* rhs, TT* out, bool forward, int divmode, int k)
    {
        const int pi = is_f64<TT>() ? 0 : 1;
        if (c->wave_faces_dirty) {  // a launch gave up waiting: faces to all-ones again
            for (int q = 0; q < 2; ++q)
                if (c->d_wface[q]) CK(cudaMemsetAsync(c->d_wface[q], 0xFF, c->wface_bytes[q], st));
            c->wave_faces_dirty = false;
        }
        const WaveGeom& g = c->wave[pi];
        char* faces = static_cast<char*>(c->d_wface[pi]);
        const size_t fa_bytes = (size_t)g.nwa * g.nwb * g.T * g.K * sizeof(TT);
        launch_wave_sweep<TT>(st, g, wave_rec<TT>(forward), rhs, out, faces, faces + fa_bytes,
                              forward, divmode, c->next_sync(), k >= 0 ? done(k) : nullptr);
    }
    // After a factorisation: the structured sweeps read the factor in the
    // stencil-SoA layout (slot 3: diagonal for the reference's division, or
    // its reciprocal for the tolerance-mode multiply).
    void prepare_box(const double* M, bool want64, bool recip64, bool want32)
    {
        soa64 = nullptr;
        soa32 = nullptr;
        if (c->rb_ok && cols.n == 1) {  // red-black records of the factor (its diagonal kept)
            if (want64 && !c->d_soa64) c->d_soa64 = dalloc<double>(8 * (size_t)P.n);
            if (want32 && !c->d_soa32) c->d_soa32 = dalloc<float>(8 * (size_t)P.n);
            ProfScope ps(c, st, PC_ILU);
            if (want64) {
                launch_rb_records<double>(st, c->rb, P.rp, c->d_rbslot, M, c->d_soa64);
                soa64 = c->d_soa64;
            }
            if (want32) {
                launch_rb_records<float>(st, c->rb, P.rp, c->d_rbslot, M, c->d_soa32);
                soa32 = c->d_soa32;
            }
            return;
        }
        if (!use_box()) return;
        if (use_serial<double>()) want64 = false;  // the serial sweep reads the CSR factor
        if (use_serial<float>()) want32 = false;
        ProfScope ps(c, st, PC_ILU);
        if (want64) {
            launch_box_to_soa<double>(st, c->hp.box.dim, P.n, P.rp, M, c->d_soa64, recip64 ? 1 : 0);
            soa64 = c->d_soa64;
            if (wave_possible(0)) {
                c->ensure_wave(0);
                launch_box_to_wave<double>(st, c->hp.box.dim, P.n, P.rp, M, c->wave[0],
                                           c->d_wrec64[0], c->d_wrec64[1], recip64 ? 1 : 0);
            }
        }
        if (want32) {
            launch_box_to_soa<float>(st, c->hp.box.dim, P.n, P.rp, M, c->d_soa32, 1);
            soa32 = c->d_soa32;
            if (wave_possible(1)) {
                c->ensure_wave(1);
                launch_box_to_wave<float>(st, c->hp.box.dim, P.n, P.rp, M, c->wave[1],
                                          c->d_wrec32[0], c->d_wrec32[1], 1);
            }
        }
    }
    // factor() + prepare_box(), or the previous solve's factor when reusing
    const double* factored(const double* A, int sweeps, bool want_dinv, bool want_fp32, int k,
                           bool want64, bool recip64, bool want32)
    {
        if (reuse && c->fac_M) {
            soa64 = c->fac_soa64;
            soa32 = c->fac_soa32;
            return c->fac_M;
        }
        const double* M = factor(A, sweeps, want_dinv, want_fp32, k);
        prepare_box(M, want64, recip64, want32);
        c->fac_checked = false;
        c->fac_M = M;
        c->fac_soa64 = soa64;
        c->fac_soa32 = soa32;
        return M;
    }
    template <typename TT>
    const TT* soa() const
    {
        if constexpr (sizeof(TT) == 8) return soa64;
        else return soa32;
    }
    // A sweep output is filled exactly when the sweep that follows runs, so a
    // finished column keeps its last vectors (the half step reads them): the
    // column-batched box sweep runs all columns (a finished column's inputs
    // no longer change, so it recomputes the same values) until every column
    // is done; the level-scheduled sweep runs per column.
    template <typename TT>
    void fill_sentinel(TT* out, int k)
    {
        const size_t bytes = sizeof(TT) * (size_t)P.n;
        if (cols.n == 1 || (use_box() && soa<TT>())) {
            launch_fill_ones(st, out, bytes * cols.n, k >= 0 ? done(k) : nullptr, cols.n,
                             kDoneStride);
        } else {
            for (int q = 0; q < cols.n; ++q)
                launch_fill_ones(st, out + q * cols.ld, bytes, k >= 0 ? done(k + q) : nullptr);
        }
    }
    template <typename TT>
    void bw(const TT* M, const TT* dinv, const TT* rhs, TT* out, int divmode, int k,
            bool prefilled = false)
    {
        if (use_serial<TT>() || use_range()) {
            ProfScope ps(c, st, is_f64<TT>() ? PC_BW64 : PC_BW32);
            for (int q = 0; q < cols.n; ++q) {
                const int* dn = k >= 0 ? done(k + q) : nullptr;
                if (!use_serial<TT>())
                    launch_range_sweep<TT>(st, P, false, M, dinv, rhs + q * cols.ld,
                                           out + q * cols.ld, divmode, dn);
                else
                    launch_serial_sweep<TT>(st, P, false, M, dinv, rhs + q * cols.ld,
                                            out + q * cols.ld, divmode, dn);
            }
            return;
        }
        const bool wave = use_box() && soa<TT>() && use_wave<TT>();
        if (!prefilled && !wave) {
            ProfScope ps(c, st, PC_FILL);
            fill_sentinel(out, k);
        }
        ProfScope ps(c, st, is_f64<TT>() ? PC_BW64 : PC_BW32);
        if (wave)
            wave_sweep<TT>(rhs, out, false, divmode, k);
        else if (use_box() && soa<TT>())
            launch_box_sweep<TT>(st, sweep_geom<TT>(), P.n, soa<TT>(), rhs, out, false, divmode,
                                 c->next_sync(), k >= 0 ? done(k) : nullptr, cols, kDoneStride);
        else
            for (int q = 0; q < cols.n; ++q)
                launch_bw_sweep<TT>(st, P, M, dinv, rhs + q * cols.ld, out + q * cols.ld, divmode,
                                    c->next_sync(), k >= 0 ? done(k + q) : nullptr);
    }
    // Enqueue `fn` (a fixed sequence of launches) through a CUDA graph keyed by
    // (kind, ptrs): captured on first use, replayed afterwards.  Returns false
    // (nothing enqueued) when graphs are off (profiling, legacy default
    // stream) or the capture failed; the caller then launches directly.
    template <typename Fn>
    bool graph_launch(int kind, std::initializer_list<const void*> ptrs, Fn&& fn)
    {
        if (!c->graphs_on || c->prof_on || c->fault_skip_pending || st == nullptr ||
            st == cudaStreamLegacy || st == cudaStreamPerThread)
            return false;
        const void* key[6] = {};
        int i = 0;
        for (const void* q : ptrs)
            if (i < 6) key[i++] = q;
        bool hit = c->graph_exec && c->graph_kind == kind;
        for (int j = 0; hit && j < 6; ++j) hit = c->graph_ptr[j] == key[j];
        if (!hit) {
            if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
            c->graph_exec = nullptr;
            if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            cudaGraph_t g = nullptr;
            try {
                fn();
            } catch (...) {
                cudaStreamEndCapture(st, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            cudaError_t e = cudaStreamEndCapture(st, &g);
            cudaGraphExec_t exec = nullptr;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            c->graph_exec = exec;
            c->graph_kind = kind;
            for (int j = 0; j < 6; ++j) c->graph_ptr[j] = key[j];
        }
        CK(cudaGraphLaunch(c->graph_exec, st));
        return true;
    }
    // OCSL_ZERO_PIVOT when the current factor has a zero or infinite
    // diagonal (synchronises once per factor; a reused factor keeps its verdict)
    int pivot_status()
    {
        if (!c->fac_checked) {
            c->fac_status = device_error() == OCSL_ZERO_PIVOT ? OCSL_ZERO_PIVOT : OCSL_OK;
            c->fac_checked = true;
        }
        return c->fac_status;
    }
    int device_error()
    {
        CK(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (*c->h_err == OCSL_TIMEOUT) c->wave_faces_dirty = true;
        return *c->h_err;
    }
};

// ------------------------------------------------------------------ reference-faithful

// CMatrix_solver::CG_solve (cmatrix_solver.cpp:635-680).
// Block 0 as a reference-faithful solve starts it: from the host (a
// synchronising upload) or, for a captured graph, from the context's device
// copy of that start state.
void reset_ref_scalars(Solve& s, bool from_device)
{
    if (from_device)
        CK(cudaMemcpyAsync(s.sc(0), s.c->d_sc_ref, sizeof(Scalars), cudaMemcpyDeviceToDevice, s.st));
    else
        s.reset_scalars(0, 0.0);
}

void run_cg_ref(Solve& s, const double* A, const double* b, double* x, bool device_reset = false)
{
    double** v = s.c->v64;
    reset_ref_scalars(s, device_reset);
    s.prepare_spmv(A, true, false);
    // r = b - A x (:652), p = r (:655), rr = <r,r>
    s.spmv<double>(A, x, v[R], 1, b, v[P], nullptr, DOT_YY, 0, EP_RC_INIT);
    double* r = v[R];
    double* rn = v[RN];
    for (int it = 0; it < kRefCgIters; ++it) {
        // q = A p (:659), a = rr / (<p,q> + 1e-40) (:660)
        s.spmv<double>(A, v[P], v[Q], 0, nullptr, nullptr, v[P], DOT_WY, 0, EP_RC_ALPHA);
        // x += a p (:662-663); r_next = r - a A p (:665); res = <r_next, r_next> (:667)
        s.vec<double>(V_RC_XR, {x, v[P], rn, v[Q], r}, 0, EP_RC_RES, it, kRefCgIters);
        // p = r_next + beta p (:674)
        s.vec<double>(V_RC_P, {v[P], rn}, 0, EP_STORE);
        std::swap(r, rn);  // :676
    }
}

// CMatrix_solver::ILU_BICGSTAB_solve (cmatrix_solver.cpp:682-762), quirks kept:
// omega in the direction update, rho never updated, the residual test on the
// r from the start of the iteration, x not updated on that exit.
void run_bicgstab_ref(Solve& s, const double* A, const double* b, double* x, int sweeps,
                      bool device_reset = false)
{
    double** v = s.c->v64;
    const size_t bytes = sizeof(double) * (size_t)s.n;
    reset_ref_scalars(s, device_reset);
    CK(cudaMemsetAsync(v[P], 0, bytes, s.st));  // Cvector(n) starts at 0 (:690-700)
    CK(cudaMemsetAsync(v[V], 0, bytes, s.st));
    const double* M = s.factored(A, sweeps, false, false, 0, true, false, false);  // :702-704
    s.prepare_spmv(A, true, false);
    // r = b - A x (:708), r0 = r (:710), iteration 0's rhon and res
    s.spmv<double>(A, x, v[R], 1, b, v[R0], nullptr, DOT_YY | DOT_ZZ, 0, EP_RB_INIT);
    for (int it = 0; it < kRefBicgIters; ++it) {
        s.vec<double>(V_RB_P, {v[P], v[V], v[R]}, 0, EP_STORE);                 // :718-720
        s.fw<double>(M, v[P], v[DUM], 0);                                       // :722
        s.bw<double>(M, nullptr, v[DUM], v[Y], 0, 0);                           // :723
        s.spmv<double>(A, v[Y], v[V], 0, nullptr, nullptr, v[R0], DOT_WY, 0, EP_RB_ALPHA);  // :725-728
        s.vec<double>(V_RB_HS, {v[H], x, v[Y], v[S], v[V], v[R]}, 0, EP_STORE);  // :731, :738
        s.fw<double>(M, v[S], v[DUM2], 0);                                      // :741 (= :747)
        s.bw<double>(M, nullptr, v[DUM2], v[Z], 0, 0);                          // :742
        s.spmv<double>(A, v[Z], v[T], 0, nullptr, nullptr, nullptr, 0, 0, EP_STORE);  // :744
        s.fw<double>(M, v[T], v[DUM], 0);                                       // :746
        s.vec<double>(V_DOT2, {v[DUM], v[DUM2]}, 0, EP_RB_OMEGA);              // :750
        s.vec<double>(V_RB_XR, {x, v[Z], v[H], v[R], v[T], v[S], v[R0]}, 0, EP_RB_RUPD, it,
                      kRefBicgIters);                                            // :753, :756
    }
}

// ------------------------------------------------------------------ tolerance mode

struct TolResult {
    int iters = 0;
    int outer = 0;
    double relres = 0.0;
    int status = OCSL_OK;
};

// A factor with a zero or infinite pivot: no iteration runs, x is unchanged.
TolResult zero_pivot_result()
{
    TolResult r;
    r.relres = NAN;
    r.status = OCSL_ZERO_PIVOT;
    return r;
}

constexpr int kBatch = 2;  // iterations enqueued between looks at the scalars

// Run enqueue(it) for at most `budget` iterations, in batches of kBatch, until
// scalars block k reports done.  Two batches are kept in flight: while the GPU
// runs one, the host inspects the scalars copied after the previous one.
// Batches enqueued after convergence cost only no-op launches.
// A full batch after the first is replayed from a CUDA graph when graph_kind
// is non-zero (the iteration's launches do not depend on `it`).
template <typename F>
Scalars run_batches(Solve& s, int k, int budget, F&& enqueue, int graph_kind = 0,
                    std::initializer_list<const void*> graph_ptrs = {})
{
    Scalars* slot = s.c->h_sc + kHostInspect;  // two pinned inspection slots of kMaxCols blocks
    const int nc = s.cols.n;
    int it = 0, issued = 0, inspected = 0;
    s.tb_prefilled = false;  // the first iteration fills its sweep outputs itself
    while (true) {
        while (issued - inspected < 2 && it < budget) {
            const int m = std::min(kBatch, budget - it);
            const bool graphed =
                graph_kind && m == kBatch && issued > 0 &&
                s.graph_launch(graph_kind, graph_ptrs, [&] {
                    for (int j = 0; j < m; ++j) enqueue(it + j);
                });
            if (!graphed)
                for (int j = 0; j < m; ++j) enqueue(it + j);
            it += m;
            CK(cudaMemcpyAsync(slot + (issued & 1) * kMaxCols, s.c->d_sc + k, nc * sizeof(Scalars),
                               cudaMemcpyDeviceToHost, s.st));
            CK(cudaEventRecord(s.c->ev_batch[issued & 1], s.st));
            ++issued;
        }
        if (inspected == issued) break;
        CK(cudaEventSynchronize(s.c->ev_batch[inspected & 1]));
        bool done = true;
        for (int q = 0; q < nc; ++q) done = done && slot[(inspected & 1) * kMaxCols + q].done != 0;
        ++inspected;
        if (done) break;
    }
    return s.read_scalars(k);
}

// Preconditioned BiCGSTAB (van der Vorst 1992) on the reference's ILU factor.
template <typename TT>
void bicgstab_iteration(Solve& s, const TT* A, const TT* M, const TT* dinv, TT* x, TT* r, TT* rh,
                        TT* p, TT* ph, TT* vv, TT* ss, TT* sh, TT* t, TT* tmp, int k)
{
    // single column: the vector kernels before each sweep pair fill the
    // pair's outputs (tmp is dead after each backward sweep, s^ after the x
    // update, p^ after the p update), so no fill launches inside the loop
    const bool fuse = s.cols.n == 1 && s.template sweeps_need_fill<TT>();
    const bool pre = fuse && s.tb_prefilled;
    TT* f0 = fuse ? tmp : nullptr;
    s.precond<TT>(M, dinv, p, tmp, ph, 1, k, pre);
    s.spmv<TT>(A, ph, vv, 0, nullptr, nullptr, rh, DOT_WY, k, EP_TB_SIGMA);
    s.vec<TT>(V_TB_S, {ss, vv, r, nullptr, nullptr, nullptr, f0, fuse ? sh : nullptr}, k,
              EP_TB_S);
    s.precond<TT>(M, dinv, ss, tmp, sh, 1, k, fuse);
    s.spmv<TT>(A, sh, t, 0, nullptr, nullptr, ss, DOT_YY | DOT_WY, k, EP_TB_OMEGA);
    s.vec<TT>(V_TB_XR, {x, ph, sh, r, t, ss, rh}, k, EP_TB_RUPD);
    s.vec<TT>(V_TB_P, {p, vv, r, nullptr, nullptr, nullptr, f0, fuse ? ph : nullptr}, k,
              EP_STORE);
    s.tb_prefilled = fuse;
}

// Restarted driver shared by BiCGSTAB and PCG: start from x, iterate until
// the recursive residual meets tol, confirm with a true FP64 residual, restart
// from the current x when they disagree or on breakdown.
template <typename Init, typename Iter, typename Half>
TolResult run_restarted(Solve& s, const double* A, const double* b, double* x, const ocsl_opts& o,
                        Init&& init, Iter&& iteration, Half&& half, int graph_kind,
                        std::initializer_list<const void*> graph_ptrs)
{
    double** v = s.c->v64;
    TolResult res;
    const double tol2 = o.tol * o.tol;
    int total = 0;
    bool converged = false;
    bool broke = false;
    for (int restart = 0; restart < 64 && !converged; ++restart) {
        s.reset_scalars(0, tol2);
        s.spmv<double>(A, x, v[R], 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, 0, EP_TB_INIT);
        init();
        Scalars st = s.read_scalars(0);
        res.relres = st.res;
        if (st.status) { res.status = st.status; break; }
        if (st.bb == 0.0) {  // b = 0: x = 0 is exact
            CK(cudaMemsetAsync(x, 0, sizeof(double) * (size_t)s.n, s.st));
            res.relres = 0.0;
            converged = true;
            break;
        }
        if (st.done) { converged = true; break; }
        if (total >= o.maxit) break;
        st = run_batches(s, 0, o.maxit - total, iteration, graph_kind, graph_ptrs);
        total += st.iters;
        broke = st.breakdown != 0;
        if (st.status) { res.status = st.status; break; }
        half();
        s.reset_scalars(2, tol2);
        s.spmv<double>(A, x, v[R], 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, 2, EP_TRUE_RES);
        const Scalars tr = s.read_scalars(2);
        res.relres = tr.res;
        if (!std::isfinite(tr.res)) { res.status = OCSL_NONFINITE; break; }
        converged = tr.rr <= tol2 * tr.bb;
        if (broke && st.iters == 0) break;  // breakdown before any progress
    }
    if (!converged && res.status == OCSL_OK) res.status = broke ? OCSL_BREAKDOWN : OCSL_NOT_CONVERGED;
    res.iters = total;
    return res;
}

TolResult run_bicgstab_tol(Solve& s, const double* A, const double* b, double* x,
                           const ocsl_opts& o)
{
    double** v = s.c->v64;
    const double* M = s.factored(A, o.ilu_sweeps, true, false, -1, true, true, false);
    if (s.pivot_status() != OCSL_OK) return zero_pivot_result();
    s.prepare_spmv(A, true, false);
    return run_restarted(
        s, A, b, x, o, [&] { s.vec<double>(V_COPY2, {v[RH], v[P], v[R]}, 0, EP_STORE); },
        [&](int) {
            bicgstab_iteration<double>(s, A, M, s.c->d_dinv, x, v[R], v[RH], v[P], v[PH], v[V],
                                       v[S], v[SH], v[T], v[TMP], 0);
        },
        [&] { s.vec<double>(V_TB_HALF, {x, v[PH]}, 0, EP_STORE); }, 1,
        {A, M, x, s.soa64, s.recA64, s.c->d_dinv});
}

TolResult run_pcg_tol(Solve& s, const double* A, const double* b, double* x, const ocsl_opts& o)
{
    double** v = s.c->v64;
    s.factored(A, 0, true, false, -1, false, false, false);  // Jacobi: dinv = 1 / A_ii
    if (s.pivot_status() != OCSL_OK) return zero_pivot_result();
    s.prepare_spmv(A, true, false);
    return run_restarted(
        s, A, b, x, o,
        [&] { s.vec<double>(V_PC_INIT, {v[Z], v[P], v[R], s.c->d_dinv}, 0, EP_PC_INIT); },
        [&](int) {
            s.spmv<double>(A, v[P], v[Q], 0, nullptr, nullptr, v[P], DOT_WY, 0, EP_PC_ALPHA);
            s.vec<double>(V_PC_XRZ, {x, v[P], v[R], v[Q], v[Z], s.c->d_dinv}, 0, EP_PC_RUPD);
            s.vec<double>(V_PC_P, {v[P], v[Z]}, 0, EP_STORE);
        },
        [] {}, 2, {A, x, s.recA64, s.c->d_dinv});
}

// FP32 inner ILU-BiCGSTAB (FP32 matrix, factor and vectors; compensated-FP32
// reductions folded to FP64; FP64 alpha / beta / omega) inside FP64
// iterative refinement: r = b - A x, x += ||r|| d in FP64.
TolResult run_bicgstab_ir32(Solve& s, const double* A, const double* b, double* x,
                            const ocsl_opts& o)
{
    ocsl_ctx* c = s.c;
    c->ensure_fp32();
    double** v = c->v64;
    float** f = c->v32;
    TolResult res;
    const double tol2 = o.tol * o.tol;
    const double* M = s.factored(A, o.ilu_sweeps, true, true, -1, false, true, true);
    if (s.pivot_status() != OCSL_OK) return zero_pivot_result();
    s.prepare_spmv(A, true, true);
    int total = 0;
    s.reset_scalars(0, tol2);
    for (int outer = 0;; ++outer) {
        // FP64 residual; EP_TB_INIT also stores ||r|| and 1/||r||
        s.spmv<double>(A, x, v[R], 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, 0, EP_TB_INIT);
        const Scalars so = s.read_scalars(0);
        res.relres = so.res;
        res.outer = outer;
        if (so.status) { res.status = so.status; break; }
        if (so.bb == 0.0) {
            CK(cudaMemsetAsync(x, 0, sizeof(double) * (size_t)s.n, s.st));
            res.relres = 0.0;
            break;
        }
        if (so.done) break;
        if (total >= o.maxit || outer >= 1000) { res.status = OCSL_NOT_CONVERGED; break; }
        // inner solve of A d = r / ||r|| in FP32 from d = 0, to the reduction
        // still missing (with a margin of 2), at most inner_tol
        const double itol = std::max(o.inner_tol, 0.5 * o.tol / so.res);
        s.reset_scalars(1, itol * itol);
        s.vec<float>(V_IR_SCALE, {v[R], f[F_RI], f[F_RH], f[F_P], f[F_D]}, 1, EP_IR_INNER_INIT);
        const int budget = std::min(o.inner_maxit, o.maxit - total);
        const Scalars si = run_batches(
            s, 1, budget,
            [&](int) {
                bicgstab_iteration<float>(s, c->d_A32, c->d_M32, c->d_dinv32, f[F_D], f[F_RI],
                                          f[F_RH], f[F_P], f[F_PH], f[F_V], f[F_S], f[F_SH],
                                          f[F_T], f[F_TMP], 1);
            },
            3, {c->d_A32, c->d_M32, s.soa32, s.recA32, c->d_dinv32});
        total += si.iters;
        s.vec<float>(V_TB_HALF, {f[F_D], f[F_PH]}, 1, EP_STORE);
        s.vec<float>(V_IR_UPDATE, {x, f[F_D]}, -1, EP_STORE);
        if (si.status == OCSL_NONFINITE) { res.status = OCSL_NONFINITE; break; }
        if (si.iters == 0 && !si.done) { res.status = OCSL_BREAKDOWN; break; }
        // the next residual reuses block 0: clear its done flag, keep tol2
        s.reset_scalars(0, tol2);
    }
    res.iters = total;
    return res;
}

// ---- The refinement loop on the device ------------------------------------
//
// run_bicgstab_ir32 with its control flow on the device: the outer
// refinement loop and the inner FP32 BiCGSTAB loop become conditional WHILE
// graph nodes, and the decisions the host takes between them (the checks on
// the FP64 residual, the next inner tolerance max(inner_tol, 0.5 tol /
// relres), the inner budget, the scalar resets, the status checks after an
// inner solve) are single-thread control kernels.  The kernels of the
// arithmetic are the same launches in the same order, so the solve is
// bit-identical to the host-driven one (no-op launches aside: an inner
// iteration after convergence returns at once in both).  One graph launch
// runs the whole solve with no host round trip.
//
// Every loop ends: each body's control kernel first sets its loop's
// condition to 0 and sets it to 1 only to continue, which needs a device
// iteration counter below its bound (inner: the budget <= inner_maxit;
// outer: 1000 steps or maxit iterations).
struct IrCtl {
    int outer, total, inner_it, budget, status, stop, zero_x, pad;
    double relres;
};

__device__ void ir_reset_block(Scalars* s, double tol2)  // the values reset_scalars stages
{
    *s = Scalars{};
    s->tol2 = tol2;
    s->alpha = 1.0;
    s->omega = 1.0;
    s->rhon = 1.0;
    s->rho = 1.0;
}

// Start of a solve; a zero or infinite pivot of the factor (flagged in *err
// by the factor kernels) runs no iteration and leaves x unchanged.
__global__ void ir_begin_kernel(Scalars* s0, double tol2, IrCtl* ctl, const int* err,
                                cudaGraphConditionalHandle h_outer)
{
    ir_reset_block(s0, tol2);
    *ctl = IrCtl{};
    if (*err == OCSL_ZERO_PIVOT) {
        ctl->status = OCSL_ZERO_PIVOT;
        ctl->relres = __longlong_as_double(0x7FF8000000000000LL);
        ctl->stop = 1;
        cudaGraphSetConditional(h_outer, 0u);
    }
}

// The iteration count and status of a solve inside the SIMPLE iteration's
// graph, into the iteration's output block; *err (a sweep wait that gave up,
// a zero pivot) takes precedence, as in a direct solve, and is cleared.
__global__ void ir_flow_out_kernel(const IrCtl* ctl, int* err, int* iters_out, int* err_out)
{
    *iters_out = ctl->total;
    *err_out = *err ? *err : ctl->status;
    *err = 0;
}

// After a refinement step's FP64 residual (EP_TB_INIT in block 0): the checks
// at the top of run_bicgstab_ir32's loop, then the inner solve's set-up.  A
// stop leaves blocks 0 and 1 done, so the rest of the pass is no-ops.
__global__ void ir_step_kernel(Scalars* s0, Scalars* s1, IrCtl* ctl,
                               cudaGraphConditionalHandle h_outer,
                               cudaGraphConditionalHandle h_inner, double tol, double inner_tol,
                               int maxit, int inner_maxit)
{
    cudaGraphSetConditional(h_outer, 0u);
    cudaGraphSetConditional(h_inner, 0u);
    bool stop = true;
    ctl->relres = s0->res;
    if (s0->status) {
        ctl->status = s0->status;
    } else if (s0->bb == 0.0) {
        ctl->zero_x = 1;
        ctl->relres = 0.0;
    } else if (s0->done) {
    } else if (ctl->total >= maxit || ctl->outer >= 1000) {
        ctl->status = OCSL_NOT_CONVERGED;
    } else {
        stop = false;
    }
    if (stop) {
        ctl->stop = 1;
        s0->done = 1;
        s1->done = 1;
        s1->half = 0;
        return;
    }
    const double q = 0.5 * tol / s0->res;
    const double itol = inner_tol < q ? q : inner_tol;  // std::max(inner_tol, q)
    ir_reset_block(s1, itol * itol);
    ctl->inner_it = 0;
    ctl->budget = min(inner_maxit, maxit - ctl->total);
    if (ctl->budget > 0) cudaGraphSetConditional(h_inner, 1u);
}

__global__ void ir_zero_x_kernel(double* x, int n, const IrCtl* ctl)
{
    if (!ctl->zero_x) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = 0.0;
}

// End of one inner iteration: continue while not converged and within budget.
__global__ void ir_inner_kernel(const Scalars* s1, IrCtl* ctl, cudaGraphConditionalHandle h_inner)
{
    cudaGraphSetConditional(h_inner, 0u);
    const int it = ctl->inner_it + 1;
    ctl->inner_it = it;
    if (!s1->done && it < ctl->budget) cudaGraphSetConditional(h_inner, 1u);
}

// After the inner solve and the update of x: the status checks at the end of
// run_bicgstab_ir32's loop, block 0 reset for the next residual.
__global__ void ir_post_kernel(Scalars* s0, const Scalars* s1, IrCtl* ctl,
                               cudaGraphConditionalHandle h_outer, double tol2)
{
    cudaGraphSetConditional(h_outer, 0u);
    if (ctl->stop) return;
    ctl->total += s1->iters;
    if (s1->status == OCSL_NONFINITE) {
        ctl->status = OCSL_NONFINITE;
        ctl->stop = 1;
        return;
    }
    if (s1->iters == 0 && !s1->done) {
        ctl->status = OCSL_BREAKDOWN;
        ctl->stop = 1;
        return;
    }
    ir_reset_block(s0, tol2);
    ctl->outer += 1;
    cudaGraphSetConditional(h_outer, 1u);
}

// A WHILE node after the work captured so far on `st`; returns its body graph
// (and the node in *node_out).
cudaGraph_t add_while_node(cudaStream_t st, cudaGraphConditionalHandle h,
                           cudaGraphNode_t* node_out = nullptr)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &nd));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, edges, nd, &p));
    CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                           cudaStreamSetCaptureDependencies));
    if (node_out) *node_out = node;
    return p.conditional.phGraph_out[0];
}

// Whether run_bicgstab_ir32 can run with its loops on the device: one column,
// a stream that can be captured, no profiling or pending fault injection.
bool device_loop_ok(const Solve& s)
{
    const ocsl_ctx* c = s.c;
    return c->device_loop && s.cols.n == 1 && !c->prof_on && !c->fault_skip_pending &&
           s.st != nullptr && s.st != cudaStreamLegacy && s.st != cudaStreamPerThread;
}

// The two loop bodies of a captured FP32-refined solve: the refinement step
// into `outer` (the body of the WHILE node of h_outer) with a nested WHILE
// node for the inner loop, captured on sb.st.
void capture_ir32_bodies(Solve& sb, cudaGraph_t outer, cudaGraphConditionalHandle h_outer,
                         const double* A, const double* b, double* x, const ocsl_opts& o,
                         IrCtl* ctl)
{
    ocsl_ctx* c = sb.c;
    double** v = c->v64;
    float** f = c->v32;
    const double tol2 = o.tol * o.tol;
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaGraph_t inner = nullptr;
    cudaGraphConditionalHandle h_inner;
    CK(cudaGraphConditionalHandleCreate(&h_inner, outer, 0u, 0u));
    CK(cudaStreamBeginCaptureToGraph(sb.st, outer, nullptr, nullptr, 0, mode));
    sb.spmv<double>(A, x, v[R], 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, 0, EP_TB_INIT);
    ir_step_kernel<<<1, 1, 0, sb.st>>>(c->d_sc, c->d_sc + 1, ctl, h_outer, h_inner, o.tol,
                                       o.inner_tol, o.maxit, o.inner_maxit);
    ir_zero_x_kernel<<<std::max(1, std::min((sb.n + 255) / 256, 1024)), 256, 0, sb.st>>>(
        x, sb.n, ctl);
    sb.vec<float>(V_IR_SCALE, {v[R], f[F_RI], f[F_RH], f[F_P], f[F_D]}, 1, EP_IR_INNER_INIT);
    inner = add_while_node(sb.st, h_inner);
    sb.vec<float>(V_TB_HALF, {f[F_D], f[F_PH]}, 1, EP_STORE);
    sb.vec<float>(V_IR_UPDATE, {x, f[F_D]}, -1, EP_STORE);
    ir_post_kernel<<<1, 1, 0, sb.st>>>(c->d_sc, c->d_sc + 1, ctl, h_outer, tol2);
    CK(cudaStreamEndCapture(sb.st, &outer));

    CK(cudaStreamBeginCaptureToGraph(sb.st, inner, nullptr, nullptr, 0, mode));
    // every pass fills its sweep outputs itself (the host loop skips the
    // fills after the first iteration: same bits either way)
    sb.tb_prefilled = false;
    bicgstab_iteration<float>(sb, c->d_A32, c->d_M32, c->d_dinv32, f[F_D], f[F_RI], f[F_RH],
                              f[F_P], f[F_PH], f[F_V], f[F_S], f[F_SH], f[F_T], f[F_TMP], 1);
    sb.tb_prefilled = false;
    ir_inner_kernel<<<1, 1, 0, sb.st>>>(c->d_sc + 1, ctl, h_inner);
    CK(cudaStreamEndCapture(sb.st, &inner));
}

void end_any_capture(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
    }
    cudaGetLastError();
}

// Captures one FP32-refined solve of A x = b from the current x into `root`
// (the factor, the FP32 copies and the stencil records already prepared),
// after node *last (none: at the root); *last becomes the solve's last node.
// Its result goes to control block `ctl`.
void capture_ir32(Solve& s, cudaGraph_t root, cudaGraphNode_t* last, const double* A,
                  const double* b, double* x, const ocsl_opts& o, IrCtl* ctl)
{
    ocsl_ctx* c = s.c;
    const double tol2 = o.tol * o.tol;
    try {
        cudaGraphConditionalHandle h_outer;
        CK(cudaGraphConditionalHandleCreate(&h_outer, root, 1u, cudaGraphCondAssignDefault));
        const bool after = last && *last;
        CK(cudaStreamBeginCaptureToGraph(s.st, root, after ? last : nullptr, nullptr,
                                         after ? 1 : 0, cudaStreamCaptureModeThreadLocal));
        ir_begin_kernel<<<1, 1, 0, s.st>>>(c->d_sc, tol2, ctl, c->d_err, h_outer);
        cudaGraphNode_t loop = nullptr;
        cudaGraph_t outer = add_while_node(s.st, h_outer, &loop);
        cudaGraph_t got = nullptr;
        CK(cudaStreamEndCapture(s.st, &got));
        if (last) *last = loop;
        capture_ir32_bodies(s, outer, h_outer, A, b, x, o, ctl);
    } catch (...) {
        end_any_capture(s.st);
        throw;
    }
}

// The same solve inserted into the capture in progress on s.st (the factor
// and records captured before it); its loop bodies are captured on `scratch`.
void capture_ir32_inline(Solve& s, cudaStream_t scratch, const double* A, const double* b,
                         double* x, const ocsl_opts& o, IrCtl* ctl)
{
    ocsl_ctx* c = s.c;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    CK(cudaStreamGetCaptureInfo(s.st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    cudaGraphConditionalHandle h_outer;
    CK(cudaGraphConditionalHandleCreate(&h_outer, g, 1u, cudaGraphCondAssignDefault));
    ir_begin_kernel<<<1, 1, 0, s.st>>>(c->d_sc, o.tol * o.tol, ctl, c->d_err, h_outer);
    cudaGraph_t outer = add_while_node(s.st, h_outer);
    Solve sb = s;
    sb.st = scratch;
    try {
        capture_ir32_bodies(sb, outer, h_outer, A, b, x, o, ctl);
    } catch (...) {
        end_any_capture(scratch);
        throw;
    }
}

// At least `count` control blocks on the context.
void ensure_irctl(ocsl_ctx* c, int count)
{
    if (c->n_irctl >= count) return;
    c->drop_graph();  // captured solves and iterations may point at the old blocks
    if (c->d_irctl) CK(cudaFree(c->d_irctl));
    c->d_irctl = nullptr;
    c->n_irctl = 0;
    CK(cudaMalloc(&c->d_irctl, sizeof(IrCtl) * (size_t)count));
    c->n_irctl = count;
}

// The result of a device-driven solve, from control block `slot` (synchronises).
TolResult read_ir_ctl(Solve& s, int slot = 0)
{
    IrCtl h;
    CK(cudaMemcpyAsync(&h, static_cast<IrCtl*>(s.c->d_irctl) + slot, sizeof h,
                       cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    TolResult r;
    r.iters = h.total;
    r.outer = h.outer;
    r.relres = h.relres;
    r.status = h.status;
    return r;
}

TolResult run_bicgstab_ir32_device(Solve& s, const double* A, const double* b, double* x,
                                   const ocsl_opts& o)
{
    ocsl_ctx* c = s.c;
    c->ensure_fp32();
    const double* M = s.factored(A, o.ilu_sweeps, true, true, -1, false, true, true);
    (void)M;
    if (s.pivot_status() != OCSL_OK) return zero_pivot_result();
    s.prepare_spmv(A, true, true);
    ensure_irctl(c, 1);
    // the graph reads these pointers and settings; it is replayed while they hold
    std::vector<unsigned char> key;
    auto add = [&](const void* p, size_t bytes) {
        const unsigned char* q = static_cast<const unsigned char*>(p);
        key.insert(key.end(), q, q + bytes);
    };
    const int kind = 3;  // the FP32-refined solve (the restarted drivers use 1, 2)
    add(&kind, sizeof kind);
    const void* ptrs[7] = {A, b, x, s.st, s.soa32, s.recA32, c->d_irctl};
    add(ptrs, sizeof ptrs);
    add(&o.tol, sizeof o.tol);
    add(&o.maxit, sizeof o.maxit);
    add(&o.inner_tol, sizeof o.inner_tol);
    add(&o.inner_maxit, sizeof o.inner_maxit);
    if (!c->ir_exec || key != c->ir_key) {
        if (c->ir_exec) cudaGraphExecDestroy(c->ir_exec);
        c->ir_exec = nullptr;
        c->ir_key.clear();
        cudaGraph_t g = nullptr;
        CK(cudaGraphCreate(&g, 0));
        try {
            capture_ir32(s, g, nullptr, A, b, x, o, static_cast<IrCtl*>(c->d_irctl));
        } catch (...) {
            cudaGraphDestroy(g);
            throw;
        }
        cudaGraphExec_t e = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&e, g, 0);
        cudaGraphDestroy(g);
        CK(ie);
        c->ir_exec = e;
        c->ir_key = key;
    }
    CK(cudaGraphLaunch(c->ir_exec, s.st));
    return read_ir_ctl(s);
}

// ---- The restarted FP64 drivers' loop on the device -------------------------
//
// run_restarted (plain FP64 ILU-BiCGSTAB and Jacobi PCG) with its control
// flow on the device, as run_bicgstab_ir32_device does for the refinement
// loop: the restart loop (at most 64 passes) and the Krylov loop (at most the
// remaining maxit iterations) as conditional WHILE nodes, the host's checks
// as single-thread control kernels over a control block (the IrCtl fields:
// outer = restarts, total, inner_it / budget of the Krylov loop, status,
// relres; pad = breakdown seen).  Same launches in the same order.
struct RsCtl {
    IrCtl k;
    int converged, pass_stop;
};

__global__ void rs_begin_kernel(RsCtl* ctl) { *ctl = RsCtl{}; }

// Top of a restart: block 0 as reset_scalars leaves it.
__global__ void rs_reset_kernel(Scalars* s0, double tol2, RsCtl* ctl)
{
    ir_reset_block(s0, tol2);
    ctl->pass_stop = 0;
}

// After the first residual (EP_TB_INIT) and the method's init: the checks at
// the top of a restart, then the Krylov loop's budget.  A stop leaves block 0
// without a pending half step and block 2 done, so the rest is no-ops.
__global__ void rs_step_kernel(Scalars* s0, Scalars* s2, RsCtl* ctl,
                               cudaGraphConditionalHandle h_inner, int maxit)
{
    cudaGraphSetConditional(h_inner, 0u);
    IrCtl& k = ctl->k;
    bool stop = true;
    k.relres = s0->res;
    if (s0->status) {
        k.status = s0->status;
    } else if (s0->bb == 0.0) {
        k.zero_x = 1;
        k.relres = 0.0;
        ctl->converged = 1;
    } else if (s0->done) {
        ctl->converged = 1;
    } else if (k.total >= maxit) {
    } else {
        stop = false;
    }
    if (stop) {
        ctl->pass_stop = 1;
        k.stop = 1;
        s0->done = 1;
        s0->half = 0;
        s2->done = 1;
        return;
    }
    k.inner_it = 0;
    k.budget = maxit - k.total;
    if (k.budget > 0) cudaGraphSetConditional(h_inner, 1u);
}

__global__ void rs_zero_x_kernel(double* x, int n, const RsCtl* ctl)
{
    if (!ctl->k.zero_x) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = 0.0;
}

// After the Krylov loop: its count, breakdown and status; block 2 reset for
// the true residual.
__global__ void rs_mid_kernel(Scalars* s0, Scalars* s2, RsCtl* ctl, double tol2)
{
    if (ctl->pass_stop) return;
    IrCtl& k = ctl->k;
    k.total += s0->iters;
    k.pad = s0->breakdown != 0;  // broke
    if (s0->status) {
        k.status = s0->status;
        ctl->pass_stop = 1;
        k.stop = 1;
        s0->half = 0;
        s2->done = 1;
        return;
    }
    ir_reset_block(s2, tol2);
}

// After the true residual (EP_TRUE_RES in block 2): converged, or restart.
__global__ void rs_post_kernel(const Scalars* s0, const Scalars* s2, RsCtl* ctl,
                               cudaGraphConditionalHandle h_outer, double tol2)
{
    cudaGraphSetConditional(h_outer, 0u);
    IrCtl& k = ctl->k;
    if (!ctl->pass_stop) {
        k.relres = s2->res;
        if (!isfinite(s2->res)) {
            k.status = OCSL_NONFINITE;
            k.stop = 1;
        } else {
            ctl->converged = s2->rr <= tol2 * s2->bb;
            k.outer += 1;
            if (ctl->converged || (k.pad && s0->iters == 0) || k.outer >= 64)
                k.stop = 1;
            else
                cudaGraphSetConditional(h_outer, 1u);
        }
    }
    if (k.stop && !ctl->converged && k.status == OCSL_OK)
        k.status = k.pad ? OCSL_BREAKDOWN : OCSL_NOT_CONVERGED;
}

template <typename Init, typename Iter, typename Half>
TolResult run_restarted_device(Solve& s, const double* A, const double* b, double* x,
                               const ocsl_opts& o, Init&& init, Iter&& iteration, Half&& half,
                               int kind, std::initializer_list<const void*> ptrs)
{
    ocsl_ctx* c = s.c;
    double** v = c->v64;
    const double tol2 = o.tol * o.tol;
    if (c->n_irctl < 2) ensure_irctl(c, 2);  // an RsCtl takes two IrCtl slots
    RsCtl* ctl = static_cast<RsCtl*>(c->d_irctl);
    static_assert(sizeof(RsCtl) <= 2 * sizeof(IrCtl), "control block size");
    std::vector<unsigned char> key;
    auto add = [&](const void* p, size_t bytes) {
        const unsigned char* q = static_cast<const unsigned char*>(p);
        key.insert(key.end(), q, q + bytes);
    };
    add(&kind, sizeof kind);
    for (const void* p : ptrs) add(&p, sizeof p);
    const void* more[5] = {A, b, x, s.st, c->d_irctl};
    add(more, sizeof more);
    add(&o.tol, sizeof o.tol);
    add(&o.maxit, sizeof o.maxit);
    if (!c->ir_exec || key != c->ir_key) {
        if (c->ir_exec) cudaGraphExecDestroy(c->ir_exec);
        c->ir_exec = nullptr;
        c->ir_key.clear();
        const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
        cudaGraph_t root = nullptr;
        CK(cudaGraphCreate(&root, 0));
        try {
            cudaGraphConditionalHandle h_outer, h_inner;
            CK(cudaGraphConditionalHandleCreate(&h_outer, root, 1u, cudaGraphCondAssignDefault));
            CK(cudaStreamBeginCaptureToGraph(s.st, root, nullptr, nullptr, 0, mode));
            rs_begin_kernel<<<1, 1, 0, s.st>>>(ctl);
            cudaGraph_t outer = add_while_node(s.st, h_outer);
            cudaGraph_t got = nullptr;
            CK(cudaStreamEndCapture(s.st, &got));

            CK(cudaGraphConditionalHandleCreate(&h_inner, outer, 0u, 0u));
            CK(cudaStreamBeginCaptureToGraph(s.st, outer, nullptr, nullptr, 0, mode));
            rs_reset_kernel<<<1, 1, 0, s.st>>>(c->d_sc, tol2, ctl);
            s.spmv<double>(A, x, v[R], 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, 0, EP_TB_INIT);
            init();
            rs_step_kernel<<<1, 1, 0, s.st>>>(c->d_sc, c->d_sc + 2, ctl, h_inner, o.maxit);
            rs_zero_x_kernel<<<std::max(1, std::min((s.n + 255) / 256, 1024)), 256, 0, s.st>>>(
                x, s.n, ctl);
            cudaGraph_t inner = add_while_node(s.st, h_inner);
            rs_mid_kernel<<<1, 1, 0, s.st>>>(c->d_sc, c->d_sc + 2, ctl, tol2);
            half();
            s.spmv<double>(A, x, v[R], 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, 2, EP_TRUE_RES);
            rs_post_kernel<<<1, 1, 0, s.st>>>(c->d_sc, c->d_sc + 2, ctl, h_outer, tol2);
            CK(cudaStreamEndCapture(s.st, &outer));

            CK(cudaStreamBeginCaptureToGraph(s.st, inner, nullptr, nullptr, 0, mode));
            s.tb_prefilled = false;  // every pass fills its sweep outputs (same bits)
            iteration(0);
            s.tb_prefilled = false;
            ir_inner_kernel<<<1, 1, 0, s.st>>>(c->d_sc, &ctl->k, h_inner);
            CK(cudaStreamEndCapture(s.st, &inner));
        } catch (...) {
            end_any_capture(s.st);
            cudaGraphDestroy(root);
            throw;
        }
        cudaGraphExec_t e = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&e, root, 0);
        cudaGraphDestroy(root);
        CK(ie);
        c->ir_exec = e;
        c->ir_key = key;
    }
    CK(cudaGraphLaunch(c->ir_exec, s.st));
    RsCtl h;
    CK(cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    TolResult r;
    r.iters = h.k.total;
    r.relres = h.k.relres;
    r.status = h.k.status;
    return r;
}

TolResult run_bicgstab_tol_device(Solve& s, const double* A, const double* b, double* x,
                                  const ocsl_opts& o)
{
    double** v = s.c->v64;
    const double* M = s.factored(A, o.ilu_sweeps, true, false, -1, true, true, false);
    if (s.pivot_status() != OCSL_OK) return zero_pivot_result();
    s.prepare_spmv(A, true, false);
    return run_restarted_device(
        s, A, b, x, o, [&] { s.vec<double>(V_COPY2, {v[RH], v[P], v[R]}, 0, EP_STORE); },
        [&](int) {
            bicgstab_iteration<double>(s, A, M, s.c->d_dinv, x, v[R], v[RH], v[P], v[PH], v[V],
                                       v[S], v[SH], v[T], v[TMP], 0);
        },
        [&] { s.vec<double>(V_TB_HALF, {x, v[PH]}, 0, EP_STORE); }, 1,
        {M, s.soa64, s.recA64, s.c->d_dinv});
}

TolResult run_pcg_tol_device(Solve& s, const double* A, const double* b, double* x,
                             const ocsl_opts& o)
{
    double** v = s.c->v64;
    s.factored(A, 0, true, false, -1, false, false, false);  // Jacobi: dinv = 1 / A_ii
    if (s.pivot_status() != OCSL_OK) return zero_pivot_result();
    s.prepare_spmv(A, true, false);
    return run_restarted_device(
        s, A, b, x, o,
        [&] { s.vec<double>(V_PC_INIT, {v[Z], v[P], v[R], s.c->d_dinv}, 0, EP_PC_INIT); },
        [&](int) {
            s.spmv<double>(A, v[P], v[Q], 0, nullptr, nullptr, v[P], DOT_WY, 0, EP_PC_ALPHA);
            s.vec<double>(V_PC_XRZ, {x, v[P], v[R], v[Q], v[Z], s.c->d_dinv}, 0, EP_PC_RUPD);
            s.vec<double>(V_PC_P, {v[P], v[Z]}, 0, EP_STORE);
        },
        [] {}, 2, {s.recA64, s.c->d_dinv});
}

// Column-batched form of run_bicgstab_ir32: nc (<= kMaxCols) right-hand
// sides b, x ([nc][n]) of one matrix in lockstep.  Every launch serves all
// columns -- the SpMV and vector kernels run nc column slices in one grid,
// the structured sweeps carry nc right-hand sides through one wavefront
// pass -- while each column keeps its own scalars, adaptive inner tolerance,
// iteration count and status; a finished column's kernels return at once.
std::vector<TolResult> run_bicgstab_ir32_cols(Solve& s, const double* A, const double* b,
                                              double* x, int nc, const ocsl_opts& o)
{
    ocsl_ctx* c = s.c;
    c->ensure_fp32();
    c->ensure_cols();
    double* R64 = c->v64c;
    float** f = c->v32c;
    const int n = s.n;
    s.cols = Cols{nc, (long long)n, 0u, c->col_batching == 2 ? 1 : 0};
    s.outer_k = kScOuterCols;
    const int KO = kScOuterCols, KI = kScInnerCols;
    std::vector<TolResult> res(nc);
    std::vector<int> fin(nc, 0), total(nc, 0);
    std::vector<double> tol2(nc, o.tol * o.tol), itol2(nc, 0.0);
    s.factored(A, o.ilu_sweeps, true, true, -1, false, true, true);
    if (s.pivot_status() != OCSL_OK) {
        for (auto& r : res) r = zero_pivot_result();
        s.cols = Cols{};
        s.outer_k = 0;
        return res;
    }
    s.prepare_spmv(A, true, true);
    s.reset_scalars_n(KO, nc, tol2.data(), nullptr);
    for (int outer = 0;; ++outer) {
        s.spmv<double>(A, x, R64, 1, b, nullptr, nullptr, DOT_YY | DOT_ZZ, KO, EP_TB_INIT);
        const Scalars* so = s.read_scalars_n(KO, nc);
        int active = 0, most = 0;
        for (int q = 0; q < nc; ++q) {
            if (fin[q]) continue;
            TolResult& r = res[q];
            r.relres = so[q].res;
            r.outer = outer;
            if (so[q].status) {
                r.status = so[q].status;
                fin[q] = 1;
            } else if (so[q].bb == 0.0) {
                CK(cudaMemsetAsync(x + (size_t)q * n, 0, sizeof(double) * (size_t)n, s.st));
                r.relres = 0.0;
                fin[q] = 1;
            } else if (so[q].done) {
                fin[q] = 1;
            } else if (total[q] >= o.maxit || outer >= 1000) {
                r.status = OCSL_NOT_CONVERGED;
                fin[q] = 1;
            } else {
                ++active;
                most = std::max(most, total[q]);
                itol2[q] = std::max(o.inner_tol, 0.5 * o.tol / so[q].res);
                itol2[q] *= itol2[q];
            }
        }
        if (active == 0) break;
        // finished columns: outer and inner blocks done, so every kernel skips
        // them (the outer blocks keep this residual's norms for the scaling)
        for (int q = 0; q < nc; ++q)
            if (fin[q] && !so[q].done) s.mark_done(KO + q);
        s.reset_scalars_n(KI, nc, itol2.data(), fin.data());
        s.vec<float>(V_IR_SCALE, {R64, f[F_RI], f[F_RH], f[F_P], f[F_D]}, KI, EP_IR_INNER_INIT);
        const int budget = std::min(o.inner_maxit, o.maxit - most);
        run_batches(
            s, KI, budget,
            [&](int) {
                bicgstab_iteration<float>(s, c->d_A32, c->d_M32, c->d_dinv32, f[F_D], f[F_RI],
                                          f[F_RH], f[F_P], f[F_PH], f[F_V], f[F_S], f[F_SH],
                                          f[F_T], f[F_TMP], KI);
            },
            5, {c->d_A32, c->d_M32, s.soa32, s.recA32, c->d_dinv32, (const void*)(intptr_t)nc});
        const Scalars* sp = s.read_scalars_n(KI, nc);
        const std::vector<Scalars> si(sp, sp + nc);
        s.vec<float>(V_TB_HALF, {f[F_D], f[F_PH]}, KI, EP_STORE);
        s.vec<float>(V_IR_UPDATE, {x, f[F_D]}, -1, EP_STORE);
        for (int q = 0; q < nc; ++q) {
            if (fin[q]) continue;
            total[q] += si[q].iters;
            if (si[q].status == OCSL_NONFINITE) {
                res[q].status = OCSL_NONFINITE;
                fin[q] = 1;
            } else if (si[q].iters == 0 && !si[q].done) {
                res[q].status = OCSL_BREAKDOWN;
                fin[q] = 1;
            }
        }
        // the next residuals reuse the outer blocks: clear done, keep tol2
        s.reset_scalars_n(KO, nc, tol2.data(), fin.data());
    }
    for (int q = 0; q < nc; ++q) res[q].iters = total[q];
    s.cols = Cols{};
    s.outer_k = 0;
    return res;
}

bool aligned8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

int check_ready(ocsl_ctx* c)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (!c->has_pattern) return fail(c, OCSL_NO_PATTERN, "ocsl_set_pattern has not been called");
    return OCSL_OK;
}

// Builds the multicolour-permuted pattern (colour_pattern) and its child
// context; the permutation and the slot map go to the device.
int ensure_coloured(ocsl_ctx* c)
{
    if (c->cctx) return OCSL_OK;
    const int n = c->P.n, nnz = c->P.nnz;
    std::vector<int> rp(n + 1), col(nnz);
    CK(cudaMemcpy(rp.data(), c->P.rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    if (nnz) CK(cudaMemcpy(col.data(), c->P.col, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    ColouredPattern cp;
    std::string err;
    if (!colour_pattern(n, rp, col, cp, err)) return fail(c, OCSL_BAD_PATTERN, err);
    ocsl_ctx* t = nullptr;
    int rc = ocsl_create(&t, c->device);
    if (rc != OCSL_OK) return fail(c, rc, "ordering context: " + g_create_error);
    t->graphs_on = c->graphs_on;
    rc = ocsl_set_pattern(t, (size_t)n, cp.rp.data(), cp.col.data());
    if (rc != OCSL_OK) {
        const std::string msg = t->last_error;
        ocsl_destroy(t);
        return fail(c, rc, "multicolour pattern: " + msg);
    }
    // Sweep colour by colour: one launch per colour (ascending forward,
    // descending backward), and the fused preconditioner (2C - 2 launches for
    // C colours).  With at most kRangeMaxLevels colours; beyond, the child
    // keeps the single-launch level-scheduled sweeps.
    DevPattern& Q = t->P;
    Q.coloured = cp.colours <= kRangeMaxLevels;
    Q.fw_nrange = Q.bw_nrange = Q.coloured ? cp.colours : 0;
    for (int k = 0; Q.coloured && k < cp.colours; ++k) {
        Q.fw_range[2 * k] = cp.start[k];
        Q.fw_range[2 * k + 1] = cp.start[k + 1];
        Q.bw_range[2 * k] = cp.start[cp.colours - 1 - k];
        Q.bw_range[2 * k + 1] = cp.start[cp.colours - k];
    }
    // red-black ordering of an even-nx box: stencil records instead of the
    // CSR, if every row of the permuted pattern is what RbGeom says it is
    std::vector<signed char> rbslot;
    std::vector<unsigned char> rbinfo;
    if (c->hp.box.ok && cp.colours == 2 && c->hp.box.dim[0] % 2 == 0 && n % 2 == 0 &&
        cp.start[1] == n / 2) {
        RbGeom g{n, n / 2, c->hp.box.dim[0], c->hp.box.dim[1], c->hp.box.dim[2],
                 c->hp.box.dim[0] / 2, nullptr};
        rbslot.assign((size_t)cp.col.size(), (signed char)-1);
        rbinfo.assign((size_t)n, 0);
        bool ok = true;
        for (int row = 0; row < n && ok; ++row) {
            const RbRow q = rb_row(g, row);
            // the natural cell of this row
            const int r = row - q.c * g.n0, rjk = r / g.hx;
            const int b = (q.c + rjk % g.ny + rjk / g.ny) & 1;
            ok = cp.perm[row] == 2 * r + b;
            unsigned char f = (unsigned char)(b << 6);
            for (int s = 0; s < 6; ++s)
                if (q.has[s]) f |= (unsigned char)(1u << s);
            rbinfo[row] = f;
            // entries in the order the kernels sum them, then phantoms
            int want[7], m = 0;
            if (q.c == 0) want[m++] = 6;
            for (int s = 0; s < 6; ++s)
                if (q.has[s]) want[m++] = s;
            if (q.c == 1) want[m++] = 6;
            int e = 0;
            for (size_t k = cp.rp[row]; k < cp.rp[row + 1] && ok; ++k) {
                if (cp.col[k] == ~size_t(0)) continue;  // phantom
                ok = e < m && (size_t)(want[e] == 6 ? row : q.nb[want[e]]) == cp.col[k];
                if (ok) rbslot[k] = (signed char)want[e++];
            }
            ok = ok && e == m;
        }
        if (ok) {
            t->rb = g;
            t->rb_ok = true;
        }
    }
    try {
        c->d_cperm = upload(cp.perm);
        c->d_cslot = upload(cp.slot);
        if (t->rb_ok) {
            CK(cudaMalloc(&t->d_rbslot, rbslot.size() + rbinfo.size()));
            CK(cudaMemcpy(t->d_rbslot, rbslot.data(), rbslot.size(), cudaMemcpyHostToDevice));
            unsigned char* info = reinterpret_cast<unsigned char*>(t->d_rbslot) + rbslot.size();
            CK(cudaMemcpy(info, rbinfo.data(), rbinfo.size(), cudaMemcpyHostToDevice));
            t->rb.info = info;
        }
    } catch (...) {
        ocsl_destroy(t);
        for (int** pp : {&c->d_cperm, &c->d_cslot}) { if (*pp) cudaFree(*pp); *pp = nullptr; }
        throw;
    }
    c->colours = cp.colours;
    c->cctx = t;
    return OCSL_OK;
}

int solve_device_impl(ocsl_ctx* c, int method, const double* A, const double* b, double* x,
                      const ocsl_opts* opts, ocsl_result* out, bool reuse_factor = false);

// A tolerance-mode solve through the multicolour ordering: the values, b and
// x0 gathered into the child context's buffers, the solve there, x scattered
// back; solve_ms covers the gathers and the scatter.
int solve_coloured(ocsl_ctx* c, int method, const double* A, const double* b, double* x,
                   const ocsl_opts* opts, ocsl_result* out, bool reuse_factor)
{
    ocsl_result r;
    std::memset(&r, 0, sizeof r);
    ocsl_ctx* t = nullptr;
    try {
        const int rc = ensure_coloured(c);
        if (rc != OCSL_OK) {
            r.status = rc;
            if (out) *out = r;
            return rc;
        }
        t = c->cctx;
        t->stream = c->stream;
        t->prof_on = c->prof_on;
        CK(cudaEventRecord(c->ev_start, c->stream));
        launch_gather_values(c->stream, t->P.nnz, c->d_cslot, A, t->d_A);
        launch_gather_values(c->stream, t->P.n, c->d_cperm, b, t->d_b);
        launch_gather_values(c->stream, t->P.n, c->d_cperm, x, t->d_x);
        CK(cudaGetLastError());
    } catch (const CudaError& e) {
        r.status = from_cuda(c, e);
        if (out) *out = r;
        return r.status;
    }
    int status = solve_device_impl(t, method, t->d_A, t->d_b, t->d_x, opts, &r, reuse_factor);
    if (status != OCSL_OK) c->last_error = t->last_error;
    if (status == OCSL_CUDA_ERROR) {
        if (out) *out = r;
        return status;
    }
    try {
        launch_scatter_values(c->stream, t->P.n, c->d_cperm, t->d_x, x);
        CK(cudaGetLastError());
        CK(cudaEventRecord(c->ev_stop, c->stream));
        CK(cudaEventSynchronize(c->ev_stop));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev_start, c->ev_stop));
        r.solve_ms = ms;
    } catch (const CudaError& e) {
        status = from_cuda(c, e);
        r.status = status;
    }
    if (out) *out = r;
    return status;
}

int solve_device_impl(ocsl_ctx* c, int method, const double* A, const double* b, double* x,
                      const ocsl_opts* opts, ocsl_result* out, bool reuse_factor)
{
    const ocsl_opts o = resolve(opts);
    ocsl_result r;
    std::memset(&r, 0, sizeof r);
    if (method < OCSL_CG_REF || method > OCSL_ILU_BICGSTAB_IR32)
        return fail(c, OCSL_BAD_ARGUMENT, "unknown method");
    if (c->P.n == 0) {
        if (out) *out = r;
        return OCSL_OK;
    }
    if (!A || !b || !x) return fail(c, OCSL_BAD_ARGUMENT, "null value, b or x pointer");
    if (!aligned8(A) || !aligned8(b) || !aligned8(x))
        return fail(c, OCSL_BAD_ARGUMENT, "device pointers must be 8-byte aligned");
    if (c->ordering == OCSL_ORDER_MULTICOLOUR && method >= OCSL_PCG)
        return solve_coloured(c, method, A, b, x, opts, out, reuse_factor);
    Solve s{c, c->stream, c->P, c->P.n};
    s.reuse = reuse_factor;
    if (!reuse_factor) c->fac_M = nullptr;
    int status = OCSL_OK;
    try {
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
        CK(cudaEventRecord(c->ev_start, c->stream));
        if (method == OCSL_CG_REF || method == OCSL_BICGSTAB_REF) {
            if (method == OCSL_CG_REF)
                run_cg_ref(s, A, b, x);
            else
                run_bicgstab_ref(s, A, b, x, o.ilu_sweeps);
            CK(cudaEventRecord(c->ev_stop, c->stream));
            const Scalars sc = s.read_scalars(0);
            r.residual = sc.res;
            r.iterations = sc.iters;
        } else {
            TolResult t;
            if (method == OCSL_PCG)
                t = device_loop_ok(s) ? run_pcg_tol_device(s, A, b, x, o)
                                      : run_pcg_tol(s, A, b, x, o);
            else if (method == OCSL_ILU_BICGSTAB)
                t = device_loop_ok(s) ? run_bicgstab_tol_device(s, A, b, x, o)
                                      : run_bicgstab_tol(s, A, b, x, o);
            else if (device_loop_ok(s))
                t = run_bicgstab_ir32_device(s, A, b, x, o);
            else
                t = run_bicgstab_ir32(s, A, b, x, o);
            CK(cudaEventRecord(c->ev_stop, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            r.residual = t.relres;
            r.iterations = t.iters;
            r.outer_iterations = t.outer;
            status = t.status;
        }
        CK(cudaEventSynchronize(c->ev_stop));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev_start, c->ev_stop));
        r.solve_ms = ms;
        const int derr = s.device_error();
        if (derr) status = derr;
        CK(cudaGetLastError());
    } catch (const CudaError& e) {
        status = from_cuda(c, e);
    }
    r.status = status;
    if (out) *out = r;
    if (status == OCSL_TIMEOUT) c->last_error = "a triangular-sweep wait hit its bound";
    if (status == OCSL_ZERO_PIVOT) c->last_error = "the factor has a zero or infinite pivot";
    return status;
}

// Builds the transposed pattern (real entries only; rows of A ascending give
// ascending columns in every row of A^T) and its child context.
int ensure_transpose(ocsl_ctx* c)
{
    if (c->tctx) return OCSL_OK;
    const int n = c->P.n, nnz = c->P.nnz;
    std::vector<int> rp(n + 1), col(nnz);
    CK(cudaMemcpy(rp.data(), c->P.rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    if (nnz) CK(cudaMemcpy(col.data(), c->P.col, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    std::vector<size_t> trp(n + 1, 0);
    for (int k = 0; k < nnz; ++k)
        if (col[k] >= 0) ++trp[col[k] + 1];
    for (int i = 0; i < n; ++i) trp[i + 1] += trp[i];
    std::vector<size_t> tcol(trp[n]), next(trp.begin(), trp.end() - 1);
    std::vector<int> perm(trp[n]);
    for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = col[k];
            if (j < 0) continue;
            const size_t q = next[j]++;
            tcol[q] = (size_t)i;
            perm[q] = k;
        }
    ocsl_ctx* t = nullptr;
    int rc = ocsl_create(&t, c->device);
    if (rc != OCSL_OK) return fail(c, rc, "adjoint context: " + g_create_error);
    ocsl_set_sweep_kernel(t, c->sweep_kernel, 0, 0);
    t->ordering = c->ordering;
    std::memcpy(t->box_tile, c->box_tile, sizeof(c->box_tile));
    std::memcpy(t->box_cluster, c->box_cluster, sizeof(c->box_cluster));
    t->graphs_on = c->graphs_on;
    rc = ocsl_set_pattern(t, (size_t)n, trp.data(), tcol.data());
    if (rc != OCSL_OK) {
        const std::string msg = t->last_error;
        ocsl_destroy(t);
        return fail(c, rc, "transposed pattern: " + msg);
    }
    try {
        c->d_tperm = upload(perm);
    } catch (...) {
        ocsl_destroy(t);
        throw;
    }
    c->nnzT = (long long)perm.size();
    c->tctx = t;
    return OCSL_OK;
}

// Names the first state field an equation needs that is NULL, else nullptr.
const char* missing_state_field(const ocsl_assembly& q, const ocsl_flow_state& s, bool has_nf,
                                bool has_nb)
{
    struct Need {
        const void* p;
        const char* name;
        bool want;
    };
    const bool mom = q.equation == OCSL_EQ_MOMENTUM, pre = q.equation == OCSL_EQ_PRESSURE,
               ent = q.equation == OCSL_EQ_ENTHALPY, heat = q.equation == OCSL_EQ_HEAT,
               flow = !heat, tr = q.transient != 0 || heat, vis = q.viscous != 0;
    const Need need[] = {
        {s.geo_aver, "geo_aver", has_nf && flow},
        {s.mdot, "mdot", has_nf && flow},
        {s.ksi_A, "ksi_A", has_nf && ((mom && vis) || ent || heat)},
        {s.stress, "stress", has_nf && mom && vis},
        {s.density, "density", has_nf && pre},
        {s.qy, "qy", has_nf && pre},
        {s.bc_type, "bc_type", has_nb && flow},
        {s.bc_mdot, "bc_mdot", has_nb && flow},
        {s.bc_wall, "bc_wall", has_nb && mom && vis},
        {s.bc_area, "bc_area", has_nb && mom && vis},
        {s.bc_area_vector, "bc_area_vector", has_nb && mom && vis},
        {s.bc_perp_dist, "bc_perp_dist", has_nb && mom && vis},
        {s.bc_velocity, "bc_velocity", has_nb && mom},
        {s.bc_supersonic, "bc_supersonic", has_nb && pre},
        {s.bc_qy, "bc_qy", has_nb && pre},
        {s.bc_density, "bc_density", has_nb && pre},
        {s.bc_temperature, "bc_temperature", has_nb && (pre || ent || heat)},
        {s.bc_enthalpy, "bc_enthalpy", has_nb && ent},
        {s.bc_ksi_A, "bc_ksi_A", has_nb && (ent || heat)},
        {s.bc_thermal, "bc_thermal", has_nb && heat},
        {s.volume, "volume", true},
        {s.delta_t, "delta_t", tr},
        {s.velocity, "velocity", mom},
        {s.velocity_last, "velocity_last", mom},
        {s.pressure_grad, "pressure_grad", mom},
        {s.density_c, "density_c", (mom && tr) || pre || ent},
        {s.density_last, "density_last", tr && (mom || pre || ent)},
        {s.temperature, "temperature", (mom && vis) || pre || ent || heat},
        {s.pressure_corr, "pressure_corr", pre},
        {s.enthalpy, "enthalpy", ent},
        {s.enthalpy_last, "enthalpy_last", ent},
        {s.pressure, "pressure", ent && tr},
        {s.pressure_last, "pressure_last", ent && tr},
    };
    for (const Need& x : need)
        if (x.want && !x.p) return x.name;
    return nullptr;
}

}  // namespace

namespace ocsl {

int ir32_graph_prepare(ocsl_ctx* c, const double* A, const ocsl_opts* opts, int slots)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (!A || !aligned8(A)) return fail(c, OCSL_BAD_ARGUMENT, "null or misaligned value pointer");
    if (c->ordering == OCSL_ORDER_MULTICOLOUR)
        return fail(c, OCSL_BAD_ARGUMENT, "the one-graph batch runs the natural ordering");
    const ocsl_opts o = resolve(opts);
    try {
        CK(cudaSetDevice(c->device));
        Solve s{c, c->stream, c->P, c->P.n};
        c->fac_M = nullptr;
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
        ensure_irctl(c, std::max(1, slots));
        if (c->P.n == 0) return OCSL_OK;
        c->ensure_fp32();
        s.factored(A, o.ilu_sweeps, true, true, -1, false, true, true);
        const int pv = s.pivot_status();
        if (pv != OCSL_OK) return pv;
        s.prepare_spmv(A, true, true);
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ir32_graph_capture(ocsl_ctx* c, cudaGraph_t root, cudaGraphNode_t* last, const double* A,
                       const double* b, double* x, const ocsl_opts* opts, int slot)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (!b || !x || !aligned8(b) || !aligned8(x))
        return fail(c, OCSL_BAD_ARGUMENT, "null or misaligned b or x pointer");
    if (slot < 0 || slot >= c->n_irctl) return fail(c, OCSL_BAD_ARGUMENT, "no such control block");
    if (c->P.n == 0) return OCSL_OK;
    if (!c->fac_M) return fail(c, OCSL_BAD_ARGUMENT, "ir32_graph_prepare first");
    if (c->prof_on || c->fault_skip_pending || c->stream == nullptr ||
        c->stream == cudaStreamLegacy || c->stream == cudaStreamPerThread)
        return fail(c, OCSL_BAD_ARGUMENT, "this context cannot capture its solve");
    const ocsl_opts o = resolve(opts);
    try {
        CK(cudaSetDevice(c->device));
        Solve s{c, c->stream, c->P, c->P.n};
        s.reuse = true;  // the prepared factor and records: no launches here
        s.factored(A, o.ilu_sweeps, true, true, -1, false, true, true);
        s.prepare_spmv(A, true, true);
        capture_ir32(s, root, last, A, b, x, o, static_cast<IrCtl*>(c->d_irctl) + slot);
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ir32_graph_result(ocsl_ctx* c, int slot, ocsl_result* r)
{
    if (!c || !r) return OCSL_BAD_ARGUMENT;
    std::memset(r, 0, sizeof *r);
    if (c->P.n == 0) return OCSL_OK;
    if (slot < 0 || slot >= c->n_irctl) return fail(c, OCSL_BAD_ARGUMENT, "no such control block");
    int status = OCSL_OK;
    try {
        Solve s{c, c->stream, c->P, c->P.n};
        const TolResult t = read_ir_ctl(s, slot);
        r->residual = t.relres;
        r->iterations = t.iters;
        r->outer_iterations = t.outer;
        status = t.status;
        const int derr = s.device_error();
        if (derr) status = derr;
    } catch (const CudaError& e) {
        status = from_cuda(c, e);
    }
    r->status = status;
    if (status == OCSL_TIMEOUT) c->last_error = "a triangular-sweep wait hit its bound";
    return status;
}

cudaStream_t ir32_graph_stream(const ocsl_ctx* c) { return c ? c->stream : nullptr; }

}  // namespace ocsl

// =================================================================== C ABI

extern "C" {

void ocsl_default_opts(ocsl_opts* o)
{
    if (!o) return;
    o->tol = 1e-10;
    o->maxit = 5000;
    o->ilu_sweeps = 3;
    o->inner_tol = 1e-5;
    o->inner_maxit = 500;
}

const char* ocsl_version(void) { return kVersion; }

const char* ocsl_status_string(int s)
{
    switch (s) {
    case OCSL_OK: return "OCSL_OK";
    case OCSL_NOT_CONVERGED: return "OCSL_NOT_CONVERGED";
    case OCSL_ZERO_PIVOT: return "OCSL_ZERO_PIVOT";
    case OCSL_NONFINITE: return "OCSL_NONFINITE";
    case OCSL_BAD_PATTERN: return "OCSL_BAD_PATTERN";
    case OCSL_TIMEOUT: return "OCSL_TIMEOUT";
    case OCSL_CUDA_ERROR: return "OCSL_CUDA_ERROR";
    case OCSL_BAD_ARGUMENT: return "OCSL_BAD_ARGUMENT";
    case OCSL_NO_PATTERN: return "OCSL_NO_PATTERN";
    case OCSL_NO_DEVICE: return "OCSL_NO_DEVICE";
    case OCSL_BREAKDOWN: return "OCSL_BREAKDOWN";
    default: return "OCSL_UNKNOWN";
    }
}

const char* ocsl_last_error(const ocsl_ctx* c)
{
    return c ? c->last_error.c_str() : g_create_error.c_str();
}

int ocsl_create(ocsl_ctx** out, int device)
{
    if (!out) return OCSL_BAD_ARGUMENT;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return OCSL_NO_DEVICE;
    }
    if (device < 0 || device >= count) {
        g_create_error = "device index out of range";
        return OCSL_BAD_ARGUMENT;
    }
    auto* c = new ocsl_ctx();
    c->device = device;
    try {
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
        c->stream = c->own_stream;
        c->d_sc = dalloc<Scalars>(kScBlocks);
        CK(cudaMemset(c->d_sc, 0, kScBlocks * sizeof(Scalars)));
        CK(cudaMallocHost(&c->h_sc, kHostSlots * sizeof(Scalars)));
        c->d_sync = dalloc<unsigned>(2);
        CK(cudaMemset(c->d_sync, 0, 2 * sizeof(unsigned)));
        c->S.ticket = c->d_sync;
        c->S.finished = c->d_sync + 1;
        c->d_err = dalloc<int>(1);
        CK(cudaMemset(c->d_err, 0, sizeof(int)));
        c->S.err = c->d_err;
        CK(cudaMallocHost(&c->h_err, sizeof(int)));
        CK(cudaEventCreate(&c->ev_start));
        CK(cudaEventCreate(&c->ev_stop));
        CK(cudaEventCreateWithFlags(&c->ev_batch[0], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->ev_batch[1], cudaEventDisableTiming));
        c->ensure_reduce(1);
    } catch (const CudaError& err) {
        g_create_error = std::string(err.what) + ": " + cudaGetErrorString(err.code);
        c->free_all();
        delete c;
        return OCSL_CUDA_ERROR;
    }
    *out = c;
    return OCSL_OK;
}

int ocsl_destroy(ocsl_ctx* c)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->free_all();
    delete c;
    return OCSL_OK;
}

int ocsl_set_stream(ocsl_ctx* c, void* stream)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    return OCSL_OK;
}

int ocsl_synchronize(ocsl_ctx* c)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(c, OCSL_CUDA_ERROR, cudaGetErrorString(e));
    return OCSL_OK;
}

int ocsl_set_pattern(ocsl_ctx* c, size_t n, const size_t* rp, const size_t* col)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    HostPattern hp;
    std::string err;
    if (!analyse_pattern(n, rp, col, hp, err)) return fail(c, OCSL_BAD_PATTERN, err);
    try {
        CK(cudaSetDevice(c->device));
        CK(cudaStreamSynchronize(c->stream));
        c->free_pattern();
        const std::vector<int>* tabs[10] = {&hp.rp, &hp.col, &hp.diag, &hp.pair_ptr, &hp.pair_k,
                                            &hp.pair_slot, &hp.fw_order, &hp.fw_chunk,
                                            &hp.bw_order, &hp.bw_chunk};
        for (int i = 0; i < 10; ++i) c->d_pat[i] = upload(*tabs[i]);
        DevPattern& P = c->P;
        P.n = hp.n;
        P.nnz = hp.nnz;
        P.rp = c->d_pat[0];
        P.col = c->d_pat[1];
        P.diag = c->d_pat[2];
        P.pair_ptr = c->d_pat[3];
        P.pair_k = c->d_pat[4];
        P.pair_slot = c->d_pat[5];
        P.fw_order = c->d_pat[6];
        P.fw_chunk = c->d_pat[7];
        P.fw_nchunks = (int)hp.fw_chunk.size() - 1;
        P.bw_order = c->d_pat[8];
        P.bw_chunk = c->d_pat[9];
        P.bw_nchunks = (int)hp.bw_chunk.size() - 1;
        P.box_ok = hp.box.ok && c->sweep_kernel != 1;
        P.fw_nrange = (int)hp.fw_range.size() / 2;
        P.bw_nrange = (int)hp.bw_range.size() / 2;
        std::copy(hp.fw_range.begin(), hp.fw_range.end(), P.fw_range);
        std::copy(hp.bw_range.begin(), hp.bw_range.end(), P.bw_range);
        c->hp.box = hp.box;
        c->rebuild_box_geoms();
        // the one-warp sweep: the solution fits its shared memory and the
        // schedule is at least a quarter as deep as the system is long
        for (int k = 0; k < 2; ++k)
            c->serial_ok[k] = (size_t)hp.n * (k ? sizeof(float) : sizeof(double)) <=
                                  (size_t)kSerialMaxBytes &&
                              4LL * P.fw_nchunks >= hp.n && 4LL * P.bw_nchunks >= hp.n;
        const size_t nn = (size_t)hp.n, nz = (size_t)hp.nnz;
        c->d_A = dalloc<double>(nz);
        c->d_b = dalloc<double>(nn);
        c->d_x = dalloc<double>(nn);
        c->d_Ma = dalloc<double>(nz);
        c->d_Mb = dalloc<double>(nz);
        c->d_dinv = dalloc<double>(nn);
        for (auto& v : c->v64) v = dalloc<double>(nn);
        if (hp.box.ok) c->d_soa64 = dalloc<double>(8 * nn);
        c->ensure_reduce((hp.n + kTile - 1) / kTile);
        // drop the large host tables, keep the facts
        c->hp.n = hp.n;
        c->hp.nnz = hp.nnz;
        c->hp.nnz_real = hp.nnz_real;
        c->hp.fw_levels = hp.fw_levels;
        c->hp.bw_levels = hp.bw_levels;
        c->has_pattern = true;
    } catch (const CudaError& e) {
        c->free_pattern();
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_check_pattern(size_t n, const size_t* rp, const size_t* col, int64_t* nnz_real,
                       int32_t* fw_levels, int32_t* bw_levels, int32_t* box_dims, char* err,
                       size_t err_len)
{
    HostPattern hp;
    std::string msg;
    const bool ok = analyse_pattern(n, rp, col, hp, msg);
    if (err && err_len) {
        std::snprintf(err, err_len, "%s", ok ? "" : msg.c_str());
    }
    if (!ok) return OCSL_BAD_PATTERN;
    if (nnz_real) *nnz_real = hp.nnz_real;
    if (fw_levels) *fw_levels = hp.fw_levels;
    if (bw_levels) *bw_levels = hp.bw_levels;
    if (box_dims)
        for (int k = 0; k < 3; ++k) box_dims[k] = hp.box.ok ? hp.box.dim[k] : 0;
    return OCSL_OK;
}

int ocsl_colour_pattern(size_t n, const size_t* rp, const size_t* col, int32_t* perm,
                        int32_t* colours, char* err, size_t err_len)
{
    HostPattern hp;
    ColouredPattern cp;
    std::string msg;
    const bool ok = analyse_pattern(n, rp, col, hp, msg) &&
                    colour_pattern(hp.n, hp.rp, hp.col, cp, msg);
    if (err && err_len) std::snprintf(err, err_len, "%s", ok ? "" : msg.c_str());
    if (!ok) return OCSL_BAD_PATTERN;
    if (perm && n) std::memcpy(perm, cp.perm.data(), n * sizeof(int32_t));
    if (colours) *colours = cp.colours;
    return OCSL_OK;
}

int ocsl_build_pattern(size_t n, int64_t n_faces, const int32_t* left, const int32_t* right,
                       int64_t n_bc, const int32_t* bc_left, size_t* row_ptr,
                       size_t* column_index, size_t* nnz)
{
    if (!nnz || (n_faces > 0 && (!left || !right)) || (n_bc > 0 && !bc_left) || n_faces < 0 ||
        n_bc < 0)
        return OCSL_BAD_ARGUMENT;
    std::vector<size_t> rp, col;
    std::string err;
    if (!build_pattern_from_faces(n, n_faces, left, right, n_bc, bc_left, rp, col, err))
        return OCSL_BAD_ARGUMENT;
    const size_t have = *nnz;
    *nnz = col.size();
    if (!row_ptr) return OCSL_OK;
    if (!column_index || have < col.size()) return OCSL_BAD_ARGUMENT;
    std::memcpy(row_ptr, rp.data(), rp.size() * sizeof(size_t));
    if (!col.empty()) std::memcpy(column_index, col.data(), col.size() * sizeof(size_t));
    return OCSL_OK;
}

int ocsl_pattern_info(const ocsl_ctx* c, int64_t* n, int64_t* nnz, int64_t* nnz_real,
                      int32_t* fw_levels, int32_t* bw_levels)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (!c->has_pattern) return OCSL_NO_PATTERN;
    if (n) *n = c->hp.n;
    if (nnz) *nnz = c->hp.nnz;
    if (nnz_real) *nnz_real = c->hp.nnz_real;
    if (fw_levels) *fw_levels = c->hp.fw_levels;
    if (bw_levels) *bw_levels = c->hp.bw_levels;
    return OCSL_OK;
}

int ocsl_solve_device(ocsl_ctx* c, int method, const double* A, const double* b, double* x,
                      const ocsl_opts* opts, ocsl_result* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, OCSL_CUDA_ERROR, "cudaSetDevice");
    return solve_device_impl(c, method, A, b, x, opts, out);
}

// nc (2..kMaxCols) right-hand sides of the FP32-inner / FP64-refined solver
// in lockstep (run_bicgstab_ir32_cols); out[nc].
int solve_cols_impl(ocsl_ctx* c, const double* A, const double* b, double* x, int nc,
                    const ocsl_opts* opts, ocsl_result* out, bool reuse_factor)
{
    const ocsl_opts o = resolve(opts);
    if (!A || !b || !x) return fail(c, OCSL_BAD_ARGUMENT, "null value, b or x pointer");
    if (!aligned8(A) || !aligned8(b) || !aligned8(x))
        return fail(c, OCSL_BAD_ARGUMENT, "device pointers must be 8-byte aligned");
    Solve s{c, c->stream, c->P, c->P.n};
    s.reuse = reuse_factor;
    if (!reuse_factor) c->fac_M = nullptr;
    int status = OCSL_OK;
    std::vector<TolResult> t;
    float ms = 0.f;
    try {
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
        CK(cudaEventRecord(c->ev_start, c->stream));
        t = run_bicgstab_ir32_cols(s, A, b, x, nc, o);
        CK(cudaEventRecord(c->ev_stop, c->stream));
        CK(cudaEventSynchronize(c->ev_stop));
        CK(cudaEventElapsedTime(&ms, c->ev_start, c->ev_stop));
        const int derr = s.device_error();
        if (derr) status = derr;
        CK(cudaGetLastError());
    } catch (const CudaError& e) {
        status = from_cuda(c, e);
    }
    for (int q = 0; q < nc; ++q) {
        ocsl_result r;
        std::memset(&r, 0, sizeof r);
        if (q < (int)t.size()) {
            r.residual = t[q].relres;
            r.iterations = t[q].iters;
            r.outer_iterations = t[q].outer;
            r.status = status != OCSL_OK ? status : t[q].status;
        } else {
            r.status = status;
        }
        r.solve_ms = ms;
        if (out) out[q] = r;
        if (status == OCSL_OK && r.status != OCSL_OK) status = r.status;
    }
    if (status == OCSL_TIMEOUT) c->last_error = "a triangular-sweep wait hit its bound";
    return status;
}

int ocsl_solve_multi_device(ocsl_ctx* c, int method, const double* A, int nrhs, const double* b,
                            double* x, const ocsl_opts* opts, ocsl_result* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (nrhs < 1) return fail(c, OCSL_BAD_ARGUMENT, "nrhs must be >= 1");
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, OCSL_CUDA_ERROR, "cudaSetDevice");
    const size_t n = (size_t)c->P.n;
    if (method == OCSL_ILU_BICGSTAB_IR32 && nrhs > 1 && n > 0 && c->col_batching &&
        c->ordering == OCSL_ORDER_NATURAL) {
        // groups of up to kMaxCols columns in lockstep; the factor is built once
        int first = OCSL_OK;
        for (int r0 = 0; r0 < nrhs; r0 += kMaxCols) {
            const int nc = std::min(kMaxCols, nrhs - r0);
            const double* bq = b ? b + r0 * n : nullptr;
            double* xq = x ? x + r0 * n : nullptr;
            ocsl_result* oq = out ? out + r0 : nullptr;
            const int st = nc == 1 ? solve_device_impl(c, method, A, bq, xq, opts, oq, r0 > 0)
                                   : solve_cols_impl(c, A, bq, xq, nc, opts, oq, r0 > 0);
            if (st == OCSL_CUDA_ERROR || st == OCSL_BAD_ARGUMENT) return st;
            if (first == OCSL_OK) first = st;
        }
        return first;
    }
    int first = OCSL_OK;
    for (int r = 0; r < nrhs; ++r) {
        ocsl_result one;
        const int st = solve_device_impl(c, method, A, b ? b + r * n : nullptr,
                                         x ? x + r * n : nullptr, opts, &one, r > 0);
        if (out) out[r] = one;
        if (st == OCSL_CUDA_ERROR || st == OCSL_BAD_ARGUMENT) return st;
        if (first == OCSL_OK) first = st;
    }
    return first;
}

int ocsl_solve(ocsl_ctx* c, int method, const double* value, const double* b, double* x,
               const ocsl_opts* opts, ocsl_result* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (c->P.n == 0) {
        if (out) std::memset(out, 0, sizeof *out);
        return OCSL_OK;
    }
    if (!value || !b || !x) return fail(c, OCSL_BAD_ARGUMENT, "null value, b or x pointer");
    const size_t n = (size_t)c->P.n, nnz = (size_t)c->P.nnz;
    try {
        CK(cudaSetDevice(c->device));
        CK(cudaMemcpyAsync(c->d_A, value, nnz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->d_b, b, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    rc = solve_device_impl(c, method, c->d_A, c->d_b, c->d_x, opts, out);
    if (rc == OCSL_CUDA_ERROR) return rc;
    try {
        CK(cudaMemcpyAsync(x, c->d_x, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return rc;
}

int ocsl_gemv_device(ocsl_ctx* c, int mode, double a, const double* val, const double* x,
                     const double* z, double* y)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (mode < 0 || mode > 2 || !val || !x || !y || (mode > 0 && !z))
        return fail(c, OCSL_BAD_ARGUMENT, "bad gemv arguments");
    if (!aligned8(val) || !aligned8(x) || !aligned8(y) || (z && !aligned8(z)))
        return fail(c, OCSL_BAD_ARGUMENT, "device pointers must be 8-byte aligned");
    try {
        CK(cudaSetDevice(c->device));
        launch_spmv<double>(c->stream, c->P, val, x, y, mode, nullptr, a, z, nullptr, nullptr, 0,
                            c->R, nullptr, EP_STORE, 0, 0);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_dot_device(ocsl_ctx* c, size_t n, const double* x, const double* y, double* result)
{
    if (!c || !result) return OCSL_BAD_ARGUMENT;
    if (n >= (size_t)INT32_MAX) return fail(c, OCSL_BAD_ARGUMENT, "n exceeds the int32 limit");
    if (n == 0) { *result = 0.0; return OCSL_OK; }
    if (!x || !y) return fail(c, OCSL_BAD_ARGUMENT, "null vector");
    if (!aligned8(x) || !aligned8(y))
        return fail(c, OCSL_BAD_ARGUMENT, "device pointers must be 8-byte aligned");
    try {
        CK(cudaSetDevice(c->device));
        c->ensure_reduce((int)((n + kTile - 1) / kTile));
        Solve s{c, c->stream, c->P, (int)n};
        s.reset_scalars(2, 0.0);
        s.vec<double>(V_DOT1, {x, y}, 2, EP_STORE);
        CK(cudaGetLastError());
        *result = s.read_scalars(2).sum[0];
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

static int vector_entry(ocsl_ctx* c, size_t n, std::initializer_list<const void*> ptrs, int op,
                        double a, double b, double* result)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (n >= (size_t)INT32_MAX) return fail(c, OCSL_BAD_ARGUMENT, "n exceeds the int32 limit");
    for (const void* p : ptrs)
        if (n > 0 && (!p || !aligned8(p)))
            return fail(c, OCSL_BAD_ARGUMENT, "null or misaligned device pointer");
    if (n == 0) {
        if (result) *result = 0.0;
        return OCSL_OK;
    }
    try {
        CK(cudaSetDevice(c->device));
        c->ensure_reduce((int)((n + kTile - 1) / kTile));
        Solve s{c, c->stream, c->P, (int)n};
        s.reset_scalars(2, 0.0);
        if (!result) {  // elementwise: a and b ride in the scalars block
            Scalars* stage = c->h_sc + kHostStage + 2;
            CK(cudaStreamSynchronize(c->stream));
            stage->alpha = a;
            stage->beta = b;
            stage->done = 0;
            CK(cudaMemcpyAsync(&c->d_sc[2].alpha, &stage->alpha, sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemcpyAsync(&c->d_sc[2].beta, &stage->beta, sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
        }
        s.vec<double>(op, ptrs, 2, EP_STORE);
        CK(cudaGetLastError());
        if (result)
            *result = s.read_scalars(2).sum[0];
        else
            CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_sum_device(ocsl_ctx* c, size_t n, const double* x, int absolute, double* result)
{
    if (!c || !result) return OCSL_BAD_ARGUMENT;
    return vector_entry(c, n, {x}, absolute ? V_ABSSUM : V_SUM, 0.0, 0.0, result);
}

int ocsl_product_device(ocsl_ctx* c, size_t n, const double* x, const double* y, double* out)
{
    return vector_entry(c, n, {x, y, out}, V_PRODUCT, 0.0, 0.0, nullptr);
}

int ocsl_axpy_device(ocsl_ctx* c, size_t n, double a, const double* x, double b, const double* y,
                     double* out)
{
    if (!y) return vector_entry(c, n, {x, x, out}, V_SCALE, a, 0.0, nullptr);
    return vector_entry(c, n, {x, y, out}, V_AXPY, a, b, nullptr);
}

int ocsl_ilu_device(ocsl_ctx* c, const double* A, double* M, int sweeps)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (!A || !M || sweeps < 0 || !aligned8(A) || !aligned8(M))
        return fail(c, OCSL_BAD_ARGUMENT, "bad ilu arguments");
    try {
        CK(cudaSetDevice(c->device));
        Solve s{c, c->stream, c->P, c->P.n};
        c->fac_M = nullptr;
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
        const double* F = s.factor(A, sweeps, false, false, -1);
        CK(cudaMemcpyAsync(M, F, sizeof(double) * (size_t)c->P.nnz, cudaMemcpyDeviceToDevice,
                           c->stream));
        CK(cudaGetLastError());
        // M is written either way (the reference has no check); the status
        // tells the caller that a diagonal of it is zero or infinite
        if (s.device_error() == OCSL_ZERO_PIVOT)
            return fail(c, OCSL_ZERO_PIVOT, "the factor has a zero or infinite pivot");
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

static int sweep_entry(ocsl_ctx* c, bool forward, const double* M, const double* in, double* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (!M || !in || !out || in == out || !aligned8(M) || !aligned8(in) || !aligned8(out))
        return fail(c, OCSL_BAD_ARGUMENT, "bad sweep arguments");
    try {
        CK(cudaSetDevice(c->device));
        Solve s{c, c->stream, c->P, c->P.n};
        c->fac_M = nullptr;
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
        s.prepare_box(M, true, false, false);  // the reference's backsub divides
        if (forward)
            s.fw<double>(M, in, out, -1);
        else
            s.bw<double>(M, nullptr, in, out, 0, -1);
        CK(cudaGetLastError());
        if (s.device_error()) return fail(c, OCSL_TIMEOUT, "a triangular-sweep wait hit its bound");
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_set_sweep_kernel(ocsl_ctx* c, int kind, int tile_a, int tile_b)
{
    if (!c || kind < 0 || kind > 3 || tile_a < 0 || tile_b < 0) return OCSL_BAD_ARGUMENT;
    if (kind == 3 && tile_a > kWaveMaxWarps) return OCSL_BAD_ARGUMENT;
    if (kind >= 2 && c->has_pattern && !c->hp.box.ok)
        return fail(c, OCSL_BAD_ARGUMENT, "the pattern is not a 7-point box stencil");
    c->drop_graph();
    c->fac_M = nullptr;  // the next solve prepares the layouts this kernel reads
    c->sweep_kernel = kind;
    for (int k = 0; k < 2; ++k) {
        if (kind == 3) {  // warps per CTA, start lag
            c->wave_req[k][0] = tile_a;
            c->wave_req[k][1] = tile_b;
        } else {
            c->box_tile[k][0] = tile_a;
            c->box_tile[k][1] = tile_b;
        }
    }
    if (c->has_pattern) {
        c->P.box_ok = c->hp.box.ok && kind != 1;
        c->rebuild_box_geoms();
    }
    return OCSL_OK;
}

int ocsl_set_sweep_cluster(ocsl_ctx* c, int cx, int cy)
{
    const bool automatic = cx == 0 && cy == 0;
    if (!c || (!automatic && (cx < 1 || cy < 1 || cx * cy > kMaxClusterTiles)))
        return OCSL_BAD_ARGUMENT;
    c->drop_graph();
    for (int k = 0; k < 2; ++k) {
        c->box_cluster[k][0] = cx;
        c->box_cluster[k][1] = cy;
    }
    if (c->has_pattern) c->rebuild_box_geoms();
    return OCSL_OK;
}

int ocsl_sweep_geometry(const ocsl_ctx* c, int fp32, int* tiles, int* cluster)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (!c->has_pattern) return OCSL_NO_PATTERN;
    const bool on = c->P.box_ok;
    const BoxGeom& g = fp32 ? c->P.box32 : c->P.box;
    if (tiles) {
        tiles[0] = on ? g.TA : 0;
        tiles[1] = on ? g.TB : 0;
    }
    if (cluster) {
        cluster[0] = on ? g.CX : 0;
        cluster[1] = on ? g.CY : 0;
    }
    return OCSL_OK;
}

int ocsl_wave_geometry(const ocsl_ctx* c, int fp32, int* on, int* warps, int* lag)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (!c->has_pattern) return OCSL_NO_PATTERN;
    const int k = fp32 ? 1 : 0;
    const bool act = c->P.box_ok && c->sweep_kernel != 2 && c->wave_fits[k] &&
                     (c->sweep_kernel == 3 || c->wave_on[k]);
    if (on) *on = act ? 1 : 0;
    if (warps) *warps = act ? c->wave[k].WB : 0;
    if (lag) *lag = act ? c->wave[k].lag : 0;
    return OCSL_OK;
}

int ocsl_autotune_device(ocsl_ctx* c, int method, const double* A, int* tile_a, int* tile_b,
                         double* sweep_us)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (tile_a) *tile_a = 0;
    if (tile_b) *tile_b = 0;
    if (sweep_us) *sweep_us = 0.0;
    if (method < OCSL_CG_REF || method > OCSL_ILU_BICGSTAB_IR32)
        return fail(c, OCSL_BAD_ARGUMENT, "unknown method");
    if (!A || !aligned8(A)) return fail(c, OCSL_BAD_ARGUMENT, "null or misaligned value pointer");
    if (!c->hp.box.ok || c->sweep_kernel == 1 || c->P.n == 0 || method == OCSL_CG_REF ||
        method == OCSL_PCG)
        return OCSL_OK;  // no structured sweep to tune
    const bool fp32 = method == OCSL_ILU_BICGSTAB_IR32;
    const bool ref = method == OCSL_CG_REF || method == OCSL_BICGSTAB_REF;
    const ocsl_opts o = resolve(nullptr);
    // candidate column tiles (one thread per column, at most 256)
    static const int kCand[][2] = {{16, 8}, {16, 16}, {32, 4}, {32, 8}, {8, 16},
                                   {8, 8},  {64, 2},  {64, 4}, {128, 1}, {128, 2}};
    // tiles per thread-block cluster (1 x 1: none)
    static const int kClus[][2] = {{1, 1}, {2, 2}, {4, 2}, {2, 4}, {4, 4}};
    const int pi = fp32 ? 1 : 0;
    BoxGeom& geo = fp32 ? c->P.box32 : c->P.box;  // the geometry this method's sweeps use
    const BoxGeom keep = geo;
    const int kind_keep = c->sweep_kernel;
    const WaveGeom wkeep = c->wave[pi];
    try {
        CK(cudaSetDevice(c->device));
        Solve s{c, c->stream, c->P, c->P.n};
        c->fac_M = nullptr;
        if (fp32) c->ensure_fp32();
        // the factor and stencil records a solve of `method` sweeps with
        // the warp-pipelined kernel's layouts are prepared too while timing it
        struct TuningFlag {
            bool& f;
            explicit TuningFlag(bool& x) : f(x) { f = true; }
            ~TuningFlag() { f = false; }
        } tuning(c->wave_tuning);
        s.factored(A, o.ilu_sweeps, !ref, fp32, -1, !fp32, !ref, fp32);
        const size_t n = (size_t)c->P.n;
        auto pair = [&] {  // one forward + backward sweep of a zero rhs
            if (fp32) {
                s.fw<float>(c->d_M32, c->v32[F_P], c->v32[F_TMP], -1);
                s.bw<float>(c->d_M32, c->d_dinv32, c->v32[F_TMP], c->v32[F_PH], 1, -1);
            } else {
                s.fw<double>(c->fac_M, c->v64[P], c->v64[TMP], -1);
                s.bw<double>(c->fac_M, c->d_dinv, c->v64[TMP], c->v64[PH], ref ? 0 : 1, -1);
            }
        };
        if (fp32)
            CK(cudaMemsetAsync(c->v32[F_P], 0, sizeof(float) * n, c->stream));
        else
            CK(cudaMemsetAsync(c->v64[P], 0, sizeof(double) * n, c->stream));
        auto timed_pair = [&]() {
            pair();  // warm-up
            double t = 1e300;
            for (int rep = 0; rep < 3; ++rep) {
                CK(cudaEventRecord(c->ev_start, c->stream));
                pair();
                CK(cudaEventRecord(c->ev_stop, c->stream));
                CK(cudaEventSynchronize(c->ev_stop));
                float ms = 0.f;
                CK(cudaEventElapsedTime(&ms, c->ev_start, c->ev_stop));
                t = std::min(t, 1000.0 * ms);
            }
            return t;
        };
        // warp-pipelined kernel: warps per CTA x start lag
        double best_wave = 1e300;
        WaveGeom bestw = wkeep;
        if (c->sweep_kernel != 2 && c->wave_fits[pi]) {
            c->sweep_kernel = 3;
            static const int kWarps[] = {1, 2, 3, 4, 6, 8};
            static const int kLags[] = {3, 6, 10};
            std::vector<std::array<int, 2>> wtried;
            for (int wb : kWarps)
            for (int lg : kLags) {
                const WaveGeom g = make_wave_geom(c->hp.box.dim, fp32 ? 4 : 8, wb, lg);
                const std::array<int, 2> key{g.WB, g.lag};
                if (std::find(wtried.begin(), wtried.end(), key) != wtried.end()) continue;
                wtried.push_back(key);
                c->wave[pi] = g;
                const double t = timed_pair();
                if (s.device_error()) {
                    c->sweep_kernel = kind_keep;
                    c->wave[pi] = wkeep;
                    return fail(c, OCSL_TIMEOUT, "a triangular-sweep wait hit its bound");
                }
                if (t < best_wave) {
                    best_wave = t;
                    bestw = g;
                }
            }
            c->sweep_kernel = 2;  // time the CTA kernel's shapes next
        }
        double best = 1e300;
        BoxGeom bestg = keep;
        std::vector<std::array<int, 4>> tried;
        for (const auto& cd : kCand)
        for (const auto& cl : kClus) {
            const BoxGeom g =
                box_with_cluster(make_box_geom(c->hp.box, cd[0], cd[1]), cl[0], cl[1]);
            const std::array<int, 4> key{g.TA, g.TB, g.CX, g.CY};
            if (std::find(tried.begin(), tried.end(), key) != tried.end()) continue;
            tried.push_back(key);
            geo = g;
            const double t = timed_pair();
            if (s.device_error()) {
                geo = keep;
                c->sweep_kernel = kind_keep;
                c->wave[pi] = wkeep;
                return fail(c, OCSL_TIMEOUT, "a triangular-sweep wait hit its bound");
            }
            if (t < best) {
                best = t;
                bestg = g;
            }
        }
        geo = bestg;
        c->drop_graph();
        c->box_tile[pi][0] = bestg.TA;
        c->box_tile[pi][1] = bestg.TB;
        c->box_cluster[pi][0] = bestg.CX;
        c->box_cluster[pi][1] = bestg.CY;
        c->sweep_kernel = kind_keep;
        const bool wave_wins = kind_keep != 2 && best_wave < best;
        // automatic choice: this precision's single-column sweeps use the
        // faster kernel (a forced kind keeps its kernel)
        if (kind_keep == 0) c->wave_on[pi] = wave_wins;
        if (wave_wins || kind_keep == 3) {
            c->wave[pi] = bestw;
            c->wave_req[pi][0] = bestw.WB;
            c->wave_req[pi][1] = bestw.lag;
        } else {
            c->wave[pi] = wkeep;
        }
        c->fac_M = nullptr;
        const int K = wave_cols_per_warp(fp32 ? 4 : 8);
        if (tile_a) *tile_a = wave_wins ? 32 : bestg.TA;
        if (tile_b) *tile_b = wave_wins ? bestw.WB * K : bestg.TB;
        if (sweep_us) *sweep_us = wave_wins ? best_wave : best;
        CK(cudaGetLastError());
    } catch (const CudaError& e) {
        geo = keep;
        c->sweep_kernel = kind_keep;
        c->wave[pi] = wkeep;
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_set_device_loop(ocsl_ctx* c, int enable)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    c->device_loop = enable != 0;
    return OCSL_OK;
}

int ocsl_set_spmv_lanes(ocsl_ctx* c, int lanes)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (lanes == 0) lanes = 1;
    if (lanes != 1 && lanes != 4 && lanes != 16)
        return fail(c, OCSL_BAD_ARGUMENT, "lanes per row must be 0, 1, 4 or 16");
    c->drop_graph();
    c->P.spmv_lanes = lanes;
    return OCSL_OK;
}

int ocsl_spmv_lanes(const ocsl_ctx* c, int* lanes)
{
    if (!c || !lanes) return OCSL_BAD_ARGUMENT;
    if (!c->has_pattern) return OCSL_NO_PATTERN;
    *lanes = c->P.spmv_lanes;
    return OCSL_OK;
}

int ocsl_autotune_spmv_device(ocsl_ctx* c, int method, const double* A, int* lanes,
                              double* spmv_us)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (lanes) *lanes = 0;
    if (spmv_us) *spmv_us = 0.0;
    if (method < OCSL_CG_REF || method > OCSL_ILU_BICGSTAB_IR32)
        return fail(c, OCSL_BAD_ARGUMENT, "unknown method");
    if (!A || !aligned8(A)) return fail(c, OCSL_BAD_ARGUMENT, "null or misaligned value pointer");
    if (c->P.n == 0) return OCSL_OK;
    const bool fp32 = method == OCSL_ILU_BICGSTAB_IR32;
    const int keep = c->P.spmv_lanes;
    try {
        CK(cudaSetDevice(c->device));
        const int n = c->P.n;
        if (fp32) {
            c->ensure_fp32();
            launch_convert_f64_f32(c->stream, c->P.nnz, A, c->d_A32);
            CK(cudaMemsetAsync(c->v32[F_P], 0, sizeof(float) * (size_t)n, c->stream));
        } else {
            CK(cudaMemsetAsync(c->v64[P], 0, sizeof(double) * (size_t)n, c->stream));
        }
        // y = A x with a dot of y, the SpMV of a Krylov step (the x values do
        // not change its time)
        auto spmv = [&] {
            if (fp32)
                launch_spmv<float>(c->stream, c->P, c->d_A32, c->v32[F_P], c->v32[F_TMP], 0,
                                   nullptr, 0.0, nullptr, nullptr, nullptr, DOT_YY, c->R,
                                   nullptr, 0, 0, 0, Cols{});
            else
                launch_spmv<double>(c->stream, c->P, A, c->v64[P], c->v64[TMP], 0, nullptr, 0.0,
                                    nullptr, nullptr, nullptr, DOT_YY, c->R, nullptr, 0, 0, 0,
                                    Cols{});
        };
        static const int kLanes[] = {1, 4, 16};
        double best = 1e300;
        int best_l = keep;
        for (int l : kLanes) {
            c->P.spmv_lanes = l;
            spmv();  // warm-up
            double t = 1e300;
            for (int rep = 0; rep < 5; ++rep) {
                CK(cudaEventRecord(c->ev_start, c->stream));
                spmv();
                CK(cudaEventRecord(c->ev_stop, c->stream));
                CK(cudaEventSynchronize(c->ev_stop));
                float ms = 0.f;
                CK(cudaEventElapsedTime(&ms, c->ev_start, c->ev_stop));
                t = std::min(t, 1000.0 * ms);
            }
            if (t < best) {
                best = t;
                best_l = l;
            }
        }
        c->drop_graph();
        c->P.spmv_lanes = best_l;
        if (lanes) *lanes = best_l;
        if (spmv_us) *spmv_us = best;
        CK(cudaGetLastError());
    } catch (const CudaError& e) {
        c->P.spmv_lanes = keep;
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_sweep_info(const ocsl_ctx* c, int* kind, int* dims, int* tiles)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (!c->has_pattern) return OCSL_NO_PATTERN;
    if (kind)
        *kind = c->sweep_kernel == 0 && c->serial_ok[0] ? 4
                : c->P.fw_nrange > 0 && c->P.bw_nrange > 0 && !c->P.box_ok && c->sweep_kernel <= 1
                    ? 5
                : !c->P.box_ok ? 1
                : (c->sweep_kernel != 2 && c->wave_fits[0] &&
                   (c->sweep_kernel == 3 || c->wave_on[0])) ? 3 : 2;
    if (dims) for (int k = 0; k < 3; ++k) dims[k] = c->hp.box.ok ? c->hp.box.dim[k] : 0;
    if (tiles) {
        tiles[0] = c->P.box_ok ? c->P.box.TA : 0;
        tiles[1] = c->P.box_ok ? c->P.box.TB : 0;
    }
    return OCSL_OK;
}

int ocsl_inject_fault(ocsl_ctx* c, int kind)
{
    if (!c || kind < OCSL_FAULT_NONE || kind > OCSL_FAULT_SKIP_FIRST_TILE) return OCSL_BAD_ARGUMENT;
    c->fault_skip_pending = kind == OCSL_FAULT_SKIP_FIRST_TILE;
    return OCSL_OK;
}

int ocsl_set_graphs(ocsl_ctx* c, int enable)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    c->graphs_on = enable != 0;
    if (!c->graphs_on) c->drop_graph();
    if (c->tctx) ocsl_set_graphs(c->tctx, enable);
    if (c->cctx) ocsl_set_graphs(c->cctx, enable);
    return OCSL_OK;
}

int ocsl_set_ordering(ocsl_ctx* c, int ordering)
{
    if (!c || (ordering != OCSL_ORDER_NATURAL && ordering != OCSL_ORDER_MULTICOLOUR))
        return OCSL_BAD_ARGUMENT;
    c->ordering = ordering;
    if (c->tctx) ocsl_set_ordering(c->tctx, ordering);  // transposed solves follow
    return OCSL_OK;
}

int ocsl_ordering_info(const ocsl_ctx* c, int* ordering, int* colours, int32_t* levels,
                       int* stencil)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (ordering) *ordering = c->ordering;
    if (colours) *colours = c->cctx ? c->colours : 0;
    if (stencil) *stencil = c->cctx && c->cctx->rb_ok ? 1 : 0;
    if (levels) {
        levels[0] = c->cctx ? c->cctx->hp.fw_levels : 0;
        levels[1] = c->cctx ? c->cctx->hp.bw_levels : 0;
    }
    return OCSL_OK;
}

int ocsl_ordering_permutation(ocsl_ctx* c, int32_t* perm, size_t n)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (n != (size_t)c->P.n || (n > 0 && !perm))
        return fail(c, OCSL_BAD_ARGUMENT, "perm must hold n entries");
    if (n == 0) return OCSL_OK;
    try {
        CK(cudaSetDevice(c->device));
        rc = ensure_coloured(c);
        if (rc) return rc;
        CK(cudaMemcpy(perm, c->d_cperm, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_set_col_batching(ocsl_ctx* c, int enable)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    if (enable < 0 || enable > 2) return OCSL_BAD_ARGUMENT;
    c->drop_graph();
    c->col_batching = enable;
    return OCSL_OK;
}

int ocsl_profile_enable(ocsl_ctx* c, int enable)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    c->prof_on = enable != 0;
    if (c->cctx) c->cctx->prof_on = c->prof_on;
    return OCSL_OK;
}

int ocsl_profile_read(ocsl_ctx* c, double* ms, int64_t* launches)
{
    if (!c) return OCSL_BAD_ARGUMENT;
    for (int k = 0; k < PC_COUNT; ++k) {
        if (ms) ms[k] = 0.0;
        if (launches) launches[k] = 0;
    }
    try {
        CK(cudaStreamSynchronize(c->stream));
        for (size_t i = 0; i < c->prof_used; ++i) {
            float t = 0.f;
            CK(cudaEventElapsedTime(&t, c->prof_ev[2 * i], c->prof_ev[2 * i + 1]));
            const int k = c->prof_cat[i];
            if (ms) ms[k] += t;
            if (launches) launches[k] += 1;
        }
    } catch (const CudaError& e) {
        c->prof_used = 0;
        c->prof_cat.clear();
        return from_cuda(c, e);
    }
    c->prof_used = 0;
    c->prof_cat.clear();
    if (c->cctx) {  // the kernels of solves through the multicolour ordering
        double cms[PC_COUNT];
        int64_t cl[PC_COUNT];
        const int rc = ocsl_profile_read(c->cctx, cms, cl);
        if (rc != OCSL_OK) return fail(c, rc, c->cctx->last_error);
        for (int k = 0; k < PC_COUNT; ++k) {
            if (ms) ms[k] += cms[k];
            if (launches) launches[k] += cl[k];
        }
    }
    return OCSL_OK;
}

const char* ocsl_profile_category_name(int k)
{
    return (k >= 0 && k < PC_COUNT) ? kProfNames[k] : "unknown";
}

int ocsl_set_faces(ocsl_ctx* c, int64_t n_faces, const int32_t* left, const int32_t* right,
                   int64_t n_bc, const int32_t* bc_left)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if ((n_faces > 0 && (!left || !right)) || (n_bc > 0 && !bc_left))
        return fail(c, OCSL_BAD_ARGUMENT, "null face array");
    try {
        CK(cudaSetDevice(c->device));
        const int n = c->P.n, nnz = c->P.nnz;
        std::vector<int> rp(n + 1), col(nnz);
        CK(cudaMemcpy(rp.data(), c->P.rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
        if (nnz) CK(cudaMemcpy(col.data(), c->P.col, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
        FaceTables ft;
        std::string err;
        if (!build_face_tables(n, rp, col, n_faces, left, right, n_bc, bc_left, ft, err))
            return fail(c, OCSL_BAD_ARGUMENT, err);
        CK(cudaStreamSynchronize(c->stream));
        for (auto& p : c->d_faces) { if (p) cudaFree(p); p = nullptr; }
        for (double** pp : {&c->d_fmu, &c->d_fpdum}) { if (*pp) cudaFree(*pp); *pp = nullptr; }
        c->drop_flow_graph();  // its launches read the old face tables and buffers
        c->has_faces = false;
        c->flow_bc_checked = nullptr;
        const std::vector<int> l(left, left + n_faces), r(right, right + n_faces),
            bl(bc_left, bc_left + n_bc);
        const std::vector<int>* tabs[8] = {&l, &r, &bl, &ft.cell_ptr, &ft.cell_ent, &ft.cell_slot,
                                           &ft.bc_ptr, &ft.bc_ent};
        for (int i = 0; i < 8; ++i) c->d_faces[i] = upload(*tabs[i]);
        DevFaces& F = c->F;
        F.nf = (int)n_faces;
        F.nb = (int)n_bc;
        F.left = c->d_faces[0];
        F.right = c->d_faces[1];
        F.bc_left = c->d_faces[2];
        F.cell_ptr = c->d_faces[3];
        F.cell_ent = c->d_faces[4];
        F.cell_slot = c->d_faces[5];
        F.bc_ptr = c->d_faces[6];
        F.bc_ent = c->d_faces[7];
        c->has_faces = true;
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

static int check_assembly(ocsl_ctx* c, const ocsl_assembly* q, const ocsl_flow_state* s)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (!c->has_faces) return fail(c, OCSL_BAD_ARGUMENT, "ocsl_set_faces has not been called");
    if (!q || !s) return fail(c, OCSL_BAD_ARGUMENT, "null assembly or state");
    if (q->equation < OCSL_EQ_MOMENTUM || q->equation > OCSL_EQ_HEAT)
        return fail(c, OCSL_BAD_ARGUMENT, "unknown equation");
    if (q->equation == OCSL_EQ_MOMENTUM && (q->dimension < 0 || q->dimension > 2))
        return fail(c, OCSL_BAD_ARGUMENT, "momentum dimension must be 0, 1 or 2");
    if (const char* m = missing_state_field(*q, *s, c->F.nf > 0, c->F.nb > 0))
        return fail(c, OCSL_BAD_ARGUMENT, std::string("state field needed but NULL: ") + m);
    return OCSL_OK;
}

int ocsl_assemble_device(ocsl_ctx* c, const ocsl_assembly* q, const ocsl_flow_state* s,
                         double* value, double* b, double* x0, double* ap, double* total_mdot)
{
    int rc = check_assembly(c, q, s);
    if (rc) return rc;
    if (c->P.n == 0) return OCSL_OK;
    if (!value || !b || !x0) return fail(c, OCSL_BAD_ARGUMENT, "null value, b or x0");
    try {
        CK(cudaSetDevice(c->device));
        launch_assemble(c->stream, c->P, c->F, *q, *s, value, b, x0, ap, total_mdot);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

// ------------------------------------------------------------------ SIMPLE iteration

// The state arrays the iteration needs, checked for presence; the FlowDev view.
static int flow_view(ocsl_ctx* c, const ocsl_assembly* q, const ocsl_flow_state* s,
                     const ocsl_flow_iteration* it, FlowDev& f)
{
    int rc = check_assembly(c, q, s);
    if (rc) return rc;
    if (!it) return fail(c, OCSL_BAD_ARGUMENT, "null iteration arguments");
    const bool nf = c->F.nf > 0, nb = c->F.nb > 0;
    for (int e : {OCSL_EQ_MOMENTUM, OCSL_EQ_PRESSURE, OCSL_EQ_ENTHALPY}) {
        ocsl_assembly qe = *q;
        qe.equation = e;
        if (const char* miss = missing_state_field(qe, *s, nf, nb))
            return fail(c, OCSL_BAD_ARGUMENT, std::string("state field ") + miss + " is NULL");
    }
    struct Need {
        const void* p;
        const char* name;
        bool want;
    };
    const Need need[] = {
        {s->density, "density", nf}, {s->qy, "qy", nf}, {s->stress, "stress", nf && q->viscous},
        {s->temperature, "temperature", true}, {s->pressure, "pressure", true},
        {s->pressure_last, "pressure_last", true},
        {s->bc_area, "bc_area", nb}, {s->bc_area_vector, "bc_area_vector", nb},
        {s->bc_mdot, "bc_mdot", nb}, {s->bc_density, "bc_density", nb}, {s->bc_qy, "bc_qy", nb},
        {s->bc_enthalpy, "bc_enthalpy", nb}, {s->bc_temperature, "bc_temperature", nb},
        {s->bc_velocity, "bc_velocity", nb}, {s->bc_supersonic, "bc_supersonic", nb},
        {it->face_area_vector, "face_area_vector", nf}, {it->face_alpha, "face_alpha", nf},
        {it->face_distance, "face_distance", nf}, {it->face_unit, "face_unit", nf},
        {it->bc_distance, "bc_distance", nb}, {it->bc_unit, "bc_unit", nb},
        {it->bc_alpha, "bc_alpha", nb}, {it->bc_out_pressure, "bc_out_pressure", nb},
        {it->bc_pressure, "bc_pressure", nb}, {it->pressure_corr_grad, "pressure_corr_grad", true},
        {it->ap, "ap", true}, {it->ap_vec, "ap_vec", true}, {it->mach, "mach", true},
        {it->total_mdot, "total_mdot", true}};
    for (const Need& x : need)
        if (x.want && !x.p) return fail(c, OCSL_BAD_ARGUMENT, std::string(x.name) + " is NULL");
    // boundary kinds within ocsl_bc_type (checked once per array)
    if (nb && c->flow_bc_checked != s->bc_type) {
        std::vector<int32_t> kind(c->F.nb);
        CK(cudaMemcpy(kind.data(), s->bc_type, sizeof(int32_t) * kind.size(),
                      cudaMemcpyDeviceToHost));
        for (int32_t k : kind)
            if (k < OCSL_BC_EMPTY || k > OCSL_BC_PRESSURE_OUTLET)
                return fail(c, OCSL_BAD_ARGUMENT, "a boundary kind outside ocsl_bc_type");
        c->flow_bc_checked = s->bc_type;
    }
    auto w = [](const double* p) { return const_cast<double*>(p); };
    f.pressure = w(s->pressure);
    f.velocity = w(s->velocity);
    f.velocity_last = w(s->velocity_last);
    f.density_c = w(s->density_c);
    f.density_last = w(s->density_last);
    f.pressure_last = w(s->pressure_last);
    f.temperature = w(s->temperature);
    f.enthalpy = w(s->enthalpy);
    f.enthalpy_last = w(s->enthalpy_last);
    f.pressure_corr = w(s->pressure_corr);
    f.pressure_grad = w(s->pressure_grad);
    f.pressure_corr_grad = it->pressure_corr_grad;
    f.ap = it->ap;
    f.ap_vec = it->ap_vec;
    f.mach = it->mach;
    f.volume = s->volume;
    f.left = c->F.left;
    f.right = c->F.right;
    f.geo_aver = s->geo_aver;
    f.area_vector = it->face_area_vector;
    f.alpha = it->face_alpha;
    f.distance = it->face_distance;
    f.unit = it->face_unit;
    f.mdot = w(s->mdot);
    f.face_density = w(s->density);
    f.qy = w(s->qy);
    f.stress = w(s->stress);
    f.bc_type = s->bc_type;
    f.bc_left = c->F.bc_left;
    f.bc_area = s->bc_area;
    f.bc_area_vector = s->bc_area_vector;
    f.bc_unit = it->bc_unit;
    f.bc_alpha = it->bc_alpha;
    f.bc_distance = it->bc_distance;
    f.bc_out_pressure = it->bc_out_pressure;
    f.bc_pressure = it->bc_pressure;
    f.bc_mdot = w(s->bc_mdot);
    f.bc_density = w(s->bc_density);
    f.bc_qy = w(s->bc_qy);
    f.bc_enthalpy = w(s->bc_enthalpy);
    f.bc_temperature = w(s->bc_temperature);
    f.bc_velocity = w(s->bc_velocity);
    f.bc_supersonic = const_cast<int*>(s->bc_supersonic);
    f.relax_p = it->relax_p;
    f.relax_u = it->relax_u;
    f.cp = it->cp;
    f.Tref = it->Tref;
    f.H_formation = it->H_formation;
    f.R = q->R_specific;
    f.gamma = q->gamma;
    f.suth0 = q->sutherland[0];
    f.suth1 = q->sutherland[1];
    return OCSL_OK;
}

}  // extern "C"

// The launches of one inner iteration on `st`, in the reference's order
// (cflow_solver.cpp:229-476).  solve(slot, method) enqueues the linear solve
// of equation slot (0-2 momentum, 3 p', 4 enthalpy) on the system in
// d_fval / d_fb / d_fx.
template <typename SolveFn>
static void enqueue_flow(ocsl_ctx* c, cudaStream_t st, const ocsl_assembly* q,
                         const ocsl_flow_state* s, const ocsl_flow_iteration* it,
                         const int* methods, const FlowDev& f, SolveFn&& solve)
{
    const int n = c->P.n, nf = c->F.nf, nb = c->F.nb;
    Solve sv{c, st, c->P, n};
    CK(cudaMemsetAsync(c->d_sc + kScFlow, 0, sizeof(Scalars), st));
    auto residual = [&](const double* v, int slot) {  // sum |v| in tile order
        sv.vec<double>(V_ABSSUM, {v}, kScFlow, EP_STORE);
        launch_take_sum(st, c->d_sc + kScFlow, c->d_fout->residual + slot);
    };
    ocsl_assembly qe = *q;
    // boundary conditions and the pressure gradient (:234-241)
    launch_flow_set_bc(st, n, nb, f);
    launch_flow_grad(st, false, n, nf, nb, f, c->F);
    CK(cudaMemsetAsync(f.ap, 0, sizeof(double) * n, st));  // :244-247
    // :250-255; and mu(T_f) per face for the momentum and enthalpy assemblies
    // (the temperature changes only in the enthalpy update at the end)
    launch_flow_stress(st, n, nf, f, q->viscous != 0);
    // momentum components (:257-302)
    for (int d = 0; d < 3; ++d) {
        qe.equation = OCSL_EQ_MOMENTUM;
        qe.dimension = d;
        launch_assemble(st, c->P, c->F, qe, *s, c->d_fval, c->d_fb, c->d_fx,
                        f.ap_vec + (size_t)d * n, it->total_mdot, f.face_mu);
        solve(d, methods[0]);
        launch_flow_velocity_update(st, n, d, c->d_fx, f, c->d_ftmp);
        residual(c->d_ftmp, d);
    }
    // face mass fluxes (:305-309), pressure correction (:316-358)
    launch_flow_face_mdot(st, n, nf, nb, f, q->blended);  // and the boundary faces', :312-315
    qe.equation = OCSL_EQ_PRESSURE;
    qe.dimension = 0;
    launch_assemble(st, c->P, c->F, qe, *s, c->d_fval, c->d_fb, c->d_fx, nullptr, it->total_mdot,
                    nullptr, f.face_pdum);
    residual(c->d_fb, 3);  // Pressure_global_residual = ABSsum(b), :346
    solve(3, methods[1]);
    launch_flow_pcorr(st, n, nb, c->d_fx, f);  // and the boundary pressures, :361-372
    // corrections (:375-426)
    launch_flow_grad(st, true, n, nf, nb, f, c->F);
    launch_flow_correct(st, n, nf, nb, f, q->blended);
    // enthalpy (:428-474)
    qe.equation = OCSL_EQ_ENTHALPY;
    launch_assemble(st, c->P, c->F, qe, *s, c->d_fval, c->d_fb, c->d_fx, nullptr, nullptr,
                    f.face_mu);
    solve(4, methods[2]);
    launch_flow_enthalpy_update(st, n, c->d_fx, f, c->d_ftmp);
    residual(c->d_ftmp, 4);
}

static bool capturable(cudaStream_t st)
{
    return st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
}

// Reference-faithful solves only: the whole iteration as one CUDA graph.  The
// solves start from the device copy of their scalars, their iteration counts
// and error words are copied aside on the device, and the outputs come back
// in one copy at the end -- no host round trip inside.  The graph runs on the
// caller's stream, or (the legacy default stream cannot be captured) on the
// context's own stream joined to the caller's by events.
static int flow_iterate_graphed(ocsl_ctx* c, const ocsl_assembly* q, const ocsl_flow_state* s,
                                const ocsl_flow_iteration* it, const int* methods,
                                const ocsl_opts& o, const FlowDev& f, ocsl_flow_report& rep)
{
    std::vector<unsigned char> key;
    auto add = [&](const void* p, size_t bytes) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + bytes);
    };
    add(q, sizeof *q);
    add(s, sizeof *s);
    add(it, sizeof *it);
    add(methods, 3 * sizeof(int));
    add(&o.ilu_sweeps, sizeof o.ilu_sweeps);
    add(&o.tol, sizeof o.tol);  // the FP32-refined solves' tolerances and budgets too
    add(&o.maxit, sizeof o.maxit);
    add(&o.inner_tol, sizeof o.inner_tol);
    add(&o.inner_maxit, sizeof o.inner_maxit);
    add(&c->stream, sizeof c->stream);
    if (key != c->flow_key) {
        c->drop_flow_graph();
        c->flow_key = key;
    }
    if (!c->d_sc_ref) {
        Scalars init;
        std::memset(&init, 0, sizeof init);
        init.alpha = init.omega = init.rhon = init.rho = 1.0;
        c->d_sc_ref = dalloc<Scalars>(1);
        CK(cudaMemcpy(c->d_sc_ref, &init, sizeof init, cudaMemcpyHostToDevice));
        CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    }
    bool ir32 = false;
    for (int e = 0; e < 3; ++e) ir32 = ir32 || methods[e] == OCSL_ILU_BICGSTAB_IR32;
    if (ir32) {  // everything a captured FP32-refined solve needs, allocated outside the capture
        c->ensure_fp32();
        ensure_irctl(c, 5);
        if (!c->capture_stream)
            CK(cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking));
    }
    const cudaStream_t caller = c->stream;
    const cudaStream_t work = capturable(caller) ? caller : c->own_stream;
    if (work != caller) {
        CK(cudaEventRecord(c->ev_fork, caller));
        CK(cudaStreamWaitEvent(work, c->ev_fork, 0));
    }
    auto enqueue = [&] {
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), work));
        enqueue_flow(c, work, q, s, it, methods, f, [&](int slot, int method) {
            Solve sv{c, work, c->P, c->P.n};
            c->fac_M = nullptr;
            if (method == OCSL_ILU_BICGSTAB_IR32) {
                cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
                CK(cudaStreamIsCapturing(work, &cs));
                if (cs == cudaStreamCaptureStatusActive) {
                    // the factor, the records and the device-driven loops
                    sv.factored(c->d_fval, o.ilu_sweeps, true, true, -1, false, true, true);
                    sv.prepare_spmv(c->d_fval, true, true);
                    IrCtl* ctl = static_cast<IrCtl*>(c->d_irctl) + slot;
                    capture_ir32_inline(sv, c->capture_stream, c->d_fval, c->d_fb, c->d_fx, o,
                                        ctl);
                    ir_flow_out_kernel<<<1, 1, 0, work>>>(ctl, c->d_err,
                                                          c->d_fout->iterations + slot,
                                                          c->d_fout->err + slot);
                } else {
                    // the first call of a key runs directly (it allocates)
                    const TolResult t =
                        run_bicgstab_ir32(sv, c->d_fval, c->d_fb, c->d_fx, o);
                    const int derr = sv.device_error();
                    const int out[2] = {t.iters, derr ? derr : t.status};
                    CK(cudaMemcpy(c->d_fout->iterations + slot, &out[0], sizeof(int),
                                  cudaMemcpyHostToDevice));
                    CK(cudaMemcpy(c->d_fout->err + slot, &out[1], sizeof(int),
                                  cudaMemcpyHostToDevice));
                    CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), work));
                }
                return;
            }
            if (method == OCSL_CG_REF)
                run_cg_ref(sv, c->d_fval, c->d_fb, c->d_fx, true);
            else
                run_bicgstab_ref(sv, c->d_fval, c->d_fb, c->d_fx, o.ilu_sweeps, true);
            CK(cudaMemcpyAsync(c->d_fout->iterations + slot, &c->d_sc[0].iters, sizeof(int),
                               cudaMemcpyDeviceToDevice, work));
            CK(cudaMemcpyAsync(c->d_fout->err + slot, c->d_err, sizeof(int),
                               cudaMemcpyDeviceToDevice, work));
            CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), work));
        });
        CK(cudaMemcpyAsync(c->h_fout, c->d_fout, sizeof *c->h_fout, cudaMemcpyDeviceToHost, work));
    };
    bool launched = false;
    if (!c->flow_exec && c->flow_seen >= 1) {
        if (cudaStreamBeginCapture(work, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            cudaGraph_t g = nullptr;
            try {
                enqueue();
            } catch (...) {
                cudaStreamEndCapture(work, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            cudaError_t e = cudaStreamEndCapture(work, &g);
            cudaGraphExec_t exec = nullptr;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e == cudaSuccess)
                c->flow_exec = exec;
            else
                cudaGetLastError();  // capture refused: run directly below
        } else {
            cudaGetLastError();
        }
    }
    if (c->flow_exec) {
        CK(cudaGraphLaunch(c->flow_exec, work));
        launched = true;
    }
    if (!launched) enqueue();
    ++c->flow_seen;
    if (work != caller) {
        CK(cudaEventRecord(c->ev_join, work));
        CK(cudaStreamWaitEvent(caller, c->ev_join, 0));
    }
    CK(cudaStreamSynchronize(work));
    CK(cudaGetLastError());
    int status = OCSL_OK;
    for (int e = 0; e < 5; ++e) {
        rep.residual[e] = c->h_fout->residual[e];
        rep.iterations[e] = c->h_fout->iterations[e];
        rep.status[e] = c->h_fout->err[e];
        if (rep.status[e] && status == OCSL_OK) status = rep.status[e];
    }
    if (status != OCSL_OK) {
        // host-side choices baked into the graph may no longer hold
        if (status == OCSL_TIMEOUT) c->wave_faces_dirty = true;
        c->drop_flow_graph();
        c->last_error = status == OCSL_TIMEOUT      ? "a triangular-sweep wait hit its bound"
                        : status == OCSL_ZERO_PIVOT ? "the factor has a zero or infinite pivot"
                                                    : ocsl_status_string(status);
    }
    return status;
}

extern "C" {

int ocsl_flow_iterate_device(ocsl_ctx* c, const ocsl_assembly* q, const ocsl_flow_state* s,
                             const ocsl_flow_iteration* it, const int* methods,
                             const ocsl_opts* opts, ocsl_flow_report* report)
{
    if (report) std::memset(report, 0, sizeof *report);
    if (!methods) return c ? fail(c, OCSL_BAD_ARGUMENT, "null methods") : OCSL_BAD_ARGUMENT;
    // one CUDA graph per iteration: the reference's solvers, and the
    // FP32-refined one with its loops on the device (ocsl_set_device_loop)
    bool graphable = true;
    for (int e = 0; e < 3; ++e) {
        if (methods[e] < OCSL_CG_REF || methods[e] > OCSL_ILU_BICGSTAB_IR32)
            return c ? fail(c, OCSL_BAD_ARGUMENT, "unknown method") : OCSL_BAD_ARGUMENT;
        graphable = graphable &&
                    (methods[e] == OCSL_CG_REF || methods[e] == OCSL_BICGSTAB_REF ||
                     (methods[e] == OCSL_ILU_BICGSTAB_IR32 && c && c->device_loop &&
                      c->ordering != OCSL_ORDER_MULTICOLOUR));
    }
    FlowDev f{};
    int status = OCSL_OK;
    ocsl_flow_report rep{};
    try {
        int rc = flow_view(c, q, s, it, f);
        if (rc) return rc;
        CK(cudaSetDevice(c->device));
        const int n = c->P.n;
        if (n == 0) {
            if (report) *report = rep;
            return OCSL_OK;
        }
        if (!c->d_fval) {
            c->d_fval = dalloc<double>((size_t)c->P.nnz);
            c->d_fb = dalloc<double>((size_t)n);
            c->d_fx = dalloc<double>((size_t)n);
            c->d_ftmp = dalloc<double>((size_t)n);
            c->d_fvolap = dalloc<double>((size_t)n);
        }
        if (!c->d_fmu && c->F.nf > 0) {
            c->d_fmu = dalloc<double>((size_t)c->F.nf);
            c->d_fpdum = dalloc<double>((size_t)c->F.nf);
        }
        f.face_mu = c->d_fmu;
        f.face_pdum = c->d_fpdum;
        f.vol_ap = c->d_fvolap;
        if (!c->d_fout) {
            c->d_fout = dalloc<ocsl_ctx::FlowOut>(1);
            CK(cudaMallocHost(&c->h_fout, sizeof *c->h_fout));
        }
        const ocsl_opts o = resolve(opts);
        if (graphable && c->graphs_on && !c->prof_on && !c->fault_skip_pending) {
            status = flow_iterate_graphed(c, q, s, it, methods, o, f, rep);
        } else {
            // solves through the ordinary entry (tolerance-mode iterations
            // look at their scalars between batches)
            const cudaStream_t st = c->stream;
            enqueue_flow(c, st, q, s, it, methods, f, [&](int slot, int method) {
                ocsl_result r;
                const int rc2 = solve_device_impl(c, method, c->d_fval, c->d_fb, c->d_fx, &o, &r);
                rep.iterations[slot] = r.iterations;
                rep.status[slot] = rc2;
                if (rc2 != OCSL_OK && status == OCSL_OK) status = rc2;
            });
            CK(cudaMemcpyAsync(c->h_fout, c->d_fout, sizeof *c->h_fout, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            std::memcpy(rep.residual, c->h_fout->residual, sizeof rep.residual);
            CK(cudaGetLastError());
        }
    } catch (const CudaError& e) {
        c->drop_flow_graph();
        status = from_cuda(c, e);
    }
    if (report) *report = rep;
    return status;
}

int ocsl_flow_end_step_device(ocsl_ctx* c, const ocsl_flow_state* s)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (!s || !s->velocity || !s->velocity_last || !s->density_c || !s->density_last ||
        !s->pressure || !s->pressure_last || !s->enthalpy || !s->enthalpy_last)
        return fail(c, OCSL_BAD_ARGUMENT, "null state field");
    try {
        CK(cudaSetDevice(c->device));
        FlowDev f{};
        auto w = [](const double* p) { return const_cast<double*>(p); };
        f.velocity = w(s->velocity);
        f.velocity_last = w(s->velocity_last);
        f.density_c = w(s->density_c);
        f.density_last = w(s->density_last);
        f.pressure = w(s->pressure);
        f.pressure_last = w(s->pressure_last);
        f.enthalpy = w(s->enthalpy);
        f.enthalpy_last = w(s->enthalpy_last);
        launch_flow_end_step(c->stream, c->P.n, f);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_bc_value_grad_device(ocsl_ctx* c, const ocsl_assembly* q, const ocsl_flow_state* s,
                              const double* lambda, double* grad)
{
    int rc = check_assembly(c, q, s);
    if (rc) return rc;
    if (c->F.nb == 0) return OCSL_OK;
    if (!lambda || !grad) return fail(c, OCSL_BAD_ARGUMENT, "null lambda or grad");
    try {
        CK(cudaSetDevice(c->device));
        launch_bc_value_grad(c->stream, c->F, *q, *s, lambda, grad);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_solve_transpose_device(ocsl_ctx* c, int method, const double* val, const double* g,
                                double* lambda, const ocsl_opts* opts, ocsl_result* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (c->P.n == 0) {
        if (out) std::memset(out, 0, sizeof *out);
        return OCSL_OK;
    }
    if (!val || !g || !lambda) return fail(c, OCSL_BAD_ARGUMENT, "null value, g or lambda pointer");
    if (!aligned8(val) || !aligned8(g) || !aligned8(lambda))
        return fail(c, OCSL_BAD_ARGUMENT, "device pointers must be 8-byte aligned");
    try {
        CK(cudaSetDevice(c->device));
        rc = ensure_transpose(c);
        if (rc) return rc;
        c->tctx->stream = c->stream;
        launch_gather_values(c->stream, c->nnzT, c->d_tperm, val, c->tctx->d_A);
        CK(cudaGetLastError());
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    rc = solve_device_impl(c->tctx, method, c->tctx->d_A, g, lambda, opts, out);
    if (rc != OCSL_OK) c->last_error = c->tctx->last_error;
    return rc;
}

int ocsl_solve_transpose(ocsl_ctx* c, int method, const double* value, const double* g,
                         double* lambda, const ocsl_opts* opts, ocsl_result* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (c->P.n == 0) {
        if (out) std::memset(out, 0, sizeof *out);
        return OCSL_OK;
    }
    if (!value || !g || !lambda) return fail(c, OCSL_BAD_ARGUMENT, "null value, g or lambda pointer");
    const size_t n = (size_t)c->P.n, nnz = (size_t)c->P.nnz;
    try {
        CK(cudaSetDevice(c->device));
        CK(cudaMemcpyAsync(c->d_A, value, nnz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->d_b, g, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->d_x, lambda, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    rc = ocsl_solve_transpose_device(c, method, c->d_A, c->d_b, c->d_x, opts, out);
    if (rc == OCSL_CUDA_ERROR || rc == OCSL_BAD_PATTERN) return rc;
    try {
        CK(cudaMemcpyAsync(lambda, c->d_x, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return rc;
}

int ocsl_pattern_outer_device(ocsl_ctx* c, double alpha, const double* u, const double* v,
                              double* out)
{
    int rc = check_ready(c);
    if (rc) return rc;
    if (c->P.n == 0) return OCSL_OK;
    if (!u || !v || !out) return fail(c, OCSL_BAD_ARGUMENT, "null u, v or out pointer");
    if (!aligned8(u) || !aligned8(v) || !aligned8(out))
        return fail(c, OCSL_BAD_ARGUMENT, "device pointers must be 8-byte aligned");
    try {
        CK(cudaSetDevice(c->device));
        launch_pattern_outer(c->stream, c->P, alpha, u, v, out);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    } catch (const CudaError& e) {
        return from_cuda(c, e);
    }
    return OCSL_OK;
}

int ocsl_forsub_device(ocsl_ctx* c, const double* M, const double* b, double* y)
{
    return sweep_entry(c, true, M, b, y);
}

int ocsl_backsub_device(ocsl_ctx* c, const double* M, const double* y, double* x)
{
    return sweep_entry(c, false, M, y, x);
}

}  // extern "C"
