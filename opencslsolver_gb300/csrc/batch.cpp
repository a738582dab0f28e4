// Batched solves of many independent systems (ocsl_batch_*, include/ocsl.h).
//
// The systems of a batch are small compared to the GPU (10^4 - 5 x 10^5 rows):
// one system's solve leaves most SMs idle -- its triangular sweeps are a
// latency-bound wavefront over a few hundred rows -- so throughput comes from
// running many solves at once.  A batch keeps one context per system (pattern
// analysed once, device memory reused from call to call) and a pool of host
// worker threads; each worker owns one CUDA stream, binds the context of the
// system it takes to that stream and drives the solve (the tolerance-mode
// drivers look at the Krylov scalars between batches of iterations, so a
// solve needs a host thread to drive it).  Workers take systems largest
// first, so the tail of the batch is short; the right-hand sides of one
// system share its factor (ocsl_solve_multi_device).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <atomic>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ocsl.h"
#include "ir32_graph.h"

struct ocsl_batch {
    int device = 0;
    std::vector<ocsl_ctx*> ctx;
    std::vector<size_t> n;
    std::vector<int> nrhs;
    std::vector<size_t> result_offset;
    std::vector<int> order;  // systems, largest first
    std::vector<cudaStream_t> streams;
    std::string last_error;
    std::mutex err_mutex;
    // one-graph mode: the instantiated graph of every solve and what it was
    // captured for (method, options, pointers, systems included)
    bool graph_mode = false;
    cudaGraphExec_t exec = nullptr;
    std::vector<const void*> key_ptrs;
    std::vector<char> key_in;
    ocsl_opts key_opts{};
};

namespace {

void destroy(ocsl_batch* b)
{
    cudaSetDevice(b->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (ocsl_ctx* c : b->ctx)
        if (c) ocsl_destroy(c);
    for (cudaStream_t s : b->streams)
        if (s) cudaStreamDestroy(s);
    delete b;
}

}  // namespace

extern "C" {

int ocsl_batch_create(ocsl_batch** out, int device, int count, const ocsl_batch_system* sys,
                      int workers)
{
    if (!out || count < 0 || (count > 0 && !sys)) return OCSL_BAD_ARGUMENT;
    *out = nullptr;
    auto* b = new ocsl_batch();
    b->device = device;
    b->ctx.assign(count, nullptr);
    size_t off = 0;
    for (int i = 0; i < count; ++i) {
        if (sys[i].nrhs < 1) {
            destroy(b);
            return OCSL_BAD_ARGUMENT;
        }
        int rc = ocsl_create(&b->ctx[i], device);
        // single-tile sweeps: the systems run concurrently on several streams,
        // and clustered sweeps would hold whole SMs per CTA
        if (rc == OCSL_OK) rc = ocsl_set_sweep_cluster(b->ctx[i], 1, 1);
        if (rc == OCSL_OK) rc = ocsl_set_pattern(b->ctx[i], sys[i].n, sys[i].row_ptr,
                                                 sys[i].column_index);
        if (rc != OCSL_OK) {
            destroy(b);
            return rc;
        }
        b->n.push_back(sys[i].n);
        b->nrhs.push_back(sys[i].nrhs);
        b->result_offset.push_back(off);
        off += (size_t)sys[i].nrhs;
    }
    b->order.resize(count);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
        return b->n[x] * (size_t)b->nrhs[x] > b->n[y] * (size_t)b->nrhs[y];
    });
    const int w = std::max(1, std::min(workers > 0 ? workers : 8, std::max(count, 1)));
    if (cudaSetDevice(device) != cudaSuccess) {
        destroy(b);
        return OCSL_CUDA_ERROR;
    }
    b->streams.assign(w, nullptr);
    for (auto& s : b->streams) {
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            destroy(b);
            return OCSL_CUDA_ERROR;
        }
    }
    *out = b;
    return OCSL_OK;
}

int ocsl_batch_destroy(ocsl_batch* b)
{
    if (!b) return OCSL_BAD_ARGUMENT;
    destroy(b);
    return OCSL_OK;
}

int ocsl_batch_set_graph(ocsl_batch* b, int enable)
{
    if (!b) return OCSL_BAD_ARGUMENT;
    b->graph_mode = enable != 0;
    return OCSL_OK;
}

}  // extern "C"

namespace {

void note_error(ocsl_batch* b, int i, int st)
{
    std::lock_guard<std::mutex> lock(b->err_mutex);
    if (b->last_error.empty())
        b->last_error = "system " + std::to_string(i) + ": " + ocsl_status_string(st) + ": " +
                        ocsl_last_error(b->ctx[i]);
}

bool same_opts(const ocsl_opts& a, const ocsl_opts& c)
{
    return a.tol == c.tol && a.maxit == c.maxit && a.ilu_sweeps == c.ilu_sweeps &&
           a.inner_tol == c.inner_tol && a.inner_maxit == c.inner_maxit;
}

// The one-graph batch (ocsl_batch_set_graph): factor every system on its
// context's own stream (worker threads), then one graph launch for every
// solve; systems whose factor failed get that status and no solve.
int solve_graph(ocsl_batch* b, const double* const* d_value, const double* const* d_b,
                double* const* d_x, const ocsl_opts* opts, ocsl_result* result)
{
    const int count = (int)b->ctx.size();
    if (count == 0) return OCSL_OK;
    ocsl_opts o;
    ocsl_default_opts(&o);
    if (opts) o = *opts;
    std::vector<int> prep(count, OCSL_OK);
    std::atomic<int> next{0};
    auto work = [&](int) {
        cudaSetDevice(b->device);
        for (int k = next.fetch_add(1); k < count; k = next.fetch_add(1)) {
            const int i = b->order[k];
            prep[i] = ocsl::ir32_graph_prepare(b->ctx[i], d_value[i], &o, b->nrhs[i]);
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < (int)b->streams.size(); ++w) pool.emplace_back(work, w);
    work(0);
    for (auto& t : pool) t.join();

    std::vector<const void*> key;
    std::vector<char> in(count);
    for (int i = 0; i < count; ++i) {
        key.push_back(d_value[i]);
        key.push_back(d_b[i]);
        key.push_back(d_x[i]);
        in[i] = prep[i] == OCSL_OK;
    }
    cudaSetDevice(b->device);
    if (!b->exec || key != b->key_ptrs || in != b->key_in || !same_opts(o, b->key_opts)) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        cudaGraph_t root = nullptr;
        if (cudaGraphCreate(&root, 0) != cudaSuccess) return OCSL_CUDA_ERROR;
        int rc = OCSL_OK;
        for (int k = 0; k < count && rc == OCSL_OK; ++k) {
            const int i = b->order[k];
            if (!in[i]) continue;
            cudaGraphNode_t last = nullptr;  // this system's solves one after another
            for (int q = 0; q < b->nrhs[i] && rc == OCSL_OK; ++q) {
                rc = ocsl::ir32_graph_capture(b->ctx[i], root, &last, d_value[i],
                                              d_b[i] + (size_t)q * b->n[i],
                                              d_x[i] + (size_t)q * b->n[i], &o, q);
                if (rc != OCSL_OK) note_error(b, i, rc);
            }
        }
        if (rc == OCSL_OK && cudaGraphInstantiate(&b->exec, root, 0) != cudaSuccess) {
            cudaGetLastError();
            b->exec = nullptr;
            rc = OCSL_CUDA_ERROR;
        }
        cudaGraphDestroy(root);
        if (rc != OCSL_OK) return rc;
        b->key_ptrs = key;
        b->key_in = in;
        b->key_opts = o;
    }
    cudaStream_t st = b->streams[0];
    if (cudaGraphLaunch(b->exec, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return OCSL_CUDA_ERROR;
    }
    int first = OCSL_OK;
    for (int i = 0; i < count; ++i) {
        for (int q = 0; q < b->nrhs[i]; ++q) {
            ocsl_result r;
            std::memset(&r, 0, sizeof r);
            int st_i = prep[i];
            if (st_i == OCSL_OK) st_i = ocsl::ir32_graph_result(b->ctx[i], q, &r);
            r.status = st_i;
            if (result) result[b->result_offset[i] + q] = r;
            if (st_i != OCSL_OK) {
                if (first == OCSL_OK) first = st_i;
                note_error(b, i, st_i);
            }
        }
    }
    return first;
}

}  // namespace

extern "C" {

int ocsl_batch_solve_device(ocsl_batch* b, int method, const double* const* d_value,
                            const double* const* d_b, double* const* d_x, const ocsl_opts* opts,
                            ocsl_result* result)
{
    if (!b || !d_value || !d_b || !d_x) return OCSL_BAD_ARGUMENT;
    if (b->graph_mode && method == OCSL_ILU_BICGSTAB_IR32) {
        b->last_error.clear();
        return solve_graph(b, d_value, d_b, d_x, opts, result);
    }
    const int count = (int)b->ctx.size();
    std::atomic<int> next{0};
    std::atomic<int> first_status{OCSL_OK};
    auto work = [&](int w) {
        cudaSetDevice(b->device);
        for (int k = next.fetch_add(1); k < count; k = next.fetch_add(1)) {
            const int i = b->order[k];
            ocsl_ctx* c = b->ctx[i];
            ocsl_set_stream(c, b->streams[w]);
            std::vector<ocsl_result> res(b->nrhs[i]);
            const int st = ocsl_solve_multi_device(c, method, d_value[i], b->nrhs[i], d_b[i],
                                                   d_x[i], opts, res.data());
            ocsl_set_stream(c, nullptr);
            if (result)
                std::copy(res.begin(), res.end(), result + b->result_offset[i]);
            if (st != OCSL_OK) {
                int expected = OCSL_OK;
                first_status.compare_exchange_strong(expected, st);
                std::lock_guard<std::mutex> lock(b->err_mutex);
                if (b->last_error.empty())
                    b->last_error = "system " + std::to_string(i) + ": " +
                                    ocsl_status_string(st) + ": " + ocsl_last_error(c);
            }
        }
    };
    b->last_error.clear();
    const int nw = (int)b->streams.size();
    std::vector<std::thread> pool;
    for (int w = 1; w < nw; ++w) pool.emplace_back(work, w);
    work(0);
    for (auto& t : pool) t.join();
    return first_status.load();
}

const char* ocsl_batch_last_error(const ocsl_batch* b)
{
    return b ? b->last_error.c_str() : "null batch";
}

}  // extern "C"
