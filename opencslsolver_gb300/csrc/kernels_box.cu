// Structured triangular sweeps for 7-point box patterns.
//
// When the pattern is exactly the natural-order 7-point stencil of an
// nx * ny * nz box (recognised on the host), a row's dependencies are its
// -1 neighbours in each dimension (+1 for the backward sweep).
//
// Factor layout.  box_to_soa_kernel copies the CSR factor into two arrays of
// packed 4-element row records: (z-, y-, x-, 0) for the forward sweep and
// (x+, y+, z+, diagonal or its reciprocal) for the backward sweep.  An absent
// neighbour is stored as an exact 0 and its dependency value is taken as 0,
// so its fma adds exactly nothing to a sum that starts at +0: the
// straight-line fma chain below equals the reference's loop over the row's
// CSR entries in storage order (cmatrix_solver.cpp:562-570 forward,
// :602-610 backward), bit for bit.  A row's record is one aligned 16-byte
// (FP32) or 32-byte (FP64) copy.
//
// Schedule.  The box is viewed in canonical coordinates (a, b, s): s spans
// the longest dimension, (a, b) are cut into TA x TB tiles; one CTA owns one
// tile of columns and all of s (see box_cta_kernel).  Tiles are handed out by
// an atomic ticket in an order where a tile's two predecessors always come
// first, so waits cannot deadlock.  The output was filled with an all-ones
// pattern, so a face value is its own ready flag (bounded wait, OCSL_TIMEOUT
// on expiry).
#include <algorithm>
#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr long kSpinLimit = 1L << 21;

// Relaxed gpu-scope accesses of the value-as-flag protocol.  `volatile` keeps
// every poll a fresh load; no "memory" clobber, since nothing else is ordered
// against them (the value is its own flag), which leaves the compiler free to
// schedule the surrounding work.
template <typename T>
struct Bits;
template <>
struct Bits<double> {
    using U = unsigned long long;
    static constexpr U kSentinel = ~0ull;
    static constexpr U kCanonicalNaN = 0x7FF8000000000000ull;
    static __device__ __forceinline__ U load(const double* p)
    {
        U v;
        asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p));
        return v;
    }
    static __device__ __forceinline__ void store(double* p, U v)
    {
        asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v));
    }
    static __device__ __forceinline__ U to(double x) { return (U)__double_as_longlong(x); }
    static __device__ __forceinline__ double from(U u) { return __longlong_as_double((long long)u); }
};
template <>
struct Bits<float> {
    using U = unsigned int;
    static constexpr U kSentinel = ~0u;
    static constexpr U kCanonicalNaN = 0x7FC00000u;
    static __device__ __forceinline__ U load(const float* p)
    {
        U v;
        asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p));
        return v;
    }
    static __device__ __forceinline__ void store(float* p, U v)
    {
        asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v));
    }
    static __device__ __forceinline__ U to(float x) { return __float_as_uint(x); }
    static __device__ __forceinline__ float from(U u) { return __uint_as_float(u); }
};

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

template <typename T>
__device__ __noinline__ T wait_value(const T* p, int* err)
{
    using B = Bits<T>;
    typename B::U u = B::load(p);
    if (u != B::kSentinel) return B::from(u);
    unsigned ns = 0;
    for (long it = 0; it < kSpinLimit; ++it) {
        if (ns) __nanosleep(ns);
        ns = it < 64 ? 0u : (ns == 0 ? 32u : (ns < 256u ? ns * 2u : 256u));
        u = B::load(p);
        if (u != B::kSentinel) return B::from(u);
        if ((it & 255) == 255 && *((volatile int*)err) != 0) break;
    }
    atomicCAS(err, 0, (int)OCSL_TIMEOUT);
    return B::from(B::kCanonicalNaN);
}

template <typename T>
__device__ __forceinline__ void publish(T* p, T v)
{
    using B = Bits<T>;
    typename B::U u = B::to(v);
    if (u == B::kSentinel) u = B::kCanonicalNaN;
    B::store(p, u);
}

// Asynchronous global -> shared copies (one element per lane).  `.ca` may
// keep the line in L1; within one launch the only copies of the output held
// there are this kernel's own earlier reads (all-ones or final values), and a
// still-all-ones word is polled again from L2, so stale data is never used.
template <typename T>
__device__ __forceinline__ void cp_async(T* smem_dst, const T* gsrc)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gsrc) : "memory");
}
// One packed 4-element record (16 bytes for FP32, 32 bytes for FP64).
template <typename T>
__device__ __forceinline__ void cp_async_vec(void* smem_dst, const void* gsrc)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    const char* s = static_cast<const char*>(gsrc);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(s) : "memory");
    if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16), "l"(s + 16) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <typename T>
struct BoxParams {
    BoxGeom g;
    int n;
    const T* soa;  // packed records [2][n][4]: (z-, y-, x-, 0), (x+, y+, z+, diagonal term)
    const T* rhs;
    T* out;
    SweepSync S;
    const int* done;   // column q's flag at done[q * done_stride]
    int done_stride;
    long long ld;      // elements between the columns of rhs and out
};

// FWD: y = L^-1 rhs (unit L); !FWD: x = U^-1 rhs, DIV: divide by the
// diagonal (the reference), else multiply by the stored reciprocal.
// SPAN: which of x (0), y (1), z (2) the canonical s dimension is; a and b
// are the other two in ascending stride.
//
// NC: right-hand sides carried through the same wavefront pass (column q's
// rhs and output ld elements after column q-1's); each row's stencil record
// is staged once and applied to all of them, and every column's arithmetic
// is exactly that of a one-column sweep.
//
// One CTA (TA x TB threads, 16 x 8 by default) sweeps one tile of columns,
// walking the wavefronts W = a + b + s of its tile with one __syncthreads per
// wavefront.  The s-neighbour is the thread's own previous row, in-tile a / b
// neighbours come from a 2-slot shared-memory ring, tile faces from the
// neighbouring CTAs' rows in global memory.
//
// Latency hiding.  A wavefront's own work is a few dependent operations, so
// every memory latency left on the per-wavefront path sets the sweep's speed:
//   * the row's packed coefficient record and rhs come from DRAM and are
//     staged kPF wavefronts ahead with cp.async into shared memory, slot
//     W mod kPF (uniform over the CTA);
//   * a tile-face value is loaded kDF wavefronts before its use into a
//     register ring (slot W mod kDF, a compile-time index after unrolling).
//     The CTA first waits until both upstream tiles have published their first
//     face row, so it runs behind them by about one L2 round trip, which is
//     more than kDF wavefronts: a prefetched face word is then normally final;
//     one still all-ones is polled again from L2 (bounded wait).
#ifndef OCSL_BOX_PF
#define OCSL_BOX_PF 16
#endif
#ifndef OCSL_BOX_DF
#define OCSL_BOX_DF 2
#endif
constexpr int kPF = OCSL_BOX_PF;
constexpr int kDF = OCSL_BOX_DF;
static_assert(kPF % kDF == 0, "the face ring must tile the record ring");
// shared memory of a 256-thread CTA, one column in FP64, must fit the 227 KB
// opt-in limit (several columns: the host narrows the tile)
static_assert((32 * kPF + 8 * (2 + kPF)) * 256 <= 227 * 1024, "staging too deep for FP64");

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    float v[4];
};
template <>
struct Vec4<double> {
    double v[4];
};

template <typename T, bool FWD, bool DIV, int SPAN, int NC>
__global__ void __launch_bounds__(256) box_cta_kernel(BoxParams<T> p)
{
    if (p.done) {
        bool all = true;
#pragma unroll
        for (int q = 0; q < NC; ++q) all = all && p.done[q * p.done_stride] != 0;
        if (all) return;
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const BoxGeom& g = p.g;
    const int TA = g.TA, TB = g.TB, NT = g.TA * g.TB;
    using V4 = Vec4<T>;
    V4* coef = reinterpret_cast<V4*>(smem_raw);         // [kPF][NT] packed row records
    T* ring = reinterpret_cast<T*>(coef + kPF * NT);    // [2][NC][NT]
    T* srhs = ring + 2 * NC * NT;                       // [kPF][NC][NT] rhs
    __shared__ int s_tile;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(p.S.ticket, 1u);
    __syncthreads();
    const int tile = s_tile;
    if (tile >= g.nta * g.ntb) {
        if (threadIdx.x == 0) atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
    } else {
        using B = Bits<T>;
        using U = typename B::U;
        const int tid = threadIdx.x;
        const int ta = tile % g.nta, tb = tile / g.nta;
        const int la = tid % TA, lb = tid / TA;
        const int ca = ta * TA + la, cb = tb * TB + lb;
        const int Da = g.D[0], Db = g.D[1], Ds = g.D[2];
        const bool col_ok = ca < Da && cb < Db;
        const int a = FWD ? ca : Da - 1 - ca;
        const int b = FWD ? cb : Db - 1 - cb;
        const int base = a * g.S[0] + b * g.S[1];
        const int sstep = FWD ? g.S[2] : -g.S[2];
        const int row0 = FWD ? base : base + (Ds - 1) * g.S[2];
        const int dstep = FWD ? -1 : 1;
        const int ta_end = min(ta * TA + TA, Da), tb_end = min(tb * TB + TB, Db);
        const int W0 = ta * TA + tb * TB;
        const int W1 = (ta_end - 1) + (tb_end - 1) + Ds - 1;
        const bool has_a = ca > 0, has_b = cb > 0;
        const bool face_a = col_ok && has_a && la == 0;
        const bool face_b = col_ok && has_b && lb == 0;
        const int off_a = dstep * g.S[0], off_b = dstep * g.S[1];
        const int c0 = ca + cb;  // the thread sweeps row cs = W - c0 at wavefront W
        const V4* pack = reinterpret_cast<const V4*>(p.soa) + (FWD ? 0 : p.n);
        // the columns' right-hand sides and outputs, ld elements apart
        const T* rhs_q[NC];
        T* out_q[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            rhs_q[q] = p.rhs + (size_t)q * p.ld;
            out_q[q] = p.out + (size_t)q * p.ld;
        }
        auto in_range = [&](int cs) { return col_ok && cs >= 0 && cs < Ds; };
        auto refill = [&](int cs, int j) {
            if (in_range(cs)) {
                const int r = row0 + cs * sstep;
                cp_async_vec<T>(&coef[j * NT + tid], pack + r);
#pragma unroll
                for (int q = 0; q < NC; ++q) cp_async(&srhs[(j * NC + q) * NT + tid], rhs_q[q] + r);
            }
            cp_async_commit();
        };
        const int Wbase = W0 - (W0 % kPF);
#pragma unroll
        for (int j = 0; j < kPF; ++j) refill(Wbase + j - c0, j);

        // Start behind the upstream tiles: thread (0, 0) waits for the first
        // face row of each (their row at s = 0 next to this tile's corner).
        if (tid == 0) {
            if (face_a) (void)wait_value(out_q[0] + row0 + off_a, p.S.err);
            if (face_b) (void)wait_value(out_q[0] + row0 + off_b, p.S.err);
        }
        __syncthreads();

        U fa[kDF][NC], fb[kDF][NC];
#pragma unroll
        for (int j = 0; j < kDF; ++j) {
            const int cs = Wbase + j - c0;
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                fa[j][q] = B::kSentinel;
                fb[j][q] = B::kSentinel;
                if (face_a && in_range(cs)) fa[j][q] = B::load(out_q[q] + row0 + cs * sstep + off_a);
                if (face_b && in_range(cs)) fb[j][q] = B::load(out_q[q] + row0 + cs * sstep + off_b);
            }
        }

        T prev[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) prev[q] = T(0);
        for (int Wb = Wbase; Wb <= W1; Wb += kPF) {
#pragma unroll
            for (int j = 0; j < kPF; ++j) {
                const int W = Wb + j;
                if (W > W1) break;  // uniform over the CTA
                const int jf = j % kDF;
                const int cs = W - c0;
                cp_async_wait<kPF - 1>();
                if (W >= W0 && in_range(cs)) {
                    const V4 cf = coef[j * NT + tid];
                    const int r = row0 + cs * sstep;
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        const T* rd = ring + (((W - 1) & 1) * NC + q) * NT;
                        T va = T(0), vb = T(0);
                        if (has_a) {
                            if (la > 0)
                                va = rd[tid - 1];
                            else
                                va = fa[jf][q] != B::kSentinel
                                         ? B::from(fa[jf][q])
                                         : wait_value(out_q[q] + r + off_a, p.S.err);
                        }
                        if (has_b) {
                            if (lb > 0)
                                vb = rd[tid - TA];
                            else
                                vb = fb[jf][q] != B::kSentinel
                                         ? B::from(fb[jf][q])
                                         : wait_value(out_q[q] + r + off_b, p.S.err);
                        }
                        const T vs = cs > 0 ? prev[q] : T(0);
                        const T vx = SPAN == 0 ? vs : va;
                        const T vy = SPAN == 0 ? va : (SPAN == 1 ? vs : vb);
                        const T vz = SPAN == 2 ? vs : vb;
                        // packed record: z-, y-, x-, (unused) | x+, y+, z+, diagonal term;
                        // the fma order is the row's CSR order
                        T sum = fma_t(cf.v[0], FWD ? vz : vx, T(0));
                        sum = fma_t(cf.v[1], vy, sum);
                        sum = fma_t(cf.v[2], FWD ? vx : vz, sum);
                        const T num = srhs[(j * NC + q) * NT + tid] - sum;
                        const T y = FWD ? num : (DIV ? num / cf.v[3] : num * cf.v[3]);
                        ring[((W & 1) * NC + q) * NT + tid] = y;
                        publish(out_q[q] + r, y);
                        prev[q] = y;
                    }
                }
                // next face words of this ring slot: wavefront W + kDF
                {
                    const int csn = cs + kDF;
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        if (face_a && in_range(csn))
                            fa[jf][q] = B::load(out_q[q] + row0 + csn * sstep + off_a);
                        if (face_b && in_range(csn))
                            fb[jf][q] = B::load(out_q[q] + row0 + csn * sstep + off_b);
                    }
                }
                refill(cs + kPF, j);
                if (W >= W0) __syncthreads();  // uniform over the CTA
            }
        }
        cp_async_wait<0>();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(p.S.finished, 1u) == gridDim.x - 1) {
            *p.S.ticket = 0u;
            *p.S.finished = 0u;
        }
    }
}

// CSR factor -> packed stencil records.  Row r's real entries are, in
// storage order, z-, y-, x-, diagonal, x+, y+, z+ (absent ones skipped), then
// phantoms; the host verified exactly this pattern.  pack[0][r] = (z-, y-,
// x-, 0), pack[1][r] = (x+, y+, z+, diagonal) with the diagonal replaced by
// 1 / diagonal (computed in FP64) when RECIP.  Absent entries are exact 0.
template <typename TO, int RECIP>
__global__ void box_to_soa_kernel(int n, int nx, int ny, int nz, const int* rp, const double* M,
                                  TO* pack)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
    const bool present[7] = {k > 0, j > 0, i > 0, true, i < nx - 1, j < ny - 1, k < nz - 1};
    double v[7];
    int q = rp[r];
#pragma unroll
    for (int d = 0; d < 7; ++d) v[d] = present[d] ? M[q++] : 0.0;
    if (RECIP) v[3] = 1.0 / v[3];
    TO* lo = pack + (size_t)4 * r;
    TO* hi = pack + (size_t)4 * n + (size_t)4 * r;
    lo[0] = (TO)v[0];
    lo[1] = (TO)v[1];
    lo[2] = (TO)v[2];
    lo[3] = (TO)0;
    hi[0] = (TO)v[4];
    hi[1] = (TO)v[5];
    hi[2] = (TO)v[6];
    hi[3] = (TO)v[3];
}

template <typename T, bool FWD, bool DIV, int SPAN, int NC>
void launch_one(cudaStream_t st, const BoxParams<T>& p)
{
    const int grid = p.g.nta * p.g.ntb;
    const int threads = p.g.TA * p.g.TB;
    const size_t smem = box_sweep_smem(threads, (int)sizeof(T), NC);
    static bool attr_set = false;  // one opt-in per instantiation
    if (!attr_set) {
        const size_t most = std::min(box_sweep_smem(256, (int)sizeof(T), NC), kBoxSmemLimit);
        cudaFuncSetAttribute(box_cta_kernel<T, FWD, DIV, SPAN, NC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
        attr_set = true;
    }
    box_cta_kernel<T, FWD, DIV, SPAN, NC><<<grid, threads, smem, st>>>(p);
}

template <typename T, bool FWD, bool DIV, int NC>
void launch_span(cudaStream_t st, int span, const BoxParams<T>& p)
{
    switch (span) {
    case 0: launch_one<T, FWD, DIV, 0, NC>(st, p); break;
    case 1: launch_one<T, FWD, DIV, 1, NC>(st, p); break;
    default: launch_one<T, FWD, DIV, 2, NC>(st, p); break;
    }
}

template <typename T, bool FWD>
void launch_cols(cudaStream_t st, int ncols, const BoxParams<T>& p)
{
    switch (ncols) {
    case 1: launch_span<T, FWD, false, 1>(st, p.g.span, p); break;
    case 2: launch_span<T, FWD, false, 2>(st, p.g.span, p); break;
    case 3: launch_span<T, FWD, false, 3>(st, p.g.span, p); break;
    default: launch_span<T, FWD, false, 4>(st, p.g.span, p); break;
    }
}

}  // namespace

size_t box_sweep_smem(int threads, int elem_size, int ncols)
{
    const size_t per = (size_t)4 * elem_size * kPF + (size_t)elem_size * ncols * (2 + kPF);
    return per * (size_t)threads;
}

template <typename T>
void launch_box_sweep(cudaStream_t st, const BoxGeom& g, int n, const T* soa, const T* rhs, T* out,
                      bool forward, int divmode, const SweepSync& S, const int* done,
                      const Cols& cols, int done_stride)
{
    BoxParams<T> p;
    p.g = g;
    p.n = n;
    p.soa = soa;
    p.rhs = rhs;
    p.out = out;
    p.S = S;
    p.done = done;
    p.done_stride = done_stride;
    p.ld = cols.ld;
    const int nc = std::max(1, std::min(cols.n, kMaxCols));
    if (divmode == 0 && !forward)
        launch_span<T, false, true, 1>(st, g.span, p);  // the reference's division: one column
    else if (forward)
        launch_cols<T, true>(st, nc, p);
    else
        launch_cols<T, false>(st, nc, p);
}

template <typename TO>
void launch_box_to_soa(cudaStream_t st, const int* dims, int n, const int* rp, const double* M,
                       TO* soa, int recip)
{
    if (n == 0) return;
    const int blocks = (n + 255) / 256;
    if (recip)
        box_to_soa_kernel<TO, 1><<<blocks, 256, 0, st>>>(n, dims[0], dims[1], dims[2], rp, M, soa);
    else
        box_to_soa_kernel<TO, 0><<<blocks, 256, 0, st>>>(n, dims[0], dims[1], dims[2], rp, M, soa);
}

template void launch_box_sweep<double>(cudaStream_t, const BoxGeom&, int, const double*,
                                       const double*, double*, bool, int, const SweepSync&,
                                       const int*, const Cols&, int);
template void launch_box_sweep<float>(cudaStream_t, const BoxGeom&, int, const float*,
                                      const float*, float*, bool, int, const SweepSync&,
                                      const int*, const Cols&, int);
template void launch_box_to_soa<double>(cudaStream_t, const int*, int, const int*, const double*,
                                        double*, int);
template void launch_box_to_soa<float>(cudaStream_t, const int*, int, const int*, const double*,
                                       float*, int);

}  // namespace ocsl
