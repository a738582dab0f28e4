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
//
// Clusters.  With BoxGeom CX x CY > 1 the tiles are grouped into
// thread-block clusters of CX x CY neighbouring tiles (one CTA each, all
// co-resident by the hardware's guarantee).  Inside a cluster a tile hands
// its face values to its downstream neighbours through distributed shared
// memory: the producing thread stores each value straight into the
// consumer's face buffer (one slot per s row, sentinel-initialised before a
// cluster barrier), and the consumer polls its own shared memory, so a hop
// costs a DSMEM store instead of an L2 store plus L2 polls.  Faces between
// clusters keep the global value-as-flag path, and clusters take tickets in
// the same dependency order as single tiles.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
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
    // own shared memory written by cluster peers / a peer's shared memory
    static __device__ __forceinline__ U load_local(unsigned saddr)
    {
        U v;
        asm volatile("ld.relaxed.cluster.shared::cta.b64 %0, [%1];" : "=l"(v) : "r"(saddr));
        return v;
    }
    static __device__ __forceinline__ void store_remote(unsigned caddr, U v)
    {
        asm volatile("st.relaxed.cluster.shared::cluster.b64 [%0], %1;" ::"r"(caddr), "l"(v));
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
    static __device__ __forceinline__ U load_local(unsigned saddr)
    {
        U v;
        asm volatile("ld.relaxed.cluster.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(saddr));
        return v;
    }
    static __device__ __forceinline__ void store_remote(unsigned caddr, U v)
    {
        asm volatile("st.relaxed.cluster.shared::cluster.b32 [%0], %1;" ::"r"(caddr), "r"(v));
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

// Face value from the cluster peer upstream: poll this CTA's own slot
// (bounded; OCSL_TIMEOUT and a NaN on expiry).
template <typename T>
__device__ __noinline__ T wait_local_slow(unsigned saddr, int* err)
{
    using B = Bits<T>;
    for (long it = 0; it < kSpinLimit; ++it) {
        const typename B::U u = B::load_local(saddr);
        if (u != B::kSentinel) return B::from(u);
        if ((it & 255) == 255 && *((volatile int*)err) != 0) break;
    }
    atomicCAS(err, 0, (int)OCSL_TIMEOUT);
    return B::from(B::kCanonicalNaN);
}
template <typename T>
__device__ __forceinline__ T wait_local(const T* slot, int* err)
{
    using B = Bits<T>;
    const unsigned a = (unsigned)__cvta_generic_to_shared(slot);
    const typename B::U u = B::load_local(a);
    return u != B::kSentinel ? B::from(u) : wait_local_slow<T>(a, err);
}
__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Every thread of every CTA of the cluster; release / acquire order shared
// memory writes before it against peers' accesses after it.
__device__ __forceinline__ void cluster_barrier()
{
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// The shared::cluster address of `local` (this CTA's shared memory) in CTA `rank`.
__device__ __forceinline__ unsigned peer_addr(const void* local, unsigned rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(r)
                 : "r"((unsigned)__cvta_generic_to_shared(local)), "r"(rank));
    return r;
}
// Hand value v (the sentinel bit pattern mapped to a NaN, as publish does)
// to the same slot of CTA `rank`.
template <typename T>
__device__ __forceinline__ void push_peer(const T* local_slot, unsigned rank, T v)
{
    using B = Bits<T>;
    typename B::U u = B::to(v);
    if (u == B::kSentinel) u = B::kCanonicalNaN;
    B::store_remote(peer_addr(local_slot, rank), u);
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
    const bool clus = g.CX * g.CY > 1;  // uniform over the grid
    using V4 = Vec4<T>;
    V4* coef = reinterpret_cast<V4*>(smem_raw);         // [kPF][NT] packed row records
    T* ring = reinterpret_cast<T*>(coef + kPF * NT);    // [2][NC][NT]
    T* srhs = ring + 2 * NC * NT;                       // [kPF][NC][NT] rhs
    // clusters only: values of the upstream tiles' faces, one slot per s row
    T* faceA = srhs + kPF * NC * NT;                    // [NC][Ds][TB] from tile (ta - 1, tb)
    T* faceB = faceA + (clus ? NC * g.D[2] * TB : 0);   // [NC][Ds][TA] from tile (ta, tb - 1)
    __shared__ int s_tile;
    int tile = -1;  // ta + tb * nta; -1: a CTA of a partial cluster with no tile
    bool overflow = false;
    unsigned rank = 0;
    if (!clus) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(p.S.ticket, 1u);
        __syncthreads();
        tile = s_tile;
        overflow = tile >= g.nta * g.ntb;
    } else {
        rank = cluster_rank();
        if (rank == 0 && threadIdx.x == 0) s_tile = (int)atomicAdd(p.S.ticket, 1u);
        using U = typename Bits<T>::U;
        U* fu = reinterpret_cast<U*>(faceA);
        const int nface = NC * g.D[2] * (TA + TB);
        for (int i = threadIdx.x; i < nface; i += blockDim.x) fu[i] = Bits<T>::kSentinel;
        // faces initialised and rank 0's ticket written before any peer access
        cluster_barrier();
        int blk;
        asm volatile("ld.shared::cluster.b32 %0, [%1];" : "=r"(blk) : "r"(peer_addr(&s_tile, 0)));
        overflow = blk >= g.nca * g.ncb;
        if (!overflow) {
            const int ta = (blk % g.nca) * g.CX + (int)rank % g.CX;
            const int tb = (blk / g.nca) * g.CY + (int)rank / g.CX;
            if (ta < g.nta && tb < g.ntb) tile = ta + tb * g.nta;
        }
    }
    if (overflow) {
        if (threadIdx.x == 0) atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
    } else if (tile >= 0) {
        using B = Bits<T>;
        using U = typename B::U;
        const int tid = threadIdx.x;
        const int ta = tile % g.nta, tb = tile / g.nta;
        const int la = tid % TA, lb = tid / TA;
        const int ca = ta * TA + la, cb = tb * TB + lb;
        const int Da = g.D[0], Db = g.D[1], Ds = g.D[2];
        // cluster position; an upstream / downstream tile inside the cluster
        // exchanges faces through shared memory
        const int rx = (int)rank % g.CX, ry = (int)rank / g.CX;
        const bool loc_a = clus && rx > 0, loc_b = clus && ry > 0;
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
        // face_*: the neighbour is in the upstream tile, read through global memory
        const bool face_a = col_ok && has_a && la == 0 && !loc_a;
        const bool face_b = col_ok && has_b && lb == 0 && !loc_b;
        // push_*: this column is the face of a downstream tile of the cluster
        const bool push_a = clus && col_ok && la == TA - 1 && rx < g.CX - 1 && ta + 1 < g.nta;
        const bool push_b = clus && col_ok && lb == TB - 1 && ry < g.CY - 1 && tb + 1 < g.ntb;
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
                            else if (loc_a)
                                va = wait_local(faceA + (q * Ds + cs) * TB + lb, p.S.err);
                            else
                                va = fa[jf][q] != B::kSentinel
                                         ? B::from(fa[jf][q])
                                         : wait_value(out_q[q] + r + off_a, p.S.err);
                        }
                        if (has_b) {
                            if (lb > 0)
                                vb = rd[tid - TA];
                            else if (loc_b)
                                vb = wait_local(faceB + (q * Ds + cs) * TA + la, p.S.err);
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
                        if (push_a) push_peer(faceA + (q * Ds + cs) * TB + lb, rank + 1, y);
                        if (push_b) push_peer(faceB + (q * Ds + cs) * TA + la, rank + g.CX, y);
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
    // no CTA leaves while a peer may still store into its faces
    if (clus) cluster_barrier();
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

// Whether a cluster launch of `kern` with this shape can run on the device
// at all (cudaOccupancyMaxActiveClusters > 0), cached per shape.
template <typename K>
bool cluster_fits(K kern, int grid, int threads, size_t smem, int csize)
{
    static std::mutex mu;
    static std::map<std::tuple<int, size_t, int>, bool> seen;
    const auto key = std::make_tuple(threads, smem, csize);
    std::lock_guard<std::mutex> lock(mu);
    const auto it = seen.find(key);
    if (it != seen.end()) return it->second;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();  // a refused query leaves no sticky error
        return false;              // not cached: the query may succeed later
    }
    seen[key] = n > 0;
    return n > 0;
}

// Dynamic shared memory above half of an SM's 228 KB (less the 1 KB each CTA
// reserves): no second CTA fits beside it.
constexpr size_t kBoxSmemOneCta = 116 * 1024;

template <typename T, bool FWD, bool DIV, int SPAN, int NC>
void launch_one(cudaStream_t st, BoxParams<T> p)
{
    auto kern = box_cta_kernel<T, FWD, DIV, SPAN, NC>;
    static std::once_flag once;  // one opt-in per instantiation
    std::call_once(once, [&] {
        // static + dynamic shared memory must stay within the opt-in limit
        cudaFuncAttributes fa{};
        size_t stat = 1024;
        bool failed = cudaFuncGetAttributes(&fa, kern) != cudaSuccess;
        if (!failed) stat = fa.sharedSizeBytes;
        failed |= cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(kBoxSmemOptin - stat)) != cudaSuccess;
        failed |= cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                  cudaSuccess;
        if (failed) (void)cudaGetLastError();  // the launch itself reports what matters
    });
    const int threads = p.g.TA * p.g.TB;
    int csize = p.g.CX * p.g.CY;
    size_t smem = box_sweep_smem(p.g, (int)sizeof(T), NC);
    if (csize > 1) {
        // one CTA per SM: a cluster's CTAs may otherwise be packed two to an
        // SM, which doubles that SM's work per wavefront
        smem = std::max(smem, kBoxSmemOneCta);
        const int grid = p.g.nca * p.g.ncb * csize;
        if (smem > kBoxSmemLimit || !cluster_fits(kern, grid, threads, smem, csize)) {
            p.g = box_with_cluster(p.g, 1, 1);  // the shape cannot run: single tiles
            csize = 1;
            smem = box_sweep_smem(p.g, (int)sizeof(T), NC);
        }
    }
    int grid = p.g.nca * p.g.ncb * csize;
    if (p.S.skip_first && grid > csize) {  // fault injection: tile / cluster 0 never runs
        preset_ticket_one(st, p.S.ticket);
        grid -= csize;
    }
    if (csize == 1) {
        kern<<<grid, threads, smem, st>>>(p);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, p);
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

size_t box_sweep_smem(const BoxGeom& g, int elem_size, int ncols)
{
    size_t b = box_sweep_smem(g.TA * g.TB, elem_size, ncols);
    if (g.CX * g.CY > 1) b += (size_t)elem_size * ncols * g.D[2] * (g.TA + g.TB);
    return b;
}

BoxGeom box_with_cluster(BoxGeom g, int cx, int cy)
{
    cx = std::max(1, std::min(cx, g.nta));
    cy = std::max(1, std::min(cy, g.ntb));
    while (cx * cy > kMaxClusterTiles) {
        if (cx >= cy)
            --cx;
        else
            --cy;
    }
    g.CX = cx;
    g.CY = cy;
    g.nca = (g.nta + cx - 1) / cx;
    g.ncb = (g.ntb + cy - 1) / cy;
    return g;
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
