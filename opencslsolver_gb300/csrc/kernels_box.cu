// Structured triangular sweeps for 7-point box patterns.
//
// When the pattern is exactly the natural-order 7-point stencil of an
// nx * ny * nz box (recognised on the host), a row's dependencies are its
// -1 neighbours in each dimension (+1 for the backward sweep).
//
// Factor layout.  box_to_soa_kernel copies the CSR factor into seven arrays
// indexed by row ("stencil SoA"): coefficient of the z-, y-, x- neighbour,
// the diagonal (or its reciprocal), x+, y+, z+.  An absent neighbour is
// stored as an exact 0 and its dependency value is taken as 0, so its fma
// adds exactly nothing to a sum that starts at +0: the straight-line fma
// chain below equals the reference's loop over the row's CSR entries in
// storage order (cmatrix_solver.cpp:562-570 forward, :602-610 backward), bit
// for bit.  Every load is affine in the row index.
//
// Schedule.  The box is viewed in canonical coordinates (a, b, s): s spans
// the longest dimension, (a, b) are cut into WA x WB tiles (8 x 4 by
// default); one warp owns one tile of columns and all of s, one lane one
// column, and the lanes run skewed in time (see box_sweep_kernel):
//   * the dependency along s is the lane's own previous row (a register);
//   * dependencies inside the tile come from the neighbouring lanes by
//     __shfl_up -- no barrier, no shared memory;
//   * the tile faces read the neighbouring tiles' rows from global memory;
//     the output was filled with an all-ones pattern, so a value is its own
//     ready flag (bounded wait, OCSL_TIMEOUT on expiry).
// Tiles are handed out by an atomic ticket in an order where a tile's two
// predecessors always come first, so waits cannot deadlock.  Row data and
// face values are prefetched kPF steps ahead with cp.async into a shared-memory
// ring whose slot is t mod kPF.
#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr long kSpinLimit = 1L << 21;
constexpr int kPF = 8;  // wavefronts of prefetch per thread

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
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <typename T>
struct BoxParams {
    BoxGeom g;
    int n;
    const T* soa;  // [7][n]: z-, y-, x-, diag or 1/diag, x+, y+, z+
    const T* rhs;
    T* out;
    SweepSync S;
    const int* done;
};

// FWD: y = L^-1 rhs (unit L); !FWD: x = U^-1 rhs, DIV: divide by the
// diagonal (the reference), else multiply by the stored reciprocal.
// SPAN: which of x (0), y (1), z (2) the canonical s dimension is; a and b
// are the other two in ascending stride.
//
// One warp sweeps one WA x WB tile of columns.  Lane (la, lb) handles column
// (ca, cb) and sweeps its row cs = t - la - lb at warp step t, so at step t
// the a-neighbour (lane - 1) and the b-neighbour (lane - WA) hold, from step
// t - 1, exactly the values this row needs: they arrive by __shfl_up, with
// no barrier and no shared memory.  The s-neighbour is the lane's own value
// from step t - 1.  Lanes on the tile's a / b faces read the neighbouring
// tiles' rows from global memory instead.
template <typename T, bool FWD, bool DIV, int SPAN>
__global__ void __launch_bounds__(32) box_sweep_kernel(BoxParams<T> p)
{
    if (p.done && *p.done) return;
    const BoxGeom& g = p.g;
    const int lane = threadIdx.x;
    int tile = 0;
    if (lane == 0) tile = (int)atomicAdd(p.S.ticket, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= g.nta * g.ntb) {
        if (lane == 0) atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
    } else {
        using B = Bits<T>;
        using U = typename B::U;
        const int WA = g.TA, WB = g.TB;
        const int ta = tile % g.nta, tb = tile / g.nta;
        const int la = lane % WA, lb = lane / WA;
        const int ca = ta * WA + la, cb = tb * WB + lb;
        const int Da = g.D[0], Db = g.D[1], Ds = g.D[2];
        const bool col_ok = lb < WB && ca < Da && cb < Db;
        const int a = FWD ? ca : Da - 1 - ca;
        const int b = FWD ? cb : Db - 1 - cb;
        const int base = a * g.S[0] + b * g.S[1];
        const int sstep = FWD ? g.S[2] : -g.S[2];  // row step along the column
        const int row0 = FWD ? base : base + (Ds - 1) * g.S[2];
        const int dstep = FWD ? -1 : 1;             // offset sign of a dependency
        const bool has_a = ca > 0, has_b = cb > 0;
        const bool face_a = col_ok && has_a && la == 0;
        const bool face_b = col_ok && has_b && lb == 0;
        const int off_a = dstep * g.S[0], off_b = dstep * g.S[1];
        const int c0 = la + lb;                     // skew: row cs = t - c0 at step t
        const int Tmax = (WA - 1) + (WB - 1) + Ds - 1;
        const int n = p.n;
        // coefficient arrays in the order of the row's CSR entries
        const T* C0 = p.soa + (size_t)(FWD ? 0 : 4) * n;  // z- | x+
        const T* C1 = p.soa + (size_t)(FWD ? 1 : 5) * n;  // y- | y+
        const T* C2 = p.soa + (size_t)(FWD ? 2 : 6) * n;  // x- | z+
        const T* CD = p.soa + (size_t)3 * n;
        auto in_range = [&](int cs) { return col_ok && cs >= 0 && cs < Ds; };

        // Prefetch ring in shared memory, slot j = t mod kPF: stage[j][f][lane]
        // holds the row's three coefficients (f 0-2), diagonal term (3), rhs
        // (4) and face values (5, 6), copied with cp.async kPF steps ahead;
        // one commit group per step, so wait_group(kPF - 1) before use leaves
        // exactly the slot of this step complete.  A face word still holding
        // the all-ones pattern is polled from L2.
        __shared__ T stage[kPF][7][32];
        auto refill = [&](int cs, int j) {
            if (in_range(cs)) {
                const int r = row0 + cs * sstep;
                cp_async(&stage[j][0][lane], C0 + r);
                cp_async(&stage[j][1][lane], C1 + r);
                cp_async(&stage[j][2][lane], C2 + r);
                if (!FWD) cp_async(&stage[j][3][lane], CD + r);
                cp_async(&stage[j][4][lane], p.rhs + r);
                if (face_a) cp_async(&stage[j][5][lane], (const T*)p.out + r + off_a);
                if (face_b) cp_async(&stage[j][6][lane], (const T*)p.out + r + off_b);
            }
            cp_async_commit();
        };
#pragma unroll
        for (int j = 0; j < kPF; ++j) refill(j - c0, j);

        T ylast = T(0);  // this lane's value from the previous step
        for (int t0 = 0; t0 <= Tmax; t0 += kPF) {
#pragma unroll
            for (int j = 0; j < kPF; ++j) {
                const int t = t0 + j;
                if (t > Tmax) break;  // warp-uniform
                const int cs = t - c0;
                const T ya = __shfl_up_sync(0xffffffffu, ylast, 1);
                const T yb = __shfl_up_sync(0xffffffffu, ylast, WA);
                cp_async_wait<kPF - 1>();
                if (in_range(cs)) {
                    const int r = row0 + cs * sstep;
                    T va = T(0), vb = T(0);
                    if (has_a) {
                        if (la > 0) {
                            va = ya;
                        } else {
                            const U u = B::to(stage[j][5][lane]);
                            va = u != B::kSentinel ? B::from(u) : wait_value(p.out + r + off_a, p.S.err);
                        }
                    }
                    if (has_b) {
                        if (lb > 0) {
                            vb = yb;
                        } else {
                            const U u = B::to(stage[j][6][lane]);
                            vb = u != B::kSentinel ? B::from(u) : wait_value(p.out + r + off_b, p.S.err);
                        }
                    }
                    const T vs = cs > 0 ? ylast : T(0);
                    // dependency values of the x, y, z neighbours
                    const T vx = SPAN == 0 ? vs : va;
                    const T vy = SPAN == 0 ? va : (SPAN == 1 ? vs : vb);
                    const T vz = SPAN == 2 ? vs : vb;
                    // CSR order: z-, y-, x- (forward); x+, y+, z+ (backward)
                    T sum = fma_t(stage[j][0][lane], FWD ? vz : vx, T(0));
                    sum = fma_t(stage[j][1][lane], vy, sum);
                    sum = fma_t(stage[j][2][lane], FWD ? vx : vz, sum);
                    const T num = stage[j][4][lane] - sum;
                    const T y = FWD ? num : (DIV ? num / stage[j][3][lane] : num * stage[j][3][lane]);
                    publish(p.out + r, y);
                    ylast = y;
                }
                __syncwarp();  // the slot's reads are done before it is refilled
                refill(cs + kPF, j);
            }
        }
        cp_async_wait<0>();
    }
    // reset the dispenser after the last tile
    __syncwarp();
    if (lane == 0) {
        __threadfence();
        if (atomicAdd(p.S.finished, 1u) == gridDim.x - 1) {
            *p.S.ticket = 0u;
            *p.S.finished = 0u;
        }
    }
}

// CSR factor -> stencil SoA.  Row r's real entries are, in storage order,
// z-, y-, x-, diagonal, x+, y+, z+ (absent ones skipped), then phantoms; the
// host verified exactly this pattern.  Slot 3 gets the diagonal (RECIP == 0)
// or 1 / diagonal computed in FP64.
template <typename TO, int RECIP>
__global__ void box_to_soa_kernel(int n, int nx, int ny, int nz, const int* rp, const double* M,
                                  TO* soa)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
    const bool present[7] = {k > 0, j > 0, i > 0, true, i < nx - 1, j < ny - 1, k < nz - 1};
    int q = rp[r];
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        double v = 0.0;
        if (present[d]) v = M[q++];
        if (d == 3 && RECIP) v = 1.0 / v;
        soa[(size_t)d * n + r] = (TO)v;
    }
}

template <typename T, bool FWD, bool DIV>
void launch_span(cudaStream_t st, int span, const BoxParams<T>& p, int threads, size_t smem,
                 int grid)
{
    switch (span) {
    case 0: box_sweep_kernel<T, FWD, DIV, 0><<<grid, threads, smem, st>>>(p); break;
    case 1: box_sweep_kernel<T, FWD, DIV, 1><<<grid, threads, smem, st>>>(p); break;
    default: box_sweep_kernel<T, FWD, DIV, 2><<<grid, threads, smem, st>>>(p); break;
    }
}

}  // namespace

template <typename T>
void launch_box_sweep(cudaStream_t st, const BoxGeom& g, int n, const T* soa, const T* rhs, T* out,
                      bool forward, int divmode, const SweepSync& S, const int* done)
{
    BoxParams<T> p;
    p.g = g;
    p.n = n;
    p.soa = soa;
    p.rhs = rhs;
    p.out = out;
    p.S = S;
    p.done = done;
    const int threads = 32;  // one warp per tile
    const size_t smem = 0;
    const int grid = g.nta * g.ntb;
    if (forward)
        launch_span<T, true, false>(st, g.span, p, threads, smem, grid);
    else if (divmode == 0)
        launch_span<T, false, true>(st, g.span, p, threads, smem, grid);
    else
        launch_span<T, false, false>(st, g.span, p, threads, smem, grid);
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
                                       const int*);
template void launch_box_sweep<float>(cudaStream_t, const BoxGeom&, int, const float*,
                                      const float*, float*, bool, int, const SweepSync&,
                                      const int*);
template void launch_box_to_soa<double>(cudaStream_t, const int*, int, const int*, const double*,
                                        double*, int);
template void launch_box_to_soa<float>(cudaStream_t, const int*, int, const int*, const double*,
                                       float*, int);

}  // namespace ocsl
