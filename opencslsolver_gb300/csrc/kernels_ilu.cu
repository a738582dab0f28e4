// ILU factor (fixed-point sweeps) and the sync-free, level-ordered triangular
// sweeps.
//
// Triangular sweeps (cmatrix_solver.cpp:555-572 forward, :595-611 backward)
// keep the reference's natural ordering.  The host builds a level schedule
// (level of a row = 1 + the deepest level it depends on) and cuts every level
// into chunks of <= 256 rows; one CTA solves one chunk, one thread one row.
// CTAs take chunks from an atomic dispenser in level order, so a CTA only
// ever waits on rows of chunks that resident CTAs already hold: the sweep
// cannot deadlock whatever the residency.
//
// The output vector is pre-filled with an all-ones bit pattern (a NaN no
// arithmetic produces; a result that happens to carry it is stored as the
// canonical NaN instead).  A row's thread reads each dependency with a relaxed
// gpu-scope load until it differs from that pattern -- the value is its own
// ready flag, so one L2 round trip serves both.  Every wait is bounded: after
// the limit the thread records OCSL_TIMEOUT, stores a NaN (so nobody waits on
// it in turn) and the host turns the flag into the solve's status.
//
// Each row's sum runs over its CSR entries in storage order with fma from 0,
// exactly as the reference's sequential loop, so the schedule does not
// change a single bit of the result.
#include <algorithm>
#include <cfloat>
#include <type_traits>

#include "division.cuh"
#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr long kSpinLimit = 1L << 21;  // polls per dependency: ~1 s with back-off

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
        asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
        return v;
    }
    static __device__ __forceinline__ void store(double* p, U v)
    {
        asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
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
        asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        return v;
    }
    static __device__ __forceinline__ void store(float* p, U v)
    {
        asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
    }
    static __device__ __forceinline__ U to(float x) { return __float_as_uint(x); }
    static __device__ __forceinline__ float from(U u) { return __uint_as_float(u); }
};

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

// Wait (bounded) until out[j] holds a value, then return it.
template <typename T>
__device__ __forceinline__ T wait_value(const T* p, int* err)
{
    using B = Bits<T>;
    typename B::U u = B::load(p);
    if (u != B::kSentinel) return B::from(u);
    unsigned ns = 0;
    for (long it = 0; it < kSpinLimit; ++it) {
        if (ns) __nanosleep(ns);
        ns = ns == 0 ? (it > 32 ? 32u : 0u) : (ns < 256u ? ns * 2u : 256u);
        u = B::load(p);
        if (u != B::kSentinel) return B::from(u);
        if ((it & 255) == 255 && *((volatile int*)err) != 0) break;  // another wait gave up
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

template <typename T>
struct SweepParams {
    int n;
    const int* rp;
    const int* col;
    const int* diag;
    const int* order;
    const int* chunk;
    int nchunks;
    const T* M;
    const T* dinv;
    const T* rhs;
    T* out;
    SweepSync S;
    const int* done;
};

__device__ __forceinline__ void sweep_epilogue(const SweepSync& S)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(S.finished, 1u) == gridDim.x - 1) {
            *S.ticket = 0u;
            *S.finished = 0u;
        }
    }
}

// y = L^-1 b with unit L (cmatrix_solver.cpp:558-571).
template <typename T>
__global__ void __launch_bounds__(kThreads) fw_sweep_kernel(SweepParams<T> p)
{
    if (p.done && *p.done) return;
    __shared__ int s_chunk;
    if (threadIdx.x == 0) s_chunk = (int)atomicAdd(p.S.ticket, 1u);
    __syncthreads();
    const int c = s_chunk;
    if (c >= p.nchunks) {  // never happens with a fresh dispenser; keeps every read in bounds
        atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
        sweep_epilogue(p.S);
        return;
    }
    const int t = __ldg(p.chunk + c) + (int)threadIdx.x;
    if (t < __ldg(p.chunk + c + 1)) {
        const int i = __ldg(p.order + t);
        const int b = __ldg(p.rp + i), d = __ldg(p.diag + i);
        T sum = T(0);
        for (int q = b; q < d; ++q) {
            const int j = __ldg(p.col + q);
            sum = fma_t(__ldg(p.M + q), wait_value(p.out + j, p.S.err), sum);
        }
        publish(p.out + i, p.rhs[i] - sum);
    }
    sweep_epilogue(p.S);
}

// x = U^-1 y (cmatrix_solver.cpp:598-610).  DIV: divide by the stored
// diagonal as the reference does; otherwise multiply by a precomputed
// reciprocal (tolerance mode).
template <typename T, bool DIV>
__global__ void __launch_bounds__(kThreads) bw_sweep_kernel(SweepParams<T> p)
{
    if (p.done && *p.done) return;
    __shared__ int s_chunk;
    if (threadIdx.x == 0) s_chunk = (int)atomicAdd(p.S.ticket, 1u);
    __syncthreads();
    const int c = s_chunk;
    if (c >= p.nchunks) {  // never happens with a fresh dispenser; keeps every read in bounds
        atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
        sweep_epilogue(p.S);
        return;
    }
    const int t = __ldg(p.chunk + c) + (int)threadIdx.x;
    if (t < __ldg(p.chunk + c + 1)) {
        const int i = __ldg(p.order + t);
        const int d = __ldg(p.diag + i), e = __ldg(p.rp + i + 1);
        T sum = T(0);
        for (int q = d + 1; q < e; ++q) {
            const int j = __ldg(p.col + q);
            if (j < 0) continue;  // phantom: the reference adds 0 * x[-1]
            sum = fma_t(__ldg(p.M + q), wait_value(p.out + j, p.S.err), sum);
        }
        const T num = p.rhs[i] - sum;
        const T xi = DIV ? num / __ldg(p.M + d) : num * __ldg(p.dinv + i);
        publish(p.out + i, xi);
    }
    sweep_epilogue(p.S);
}

// Sweeps over schedules whose levels are contiguous row ranges (multicolour
// orderings: a row's lower neighbours all lie in lower colours, its upper
// ones in higher colours).  One launch per level, one thread per row: every
// dependency lies in a level an earlier launch finished, so plain read-only
// loads serve, nothing is prefilled and nothing waits.  A row's first
// triangle entries (preload_width below) are loaded together, then their
// neighbour values, then the fma chain runs (CSR order from 0, as above).
//
// KIND 0: forward, y_i = rhs_i - sum_{j<i} M_ij y_j.
// KIND 2: backward, x_i = (y_i - sum_{j>i} M_ij x_j) / M_ii (DIV) or * dinv_i.
// KIND 1: both for a level whose rows have no upper entries (the last colour):
//         x_i = y_i / M_ii or * dinv_i, y_i not stored.
// Rows below rhs_end take y from rhs: level 0 of the forward sweep has no
// lower entries, so its y equals rhs bit for bit (rhs - 0.0) and the
// preconditioner skips that level's copy.
template <typename T>
struct RangeParams {
    const int* rp;
    const int* col;
    const int* diag;
    const T* M;
    const T* dinv;
    const T* rhs;
    T* y;
    T* x;
    int r0, r1, rhs_end;
    const int* done;
};

template <typename T>
__device__ __forceinline__ T y_of(const RangeParams<T>& p, int j)
{
    return j < p.rhs_end ? __ldg(p.rhs + j) : __ldg(p.y + j);
}

// Triangle entries preloaded per row: 4 (a 7-point row has at most 3 per
// triangle, a tetrahedral cell 4 face neighbours), so the kernel stays at 32
// registers, 8 CTAs per SM, without spills; longer rows continue the same
// chain in a loop.
template <typename T>
__host__ __device__ constexpr int preload_width()
{
    return 4;
}

template <typename T>
__device__ __forceinline__ T lower_sum(const RangeParams<T>& p, int b, int d)
{
    constexpr int K = preload_width<T>();
    int c[K];
    T v[K], yv[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        c[k] = b + k < d ? __ldg(p.col + b + k) : 0;
        v[k] = b + k < d ? __ldg(p.M + b + k) : T(0);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) yv[k] = b + k < d ? y_of(p, c[k]) : T(0);
    T sum = T(0);
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (b + k < d) sum = fma_t(v[k], yv[k], sum);
    for (int q = b + K; q < d; ++q) sum = fma_t(__ldg(p.M + q), y_of(p, __ldg(p.col + q)), sum);
    return sum;
}

template <typename T>
__device__ __forceinline__ T upper_sum(const RangeParams<T>& p, int d, int e)
{
    constexpr int K = preload_width<T>();
    const int b = d + 1;
    int c[K];
    T v[K], xv[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        c[k] = b + k < e ? __ldg(p.col + b + k) : -1;
        v[k] = b + k < e ? __ldg(p.M + b + k) : T(0);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) xv[k] = c[k] >= 0 ? __ldg(p.x + c[k]) : T(0);
    T sum = T(0);
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (c[k] >= 0) sum = fma_t(v[k], xv[k], sum);  // phantoms skipped
    for (int q = b + K; q < e; ++q) {
        const int j = __ldg(p.col + q);
        if (j >= 0) sum = fma_t(__ldg(p.M + q), __ldg(p.x + j), sum);
    }
    return sum;
}

template <typename T, int KIND, bool DIV>
__global__ void __launch_bounds__(kThreads, 8) range_sweep_kernel(RangeParams<T> p)
{
    if (p.done && *p.done) return;
    const int i = p.r0 + (int)(blockIdx.x * kThreads + threadIdx.x);
    if (i >= p.r1) return;
    const int d = __ldg(p.diag + i);
    if constexpr (KIND == 2) {
        const T num = y_of(p, i) - upper_sum(p, d, __ldg(p.rp + i + 1));
        p.x[i] = DIV ? num / __ldg(p.M + d) : num * __ldg(p.dinv + i);
    } else {
        const T yi = __ldg(p.rhs + i) - lower_sum(p, __ldg(p.rp + i), d);
        if constexpr (KIND == 0)
            p.y[i] = yi;
        else
            p.x[i] = DIV ? yi / __ldg(p.M + d) : yi * __ldg(p.dinv + i);
    }
}

template <typename T, int KIND>
void range_launch(cudaStream_t st, RangeParams<T> p, int r0, int r1, bool div)
{
    if (r1 <= r0) return;
    p.r0 = r0;
    p.r1 = r1;
    const int grid = (r1 - r0 + kThreads - 1) / kThreads;
    if (div)
        range_sweep_kernel<T, KIND, true><<<grid, kThreads, 0, st>>>(p);
    else
        range_sweep_kernel<T, KIND, false><<<grid, kThreads, 0, st>>>(p);
}

template <typename T>
RangeParams<T> make_range(const DevPattern& P, const T* M, const T* dinv, const T* rhs, T* y,
                          T* x, const int* done)
{
    RangeParams<T> p;
    p.rp = P.rp;
    p.col = P.col;
    p.diag = P.diag;
    p.M = M;
    p.dinv = dinv;
    p.rhs = rhs;
    p.y = y;
    p.x = x;
    p.r0 = p.r1 = 0;
    p.rhs_end = 0;
    p.done = done;
    return p;
}

// The preconditioner on a red-black box's records (RbGeom), arithmetic of
// range_sweep_kernel: colour 1 (KIND 1: y = rhs - sum over z-, y-, x-, x+,
// y+, z+ of M y with y = rhs on colour 0, then x = y / M_ii or y dinv),
// colour 0 (KIND 2: x = (rhs - sum over the same neighbours of M x) / M_ii or
// dinv); neighbour rows computed, not read.
template <typename T, int KIND, bool DIV>
__global__ void __launch_bounds__(kThreads, 8) rb_precond_kernel(RbGeom g, const T* rec,
                                                                 const T* dinv, const T* rhs,
                                                                 T* out, const int* done)
{
    if (done && *done) return;
    using V = typename std::conditional<sizeof(T) == 8, double4, float4>::type;
    const int t = (KIND == 1 ? g.n0 : 0) + (int)(blockIdx.x * kThreads + threadIdx.x);
    if (t >= (KIND == 1 ? g.n : g.n0)) return;
    const RbRow q = rb_row_info(g, t);
    const V* lo = reinterpret_cast<const V*>(rec);
    const V l = lo[t], h = lo[g.n + t];
    const T v[6] = {l.x, l.y, l.z, l.w, h.x, h.y};
    const T* src = KIND == 1 ? rhs : out;  // colour 0's y is rhs; colour 1's x is out
    T xn[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) xn[s] = q.has[s] ? __ldg(src + q.nb[s]) : T(0);
    T sum = T(0);
#pragma unroll
    for (int s = 0; s < 6; ++s)
        if (q.has[s]) sum = fma_t(v[s], xn[s], sum);
    const T num = __ldg(rhs + t) - sum;
    out[t] = DIV ? num / h.z : num * __ldg(dinv + t);
}

// CSR values -> red-black stencil records through the slot map.
template <typename TO>
__global__ void __launch_bounds__(kThreads) rb_records_kernel(int n, const int* rp,
                                                              const signed char* slot,
                                                              const double* M, TO* rec)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    for (int q = __ldg(rp + t); q < __ldg(rp + t + 1); ++q) {
        const int s = slot[q];
        if (s >= 0) rec[((size_t)(s >> 2) * n + t) * 4 + (s & 3)] = (TO)M[q];
    }
}

// Tiny systems with a deep schedule (the 1D shock tube's chain: one row per
// level): a single warp walks the rows in natural order (reverse order for
// the backward sweep), a topological order of either triangle, so there is
// nothing to wait for.  Rows are taken 32 at a time: lane k loads row k's
// triangle entries (up to kSerialK of them), right-hand side, divisor and
// the divisor's reciprocal into shared memory in one parallel round trip;
// then lane 0 alone runs the rows' chain (the other lanes would only repeat
// its FP64 work), with the solution in shared memory and the last row's
// value in a register (a chain row depends on the row before it).  Sums run
// over the entries in storage order with fma from 0, and a result with the
// all-ones pattern is stored as the canonical NaN, as in the level-scheduled
// kernels: the results are the same bits.
constexpr int kSerialK = 4;

// a / b, correctly rounded, by Markstein's method (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990).  Off the chain, per row: y =
// RN(1/b) and y_lo = RN((1 - b y) y), so y + y_lo is 1/b to about 2^-104
// (1 - b y is exact in an fma).  On the chain: q = RN(a y + a y_lo) is within
// an ulp of a/b, and one residual correction q + (a - b q) y is, by
// Markstein's theorem (y within half an ulp of 1/b, q within an ulp of a/b),
// the correctly rounded quotient; the residual a - b q is an exact fma.
// Operands outside [2^-500, 2^500] in magnitude (zeros, subnormals,
// infinities, NaN, values near over- or underflow) take the IEEE division.
// Four dependent FP64 operations instead of a division, which costs about
// nine times one of them on this GPU.
__device__ __forceinline__ double div_rcp(double a, double b, double y, double ylo, bool b_ok)
{
    return divide(a, Recip{b, y, ylo, b_ok});  // division.cuh
}

__device__ __forceinline__ float div_rcp(float a, float b, float, float, bool) { return a / b; }

template <typename T, bool FW, bool DIV>
__global__ void __launch_bounds__(32) serial_sweep_kernel(SweepParams<T> p)
{
    if (p.done && *p.done) return;
    extern __shared__ __align__(16) unsigned char serial_smem[];
    T* xs = reinterpret_cast<T*>(serial_smem);
    __shared__ int s_row[32], s_q0[32], s_q1[32], s_ok[32];
    __shared__ int s_col[kSerialK][32];
    __shared__ T s_rhs[32], s_div[32], s_rcp[32], s_rlo[32];
    __shared__ T s_m[kSerialK][32];
    using B = Bits<T>;
    const int lane = (int)threadIdx.x;
    const int n = p.n;
    int last_i = -1;
    T last = T(0);
    for (int base = 0; base < n; base += 32) {
        const int r = base + lane;
        if (r < n) {
            const int i = FW ? r : n - 1 - r;
            const int d = __ldg(p.diag + i);
            const int q0 = FW ? __ldg(p.rp + i) : d + 1;
            const int q1 = FW ? d : __ldg(p.rp + i + 1);
            s_row[lane] = i;
            s_q0[lane] = q0;
            s_q1[lane] = q1;
            s_rhs[lane] = p.rhs[i];
            if (!FW) {
                const T dv = DIV ? __ldg(p.M + d) : __ldg(p.dinv + i);
                s_div[lane] = dv;
                if (DIV) {
                    const T y = T(1) / dv;
                    s_rcp[lane] = y;
                    s_rlo[lane] = fma_t(-dv, y, T(1)) * y;
                    if constexpr (sizeof(T) == 8) s_ok[lane] = markstein_range(dv) ? 1 : 0;
                    else s_ok[lane] = 0;
                }
            }
#pragma unroll
            for (int t = 0; t < kSerialK; ++t) {
                const bool in = q0 + t < q1;
                s_col[t][lane] = in ? __ldg(p.col + q0 + t) : -1;
                s_m[t][lane] = in ? __ldg(p.M + q0 + t) : T(0);
            }
        }
        __syncwarp();
        if (lane == 0) {
            const int cnt = min(32, n - base);
            for (int k = 0; k < cnt; ++k) {
                const int ik = s_row[k];
                T sum = T(0);
#pragma unroll
                for (int t = 0; t < kSerialK; ++t) {
                    const int j = s_col[t][k];
                    if (j >= 0) sum = fma_t(s_m[t][k], j == last_i ? last : xs[j], sum);
                }
                for (int q = s_q0[k] + kSerialK; q < s_q1[k]; ++q) {  // rows with more entries
                    const int j = __ldg(p.col + q);
                    if (j < 0) continue;  // phantom: the reference adds 0 * x[-1]
                    sum = fma_t(__ldg(p.M + q), j == last_i ? last : xs[j], sum);
                }
                const T num = s_rhs[k] - sum;
                T v = num;
                if (!FW)
                    v = DIV ? div_rcp(num, s_div[k], s_rcp[k], s_rlo[k], s_ok[k] != 0)
                            : num * s_div[k];
                if (B::to(v) == B::kSentinel) v = B::from(B::kCanonicalNaN);
                xs[ik] = v;
                p.out[ik] = v;
                last_i = ik;
                last = v;
            }
        }
        __syncwarp();
    }
}

struct IluParams {
    int n;
    const int* rp;
    const int* col;
    const int* diag;
    const int* pair_ptr;
    const int* pair_k;
    const int* pair_slot;
    const double* A;
    const double* Mold;
    double* Mnew;
    double* dinv;
    float* M32;
    float* dinv32;
    float* A32;
    const int* done;
    int* pivot_err;  // last sweep: OCSL_ZERO_PIVOT on a zero or infinite M_ii
};

// A broken-down pivot: zero or infinite (for the FP32 inner solver also an
// infinite FP32 reciprocal).  The reference's own check of the sequential
// factor tests M_ii == 0 (cmatrix_solver.cpp:495-500, commented out there);
// the fixed-point factor turns a zero pivot into infinities in the sweeps
// after it.  A NaN pivot comes from NaN / Inf in the matrix itself, which the
// iteration reports as OCSL_NONFINITE.
__device__ __forceinline__ void check_pivot(double m, const float* r32, int* err)
{
    const bool bad = m == 0.0 || isinf(m) || (r32 && isinf(*r32));
    if (bad) atomicCAS(err, 0, (int)OCSL_ZERO_PIVOT);
}

// One Jacobi sweep of the reference's fixed-point ILU (cmatrix_solver.cpp:525-549):
//   lower  (col < i):  Mnew_ij = (A_ij - sum_k M_ik M_kj) / M_jj
//   other           :  Mnew_ij =  A_ij - sum_k M_ik M_kj
// with the products listed by the host in the reference's k order (the
// table omits products whose CCSR::get_element would return 0).  Optional
// outputs of the last sweep: reciprocal diagonal and FP32 copies.
__global__ void __launch_bounds__(kThreads) ilu_sweep_kernel(IluParams p)
{
    if (p.done && *p.done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const int b = __ldg(p.rp + i), e = __ldg(p.rp + i + 1), di = __ldg(p.diag + i);
    for (int j = b; j < e; ++j) {
        const int c = __ldg(p.col + j);
        double dum = 0.0;
        const int q1 = __ldg(p.pair_ptr + j + 1);
        for (int q = __ldg(p.pair_ptr + j); q < q1; ++q)
            dum = fma(p.Mold[__ldg(p.pair_k + q)], p.Mold[__ldg(p.pair_slot + q)], dum);
        const double a = p.A[j];
        const double m = (c >= 0 && c < i) ? (a - dum) / p.Mold[__ldg(p.diag + c)] : a - dum;
        p.Mnew[j] = m;
        if (p.M32) p.M32[j] = (float)m;
        if (p.A32) p.A32[j] = (float)a;
        if (j == di) {
            float r32 = 0.f;
            if (p.dinv) {
                const double r = 1.0 / m;
                p.dinv[i] = r;
                r32 = (float)r;
                if (p.dinv32) p.dinv32[i] = r32;
            }
            if (p.pivot_err) check_pivot(m, p.dinv32 ? &r32 : nullptr, p.pivot_err);
        }
    }
}

__global__ void factor_outputs_kernel(int n, const int* rp, const int* diag, const double* M,
                                      const double* A, double* dinv, float* M32, float* dinv32,
                                      float* A32, int* pivot_err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = rp[i], e = rp[i + 1];
    for (int j = b; j < e; ++j) {
        if (M32) M32[j] = (float)M[j];
        if (A32) A32[j] = (float)A[j];
    }
    const double m = M[diag[i]];
    const double r = 1.0 / m;
    const float r32 = (float)r;
    if (dinv) dinv[i] = r;
    if (dinv32) dinv32[i] = r32;
    if (pivot_err) check_pivot(m, dinv32 ? &r32 : nullptr, pivot_err);
}

// Fill a sweep's output with the all-ones pattern, unless the solve is done:
// a batch queued after convergence must not clobber vectors still in use.
// `head` 32-bit words bring the pointer to a 16-byte boundary, then 16-byte
// stores, then `tail` words.
__global__ void __launch_bounds__(kThreads) fill_ones_kernel(unsigned* out, int head,
                                                            long long n16, int tail,
                                                            const int* done, int ndone,
                                                            int done_stride)
{
    if (done) {  // skipped once every listed flag is set
        bool all = true;
        for (int q = 0; q < ndone; ++q) all = all && done[q * done_stride] != 0;
        if (all) return;
    }
    const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (gid < head) out[gid] = ~0u;
    uint4* body = reinterpret_cast<uint4*>(out + head);
    const uint4 ones = make_uint4(~0u, ~0u, ~0u, ~0u);
    for (long long i = gid; i < n16; i += (long long)gridDim.x * blockDim.x) body[i] = ones;
    if (gid < tail) out[head + 4 * n16 + gid] = ~0u;
}

template <typename T>
SweepParams<T> make_sweep(const DevPattern& P, bool forward, const T* M, const T* dinv,
                          const T* rhs, T* out, const SweepSync& S, const int* done)
{
    SweepParams<T> p;
    p.n = P.n;
    p.rp = P.rp;
    p.col = P.col;
    p.diag = P.diag;
    p.order = forward ? P.fw_order : P.bw_order;
    p.chunk = forward ? P.fw_chunk : P.bw_chunk;
    p.nchunks = forward ? P.fw_nchunks : P.bw_nchunks;
    p.M = M;
    p.dinv = dinv;
    p.rhs = rhs;
    p.out = out;
    p.S = S;
    p.done = done;
    return p;
}

// Fault injection (SweepSync::skip_first): the dispenser starts at 1 and the
// grid is one chunk short, so chunk 0 is never solved.  Returns the chunks
// left out (0 when there is only one).
int skip_chunks(cudaStream_t st, const SweepSync& S, int nchunks)
{
    if (!S.skip_first || nchunks < 2) return 0;
    preset_ticket_one(st, S.ticket);
    return 1;
}

}  // namespace

void preset_ticket_one(cudaStream_t st, unsigned* ticket)
{
    // little-endian word 0 -> 1: only its lowest byte changes
    cudaMemsetAsync(ticket, 1, 1, st);
}

template <typename T>
void launch_fw_sweep(cudaStream_t st, const DevPattern& P, const T* M, const T* rhs, T* out,
                     const SweepSync& S, const int* done)
{
    if (P.n == 0) return;  // `out` holds the all-ones pattern (filled by the caller)
    auto p = make_sweep<T>(P, true, M, nullptr, rhs, out, S, done);
    fw_sweep_kernel<T><<<p.nchunks - skip_chunks(st, S, p.nchunks), kThreads, 0, st>>>(p);
}

template <typename T>
void launch_range_sweep(cudaStream_t st, const DevPattern& P, bool forward, const T* M,
                        const T* dinv, const T* rhs, T* out, int divmode, const int* done)
{
    const int nr = forward ? P.fw_nrange : P.bw_nrange;
    const int* rg = forward ? P.fw_range : P.bw_range;
    // forward: y = out, rhs the input; backward: y = the input, x = out
    const auto p = forward ? make_range<T>(P, M, dinv, rhs, out, nullptr, done)
                           : make_range<T>(P, M, dinv, nullptr, const_cast<T*>(rhs), out, done);
    for (int l = 0; l < nr; ++l) {
        if (forward)
            range_launch<T, 0>(st, p, rg[2 * l], rg[2 * l + 1], false);
        else
            range_launch<T, 2>(st, p, rg[2 * l], rg[2 * l + 1], divmode == 0);
    }
}

template <typename T>
void launch_rb_precond(cudaStream_t st, const RbGeom& g, const T* rec, const T* dinv,
                       const T* rhs, T* out, int divmode, const int* done)
{
    const int n1 = g.n - g.n0;
    const bool div = divmode == 0;
    if (n1 > 0) {
        const int grid = (n1 + kThreads - 1) / kThreads;
        if (div) rb_precond_kernel<T, 1, true><<<grid, kThreads, 0, st>>>(g, rec, dinv, rhs, out, done);
        else rb_precond_kernel<T, 1, false><<<grid, kThreads, 0, st>>>(g, rec, dinv, rhs, out, done);
    }
    if (g.n0 > 0) {
        const int grid = (g.n0 + kThreads - 1) / kThreads;
        if (div) rb_precond_kernel<T, 2, true><<<grid, kThreads, 0, st>>>(g, rec, dinv, rhs, out, done);
        else rb_precond_kernel<T, 2, false><<<grid, kThreads, 0, st>>>(g, rec, dinv, rhs, out, done);
    }
}

template <typename TO>
void launch_rb_records(cudaStream_t st, const RbGeom& g, const int* rp, const signed char* slot,
                       const double* M, TO* rec)
{
    if (g.n > 0)
        rb_records_kernel<TO><<<(g.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(g.n, rp, slot,
                                                                                  M, rec);
}

template <typename T>
void launch_coloured_precond(cudaStream_t st, const DevPattern& P, const T* M, const T* dinv,
                             const T* rhs, T* tmp, T* out, int divmode, const int* done)
{
    const int C = P.fw_nrange;  // colours; fw_range holds them in ascending order
    if (C == 0) return;
    auto p = make_range<T>(P, M, dinv, rhs, tmp, out, done);
    p.rhs_end = P.fw_range[1];  // colour 0: y = rhs
    const bool div = divmode == 0;
    for (int c = 1; c < C - 1; ++c) range_launch<T, 0>(st, p, P.fw_range[2 * c], P.fw_range[2 * c + 1], false);
    range_launch<T, 1>(st, p, P.fw_range[2 * (C - 1)], P.fw_range[2 * C - 1], div);
    for (int c = C - 2; c >= 0; --c) range_launch<T, 2>(st, p, P.fw_range[2 * c], P.fw_range[2 * c + 1], div);
}

template <typename T>
void launch_bw_sweep(cudaStream_t st, const DevPattern& P, const T* M, const T* dinv,
                     const T* rhs, T* out, int divmode, const SweepSync& S, const int* done)
{
    if (P.n == 0) return;  // `out` holds the all-ones pattern (filled by the caller)
    auto p = make_sweep<T>(P, false, M, dinv, rhs, out, S, done);
    const int grid = p.nchunks - skip_chunks(st, S, p.nchunks);
    if (divmode == 0)
        bw_sweep_kernel<T, true><<<grid, kThreads, 0, st>>>(p);
    else
        bw_sweep_kernel<T, false><<<grid, kThreads, 0, st>>>(p);
}

template <typename T>
void launch_serial_sweep(cudaStream_t st, const DevPattern& P, bool forward, const T* M,
                         const T* dinv, const T* rhs, T* out, int divmode, const int* done)
{
    if (P.n == 0) return;
    SweepSync none{};
    auto p = make_sweep<T>(P, forward, M, dinv, rhs, out, none, done);
    const size_t smem = sizeof(T) * (size_t)P.n;
    if (forward)
        serial_sweep_kernel<T, true, true><<<1, 32, smem, st>>>(p);
    else if (divmode == 0)
        serial_sweep_kernel<T, false, true><<<1, 32, smem, st>>>(p);
    else
        serial_sweep_kernel<T, false, false><<<1, 32, smem, st>>>(p);
}

template <typename T>
void launch_ilu_sweep(cudaStream_t st, const DevPattern& P, const T* A, const T* Mold, T* Mnew,
                      double* dinv, float* M32, float* dinv32, float* A32, const int* done,
                      int* pivot_err)
{
    static_assert(sizeof(T) == 8, "the ILU factor is computed in FP64");
    if (P.n == 0) return;
    IluParams p;
    p.n = P.n;
    p.rp = P.rp;
    p.col = P.col;
    p.diag = P.diag;
    p.pair_ptr = P.pair_ptr;
    p.pair_k = P.pair_k;
    p.pair_slot = P.pair_slot;
    p.A = A;
    p.Mold = Mold;
    p.Mnew = Mnew;
    p.dinv = dinv;
    p.M32 = M32;
    p.dinv32 = dinv32;
    p.A32 = A32;
    p.done = done;
    p.pivot_err = pivot_err;
    ilu_sweep_kernel<<<(P.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(p);
}

void launch_fill_ones(cudaStream_t st, void* out, size_t bytes, const int* done, int ndone,
                      int done_stride)
{
    // `out` is element-aligned (4 or 8 bytes); the entry points check that.
    const size_t words = bytes / 4;
    if (words == 0) return;
    const uintptr_t a = reinterpret_cast<uintptr_t>(out);
    size_t head = ((16 - (a & 15)) & 15) / 4;
    if (head > words) head = words;
    const long long n16 = (long long)((words - head) / 4);
    const int tail = (int)(words - head - 4 * (size_t)n16);
    long long blocks = (n16 + kThreads - 1) / kThreads;
    if (blocks < 1) blocks = 1;
    if (blocks > 4096) blocks = 4096;
    fill_ones_kernel<<<(int)blocks, kThreads, 0, st>>>(static_cast<unsigned*>(out), (int)head,
                                                       n16, tail, done, ndone, done_stride);
}

void launch_factor_outputs(cudaStream_t st, const DevPattern& P, const double* M, const double* A,
                           double* dinv, float* M32, float* dinv32, float* A32, int* pivot_err)
{
    if (P.n == 0) return;
    factor_outputs_kernel<<<(P.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        P.n, P.rp, P.diag, M, A, dinv, M32, dinv32, A32, pivot_err);
}

template void launch_fw_sweep<double>(cudaStream_t, const DevPattern&, const double*,
                                      const double*, double*, const SweepSync&, const int*);
template void launch_fw_sweep<float>(cudaStream_t, const DevPattern&, const float*, const float*,
                                     float*, const SweepSync&, const int*);
template void launch_bw_sweep<double>(cudaStream_t, const DevPattern&, const double*,
                                      const double*, const double*, double*, int,
                                      const SweepSync&, const int*);
template void launch_bw_sweep<float>(cudaStream_t, const DevPattern&, const float*, const float*,
                                     const float*, float*, int, const SweepSync&, const int*);
template void launch_range_sweep<double>(cudaStream_t, const DevPattern&, bool, const double*,
                                         const double*, const double*, double*, int, const int*);
template void launch_range_sweep<float>(cudaStream_t, const DevPattern&, bool, const float*,
                                        const float*, const float*, float*, int, const int*);
template void launch_rb_precond<double>(cudaStream_t, const RbGeom&, const double*,
                                        const double*, const double*, double*, int, const int*);
template void launch_rb_precond<float>(cudaStream_t, const RbGeom&, const float*, const float*,
                                       const float*, float*, int, const int*);
template void launch_rb_records<double>(cudaStream_t, const RbGeom&, const int*,
                                        const signed char*, const double*, double*);
template void launch_rb_records<float>(cudaStream_t, const RbGeom&, const int*,
                                       const signed char*, const double*, float*);
template void launch_coloured_precond<double>(cudaStream_t, const DevPattern&, const double*,
                                              const double*, const double*, double*, double*, int,
                                              const int*);
template void launch_coloured_precond<float>(cudaStream_t, const DevPattern&, const float*,
                                             const float*, const float*, float*, float*, int,
                                             const int*);
template void launch_serial_sweep<double>(cudaStream_t, const DevPattern&, bool, const double*,
                                          const double*, const double*, double*, int,
                                          const int*);
template void launch_serial_sweep<float>(cudaStream_t, const DevPattern&, bool, const float*,
                                         const float*, const float*, float*, int, const int*);
template void launch_ilu_sweep<double>(cudaStream_t, const DevPattern&, const double*,
                                       const double*, double*, double*, float*, float*, float*,
                                       const int*, int*);

}  // namespace ocsl
