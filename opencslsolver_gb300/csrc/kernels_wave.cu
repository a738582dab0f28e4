// Warp-pipelined structured sweeps for 7-point box patterns (one right-hand
// side).
//
// The forward sweep of a natural-order 7-point stencil, y = L^-1 rhs
// (cmatrix_solver.cpp:555-572), is a chain of wavefronts W = a + b + s: row
// (a, b, s) needs the rows (a-1, b, s), (a, b-1, s) and (a, b, s-1).  The
// backward sweep (:595-611) is the same with every coordinate mirrored.
//
// Here one warp owns a column tile of K (along a) x 32 (along b, one lane
// each) columns and walks its own steps t = 0, 1, ...: at step t, column k of
// lane l solves row s = t - k - l.  Every dependency of that row was solved
// at step t - 1 inside the same warp:
//   (a-1, b, s): column k-1 of the same lane         -> a register
//   (a, b-1, s): column k of lane l-1                 -> one warp shuffle
//   (a, b, s-1): column k of the same lane            -> a register
// so a step is K independent fma chains, no barrier and no memory round trip
// on the critical path.  Only the tile's faces come from outside: column 0's
// a-neighbour from the warp to the left (same CTA: one shared-memory slot per
// s row; other CTA: the output vector in global memory) and lane 0's
// b-neighbours from the tile below (global memory).  Values crossing a CTA
// use the value-as-flag protocol of the other sweeps -- the output is
// pre-filled with all-ones, every wait is bounded (OCSL_TIMEOUT and a NaN
// when it runs out) -- and are fetched a few steps ahead into a register
// ring; shared-memory faces are filled with the same sentinel at the start.
//
// A row's arithmetic is the packed record's fma chain in CSR order (z-, y-,
// x-), then rhs - sum (and the division by, or the product with the
// reciprocal of, the diagonal backward), exactly as in box_cta_kernel, so
// results are bit-identical to the oracle whatever the tile shape.
//
// Records and right-hand sides are staged with per-lane cp.async into a
// P-step ring in shared memory; each lane reads back only what it copied
// itself, so no barrier is needed there either.  CTAs take tiles from an
// atomic ticket in row-major tile order (a tile's upstream neighbours come
// first), so a waiting CTA never waits on an unscheduled one.
#include <algorithm>
#include <mutex>

#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr long kSpinLimit = 1L << 21;
constexpr int kP = 12;   // cp.async ring depth (steps)
constexpr int kDF = 4;   // global face values fetched this many steps ahead
constexpr int kWaveLag = kDF + 2;    // default start lag behind an upstream CTA (rows)
constexpr int kWaveLagShared = 1;    // ... behind the warp to the left

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

template <typename U>
__device__ __forceinline__ U vload_shared(const U* p)
{
    if constexpr (sizeof(U) == 8) {
        U v;
        asm volatile("ld.volatile.shared.b64 %0, [%1];"
                     : "=l"(v)
                     : "r"((unsigned)__cvta_generic_to_shared(p)));
        return v;
    } else {
        U v;
        asm volatile("ld.volatile.shared.b32 %0, [%1];"
                     : "=r"(v)
                     : "r"((unsigned)__cvta_generic_to_shared(p)));
        return v;
    }
}
template <typename U>
__device__ __forceinline__ void vstore_shared(U* p, U v)
{
    if constexpr (sizeof(U) == 8)
        asm volatile("st.volatile.shared.b64 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)),
                     "l"(v));
    else
        asm volatile("st.volatile.shared.b32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)),
                     "r"(v));
}

// Bounded polls (OCSL_TIMEOUT and a NaN when they run out, or as soon as
// another wait of the launch has given up).
template <typename T>
__device__ __noinline__ T wait_global(const T* p, int* err)
{
    using B = Bits<T>;
    unsigned ns = 0;
    for (long it = 0; it < kSpinLimit; ++it) {
        const typename B::U u = B::load(p);
        if (u != B::kSentinel) return B::from(u);
        if (ns) __nanosleep(ns);
        ns = it < 64 ? 0u : (ns == 0 ? 32u : (ns < 256u ? ns * 2u : 256u));
        if ((it & 255) == 255 && *((volatile int*)err) != 0) break;
    }
    atomicCAS(err, 0, (int)OCSL_TIMEOUT);
    return B::from(B::kCanonicalNaN);
}
template <typename T>
__device__ __noinline__ T wait_shared(const typename Bits<T>::U* p, int* err)
{
    using B = Bits<T>;
    for (long it = 0; it < kSpinLimit; ++it) {
        const typename B::U u = vload_shared(p);
        if (u != B::kSentinel) return B::from(u);
        if ((it & 255) == 255 && *((volatile int*)err) != 0) break;
    }
    atomicCAS(err, 0, (int)OCSL_TIMEOUT);
    return B::from(B::kCanonicalNaN);
}
template <typename T>
__device__ __forceinline__ typename Bits<T>::U to_bits(T v)
{
    using B = Bits<T>;
    typename B::U u = B::to(v);
    return u == B::kSentinel ? B::kCanonicalNaN : u;
}

template <typename T>
struct Rec;
template <>
struct alignas(16) Rec<float> {
    float v[4];
};
template <>
struct alignas(32) Rec<double> {
    double v[4];
};

template <typename T>
__device__ __forceinline__ void cp_rec(Rec<T>* dst, const Rec<T>* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const char* s = reinterpret_cast<const char*>(src);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(s) : "memory");
    if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16), "l"(s + 16) : "memory");
}
template <typename T>
__device__ __forceinline__ void cp_val(T* dst, const T* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <typename T>
struct WaveParams {
    WaveGeom g;
    int n;
    const T* soa;  // packed records [2][n][4]: (z-, y-, x-, 0), (x+, y+, z+, diagonal term)
    const T* rhs;
    T* out;
    SweepSync S;
    const int* done;
};

// FWD: y = L^-1 rhs (unit L); !FWD: x = U^-1 rhs, DIV: divide by the
// diagonal (the reference), else multiply by the stored reciprocal.  SPAN:
// which of x (0), y (1), z (2) the canonical s dimension is.
template <typename T, bool FWD, bool DIV, int SPAN, int K>
__global__ void __launch_bounds__(32 * kWaveMaxWarps) wave_sweep_kernel(WaveParams<T> p)
{
    if (p.done && *p.done) return;
    using B = Bits<T>;
    using U = typename B::U;
    using R = Rec<T>;
    extern __shared__ __align__(32) unsigned char smem_raw[];
    const WaveGeom& g = p.g;
    const int WA = g.WA;
    const int w = (int)threadIdx.x >> 5, l = (int)threadIdx.x & 31;
    const int Da = g.D[0], Db = g.D[1], Ds = g.D[2];
    R* ring = reinterpret_cast<R*>(smem_raw);                 // [WA][kP][K][32]
    T* rring = reinterpret_cast<T*>(ring + WA * kP * K * 32); // [WA][kP][K][32]
    U* faceA = reinterpret_cast<U*>(rring + WA * kP * K * 32); // [WA-1][Ds][32]
    __shared__ int s_tile;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(p.S.ticket, 1u);
    for (int i = threadIdx.x; i < (WA - 1) * Ds * 32; i += blockDim.x) faceA[i] = B::kSentinel;
    __syncthreads();
    const int tile = s_tile;
    if (tile >= g.nta * g.ntb) {  // never with a fresh dispenser; keeps every access in bounds
        if (threadIdx.x == 0) atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
    } else {
        const int ta = tile % g.nta, tb = tile / g.nta;
        const int a0 = (ta * WA + w) * K;  // canonical a of column 0
        const int b = tb * 32 + l;
        const bool b_ok = b < Db;
        const int dstep = FWD ? -1 : 1;    // physical offset of an upstream neighbour
        const int off_a = dstep * g.S[0], off_b = dstep * g.S[1];
        const int sstep = FWD ? g.S[2] : -g.S[2];
        // physical row of column k at s = 0
        int base[K];
        bool ok[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int a = a0 + k;
            ok[k] = b_ok && a < Da;
            const int pa = FWD ? a : Da - 1 - a;
            const int pb = FWD ? b : Db - 1 - b;
            base[k] = pa * g.S[0] + pb * g.S[1] + (FWD ? 0 : (Ds - 1) * g.S[2]);
        }
        const bool has_b = b > 0;          // lane l-1 or the tile below holds (a, b-1)
        const bool face_b = has_b && l == 0;   // ... the tile below (global)
        const bool has_a = a0 > 0;         // column 0's a-neighbour exists
        const bool face_a_sh = has_a && w > 0;   // ... in the warp to the left (shared)
        const bool face_a_gl = has_a && w == 0;  // ... in the CTA to the left (global)
        const bool push_a = w < WA - 1;    // column K-1 feeds the warp to the right
        const R* recs = reinterpret_cast<const R*>(p.soa) + (FWD ? 0 : p.n);
        R* my_ring = ring + w * kP * K * 32;
        T* my_rr = rring + w * kP * K * 32;
        const U* fa_in = faceA + (w - 1) * Ds * 32;  // valid when w > 0
        U* fa_out = faceA + w * Ds * 32;             // valid when w < WA - 1
        int* err = p.S.err;

        auto refill = [&](int t, int j) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int s = t - k - l;
                if (ok[k] && s >= 0 && s < Ds) {
                    const int r = base[k] + s * sstep;
                    cp_rec<T>(&my_ring[(j * K + k) * 32 + l], recs + r);
                    cp_val<T>(&my_rr[(j * K + k) * 32 + l], p.rhs + r);
                }
            }
            cp_commit();
        };
#pragma unroll
        for (int j = 0; j < kP; ++j) refill(j, j);

        // Start behind the upstream tiles: wait for their face values at
        // s = lag next to this tile (lane 0, column 0), so that the values
        // fetched kDF steps ahead are normally final; behind the warp to the
        // left by lag_sh rows.
        {
            const int sg = min(g.lag, Ds - 1), ss = min(g.lag_sh, Ds - 1);
            if (face_a_gl && l == 0 && ok[0]) (void)wait_global(p.out + base[0] + sg * sstep + off_a, err);
            if (face_b && ok[0]) (void)wait_global(p.out + base[0] + sg * sstep + off_b, err);
            if (face_a_sh && l == 0 && ok[0]) {
                const U* slot = fa_in + ss * 32;
                if (vload_shared(slot) == B::kSentinel) (void)wait_shared<T>(slot, err);
            }
        }
        __syncwarp();

        // global face values, kDF steps ahead: fa (column 0, a-1), fb (lane 0, b-1)
        U fa[kDF], fb[kDF][K];
        auto fetch = [&](int t, int j) {
            fa[j] = B::kSentinel;
            if (face_a_gl) {
                const int s = t - l;
                if (ok[0] && s >= 0 && s < Ds) fa[j] = B::load(p.out + base[0] + s * sstep + off_a);
            }
#pragma unroll
            for (int k = 0; k < K; ++k) {
                fb[j][k] = B::kSentinel;
                const int s = t - k;
                if (face_b && ok[k] && s >= 0 && s < Ds)
                    fb[j][k] = B::load(p.out + base[k] + s * sstep + off_b);
            }
        };
#pragma unroll
        for (int j = 0; j < kDF; ++j) fetch(j, j);

        T cur[K];
#pragma unroll
        for (int k = 0; k < K; ++k) cur[k] = T(0);
        // one past the last step of the warp's last column in range
        const int kmax = min(K - 1, max(Da - 1 - a0, 0));
        const int lmax = min(31, max(Db - 1 - tb * 32, 0));
        const int T_end = Ds + kmax + lmax;
        for (int tb0 = 0; tb0 < T_end; tb0 += kP) {
#pragma unroll
            for (int j = 0; j < kP; ++j) {
                const int t = tb0 + j;
                if (t >= T_end) break;  // uniform over the warp
                const int jf = j % kDF;
                cp_wait<kP - 1>();
                T up[K];  // lane l-1's values of the previous step (b-neighbours)
#pragma unroll
                for (int k = 0; k < K; ++k) up[k] = __shfl_up_sync(0xffffffffu, cur[k], 1);
                T nv[K];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    nv[k] = cur[k];
                    const int s = t - k - l;
                    if (ok[k] && s >= 0 && s < Ds) {
                        const R cf = my_ring[(j * K + k) * 32 + l];
                        const T rh = my_rr[(j * K + k) * 32 + l];
                        T va = T(0), vb = T(0);
                        if (k > 0) {
                            va = cur[k - 1];  // a0 + k > 0 always
                        } else if (face_a_sh) {
                            const U* slot = fa_in + s * 32 + l;
                            const U u = vload_shared(slot);
                            va = u != B::kSentinel ? B::from(u) : wait_shared<T>(slot, err);
                        } else if (face_a_gl) {
                            va = fa[jf] != B::kSentinel
                                     ? B::from(fa[jf])
                                     : wait_global(p.out + base[0] + s * sstep + off_a, err);
                        }
                        if (l > 0) {
                            vb = up[k];
                        } else if (face_b) {
                            vb = fb[jf][k] != B::kSentinel
                                     ? B::from(fb[jf][k])
                                     : wait_global(p.out + base[k] + s * sstep + off_b, err);
                        }
                        const T vs = s > 0 ? cur[k] : T(0);
                        const T vx = SPAN == 0 ? vs : va;
                        const T vy = SPAN == 0 ? va : (SPAN == 1 ? vs : vb);
                        const T vz = SPAN == 2 ? vs : vb;
                        // record: z-, y-, x-, (unused) | x+, y+, z+, diagonal term;
                        // the fma order is the row's CSR order
                        T sum = fma_t(cf.v[0], FWD ? vz : vx, T(0));
                        sum = fma_t(cf.v[1], vy, sum);
                        sum = fma_t(cf.v[2], FWD ? vx : vz, sum);
                        const T num = rh - sum;
                        const T y = FWD ? num : (DIV ? num / cf.v[3] : num * cf.v[3]);
                        nv[k] = y;
                        const U bits = to_bits(y);
                        B::store(p.out + base[k] + s * sstep, bits);
                        if (k == K - 1 && push_a) vstore_shared(fa_out + s * 32 + l, bits);
                    }
                }
#pragma unroll
                for (int k = 0; k < K; ++k) cur[k] = nv[k];
                fetch(t + kDF, jf);
                refill(t + kP, j);
            }
        }
        cp_wait<0>();
    }
    // every warp of the CTA done with the face buffers before the CTA retires
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(p.S.finished, 1u) == gridDim.x - 1) {
            *p.S.ticket = 0u;
            *p.S.finished = 0u;
        }
    }
}

template <typename T>
constexpr int wave_k()
{
    return sizeof(T) == 8 ? 2 : 4;
}

template <typename T, bool FWD, bool DIV, int SPAN>
void launch_wave_one(cudaStream_t st, WaveParams<T> p)
{
    constexpr int K = wave_k<T>();
    auto kern = wave_sweep_kernel<T, FWD, DIV, SPAN, K>;
    static std::once_flag once;
    std::call_once(once, [&] {
        cudaFuncAttributes fa{};
        size_t stat = 1024;
        bool failed = cudaFuncGetAttributes(&fa, kern) != cudaSuccess;
        if (!failed) stat = fa.sharedSizeBytes;
        failed |= cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(kBoxSmemOptin - stat)) != cudaSuccess;
        if (failed) (void)cudaGetLastError();  // the launch itself reports what matters
    });
    const size_t smem = wave_sweep_smem(p.g, (int)sizeof(T));
    int grid = p.g.nta * p.g.ntb;
    if (p.S.skip_first && grid > 1) {  // fault injection: tile 0 never runs
        preset_ticket_one(st, p.S.ticket);
        grid -= 1;
    }
    kern<<<grid, 32 * p.g.WA, smem, st>>>(p);
}

template <typename T, bool FWD, bool DIV>
void launch_wave_span(cudaStream_t st, int span, const WaveParams<T>& p)
{
    switch (span) {
    case 0: launch_wave_one<T, FWD, DIV, 0>(st, p); break;
    case 1: launch_wave_one<T, FWD, DIV, 1>(st, p); break;
    default: launch_wave_one<T, FWD, DIV, 2>(st, p); break;
    }
}

}  // namespace

int wave_cols_per_warp(int elem_size) { return elem_size == 8 ? wave_k<double>() : wave_k<float>(); }

size_t wave_sweep_smem(const WaveGeom& g, int elem_size)
{
    const int K = wave_cols_per_warp(elem_size);
    const size_t rec = (size_t)4 * elem_size;
    return (size_t)g.WA * kP * K * 32 * (rec + elem_size) +
           (size_t)(g.WA - 1) * g.D[2] * 32 * elem_size;
}

WaveGeom make_wave_geom(const BoxGeom& box, int elem_size, int warps, int lag)
{
    WaveGeom g{};
    for (int k = 0; k < 3; ++k) {
        g.D[k] = box.D[k];
        g.S[k] = box.S[k];
    }
    g.span = box.span;
    const int K = wave_cols_per_warp(elem_size);
    const int need = (g.D[0] + K - 1) / K;  // warps to cover a
    int wa = std::max(1, std::min({warps, kWaveMaxWarps, need}));
    g.WA = wa;
    while (g.WA > 1 && wave_sweep_smem(g, elem_size) > kBoxSmemLimit) --g.WA;
    wa = g.WA;
    g.lag = lag > 0 ? lag : kWaveLag;
    g.lag_sh = kWaveLagShared;
    g.nta = (g.D[0] + wa * K - 1) / (wa * K);
    g.ntb = (g.D[1] + 31) / 32;
    return g;
}

template <typename T>
void launch_wave_sweep(cudaStream_t st, const WaveGeom& g, int n, const T* soa, const T* rhs,
                       T* out, bool forward, int divmode, const SweepSync& S, const int* done)
{
    if (n == 0) return;
    WaveParams<T> p;
    p.g = g;
    p.n = n;
    p.soa = soa;
    p.rhs = rhs;
    p.out = out;
    p.S = S;
    p.done = done;
    if (forward)
        launch_wave_span<T, true, false>(st, g.span, p);
    else if (divmode == 0)
        launch_wave_span<T, false, true>(st, g.span, p);
    else
        launch_wave_span<T, false, false>(st, g.span, p);
}

template void launch_wave_sweep<double>(cudaStream_t, const WaveGeom&, int, const double*,
                                        const double*, double*, bool, int, const SweepSync&,
                                        const int*);
template void launch_wave_sweep<float>(cudaStream_t, const WaveGeom&, int, const float*,
                                       const float*, float*, bool, int, const SweepSync&,
                                       const int*);

}  // namespace ocsl
