// Warp-pipelined structured sweeps for 7-point box patterns (one right-hand
// side), with every memory access coalesced.
//
// The forward sweep of a natural-order 7-point stencil, y = L^-1 rhs
// (cmatrix_solver.cpp:555-572), is a chain of wavefronts: row (a, b, s) needs
// (a-1, b, s), (a, b-1, s) and (a, b, s-1).  The backward sweep (:595-611) is
// the same with every coordinate mirrored.  Canonical coordinates here: a = x
// (unit stride), s = the longer of y and z, b = the other one.
//
// One warp owns a tile of 32 (along a, one lane each) x K (along b) columns
// and walks steps t = 0 .. T-1, T = Ds + K - 1 + 31: at step t, column k of
// lane l solves row s = t - k - l.  Every dependency inside the tile was
// solved at step t - 1 by the same warp:
//   (a-1, b, s): column k of lane l-1   -> one warp shuffle
//   (a, b-1, s): column k-1 of lane l   -> a register
//   (a, b, s-1): column k of lane l     -> a register
// so a step is K independent fma chains with no barrier.
//
// Memory.  Rows solved in the same step lie on a diagonal of the box, so
// per-lane loads and stores of natural-order vectors would touch a different
// cache line per lane -- the load/store pipe, not DRAM, then sets the speed.
// Instead:
//   * the factor's stencil records are stored in the sweep's own step order
//     ([tile][t][k][lane], written once per factorisation by
//     box_to_wave_kernel), so each step reads K contiguous 32-record blocks;
//   * the right-hand side and the output go through a ring of s-slices in
//     shared memory: slice s of the tile (K rows of 32 consecutive a) is
//     loaded with one coalesced access per row kP steps before step s, each
//     row's result overwrites its right-hand side in place, and the slice is
//     written back with coalesced stores once its last row is solved (step
//     s + K - 1 + 31);
//   * faces between tiles are exchanged through buffers indexed by the
//     producer's step ([d][k] for the a-face: lane 31 of the tile to the left,
//     [d][lane] for the b-face: column K-1 of the tile below), so that the
//     producer's stores and the consumer's loads are contiguous too.  Faces
//     between the warps of a CTA live in shared memory; faces between CTAs in
//     global memory, where a value is its own ready flag (all-ones = not
//     yet), every wait is bounded (OCSL_TIMEOUT and a NaN when it runs out),
//     values are fetched kDF steps ahead, and the consumer writes the
//     sentinel back after use, so the buffers are ready for the next launch
//     without a fill (after a launch that timed out the host refills them).
//
// A row's arithmetic is the record's fma chain in CSR order (z-, y-, x-),
// then rhs - sum (and the division by, or the product with the reciprocal
// of, the diagonal backward), exactly as in box_cta_kernel: results are
// bit-identical to the oracle whatever the tiling.
//
// A CTA holds WB warps stacked along b; CTAs take tiles from an atomic ticket
// in row-major tile order, so a tile's upstream neighbours always hold
// earlier tickets and a waiting CTA never waits on an unscheduled one.
#include <algorithm>
#include <mutex>

#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr long kSpinLimit = 1L << 21;
constexpr int kP = 8;     // prefetch depth of records and right-hand-side slices (steps)
constexpr int kDF = 4;    // global face values fetched this many steps ahead
constexpr int kWaveLag = kDF + 3;   // default start lag behind an upstream CTA (rows)
// the face ring slot of step t is (t mod kP) mod kDF: equal to t mod kDF only
// when kDF divides kP
static_assert(kP % kDF == 0, "the face ring must tile the step ring");
constexpr int kWaveLagShared = 1;   // ... behind the warp below in the same CTA

template <typename T>
struct Bits;
template <>
struct Bits<double> {
    using U = unsigned long long;
    static constexpr U kSentinel = ~0ull;
    static constexpr U kCanonicalNaN = 0x7FF8000000000000ull;
    static __device__ __forceinline__ U load(const U* p)
    {
        U v;
        asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p));
        return v;
    }
    static __device__ __forceinline__ void store(U* p, U v)
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
    static __device__ __forceinline__ U load(const U* p)
    {
        U v;
        asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p));
        return v;
    }
    static __device__ __forceinline__ void store(U* p, U v)
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
    U v;
    if constexpr (sizeof(U) == 8)
        asm volatile("ld.volatile.shared.b64 %0, [%1];"
                     : "=l"(v)
                     : "r"((unsigned)__cvta_generic_to_shared(p)));
    else
        asm volatile("ld.volatile.shared.b32 %0, [%1];"
                     : "=r"(v)
                     : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
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

// Bounded polls: OCSL_TIMEOUT and a NaN when they run out, or as soon as
// another wait of the launch has given up.
template <typename T>
__device__ __noinline__ T wait_global(const typename Bits<T>::U* p, int* err)
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
    const typename B::U u = B::to(v);
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
    const T* rec;   // this direction's records in step order [nwb][nwa][T][K][32]
    const T* rhs;   // natural order
    T* out;         // natural order
    typename Bits<T>::U* faceA;  // [tiles][T][K]  lane 31 of a tile, by producer step
    typename Bits<T>::U* faceB;  // [tiles][T][32] column K-1 of a tile, by producer step
    SweepSync S;
    const int* done;
};

// FWD: y = L^-1 rhs (unit L); !FWD: x = U^-1 rhs, DIV: divide by the
// diagonal (the reference), else multiply by the stored reciprocal.
// SPAN: 2 when s = z (b = y), 1 when s = y (b = z).
template <typename T, bool FWD, bool DIV, int SPAN, int K>
__global__ void __launch_bounds__(32 * kWaveMaxWarps) wave_sweep_kernel(WaveParams<T> p)
{
    if (p.done && *p.done) return;
    using B = Bits<T>;
    using U = typename B::U;
    using R = Rec<T>;
    constexpr int RS = kP + K + 31;  // slice ring: loaded kP steps ahead, kept until flushed
    extern __shared__ __align__(32) unsigned char smem_raw[];
    const WaveGeom& g = p.g;
    const int WB = g.WB, T_ = g.T;
    const int w = (int)threadIdx.x >> 5, l = (int)threadIdx.x & 31;
    const int Da = g.D[0], Db = g.D[1], Ds = g.D[2];
    R* rring = reinterpret_cast<R*>(smem_raw);                    // [WB][kP][K][32]
    T* sring = reinterpret_cast<T*>(rring + WB * kP * K * 32);    // [WB][RS][K][32]
    U* sface = reinterpret_cast<U*>(sring + WB * RS * K * 32);    // [WB-1][T][32]
    __shared__ int s_tile;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(p.S.ticket, 1u);
    for (int i = threadIdx.x; i < (WB - 1) * T_ * 32; i += blockDim.x) sface[i] = B::kSentinel;
    __syncthreads();
    const int tile = s_tile;
    const int wa = tile % g.nta, tb = tile / g.nta;
    const int wb = tb * WB + w;
    if (tile >= g.nta * g.ntb) {  // never with a fresh dispenser; keeps every access in bounds
        if (threadIdx.x == 0) atomicCAS(p.S.err, 0, (int)OCSL_TIMEOUT);
    } else if (wb < g.nwb) {  // uniform over the warp
        int* err = p.S.err;
        const int a = wa * 32 + l;
        const bool a_ok = a < Da;
        const int sstep = FWD ? g.S[2] : -g.S[2];
        const int pa = FWD ? a : Da - 1 - a;
        int base[K];
        bool ok[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int b = wb * K + k;
            ok[k] = a_ok && b < Db;
            const int pb = FWD ? b : Db - 1 - b;
            base[k] = ok[k] ? pa * g.S[0] + pb * g.S[1] + (FWD ? 0 : (Ds - 1) * g.S[2]) : 0;
        }
        const int wt = wb * g.nwa + wa;  // tile index of the step-order layouts
        const R* recs = reinterpret_cast<const R*>(p.rec) + (size_t)wt * T_ * K * 32;
        R* my_rr = rring + w * kP * K * 32;
        T* my_sr = sring + w * RS * K * 32;
        // faces in: a from the tile to the left (another CTA), b from the tile
        // below (the warp below, or the CTA below for warp 0)
        const bool has_a = wa > 0;
        const bool has_b = wb > 0;
        const U* fa_in = has_a ? p.faceA + (size_t)(wt - 1) * T_ * K : nullptr;
        const U* fb_in_sh = (has_b && w > 0) ? sface + (w - 1) * T_ * 32 : nullptr;
        const U* fb_in_gl = (has_b && w == 0) ? p.faceB + (size_t)(wt - g.nwa) * T_ * 32 : nullptr;
        // faces out
        const bool push_a = wa + 1 < g.nwa && l == 31;
        U* fa_out = p.faceA + (size_t)wt * T_ * K;
        const bool push_b = wb + 1 < g.nwb;
        U* fb_out_sh = (push_b && w < WB - 1) ? sface + w * T_ * 32 : nullptr;
        U* fb_out_gl = (push_b && w == WB - 1) ? p.faceB + (size_t)wt * T_ * 32 : nullptr;

        // Ring slots are tracked incrementally (RS is not a power of two):
        // rs_l = (t - l) mod RS, so row (k, s = t - k - l) sits in slot
        // rs_l - k (mod RS); rs_fl = (t - K + 1 - 31) mod RS is the slice that
        // completes at step t; rs_in = (t + kP) mod RS is the slice issued at t.
        const T* rhs_k[K];
#pragma unroll
        for (int k = 0; k < K; ++k) rhs_k[k] = p.rhs + base[k];
        auto issue = [&](int t, int rs) {  // records of step t and right-hand-side slice t
            if (t < T_) {  // uniform over the warp
                const int j = t % kP;
                const R* src = recs + (size_t)t * K * 32 + l;
#pragma unroll
                for (int k = 0; k < K; ++k) cp_rec<T>(&my_rr[(j * K + k) * 32 + l], src + k * 32);
            }
            if (t < Ds) {
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if (ok[k]) cp_val<T>(&my_sr[(rs * K + k) * 32 + l], rhs_k[k] + t * sstep);
            }
            cp_commit();
        };
#pragma unroll
        for (int j = 0; j < kP; ++j) issue(j, j);

        // Start behind the upstream tiles: wait for their face values of row
        // s = lag next to this tile (lane 0, column 0), so that values fetched
        // kDF steps ahead are normally final.
        {
            const int sg = min(g.lag, Ds - 1), ss = min(g.lag_sh, Ds - 1);
            if (l == 0 && ok[0]) {
                if (fa_in && B::load(fa_in + (size_t)(sg + 31) * K) == B::kSentinel)
                    (void)wait_global<T>(fa_in + (size_t)(sg + 31) * K, err);
                if (fb_in_gl && B::load(fb_in_gl + (size_t)(sg + K - 1) * 32) == B::kSentinel)
                    (void)wait_global<T>(fb_in_gl + (size_t)(sg + K - 1) * 32, err);
                if (fb_in_sh && vload_shared(fb_in_sh + (ss + K - 1) * 32) == B::kSentinel)
                    (void)wait_shared<T>(fb_in_sh + (ss + K - 1) * 32, err);
            }
        }
        __syncwarp();

        // global face values kDF steps ahead: fa (lane 0, the K a-neighbours of
        // step t at d = t + 31), fb (column 0's b-neighbour at d = t + K - 1)
        const bool get_a = fa_in != nullptr && l == 0;
        U fa[kDF][K], fb[kDF];
        auto fetch = [&](int t, int j) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                fa[j][k] = (get_a && t + 31 < T_) ? B::load(fa_in + (size_t)(t + 31) * K + k)
                                                  : B::kSentinel;
            fb[j] = (fb_in_gl && t + K - 1 < T_) ? B::load(fb_in_gl + (size_t)(t + K - 1) * 32 + l)
                                                 : B::kSentinel;
        };
#pragma unroll
        for (int j = 0; j < kDF; ++j) fetch(j, j);

        T cur[K];
#pragma unroll
        for (int k = 0; k < K; ++k) cur[k] = T(0);
        int rs_l = l == 0 ? 0 : RS - l;
        int rs_fl = RS - (K - 1) - 31;
        int rs_in = kP;
        for (int t0 = 0; t0 < T_; t0 += kP) {
#pragma unroll
            for (int j = 0; j < kP; ++j) {
                const int t = t0 + j;
                if (t >= T_) break;  // uniform over the warp
                const int jf = j % kDF;
                cp_wait<kP - 1>();
                // rows of this step and their slots
                bool act[K];
                int slot_i[K];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const int s = t - k - l;
                    act[k] = ok[k] && (unsigned)s < (unsigned)Ds;
                    const int sk = rs_l - k;
                    slot_i[k] = ((sk < 0 ? sk + RS : sk) * K + k) * 32 + l;
                }
                // faces of this step; a face value that is not there yet is
                // waited for on the rare slow path
                T fa_v[K], fb_v = T(0);
                bool slow = false;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    fa_v[k] = get_a ? B::from(fa[jf][k]) : T(0);
                    slow |= get_a && act[k] && fa[jf][k] == B::kSentinel;
                }
                U fbu = B::kSentinel;
                if (fb_in_sh) {
                    if (t + K - 1 < T_) fbu = vload_shared(fb_in_sh + (t + K - 1) * 32 + l);
                } else if (fb_in_gl) {
                    fbu = fb[jf];
                }
                if (fb_in_sh || fb_in_gl) {
                    fb_v = B::from(fbu);
                    slow |= act[0] && fbu == B::kSentinel;
                }
                if (slow) {
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (get_a && act[k] && fa[jf][k] == B::kSentinel)
                            fa_v[k] = wait_global<T>(fa_in + (size_t)(t + 31) * K + k, err);
                    // only a tile with a b-face waits for one (fbu keeps the
                    // all-ones default on the bottom tile row)
                    if ((fb_in_sh || fb_in_gl) && act[0] && fbu == B::kSentinel) {
                        if (fb_in_sh)
                            fb_v = wait_shared<T>(fb_in_sh + (t + K - 1) * 32 + l, err);
                        else
                            fb_v = wait_global<T>(fb_in_gl + (size_t)(t + K - 1) * 32 + l, err);
                    }
                }
                T up[K];  // lane l-1's values of the previous step: a-neighbours
#pragma unroll
                for (int k = 0; k < K; ++k) up[k] = __shfl_up_sync(0xffffffffu, cur[k], 1);
                // K independent rows, straight-line (inactive rows compute on
                // stale slot contents and are discarded)
                T nv[K];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const R cf = my_rr[(j * K + k) * 32 + l];
                    const T rh = my_sr[slot_i[k]];
                    const int s = t - k - l;
                    const T va = l > 0 ? up[k] : fa_v[k];
                    const T vb = k > 0 ? cur[k > 0 ? k - 1 : 0] : fb_v;
                    const T vs = s > 0 ? cur[k] : T(0);
                    const T vx = va;
                    const T vy = SPAN == 2 ? vb : vs;
                    const T vz = SPAN == 2 ? vs : vb;
                    // record: z-, y-, x-, (unused) | x+, y+, z+, diagonal term;
                    // the fma order is the row's CSR order
                    T sum = fma_t(cf.v[0], FWD ? vz : vx, T(0));
                    sum = fma_t(cf.v[1], vy, sum);
                    sum = fma_t(cf.v[2], FWD ? vx : vz, sum);
                    const T num = rh - sum;
                    T y;
                    if constexpr (FWD)
                        y = num;
                    else if constexpr (DIV)
                        y = num / (act[k] ? cf.v[3] : T(1));
                    else
                        y = num * cf.v[3];
                    nv[k] = act[k] ? y : cur[k];
                    if (act[k]) my_sr[slot_i[k]] = y;  // kept until the slice is written back
                }
                // faces out: column K-1 to the tile above, lane 31 to the right
                if (act[K - 1]) {
                    const U bits = to_bits(nv[K - 1]);
                    if (fb_out_sh) vstore_shared(fb_out_sh + t * 32 + l, bits);
                    else if (fb_out_gl) B::store(fb_out_gl + (size_t)t * 32 + l, bits);
                }
                if (push_a) {
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (act[k]) B::store(fa_out + (size_t)t * K + k, to_bits(nv[k]));
                }
                // consumed global faces go back to the sentinel for the next launch
                if (get_a) {
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (act[k])
                            B::store(const_cast<U*>(fa_in) + (size_t)(t + 31) * K + k, B::kSentinel);
                }
                if (fb_in_gl && act[0])
                    B::store(const_cast<U*>(fb_in_gl) + (size_t)(t + K - 1) * 32 + l, B::kSentinel);
#pragma unroll
                for (int k = 0; k < K; ++k) cur[k] = nv[k];
                // slice t - (K-1) - 31 is complete: write it back, coalesced
                if (t >= K - 1 + 31 && t - (K - 1) - 31 < Ds) {  // uniform over the warp
                    const int sf = t - (K - 1) - 31;
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (ok[k]) p.out[base[k] + sf * sstep] = my_sr[(rs_fl * K + k) * 32 + l];
                }
                fetch(t + kDF, jf);
                issue(t + kP, rs_in);
                rs_l = rs_l + 1 == RS ? 0 : rs_l + 1;
                rs_fl = rs_fl + 1 == RS ? 0 : rs_fl + 1;
                rs_in = rs_in + 1 == RS ? 0 : rs_in + 1;
            }
        }
        cp_wait<0>();
    }
    // every warp of the CTA done with the shared faces before the CTA retires
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(p.S.finished, 1u) == gridDim.x - 1) {
            *p.S.ticket = 0u;
            *p.S.finished = 0u;
        }
    }
}

// CSR factor -> stencil records in each direction's step order (see above).
// Row r's real entries are, in storage order, z-, y-, x-, diagonal, x+, y+,
// z+ (absent ones skipped), then phantoms; the host verified exactly this
// pattern.  fw gets (z-, y-, x-, 0), bw gets (x+, y+, z+, diagonal) with the
// diagonal replaced by 1 / diagonal (computed in FP64) when RECIP.  Absent
// entries are exact 0.  Slots of the layout that belong to no row (the
// skewed ends of each tile) are never read as a row's record.
template <typename TO, int RECIP>
__global__ void box_to_wave_kernel(int n, int nx, int ny, int nz, const int* rp, const double* M,
                                   WaveGeom g, TO* fw, TO* bw)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int i = r % nx, j = (r / nx) % ny, kz = r / (nx * ny);
    const bool present[7] = {kz > 0, j > 0, i > 0, true, i < nx - 1, j < ny - 1, kz < nz - 1};
    double v[7];
    int q = rp[r];
#pragma unroll
    for (int d = 0; d < 7; ++d) v[d] = present[d] ? M[q++] : 0.0;
    if (RECIP) v[3] = 1.0 / v[3];
    const int K = g.K;
    const int a = i, b = g.span == 2 ? j : kz, s = g.span == 2 ? kz : j;
    auto index = [&](int ca, int cb, int cs) {
        const int wa = ca >> 5, l = ca & 31, wb = cb / K, k = cb % K;
        const size_t wt = (size_t)wb * g.nwa + wa;
        return ((wt * g.T + (size_t)(cs + k + l)) * K + k) * 32 + l;
    };
    TO* lo = fw + 4 * index(a, b, s);
    TO* hi = bw + 4 * index(g.D[0] - 1 - a, g.D[1] - 1 - b, g.D[2] - 1 - s);
    lo[0] = (TO)v[0];
    lo[1] = (TO)v[1];
    lo[2] = (TO)v[2];
    lo[3] = (TO)0;
    hi[0] = (TO)v[4];
    hi[1] = (TO)v[5];
    hi[2] = (TO)v[6];
    hi[3] = (TO)v[3];
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
    kern<<<grid, 32 * p.g.WB, smem, st>>>(p);
}

template <typename T, bool FWD, bool DIV>
void launch_wave_span(cudaStream_t st, const WaveParams<T>& p)
{
    if (p.g.span == 2)
        launch_wave_one<T, FWD, DIV, 2>(st, p);
    else
        launch_wave_one<T, FWD, DIV, 1>(st, p);
}

}  // namespace

int wave_cols_per_warp(int elem_size) { return elem_size == 8 ? wave_k<double>() : wave_k<float>(); }

size_t wave_sweep_smem(const WaveGeom& g, int elem_size)
{
    const int K = wave_cols_per_warp(elem_size);
    const int RS = kP + K + 31;
    return (size_t)g.WB * kP * K * 32 * (4 * elem_size) + (size_t)g.WB * RS * K * 32 * elem_size +
           (size_t)(g.WB - 1) * g.T * 32 * elem_size;
}

WaveGeom make_wave_geom(const int* dims, int elem_size, int warps, int lag)
{
    WaveGeom g{};
    const int nx = dims[0], ny = dims[1], nz = dims[2];
    g.span = nz >= ny ? 2 : 1;  // s = the longer of y and z
    g.D[0] = nx;
    g.D[1] = g.span == 2 ? ny : nz;
    g.D[2] = g.span == 2 ? nz : ny;
    g.S[0] = 1;
    g.S[1] = g.span == 2 ? nx : nx * ny;
    g.S[2] = g.span == 2 ? nx * ny : nx;
    g.K = wave_cols_per_warp(elem_size);
    g.nwa = (g.D[0] + 31) / 32;
    g.nwb = (g.D[1] + g.K - 1) / g.K;
    g.T = g.D[2] + g.K - 1 + 31;
    g.WB = std::max(1, std::min({warps > 0 ? warps : 4, kWaveMaxWarps, g.nwb}));
    while (g.WB > 1 && wave_sweep_smem(g, elem_size) > kBoxSmemLimit) --g.WB;
    g.nta = g.nwa;
    g.ntb = (g.nwb + g.WB - 1) / g.WB;
    g.lag = lag > 0 ? lag : kWaveLag;
    g.lag_sh = kWaveLagShared;
    return g;
}

size_t wave_layout_elems(const WaveGeom& g)
{
    return (size_t)g.nwa * g.nwb * g.T * g.K * 32;
}

template <typename T>
void launch_wave_sweep(cudaStream_t st, const WaveGeom& g, const T* rec, const T* rhs, T* out,
                       void* face_a, void* face_b, bool forward, int divmode, const SweepSync& S,
                       const int* done)
{
    if (g.D[0] * g.D[1] * g.D[2] == 0) return;
    WaveParams<T> p;
    p.g = g;
    p.rec = rec;
    p.rhs = rhs;
    p.out = out;
    p.faceA = static_cast<typename Bits<T>::U*>(face_a);
    p.faceB = static_cast<typename Bits<T>::U*>(face_b);
    p.S = S;
    p.done = done;
    if (forward)
        launch_wave_span<T, true, false>(st, p);
    else if (divmode == 0)
        launch_wave_span<T, false, true>(st, p);
    else
        launch_wave_span<T, false, false>(st, p);
}

template <typename TO>
void launch_box_to_wave(cudaStream_t st, const int* dims, int n, const int* rp, const double* M,
                        const WaveGeom& g, TO* fw, TO* bw, int recip)
{
    if (n == 0) return;
    const int blocks = (n + 255) / 256;
    if (recip)
        box_to_wave_kernel<TO, 1><<<blocks, 256, 0, st>>>(n, dims[0], dims[1], dims[2], rp, M, g,
                                                          fw, bw);
    else
        box_to_wave_kernel<TO, 0><<<blocks, 256, 0, st>>>(n, dims[0], dims[1], dims[2], rp, M, g,
                                                          fw, bw);
}

template void launch_wave_sweep<double>(cudaStream_t, const WaveGeom&, const double*,
                                        const double*, double*, void*, void*, bool, int,
                                        const SweepSync&, const int*);
template void launch_wave_sweep<float>(cudaStream_t, const WaveGeom&, const float*, const float*,
                                       float*, void*, void*, bool, int, const SweepSync&,
                                       const int*);
template void launch_box_to_wave<double>(cudaStream_t, const int*, int, const int*, const double*,
                                         const WaveGeom&, double*, double*, int);
template void launch_box_to_wave<float>(cudaStream_t, const int*, int, const int*, const double*,
                                        const WaveGeom&, float*, float*, int);

}  // namespace ocsl
