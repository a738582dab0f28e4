// SpMV, fused vector updates and tile-order reductions for the Krylov solvers.
//
// Every kernel here is a "tile kernel": CTA b owns rows / elements
// [2048 b, 2048 b + 2048); thread t handles 2048 b + 256 j + t for j = 0..7,
// so all global traffic is coalesced and every fused dot product is
// accumulated in the tile order the CPU oracle restates (ocsl_oracle.h).
// The last CTA to finish (atomic ticket) reduces the per-tile partial sums and
// applies a small scalar epilogue (alpha, omega, convergence tests), so the
// Krylov scalars never leave the device.
//
// Rounding follows the reference's expressions (cmatrix_solver.cpp): fma where
// the reference computes a*x + y, separately rounded operations elsewhere;
// the library is compiled with --fmad=false so that only explicit fma fuses.
#include <cfloat>
#include <cstdio>

#include <type_traits>

#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

template <int MASK>
struct DotCount {
    static constexpr int value = ((MASK & 1) ? 1 : 0) + ((MASK & 2) ? 1 : 0) + ((MASK & 4) ? 1 : 0);
};

// Per-thread dot accumulator.  FP64 vectors: fma chain from 0.0 (tile order).
// FP32 vectors: compensated FP32 (exact product split + TwoSum, Ogita, Rump &
// Oishi 2005), folded into FP64 before the warp butterfly.
template <typename T>
struct DotAcc;

template <>
struct DotAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};

template <>
struct DotAcc<float> {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float a, float b)
    {
        const float p = a * b;
        const float e = fmaf(a, b, -p);
        const float t = s + p;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (p - bp);
        s = t;
        c = c + (err + e);
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ double warp_butterfly(double v)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Reduce ND lane values of a CTA to ND sums (valid in thread 0):
// butterfly per warp, then the 8 warp sums in order.
template <int ND>
__device__ __forceinline__ void cta_sum(double (&v)[ND], double* s_red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < ND; ++k) {
        const double w = warp_butterfly(v[k]);
        if (lane == 0) s_red[k * 8 + warp] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            double s = s_red[k * 8];
            for (int w = 1; w < kThreads / 32; ++w) s = s + s_red[k * 8 + w];
            v[k] = s;
        }
    }
    __syncthreads();
}

__device__ void apply_epilogue(int epi, const double* s, int nd, Scalars* sc, int it, int maxit)
{
    for (int k = 0; k < nd && k < 4; ++k) sc->sum[k] = s[k];
    switch (epi) {
    // ---- CG_solve, cmatrix_solver.cpp:635-680
    case EP_RC_INIT:
        sc->rr = s[0];
        sc->iters = 0;
        break;
    case EP_RC_ALPHA:  // a = norm(r,r) / (norm(p,dum) + 1e-40), :660
        sc->alpha = sc->rr / (s[0] + 1.0e-40);
        break;
    case EP_RC_RES:  // res = norm(r_next, r_next); exit if < 1e-6, :667-672
        sc->res = s[0];
        sc->iters = it + 1;
        if (s[0] < 1.0e-6) {
            sc->done = 1;
        } else {
            sc->beta = s[0] / (sc->rr + 1.0e-40);
            sc->rr = s[0];
        }
        break;
    // ---- ILU_BICGSTAB_solve, cmatrix_solver.cpp:682-762
    case EP_RB_INIT: {  // r = b - A x; r0 = r; iteration 0's rhon and res
        sc->rr = s[0];
        sc->bb = s[1];
        sc->rhon = s[0];
        const double res = s[0] / s[1] + DBL_MIN;  // :733
        sc->res = res;
        sc->iters = 0;
        if (res < 1.0e-20) sc->done = 1;           // :734-735
        break;
    }
    case EP_RB_ALPHA:  // alpha = rhon / (norm(r0, v) + DBL_MIN), :727-728
        sc->alpha = sc->rhon / (s[0] + DBL_MIN);
        break;
    case EP_RB_OMEGA:  // omega = norm(dum, dum2) / (norm(dum, dum) + 1e-40), :750
        sc->omega = s[0] / (s[1] + 1.0e-40);
        break;
    case EP_RB_RUPD:  // end of iteration `it`: next iteration's rhon and res
        sc->iters = it + 1;
        if (it + 1 < maxit) {
            sc->rhon = s[0];
            sc->rr = s[1];
            const double res = s[1] / sc->bb + DBL_MIN;
            sc->res = res;
            if (res < 1.0e-20) sc->done = 1;
        }
        break;
    // ---- tolerance-mode BiCGSTAB (van der Vorst 1992)
    case EP_TB_INIT:  // s0 = <r,r>, s1 = <b,b>
        sc->rr = s[0];
        sc->bb = s[1];
        sc->rnorm = sqrt(s[0]);
        sc->res = s[1] > 0.0 ? sqrt(s[0] / s[1]) : 0.0;
        sc->rho = s[0];
        sc->sum[3] = sc->rnorm > 0.0 ? 1.0 / sc->rnorm : 0.0;
        if (!isfinite(s[0]) || !isfinite(s[1])) {
            sc->status = OCSL_NONFINITE;
            sc->done = 1;
        } else if (s[1] == 0.0 || s[0] <= sc->tol2 * s[1]) {
            sc->done = 1;
        }
        break;
    case EP_TB_SIGMA:  // sigma = <r^, v>
        sc->sigma = s[0];
        if (s[0] == 0.0 || !isfinite(s[0])) {
            sc->breakdown = 1;
            sc->done = 1;
        } else {
            sc->alpha = sc->rho / s[0];
        }
        break;
    case EP_TB_S:  // <s,s>: half-step convergence test
        sc->ss = s[0];
        sc->iters += 1;
        if (!isfinite(s[0])) {
            sc->status = OCSL_NONFINITE;
            sc->done = 1;
        } else if (s[0] <= sc->tol2 * sc->bb) {
            sc->half = 1;
            sc->done = 1;
        }
        break;
    case EP_TB_OMEGA:  // s0 = <t,t>, s1 = <s,t>
        sc->omega = s[0] != 0.0 ? s[1] / s[0] : 0.0;
        break;
    case EP_TB_RUPD: {  // s0 = <r,r>, s1 = <r^,r>
        sc->rr = s[0];
        if (!isfinite(s[0])) {
            sc->status = OCSL_NONFINITE;
            sc->done = 1;
        } else if (s[0] <= sc->tol2 * sc->bb) {
            sc->done = 1;
        } else if (sc->omega == 0.0 || sc->rho == 0.0) {
            sc->breakdown = 1;
            sc->done = 1;
        } else {
            sc->beta = (s[1] / sc->rho) * (sc->alpha / sc->omega);
            sc->rho = s[1];
        }
        break;
    }
    case EP_TRUE_RES:
        sc->rr = s[0];
        sc->res = s[1] > 0.0 ? sqrt(s[0] / s[1]) : 0.0;
        break;
    // ---- tolerance-mode Jacobi PCG
    case EP_PC_INIT:  // rho = <r,z>
        sc->rho = s[0];
        break;
    case EP_PC_ALPHA:  // <p, q>
        if (s[0] == 0.0 || !isfinite(s[0])) {
            sc->breakdown = 1;
            sc->done = 1;
        } else {
            sc->alpha = sc->rho / s[0];
        }
        break;
    case EP_PC_RUPD:  // s0 = <r,r>, s1 = <r,z>
        sc->rr = s[0];
        sc->iters += 1;
        if (!isfinite(s[0])) {
            sc->status = OCSL_NONFINITE;
            sc->done = 1;
        } else if (s[0] <= sc->tol2 * sc->bb) {
            sc->done = 1;
        } else if (sc->rho == 0.0) {
            sc->breakdown = 1;
            sc->done = 1;
        } else {
            sc->beta = s[1] / sc->rho;
            sc->rho = s[1];
        }
        break;
    case EP_IR_INNER_INIT:  // inner residual target relative to ||r32||^2
        sc->rr = s[0];
        sc->bb = s[0];
        sc->rho = s[0];
        if (!(s[0] > 0.0) || !isfinite(s[0])) sc->done = 1;
        break;
    default:
        break;
    }
}

// Store this CTA's tile partials; if it is the last CTA, reduce all tiles and
// apply the epilogue.  Must be reached by every thread of every CTA.
// Column `col` of a column-batched launch has its own partials and counter.
template <int ND>
__device__ __forceinline__ void finish_reduction(double (&v)[ND], int tile, int ntiles, int col,
                                                 const ReduceState& R, Scalars* sc, int epi,
                                                 int it, int maxit, double* s_red, int* s_last)
{
    double* partials = R.partials + (size_t)col * kMaxDots * R.max_tiles;
    unsigned* counter = R.counter + col;
    cta_sum<ND>(v, s_red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < ND; ++k) partials[k * R.max_tiles + tile] = v[k];
        __threadfence();
        const unsigned prev = atomicAdd(counter, 1u);
        *s_last = (prev == (unsigned)ntiles - 1u);
    }
    __syncthreads();
    if (!*s_last) return;
    __threadfence();
    double acc[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
        double a = 0.0;
        for (int t = threadIdx.x; t < ntiles; t += kThreads) a = a + __ldcg(partials + k * R.max_tiles + t);
        acc[k] = a;
    }
    cta_sum<ND>(acc, s_red);
    if (threadIdx.x == 0) {
        if (sc) apply_epilogue(epi, acc, ND, sc, it, maxit);
        *counter = 0u;
    }
}

// Column and tile of this CTA in a launch of ntiles * cols.n CTAs.
struct ColTile {
    int col, tile, ntiles;
    size_t off;  // element offset of the column's vectors
};
__device__ __forceinline__ ColTile col_tile(const Cols& c)
{
    ColTile t;
    t.col = (int)(blockIdx.x % (unsigned)c.n);
    t.tile = (int)(blockIdx.x / (unsigned)c.n);
    t.ntiles = (int)(gridDim.x / (unsigned)c.n);
    t.off = (size_t)t.col * (size_t)c.ld;
    return t;
}
template <typename P>
__device__ __forceinline__ P* at(P* p, size_t off)
{
    return p ? p + off : p;
}

template <typename T>
struct SpmvParams {
    int n;
    const int* rp;
    const int* col;
    const T* val;
    const T* x;
    T* y;
    const T* z;
    T* y_copy;
    const T* w;
    T a;
    ReduceState R;
    Scalars* sc;
    int epi, it, maxit;
    Cols cols;
    int lanes;  // lanes per row: 1 (spmv_kernel), 4 or 16 (spmv_lanes_kernel)
};

// y = A x (MODE 0), y = z - A x (MODE 1), y = fma(a, A x, z) (MODE 2);
// cmatrix_solver.cpp:338-453.  Thread t of tile k owns rows k * 2048 + j * 256
// + t (j = 0..7) and sums each in CSR storage order with fma from 0.0
// (:346-350), skipping phantom columns.  Entries are loaded directly: a
// warp's 32 consecutive rows cover one contiguous stretch of the CSR arrays,
// so the loads coalesce in L1.  A row's first 8 entries are loaded together
// (predicated loads), then their x values, then the chain runs; entries past
// the 8th continue the same chain after.  One row at a time keeps the kernel
// at 32-40 registers and the SMs full of warps, which measured faster than
// more rows in flight per thread (2 rows: 1.26x, 4 rows: 1.5x slower at 64-205
// registers) and than staging each 256-row slab through shared memory first
// (1.4x slower: two barriers per slab).
template <typename T, int MODE, int DOTS>
__global__ void __launch_bounds__(kThreads) spmv_kernel(SpmvParams<T> p)
{
    constexpr int G = 1;
    const ColTile ct = col_tile(p.cols);
    Scalars* const sc = at(p.sc, ct.col);
    if (sc && sc->done) return;
    constexpr int ND = DotCount<DOTS>::value;
    constexpr int K = 8;
    __shared__ double s_red[kMaxDots * 8];
    __shared__ int s_last;
    const int tile = ct.tile;
    const int n = p.n;
    const T* const xv = p.x + ct.off;
    T* const yv = p.y + ct.off;
    const T* const zvec = at(p.z, ct.off);
    T* const ycp = at(p.y_copy, ct.off);
    const T* const wv = at(p.w, ct.off);
    DotAcc<T> acc[ND > 0 ? ND : 1];

#pragma unroll 1
    for (int j0 = 0; j0 < kRowsPerThread; j0 += G) {
        int row[G], b[G], e[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            row[g] = tile * kTile + (j0 + g) * kThreads + (int)threadIdx.x;
            const bool in = row[g] < n;
            b[g] = in ? __ldg(p.rp + row[g]) : 0;
            e[g] = in ? __ldg(p.rp + row[g] + 1) : 0;
        }
        int c[G][K];
        T v[G][K], xk[G][K];
#pragma unroll
        for (int g = 0; g < G; ++g)
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const bool in = b[g] + k < e[g];
                c[g][k] = in ? __ldg(p.col + b[g] + k) : -1;
                v[g][k] = in ? __ldg(p.val + b[g] + k) : T(0);
            }
#pragma unroll
        for (int g = 0; g < G; ++g)
#pragma unroll
            for (int k = 0; k < K; ++k) xk[g][k] = c[g][k] >= 0 ? __ldg(xv + c[g][k]) : T(0);
#pragma unroll
        for (int g = 0; g < G; ++g) {
            if (row[g] >= n) continue;
            T dum = T(0);
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (c[g][k] >= 0) dum = fma_t(v[g][k], xk[g][k], dum);
            for (int q = b[g] + K; q < e[g]; ++q) {  // rows longer than K entries
                const int cq = __ldg(p.col + q);
                if (cq >= 0) dum = fma_t(__ldg(p.val + q), __ldg(xv + cq), dum);
            }
            T y, zv = T(0);
            if constexpr (MODE == 0) {
                y = dum;
            } else if constexpr (MODE == 1) {
                zv = __ldg(zvec + row[g]);
                y = zv - dum;
            } else {
                zv = __ldg(zvec + row[g]);
                y = fma_t(p.a, dum, zv);
            }
            yv[row[g]] = y;
            if (MODE == 1 && ycp) ycp[row[g]] = y;
            int k = 0;
            if constexpr ((DOTS & DOT_YY) != 0) acc[k++].add(y, y);
            if constexpr ((DOTS & DOT_ZZ) != 0) acc[k++].add(zv, zv);
            if constexpr ((DOTS & DOT_WY) != 0) acc[k++].add(__ldg(wv + row[g]), y);
            (void)k;
        }
    }
    if constexpr (ND > 0) {
        double vals[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) vals[k] = acc[k].value();
        finish_reduction<ND>(vals, tile, ct.ntiles, ct.col, p.R, sc, p.epi, p.it, p.maxit, s_red,
                             &s_last);
    }
}

// spmv_kernel with L lanes per row (32 / L rows per warp): the lanes of a
// row group load the row's entries side by side (lane l takes entries
// b + l, b + l + L, ...), so a warp's loads of values and column indices
// cover contiguous stretches of the CSR arrays for rows of any length; the
// group's first lane runs the row's fma chain in CSR order from 0.0 with the
// entries handed over by shuffles, skipping phantoms, so y is spmv_kernel's
// bit for bit.  The tile's results go to shared memory, and the fused dots
// are then accumulated exactly as spmv_kernel does (thread t: rows t + 256 j
// in j order), so the partial sums are unchanged too.  For the short rows of
// finite-volume stencils one lane per row (spmv_kernel) is faster; longer
// rows gain from more lanes -- the autotuner times them per matrix.
template <typename T, int MODE, int DOTS, int L>
__global__ void __launch_bounds__(kThreads) spmv_lanes_kernel(SpmvParams<T> p)
{
    const ColTile ct = col_tile(p.cols);
    Scalars* const sc = at(p.sc, ct.col);
    if (sc && sc->done) return;
    constexpr int ND = DotCount<DOTS>::value;
    constexpr int kGroups = kThreads / L;  // rows per CTA pass
    __shared__ double s_red[kMaxDots * 8];
    __shared__ int s_last;
    __shared__ T s_y[kTile];
    const int tile = ct.tile;
    const int n = p.n;
    const T* const xv = p.x + ct.off;
    T* const yv = p.y + ct.off;
    const T* const zvec = at(p.z, ct.off);
    T* const ycp = at(p.y_copy, ct.off);
    const T* const wv = at(p.w, ct.off);
    const int lane = (int)threadIdx.x & 31;
    const int g = (int)threadIdx.x / L, l = (int)threadIdx.x % L;
    const int gbase = lane - l;  // the group's first lane within the warp
#pragma unroll 1
    for (int r0 = 0; r0 < kTile; r0 += kGroups) {
        const int row = tile * kTile + r0 + g;
        const bool in = row < n;
        const int b = in ? __ldg(p.rp + row) : 0;
        const int e = in ? __ldg(p.rp + row + 1) : 0;
        // the longest row of the warp bounds the warp's uniform block loop
        int span = e - b;
#pragma unroll
        for (int off = L; off < 32; off <<= 1) span = max(span, __shfl_xor_sync(0xffffffffu, span, off));
        T dum = T(0);
        for (int k0 = 0; k0 < span; k0 += L) {
            const int q = b + k0 + l;
            const bool has = q < e;
            const int c = has ? __ldg(p.col + q) : -1;
            const T v = has ? __ldg(p.val + q) : T(0);
            const T xk = c >= 0 ? __ldg(xv + c) : T(0);
#pragma unroll
            for (int s = 0; s < L; ++s) {
                const int cs = __shfl_sync(0xffffffffu, c, gbase + s);
                const T vs = __shfl_sync(0xffffffffu, v, gbase + s);
                const T xs = __shfl_sync(0xffffffffu, xk, gbase + s);
                if (cs >= 0) dum = fma_t(vs, xs, dum);  // only the first lane's chain is used
            }
        }
        if (l == 0 && in) {
            T y;
            if constexpr (MODE == 0) {
                y = dum;
            } else if constexpr (MODE == 1) {
                y = __ldg(zvec + row) - dum;
            } else {
                y = fma_t(p.a, dum, __ldg(zvec + row));
            }
            yv[row] = y;
            if (MODE == 1 && ycp) ycp[row] = y;
            if constexpr (ND > 0) s_y[r0 + g] = y;
        }
    }
    if constexpr (ND > 0) {
        __syncthreads();
        DotAcc<T> acc[ND];
#pragma unroll 1
        for (int j = 0; j < kRowsPerThread; ++j) {
            const int row = tile * kTile + j * kThreads + (int)threadIdx.x;
            if (row >= n) continue;
            const T y = s_y[j * kThreads + (int)threadIdx.x];
            int k = 0;
            if constexpr ((DOTS & DOT_YY) != 0) acc[k++].add(y, y);
            if constexpr ((DOTS & DOT_ZZ) != 0) {
                const T zv = MODE == 0 ? T(0) : __ldg(zvec + row);
                acc[k++].add(zv, zv);
            }
            if constexpr ((DOTS & DOT_WY) != 0) acc[k++].add(__ldg(wv + row), y);
            (void)k;
        }
        double vals[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) vals[k] = acc[k].value();
        finish_reduction<ND>(vals, tile, ct.ntiles, ct.col, p.R, sc, p.epi, p.it, p.maxit, s_red,
                             &s_last);
    }
}

// SpMV on the packed stencil records of a natural-order 7-point box pattern
// (the layout of the structured sweeps: [2][n][4] = (z-, y-, x-, 0) and
// (x+, y+, z+, diagonal) per row, absent neighbours exact 0).  Same tile and
// row assignment, same fused dots and epilogues as spmv_kernel, and the same
// fma chain in the row's CSR order (z-, y-, x-, diagonal, x+, y+, z+): an
// absent neighbour multiplies an exact 0 by a finite x from a clamped address
// and adds nothing, so y equals the CSR kernel's bit for bit while no column
// index is read and every load is coalesced (32 or 64 B of records per row,
// x at seven shifted, contiguous offsets).
// In both SpMV kernels z and w are read through the read-only path: no
// launch writes them (y may equal z only element-wise, each row's z read
// coming before its y store in the same thread), so later rows' loads can be
// issued ahead of earlier rows' stores.
template <typename T>
struct BoxSpmvParams {
    int n, sy, sz;  // rows, y and z strides (nx, nx*ny)
    const T* rec;   // [2][n][4]
    const T* x;
    T* y;
    const T* z;
    T* y_copy;
    const T* w;
    T a;
    ReduceState R;
    Scalars* sc;
    int epi, it, maxit;
    Cols cols;
};

template <typename T>
struct Rec4;
template <>
struct Rec4<float> {
    using V = float4;
};
template <>
struct Rec4<double> {
    using V = double4;
};

#ifndef OCSL_BOX_SPMV_UNROLL
#define OCSL_BOX_SPMV_UNROLL 4
#endif
constexpr int kBoxSpmvUnroll = OCSL_BOX_SPMV_UNROLL;

template <typename T, int MODE, int DOTS>
__global__ void __launch_bounds__(kThreads) box_spmv_kernel(BoxSpmvParams<T> p)
{
    const ColTile ct = col_tile(p.cols);
    Scalars* const sc = at(p.sc, ct.col);
    if (sc && sc->done) return;
    constexpr int ND = DotCount<DOTS>::value;
    using V = typename Rec4<T>::V;
    __shared__ double s_red[kMaxDots * 8];
    __shared__ int s_last;
    const int tile = ct.tile;
    const int n = p.n;
    const T* const xv = p.x + ct.off;
    T* const yv = p.y + ct.off;
    const T* const zvec = at(p.z, ct.off);
    T* const ycp = at(p.y_copy, ct.off);
    const T* const wv = at(p.w, ct.off);
    const V* lo = reinterpret_cast<const V*>(p.rec);
    const V* hi = lo + n;
    DotAcc<T> acc[ND > 0 ? ND : 1];
#pragma unroll kBoxSpmvUnroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int row = tile * kTile + j * kThreads + (int)threadIdx.x;
        if (row >= n) continue;
        const V l = lo[row], h = hi[row];
        const T* x = xv;
        const T xzm = __ldg(x + max(row - p.sz, 0)), xym = __ldg(x + max(row - p.sy, 0));
        const T xxm = __ldg(x + max(row - 1, 0)), xc = __ldg(x + row);
        const T xxp = __ldg(x + min(row + 1, n - 1)), xyp = __ldg(x + min(row + p.sy, n - 1));
        const T xzp = __ldg(x + min(row + p.sz, n - 1));
        T dum = fma_t(l.x, xzm, T(0));
        dum = fma_t(l.y, xym, dum);
        dum = fma_t(l.z, xxm, dum);
        dum = fma_t(h.w, xc, dum);
        dum = fma_t(h.x, xxp, dum);
        dum = fma_t(h.y, xyp, dum);
        dum = fma_t(h.z, xzp, dum);
        T y, zv = T(0);
        if constexpr (MODE == 0) {
            y = dum;
        } else if constexpr (MODE == 1) {
            zv = __ldg(zvec + row);
            y = zv - dum;
        } else {
            zv = __ldg(zvec + row);
            y = fma_t(p.a, dum, zv);
        }
        yv[row] = y;
        if (MODE == 1 && ycp) ycp[row] = y;
        int k = 0;
        if constexpr ((DOTS & DOT_YY) != 0) acc[k++].add(y, y);
        if constexpr ((DOTS & DOT_ZZ) != 0) acc[k++].add(zv, zv);
        if constexpr ((DOTS & DOT_WY) != 0) acc[k++].add(__ldg(wv + row), y);
        (void)k;
    }
    if constexpr (ND > 0) {
        double v[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) v[k] = acc[k].value();
        finish_reduction<ND>(v, tile, ct.ntiles, ct.col, p.R, sc, p.epi, p.it, p.maxit, s_red,
                             &s_last);
    }
}

// box_spmv_kernel for NC right-hand sides sharing the matrix (the lockstep
// columns of ocsl_solve_multi_device), SpMM-style: one CTA per tile loads
// each row's stencil record once and applies it to every live column, instead
// of one CTA per (tile, column) each fetching the records again.  Column q's
// vectors sit q * ld elements after column 0's, its scalars at sc + q, its
// partial sums and counter in its own slot; a column whose solve is done
// when the launch starts is skipped whole, as its own launch would return.
// Each column's arithmetic, stores and tile partials are exactly those of
// box_spmv_kernel, so results are bit-identical.
template <typename T, int MODE, int DOTS, int NC>
__global__ void __launch_bounds__(kThreads) box_spmm_kernel(BoxSpmvParams<T> p)
{
    constexpr int ND = DotCount<DOTS>::value;
    using V = typename Rec4<T>::V;
    __shared__ double s_red[kMaxDots * 8];
    __shared__ int s_last;
    bool live[NC];
    bool any = false;
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        live[q] = !(p.sc && p.sc[q].done);
        any = any || live[q];
    }
    if (!any) return;
    const int tile = (int)blockIdx.x;
    const int ntiles = (int)gridDim.x;
    const int n = p.n;
    const V* lo = reinterpret_cast<const V*>(p.rec);
    const V* hi = lo + n;
    DotAcc<T> acc[NC][ND > 0 ? ND : 1];
#pragma unroll 2
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int row = tile * kTile + j * kThreads + (int)threadIdx.x;
        if (row >= n) continue;
        const V l = lo[row], h = hi[row];
        const int izm = max(row - p.sz, 0), iym = max(row - p.sy, 0), ixm = max(row - 1, 0);
        const int ixp = min(row + 1, n - 1), iyp = min(row + p.sy, n - 1);
        const int izp = min(row + p.sz, n - 1);
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            if (!live[q]) continue;
            const size_t off = (size_t)q * (size_t)p.cols.ld;
            const T* x = p.x + off;
            T dum = fma_t(l.x, __ldg(x + izm), T(0));
            dum = fma_t(l.y, __ldg(x + iym), dum);
            dum = fma_t(l.z, __ldg(x + ixm), dum);
            dum = fma_t(h.w, __ldg(x + row), dum);
            dum = fma_t(h.x, __ldg(x + ixp), dum);
            dum = fma_t(h.y, __ldg(x + iyp), dum);
            dum = fma_t(h.z, __ldg(x + izp), dum);
            T y, zv = T(0);
            if constexpr (MODE == 0) {
                y = dum;
            } else if constexpr (MODE == 1) {
                zv = __ldg(p.z + off + row);
                y = zv - dum;
            } else {
                zv = __ldg(p.z + off + row);
                y = fma_t(p.a, dum, zv);
            }
            p.y[off + row] = y;
            if (MODE == 1 && p.y_copy) p.y_copy[off + row] = y;
            int k = 0;
            if constexpr ((DOTS & DOT_YY) != 0) acc[q][k++].add(y, y);
            if constexpr ((DOTS & DOT_ZZ) != 0) acc[q][k++].add(zv, zv);
            if constexpr ((DOTS & DOT_WY) != 0) acc[q][k++].add(__ldg(p.w + off + row), y);
            (void)k;
        }
    }
    if constexpr (ND > 0) {
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            if (!live[q]) continue;  // uniform over the CTA
            double v[ND];
#pragma unroll
            for (int k = 0; k < ND; ++k) v[k] = acc[q][k].value();
            finish_reduction<ND>(v, tile, ntiles, q, p.R, p.sc ? p.sc + q : nullptr, p.epi, p.it,
                                 p.maxit, s_red, &s_last);
        }
    }
}

// spmv_kernel on the red-black stencil records (RbGeom): the neighbours'
// rows computed, not read; each row's chain in its CSR order (colour 0: the
// diagonal, then z-, y-, x-, x+, y+, z+; colour 1: the neighbours, then the
// diagonal), absent neighbours skipped -- bit-identical to spmv_kernel on
// the permuted CSR, without column indices or row pointers.
template <typename T>
struct RbSpmvParams {
    RbGeom g;
    const T* rec;  // [2][n][4]
    const T* x;
    T* y;
    const T* z;
    T* y_copy;
    const T* w;
    T a;
    ReduceState R;
    Scalars* sc;
    int epi, it, maxit;
};

template <typename T, int MODE, int DOTS>
__global__ void __launch_bounds__(kThreads) rb_spmv_kernel(RbSpmvParams<T> p)
{
    Scalars* const sc = p.sc;
    if (sc && sc->done) return;
    constexpr int ND = DotCount<DOTS>::value;
    using V = typename Rec4<T>::V;
    __shared__ double s_red[kMaxDots * 8];
    __shared__ int s_last;
    const int tile = blockIdx.x;
    const int n = p.g.n;
    const V* lo = reinterpret_cast<const V*>(p.rec);
    const V* hi = lo + n;
    DotAcc<T> acc[ND > 0 ? ND : 1];
#pragma unroll 1
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int row = tile * kTile + j * kThreads + (int)threadIdx.x;
        if (row >= n) continue;
        const RbRow q = rb_row_info(p.g, row);
        const V l = lo[row], h = hi[row];
        const T v[6] = {l.x, l.y, l.z, l.w, h.x, h.y};
        T xn[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) xn[s] = q.has[s] ? __ldg(p.x + q.nb[s]) : T(0);
        const T xc = __ldg(p.x + row);
        T dum = T(0);
        if (q.c == 0) dum = fma_t(h.z, xc, dum);
#pragma unroll
        for (int s = 0; s < 6; ++s)
            if (q.has[s]) dum = fma_t(v[s], xn[s], dum);
        if (q.c == 1) dum = fma_t(h.z, xc, dum);
        T y, zv = T(0);
        if constexpr (MODE == 0) {
            y = dum;
        } else if constexpr (MODE == 1) {
            zv = __ldg(p.z + row);
            y = zv - dum;
        } else {
            zv = __ldg(p.z + row);
            y = fma_t(p.a, dum, zv);
        }
        p.y[row] = y;
        if (MODE == 1 && p.y_copy) p.y_copy[row] = y;
        int k = 0;
        if constexpr ((DOTS & DOT_YY) != 0) acc[k++].add(y, y);
        if constexpr ((DOTS & DOT_ZZ) != 0) acc[k++].add(zv, zv);
        if constexpr ((DOTS & DOT_WY) != 0) acc[k++].add(__ldg(p.w + row), y);
        (void)k;
    }
    if constexpr (ND > 0) {
        double vals[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) vals[k] = acc[k].value();
        finish_reduction<ND>(vals, tile, (int)gridDim.x, 0, p.R, sc, p.epi, p.it, p.maxit, s_red,
                             &s_last);
    }
}

template <int OP>
struct OpDots {
    static constexpr int value =
        (OP == V_RB_XR || OP == V_DOT2 || OP == V_TB_XR || OP == V_PC_XRZ) ? 2
        : (OP == V_DOT1 || OP == V_RC_XR || OP == V_TB_S || OP == V_PC_INIT || OP == V_IR_SCALE ||
           OP == V_SUM || OP == V_ABSSUM) ? 1
                                          : 0;
};

struct VecParams {
    int n;
    VecPtrs p;
    ReduceState R;
    Scalars* sc;
    const Scalars* outer;
    int epi, it, maxit;
    Cols cols;
};

// V_TB_S / V_TB_P also leave the all-ones sweep sentinel in up to two dead
// vectors (v[6], v[7]: the outputs of the two sweeps that follow), in place
// of separate fill launches.
template <typename T>
__device__ __forceinline__ void fill_sentinels(T* f0, T* f1, int e)
{
    using U = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned>::type;
    if (f0) reinterpret_cast<U*>(f0)[e] = ~U(0);
    if (f1) reinterpret_cast<U*>(f1)[e] = ~U(0);
}

// Vectors (bit k = v[k]) each op reads, and whether it reads v64[0].
template <int OP>
struct VecReads {
    static constexpr unsigned mask =
        OP == V_RB_P ? 0x07u : OP == V_RB_HS ? 0x36u : OP == V_RB_XR ? 0x76u
      : OP == V_DOT2 || OP == V_DOT1 ? 0x03u : OP == V_RC_XR ? 0x1Bu : OP == V_RC_P ? 0x03u
      : OP == V_TB_S ? 0x06u : OP == V_TB_XR ? 0x77u : OP == V_TB_P ? 0x07u
      : OP == V_TB_HALF ? 0x03u : OP == V_COPY2 ? 0x04u : OP == V_PC_INIT ? 0x0Cu
      : OP == V_PC_XRZ ? 0x2Fu : OP == V_PC_P ? 0x03u : OP == V_IR_SCALE ? 0x00u
      : OP == V_IR_UPDATE ? 0x02u : OP == V_SUM || OP == V_ABSSUM ? 0x01u
      : OP == V_PRODUCT || OP == V_AXPY ? 0x03u : OP == V_SCALE ? 0x01u : 0xFFu;
    static constexpr bool f64 = OP == V_IR_SCALE || OP == V_IR_UPDATE;
};

template <typename T, int OP>
__global__ void __launch_bounds__(kThreads) vec_kernel(VecParams P)
{
    const ColTile ct = col_tile(P.cols);
    Scalars* const sc = at(P.sc, ct.col);
    const Scalars* const outer = at(P.outer, ct.col);
    if constexpr (OP == V_TB_HALF) {
        if (!sc->half) return;
    } else if constexpr (OP == V_IR_SCALE || OP == V_IR_UPDATE) {
        if (outer->done) return;
    } else if (sc && sc->done) {
        return;
    }
    constexpr int ND = OpDots<OP>::value;
    __shared__ double s_red[kMaxDots * 8];
    __shared__ int s_last;
    const int tile = ct.tile;
    const int n = P.n;
    // this column's vectors (element offsets in each pointer's own type)
    T* v[8];
    double* v64[2];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const size_t o = ((P.cols.shared >> i) & 1u) ? 0 : ct.off;
        v[i] = at(reinterpret_cast<T*>(P.p.v[i]), o);
        if (i < 2) v64[i] = at(reinterpret_cast<double*>(P.p.v[i]), o);
    }

    // Scalars of this step, read once per thread (written by earlier kernels).
    const double alpha = sc ? sc->alpha : 0.0;
    const double omega = sc ? sc->omega : 0.0;
    const double beta = sc ? sc->beta : 0.0;
    const T a = (T)alpha, w = (T)omega, be = (T)beta;
    DotAcc<T> acc[ND > 0 ? ND : 1];

    // Two phases: every input element of this thread first (all loads in
    // flight together), then the updates and dot terms in element order, so
    // results and reduction order are those of one element at a time.  Every
    // op reads each element of a vector before it writes that element.
    constexpr unsigned RM = VecReads<OP>::mask;
    T in[kRowsPerThread][8];
    double in64[kRowsPerThread];
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int e = tile * kTile + j * kThreads + (int)threadIdx.x;
        const bool ok = e < n;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if ((RM >> k) & 1u) in[j][k] = ok ? v[k][e] : T(0);
        if constexpr (VecReads<OP>::f64) in64[j] = ok ? v64[0][e] : 0.0;
    }
#pragma unroll
    for (int j = 0; j < kRowsPerThread; ++j) {
        const int e = tile * kTile + j * kThreads + (int)threadIdx.x;
        if (e >= n) continue;
        if constexpr (OP == V_RB_P) {  // :718-720
            const T dum = fma_t(-w, in[j][1], in[j][0]);
            v[0][e] = fma_t(w, dum, in[j][2]);
        } else if constexpr (OP == V_RB_HS) {  // :731, :738
            v[0][e] = fma_t(a, in[j][2], in[j][1]);
            v[3][e] = fma_t(-a, in[j][4], in[j][5]);
        } else if constexpr (OP == V_RB_XR) {  // :753, :756, next :714 and :733
            v[0][e] = fma_t(w, in[j][1], in[j][2]);
            const T r = fma_t(-w, in[j][4], in[j][5]);
            v[3][e] = r;
            acc[0].add(in[j][6], r);
            acc[1].add(r, r);
        } else if constexpr (OP == V_DOT2) {
            const T x = in[j][0];
            acc[0].add(x, in[j][1]);
            acc[1].add(x, x);
        } else if constexpr (OP == V_DOT1) {
            acc[0].add(in[j][0], in[j][1]);
        } else if constexpr (OP == V_RC_XR) {  // :662-667
            v[0][e] = fma_t(a, in[j][1], in[j][0]);
            const T rn = fma_t(-a, in[j][3], in[j][4]);
            v[2][e] = rn;
            acc[0].add(rn, rn);
        } else if constexpr (OP == V_RC_P) {  // :674
            v[0][e] = fma_t(be, in[j][0], in[j][1]);
        } else if constexpr (OP == V_TB_S) {
            const T s = fma_t(-a, in[j][1], in[j][2]);
            v[0][e] = s;
            acc[0].add(s, s);
            fill_sentinels(v[6], v[7], e);
        } else if constexpr (OP == V_TB_XR) {
            v[0][e] = fma_t(w, in[j][2], fma_t(a, in[j][1], in[j][0]));
            const T r = fma_t(-w, in[j][4], in[j][5]);
            v[3][e] = r;
            acc[0].add(r, r);
            acc[1].add(in[j][6], r);
        } else if constexpr (OP == V_TB_P) {
            v[0][e] = fma_t(be, fma_t(-w, in[j][1], in[j][0]), in[j][2]);
            fill_sentinels(v[6], v[7], e);
        } else if constexpr (OP == V_TB_HALF) {
            v[0][e] = fma_t(a, in[j][1], in[j][0]);
        } else if constexpr (OP == V_COPY2) {
            const T r = in[j][2];
            v[0][e] = r;
            v[1][e] = r;
        } else if constexpr (OP == V_PC_INIT) {
            const T r = in[j][2];
            const T z = r * in[j][3];
            v[0][e] = z;
            v[1][e] = z;
            acc[0].add(r, z);
        } else if constexpr (OP == V_PC_XRZ) {
            v[0][e] = fma_t(a, in[j][1], in[j][0]);
            const T r = fma_t(-a, in[j][3], in[j][2]);
            v[2][e] = r;
            const T z = r * in[j][5];
            v[4][e] = z;
            acc[0].add(r, r);
            acc[1].add(r, z);
        } else if constexpr (OP == V_PC_P) {
            v[0][e] = fma_t(be, in[j][0], in[j][1]);
        } else if constexpr (OP == V_IR_SCALE) {  // v[0] is FP64
            const float f = (float)(in64[j] * outer->sum[3]);
            v[1][e] = f;
            v[2][e] = f;
            v[3][e] = f;
            v[4][e] = 0.0f;
            acc[0].add(f, f);
        } else if constexpr (OP == V_IR_UPDATE) {  // v[0] is FP64
            const float d = in[j][1];
            v64[0][e] = fma((double)d, outer->rnorm, in64[j]);
        } else if constexpr (OP == V_SUM) {  // fma(x, 1, s) == s + x exactly
            acc[0].add(in[j][0], T(1));
        } else if constexpr (OP == V_ABSSUM) {
            acc[0].add(fabs(in[j][0]), T(1));
        } else if constexpr (OP == V_PRODUCT) {
            v[2][e] = in[j][0] * in[j][1];
        } else if constexpr (OP == V_SCALE) {
            v[2][e] = a * in[j][0];
        } else if constexpr (OP == V_AXPY) {
            // a = alpha, b = beta of the scalars block; the reference's branches
            const T x = in[j][0], y = in[j][1];
            T o;
            if (be == T(1)) {
                o = a == T(1) ? x + y : (a == T(-1) ? y - x : fma_t(a, x, y));
            } else if (be == T(-1)) {
                o = a == T(1) ? x - y : (a == T(-1) ? -y - x : fma_t(a, x, -y));
            } else {
                o = fma_t(a, x, be * y);
            }
            v[2][e] = o;
        }
    }
    if constexpr (ND > 0) {
        double vals[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) vals[k] = acc[k].value();
        finish_reduction<ND>(vals, tile, ct.ntiles, ct.col, P.R, sc, P.epi, P.it, P.maxit, s_red,
                             &s_last);
    }
}

__global__ void convert_kernel(int n, const double* in, float* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

inline int ntiles_of(int n) { return (n + kTile - 1) / kTile; }

template <typename T, int MODE, int DOTS>
void spmv_dispatch(cudaStream_t st, const SpmvParams<T>& p)
{
    const int nt = ntiles_of(p.n);
    if (nt == 0) return;
    const unsigned grid = (unsigned)(nt * p.cols.n);
    switch (p.lanes) {
    case 4: spmv_lanes_kernel<T, MODE, DOTS, 4><<<grid, kThreads, 0, st>>>(p); break;
    case 16: spmv_lanes_kernel<T, MODE, DOTS, 16><<<grid, kThreads, 0, st>>>(p); break;
    default: spmv_kernel<T, MODE, DOTS><<<grid, kThreads, 0, st>>>(p); break;
    }
}

template <typename T, int MODE>
void spmv_dots(cudaStream_t st, const SpmvParams<T>& p, int dots)
{
    switch (dots) {
    case 0: spmv_dispatch<T, MODE, 0>(st, p); break;
    case DOT_YY: spmv_dispatch<T, MODE, DOT_YY>(st, p); break;
    case DOT_YY | DOT_ZZ: spmv_dispatch<T, MODE, DOT_YY | DOT_ZZ>(st, p); break;
    case DOT_WY: spmv_dispatch<T, MODE, DOT_WY>(st, p); break;
    case DOT_YY | DOT_WY: spmv_dispatch<T, MODE, DOT_YY | DOT_WY>(st, p); break;
    default: break;
    }
}

template <typename T, int MODE, int DOTS>
void box_spmv_dispatch(cudaStream_t st, const BoxSpmvParams<T>& p)
{
    const int nt = ntiles_of(p.n);
    if (nt == 0) return;
    if (p.cols.spmm && p.cols.n > 1) {
        switch (p.cols.n) {
        case 2: box_spmm_kernel<T, MODE, DOTS, 2><<<nt, kThreads, 0, st>>>(p); return;
        case 3: box_spmm_kernel<T, MODE, DOTS, 3><<<nt, kThreads, 0, st>>>(p); return;
        case 4: box_spmm_kernel<T, MODE, DOTS, 4><<<nt, kThreads, 0, st>>>(p); return;
        default: break;
        }
    }
    box_spmv_kernel<T, MODE, DOTS><<<nt * p.cols.n, kThreads, 0, st>>>(p);
}

template <typename T, int MODE>
void box_spmv_dots(cudaStream_t st, const BoxSpmvParams<T>& p, int dots)
{
    switch (dots) {
    case 0: box_spmv_dispatch<T, MODE, 0>(st, p); break;
    case DOT_YY: box_spmv_dispatch<T, MODE, DOT_YY>(st, p); break;
    case DOT_YY | DOT_ZZ: box_spmv_dispatch<T, MODE, DOT_YY | DOT_ZZ>(st, p); break;
    case DOT_WY: box_spmv_dispatch<T, MODE, DOT_WY>(st, p); break;
    case DOT_YY | DOT_WY: box_spmv_dispatch<T, MODE, DOT_YY | DOT_WY>(st, p); break;
    default: break;
    }
}

template <typename T, int OP>
void vec_dispatch(cudaStream_t st, const VecParams& P)
{
    const int nt = ntiles_of(P.n);
    if (nt == 0) return;
    vec_kernel<T, OP><<<nt * P.cols.n, kThreads, 0, st>>>(P);
}

}  // namespace

template <typename T>
void launch_spmv(cudaStream_t st, const DevPattern& P, const T* val, const T* x, T* y, int mode,
                 const double* /*scal_a*/, double a_const, const T* z, T* y_copy, const T* w,
                 int dots, const ReduceState& R, Scalars* sc, int epi, int it, int maxit,
                 const Cols& cols)
{
    SpmvParams<T> p;
    p.cols = cols;
    p.lanes = P.spmv_lanes;
    p.n = P.n;
    p.rp = P.rp;
    p.col = P.col;
    p.val = val;
    p.x = x;
    p.y = y;
    p.z = z;
    p.y_copy = y_copy;
    p.w = w;
    p.a = (T)a_const;
    p.R = R;
    p.sc = sc;
    p.epi = epi;
    p.it = it;
    p.maxit = maxit;
    switch (mode) {
    case 0: spmv_dots<T, 0>(st, p, dots); break;
    case 1: spmv_dots<T, 1>(st, p, dots); break;
    default: spmv_dots<T, 2>(st, p, dots); break;
    }
}

template <typename T>
void launch_box_spmv(cudaStream_t st, int n, const int* dims, const T* rec, const T* x, T* y,
                     int mode, double a_const, const T* z, T* y_copy, const T* w, int dots,
                     const ReduceState& R, Scalars* sc, int epi, int it, int maxit,
                     const Cols& cols)
{
    BoxSpmvParams<T> p;
    p.cols = cols;
    p.n = n;
    p.sy = dims[0];
    p.sz = dims[0] * dims[1];
    p.rec = rec;
    p.x = x;
    p.y = y;
    p.z = z;
    p.y_copy = y_copy;
    p.w = w;
    p.a = (T)a_const;
    p.R = R;
    p.sc = sc;
    p.epi = epi;
    p.it = it;
    p.maxit = maxit;
    switch (mode) {
    case 0: box_spmv_dots<T, 0>(st, p, dots); break;
    case 1: box_spmv_dots<T, 1>(st, p, dots); break;
    default: box_spmv_dots<T, 2>(st, p, dots); break;
    }
}

template <typename T, int MODE, int DOTS>
void rb_spmv_dispatch(cudaStream_t st, const RbSpmvParams<T>& p)
{
    const int nt = ntiles_of(p.g.n);
    if (nt > 0) rb_spmv_kernel<T, MODE, DOTS><<<nt, kThreads, 0, st>>>(p);
}

template <typename T, int MODE>
void rb_spmv_dots(cudaStream_t st, const RbSpmvParams<T>& p, int dots)
{
    switch (dots) {
    case 0: rb_spmv_dispatch<T, MODE, 0>(st, p); break;
    case DOT_YY: rb_spmv_dispatch<T, MODE, DOT_YY>(st, p); break;
    case DOT_YY | DOT_ZZ: rb_spmv_dispatch<T, MODE, DOT_YY | DOT_ZZ>(st, p); break;
    case DOT_WY: rb_spmv_dispatch<T, MODE, DOT_WY>(st, p); break;
    case DOT_YY | DOT_WY: rb_spmv_dispatch<T, MODE, DOT_YY | DOT_WY>(st, p); break;
    default: break;
    }
}

template <typename T>
void launch_rb_spmv(cudaStream_t st, const RbGeom& g, const T* rec, const T* x, T* y, int mode,
                    double a_const, const T* z, T* y_copy, const T* w, int dots,
                    const ReduceState& R, Scalars* sc, int epi, int it, int maxit)
{
    RbSpmvParams<T> p;
    p.g = g;
    p.rec = rec;
    p.x = x;
    p.y = y;
    p.z = z;
    p.y_copy = y_copy;
    p.w = w;
    p.a = (T)a_const;
    p.R = R;
    p.sc = sc;
    p.epi = epi;
    p.it = it;
    p.maxit = maxit;
    switch (mode) {
    case 0: rb_spmv_dots<T, 0>(st, p, dots); break;
    case 1: rb_spmv_dots<T, 1>(st, p, dots); break;
    default: rb_spmv_dots<T, 2>(st, p, dots); break;
    }
}

template <typename T>
void launch_vec(cudaStream_t st, int op, int n, const VecPtrs& ptrs, const ReduceState& R,
                Scalars* sc, const Scalars* sc_outer, int epi, int it, int maxit,
                const Cols& cols)
{
    VecParams P;
    P.cols = cols;
    P.n = n;
    P.p = ptrs;
    P.R = R;
    P.sc = sc;
    P.outer = sc_outer;
    P.epi = epi;
    P.it = it;
    P.maxit = maxit;
    switch (op) {
    case V_RB_P: vec_dispatch<T, V_RB_P>(st, P); break;
    case V_RB_HS: vec_dispatch<T, V_RB_HS>(st, P); break;
    case V_RB_XR: vec_dispatch<T, V_RB_XR>(st, P); break;
    case V_DOT2: vec_dispatch<T, V_DOT2>(st, P); break;
    case V_DOT1: vec_dispatch<T, V_DOT1>(st, P); break;
    case V_RC_XR: vec_dispatch<T, V_RC_XR>(st, P); break;
    case V_RC_P: vec_dispatch<T, V_RC_P>(st, P); break;
    case V_TB_S: vec_dispatch<T, V_TB_S>(st, P); break;
    case V_TB_XR: vec_dispatch<T, V_TB_XR>(st, P); break;
    case V_TB_P: vec_dispatch<T, V_TB_P>(st, P); break;
    case V_TB_HALF: vec_dispatch<T, V_TB_HALF>(st, P); break;
    case V_COPY2: vec_dispatch<T, V_COPY2>(st, P); break;
    case V_PC_INIT: vec_dispatch<T, V_PC_INIT>(st, P); break;
    case V_PC_XRZ: vec_dispatch<T, V_PC_XRZ>(st, P); break;
    case V_PC_P: vec_dispatch<T, V_PC_P>(st, P); break;
    case V_IR_SCALE: vec_dispatch<float, V_IR_SCALE>(st, P); break;
    case V_IR_UPDATE: vec_dispatch<float, V_IR_UPDATE>(st, P); break;
    case V_SUM: vec_dispatch<T, V_SUM>(st, P); break;
    case V_ABSSUM: vec_dispatch<T, V_ABSSUM>(st, P); break;
    case V_PRODUCT: vec_dispatch<T, V_PRODUCT>(st, P); break;
    case V_AXPY: vec_dispatch<T, V_AXPY>(st, P); break;
    case V_SCALE: vec_dispatch<T, V_SCALE>(st, P); break;
    default: break;
    }
}

void launch_convert_f64_f32(cudaStream_t st, int n, const double* in, float* out)
{
    if (n <= 0) return;
    convert_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, in, out);
}

template void launch_spmv<double>(cudaStream_t, const DevPattern&, const double*, const double*,
                                  double*, int, const double*, double, const double*, double*,
                                  const double*, int, const ReduceState&, Scalars*, int, int, int,
                                  const Cols&);
template void launch_spmv<float>(cudaStream_t, const DevPattern&, const float*, const float*,
                                 float*, int, const double*, double, const float*, float*,
                                 const float*, int, const ReduceState&, Scalars*, int, int, int,
                                 const Cols&);
template void launch_rb_spmv<double>(cudaStream_t, const RbGeom&, const double*, const double*,
                                     double*, int, double, const double*, double*, const double*,
                                     int, const ReduceState&, Scalars*, int, int, int);
template void launch_rb_spmv<float>(cudaStream_t, const RbGeom&, const float*, const float*,
                                    float*, int, double, const float*, float*, const float*, int,
                                    const ReduceState&, Scalars*, int, int, int);
template void launch_box_spmv<double>(cudaStream_t, int, const int*, const double*,
                                      const double*, double*, int, double, const double*,
                                      double*, const double*, int, const ReduceState&, Scalars*,
                                      int, int, int, const Cols&);
template void launch_box_spmv<float>(cudaStream_t, int, const int*, const float*, const float*,
                                     float*, int, double, const float*, float*, const float*, int,
                                     const ReduceState&, Scalars*, int, int, int, const Cols&);
template void launch_vec<double>(cudaStream_t, int, int, const VecPtrs&, const ReduceState&,
                                 Scalars*, const Scalars*, int, int, int, const Cols&);
template void launch_vec<float>(cudaStream_t, int, int, const VecPtrs&, const ReduceState&,
                                Scalars*, const Scalars*, int, int, int, const Cols&);

}  // namespace ocsl
