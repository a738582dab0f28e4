// Correctly rounded FP64 quotients a / b for several a over one b, with one
// IEEE division per divisor instead of one per quotient.
//
// GB300 runs FP64 at a small fraction of its FP32 rate and an IEEE FP64
// division is a multi-instruction sequence (measured 562 cycles of latency),
// so kernels that divide several values by one distance or one diagonal are
// FP64-throughput bound.  Markstein's method (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): with y = RN(1/b) and its correction y_lo = RN((1 - b y) y)
// taken once per divisor, each quotient is
//     q = RN(a y + a y_lo),  r = a - b q (exact by fma),  RN(q + r y),
// which is the correctly rounded a / b -- the IEEE quotient bit for bit --
// while no intermediate overflows or underflows; operands outside
// [2^-500, 2^500] (zeros, subnormals, infinities and NaNs among them) take
// the IEEE division instead.  The serial sweep's backward division and its
// test against IEEE division over 12M quotients use the same code.
#pragma once

#include <cuda_runtime.h>

namespace ocsl {

__device__ __forceinline__ bool markstein_range(double v)
{
    const int e = (__double2hiint(v) >> 20) & 0x7ff;  // biased exponent
    return e >= 1023 - 500 && e <= 1023 + 500;
}

struct Recip {
    double b, y, ylo;
    bool ok;
};

__device__ __forceinline__ Recip recip(double b)
{
    Recip r;
    r.b = b;
    r.y = 1.0 / b;
    r.ylo = fma(-b, r.y, 1.0) * r.y;
    r.ok = markstein_range(b);
    return r;
}

__device__ __forceinline__ double divide(double a, const Recip& d)
{
    if (!d.ok || !markstein_range(a)) return a / d.b;
    const double q = fma(a, d.y, a * d.ylo);
    const double r = fma(-d.b, q, a);
    return fma(r, d.y, q);
}

}  // namespace ocsl
