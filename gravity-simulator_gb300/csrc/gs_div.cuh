// gs_div.cuh -- correctly rounded FP64 quotients from a correctly rounded
// reciprocal, for the FP64 parity kernels (whose quotients must equal the
// reference's a / b bit for bit).
//
// Method (Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990; restated as the
// theorem on division from a reciprocal in Muller et al., "Handbook of
// Floating-Point Arithmetic"): with y = RN(1/b) and q within one ulp of
// a/b, the residual r = a - b q is exactly representable (one FMA gives it
// exactly) and RN(q + r y) = RN(a / b), barring underflow and overflow.
// q0 = RN(a y) is within about 1.5 ulp of a / b, so one correction step
// brings it within one ulp and a second one gives the correctly rounded
// quotient: one product and four FMAs.  Operands outside [2^-900, 2^900] in
// magnitude (and zeros, infinities, NaNs) take __ddiv_rn, so the result
// equals __ddiv_rn(a, b) for every input.
//
// This pays where several quotients share a denominator (one reciprocal,
// then five operations per quotient instead of a full division each) and
// for the fixed divisors of the Stumpff series, whose reciprocals are
// compile-time constants.  Division by a power of two is exact and written
// as the multiplication it equals.
#pragma once

namespace gs {

__device__ __forceinline__ double div_rcp(double a, double b, double y)
{
    const double aa = fabs(a), ab = fabs(b);
    if (!(aa >= 0x1p-900 && aa <= 0x1p900 && ab >= 0x1p-900 && ab <= 0x1p900))
        return __ddiv_rn(a, b);
    double q = __dmul_rn(a, y);
    double r = __fma_rn(-q, b, a);
    q = __fma_rn(r, y, q);
    r = __fma_rn(-q, b, a);
    return __fma_rn(r, y, q);
}

}  // namespace gs
