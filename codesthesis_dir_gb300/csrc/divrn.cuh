// Correctly rounded FP64 division by a stored reciprocal (sm_103a).
//
// The bit-exact line eliminations divide by the pivots of a matrix that is
// factored once, and each division sits on the elimination's dependent
// chain, where an IEEE division costs several times a fused multiply-add.
// With y = RN(1/b) formed once when the matrix is factored (an IEEE
// division, off the chain), the quotient follows from one multiplication
// and two fused multiply-adds (Markstein's correction, IBM J. Res. Dev.
// 34(1), 1990; the division theorem of Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 4):
//   q0 = RN(a y)            within one ulp of a / b,
//   r  = a - b q0           exact in one fused multiply-add,
//   q  = RN(q0 + r y)       = RN(a / b).
// The result is the IEEE quotient bit for bit as long as neither the
// quotient nor the remainder leaves the normal range (the eliminations here
// work far inside it).  A zero remainder means q0 is the exact quotient; it
// is returned as is, which also keeps the sign of a zero quotient.  The
// library's gb_check_division compares this with the hardware division on
// seeded operands over the normal range.
#pragma once

#include <cuda_runtime.h>

__device__ __forceinline__ double div_by_rcp(double a, double b, double y)
{
    const double q0 = __dmul_rn(a, y);
    const double r = __fma_rn(-b, q0, a);
    return r == 0.0 ? q0 : __fma_rn(r, y, q0);
}
