// Correctly rounded division by a divisor fixed for a whole launch.
//
// The snapshot store divides every cell by dt ((p_3 - p_1)*0.5/dt,
// solver_acoustic_SS.f90:447).  A full IEEE division per cell costs the
// forward snapshot passes about a third of their time, so the quotient is
// formed from y = RN(1/b), computed once on the host, with two refinement
// steps q <- q + (a - b*q)*y in fused multiply-adds (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990).  q0 = RN(a*y) is within two
// units in the last place of a/b; the first step makes q faithful (within one
// unit); for a faithful q the remainder a - b*q is exactly representable and
// the second step returns RN(a/b), the round-to-nearest-even quotient.  The
// argument assumes that neither the remainder nor the quotient leaves the
// normal range, so a outside [2^-100, 2^100] in magnitude (subnormal and
// huge values, Inf, NaN) and a missing reciprocal (y = 0) take the division
// itself; a zero dividend (b > 0) is its own quotient.  The refinement runs
// for every lane and the rare exceptions are selected afterwards, so that
// the zeros of a wavefield not yet reached by the wave cost no branch.
// tests/test_gpu_division.py compares the result bit for bit with the
// division of CUDA over all 2^32 values of a for the time steps of the
// benchmark workloads and a set of seeded random ones.
#pragma once

namespace fwi {

__device__ __forceinline__ float div_by_const(float a, float b, float y) {
    const float m = fabsf(a);
    float q = __fmul_rn(a, y);
    float r = __fmaf_rn(-q, b, a);
    q = __fmaf_rn(r, y, q);
    r = __fmaf_rn(-q, b, a);
    q = __fmaf_rn(r, y, q);
    if (m == 0.f) q = a;
    else if (!(m >= 0x1p-100f && m <= 0x1p100f) || y == 0.f) q = __fdiv_rn(a, b);
    return q;
}

}  // namespace fwi
