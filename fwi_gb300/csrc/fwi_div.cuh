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
// normal range, so it serves 2^-100 <= |a| <= 2^100.  Smaller nonzero
// dividends (the numerical precursor of the finite-difference stencil fills
// the wavefield ahead of the wave with them) take div_tiny below; a zero
// dividend (b > 0) is its own quotient; Inf, NaN, huge values and a missing
// reciprocal (y = 0) take the division itself.  The refinement runs for every
// lane and the exceptions are selected afterwards, so that the zeros of a
// wavefield not yet reached by the wave cost no branch.
// tests/test_gpu_division.py compares the result bit for bit with the
// division of CUDA over all 2^32 values of a for the time steps of the
// benchmark workloads and a set of seeded random ones.
#pragma once

namespace fwi {

__device__ __forceinline__ float div_main(float a, float b, float y) {
    float q = __fmul_rn(a, y);
    float r = __fmaf_rn(-q, b, a);
    q = __fmaf_rn(r, y, q);
    r = __fmaf_rn(-q, b, a);
    return __fmaf_rn(r, y, q);
}

// RN(a/b) for 0 < |a| < 2^-100.  A normal quotient is that of a*2^64 (a
// normal dividend) scaled back by 2^-64, exactly.  A quotient below 2^-126
// lies on the grid of multiples of 2^-149: n = the integer nearest to
// s/b, s = a*2^149 (exact), ties to even, from c = RN(s/b) rounded to an
// integer n0 and the exact remainder r = s - n0*b (one FMA): |r| > b/2 moves
// n0 one step towards r, |r| = b/2 is a tie; the quotient is n*2^-149 with
// the sign of a.
__device__ __forceinline__ float div_tiny(float a, float b, float y) {
    const float qs = __fmul_rn(div_main(__fmul_rn(a, 0x1p64f), b, y), 0x1p-64f);
    const float s = __fmul_rn(__fmul_rn(a, 0x1p100f), 0x1p49f);
    const float n0 = rintf(div_main(s, b, y));
    const float r = __fmaf_rn(-n0, b, s);
    const float hb = __fmul_rn(0.5f, b), ar = fabsf(r);
    const float h = __fmul_rn(n0, 0.5f);
    const bool up = ar > hb || (ar == hb && truncf(h) != h);
    const float n = up ? __fadd_rn(n0, copysignf(1.f, r)) : n0;
    const float qi = copysignf(__fmul_rn(n, 0x1p-149f), a);
    return fabsf(qs) >= 0x1p-126f ? qs : qi;
}

__device__ __forceinline__ float div_by_const(float a, float b, float y) {
    const float m = fabsf(a);
    float q = div_main(a, b, y);
    if (m == 0.f) q = a;
    else if (m < 0x1p-100f && y != 0.f) q = div_tiny(a, b, y);
    else if (!(m <= 0x1p100f) || y == 0.f) q = __fdiv_rn(a, b);
    return q;
}

}  // namespace fwi
