// The fast FP64 form's reciprocal: the hardware's approximate reciprocal
// (rcp.approx.ftz.f64) refined by two Newton-Raphson steps, r' = r + r (1 - b r), each
// roughly doubling the correct bits — within about an ulp of 1 / b, in five FP64
// instructions against the ten or so of an IEEE division.  For normal, finite b (the
// callers' denominators are at least 1e-20); not the reference's rounding.
#pragma once
#include <cuda_runtime.h>

namespace vx {

__device__ __forceinline__ double rcp_nr(double b) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
    double e = __fma_rn(-b, r, 1.0);
    r = __fma_rn(r, e, r);
    e = __fma_rn(-b, r, 1.0);
    return __fma_rn(r, e, r);
}

}  // namespace vx
