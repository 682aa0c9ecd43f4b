// Order tests of doubles evaluated on the integer pipe. On GB300 the FP64 pipe executes 2 DFMA per
// clock per SM and is what bounds the vehicle step; comparisons, minima and maxima of doubles
// occupy it as well. These helpers give exactly the results of the floating-point tests for every
// non-NaN operand.
#pragma once

#include <cuda_runtime.h>

namespace lfdm {

// Non-negative operands: a positive double's bit pattern is a positive int64, and the patterns of
// non-negative doubles (+0 included, -0 excluded) are ordered as their values.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool gt0(double x) { return dbits(x) > 0; }                    // x > 0
__device__ __forceinline__ bool gt_nn(double a, double b) { return dbits(a) > dbits(b); }  // a > b, a, b >= +0
__device__ __forceinline__ double max_nn(double a, double b) { return gt_nn(a, b) ? a : b; }
__device__ __forceinline__ double min_nn(double a, double b) { return gt_nn(a, b) ? b : a; }
__device__ __forceinline__ double pos_part(double x) { return gt0(x) ? x : 0.0; }         // max(x, 0)
__device__ __forceinline__ bool is_zero(double x) { return (static_cast<unsigned long long>(dbits(x)) << 1) == 0; }
// Operands of any sign: the total-order key maps a double to an int64 ordered as the values, with
// both zeros at 0, so that <, <=, ==, >= and > of the keys are those of the non-NaN values.
__device__ __forceinline__ long long okey(double x) {
    const long long b = dbits(x);
    return b >= 0 ? b : -(b & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ bool lt_(double a, double b) { return okey(a) < okey(b); }
// min(max(g, -m), m) for m > 0
__device__ __forceinline__ double clamp_sym(double g, double m) {
    const long long kg = okey(g), km = okey(m);
    return kg > km ? m : (kg < -km ? -m : g);
}

}  // namespace lfdm
