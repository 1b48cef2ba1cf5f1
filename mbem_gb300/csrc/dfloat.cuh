// Double-float (hi + lo FP32 pair) helpers shared by the mixed-precision
// kernels: the split of an FP64 value and the error-free accumulation of an
// FP32 entry times a double-float value (TwoProd by FMA, Knuth's TwoSum).
// The _rn intrinsics keep the compiler from contracting or reassociating
// the error-free steps.
#pragma once

namespace mbem {

struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 split_d(double v) {
    F2 r;
    r.hi = (float)v;
    r.lo = (float)(v - (double)r.hi);
    return r;
}

// (sh + sl) += a * (xh + xl), a an FP32 value taken as exact
__device__ __forceinline__ void df_acc(float& sh, float& sl, float a, float xh, float xl) {
    const float p = __fmul_rn(a, xh);
    const float e = __fmaf_rn(a, xh, -p);      // exact product error (TwoProd)
    const float q = __fmaf_rn(a, xl, e);
    const float s = __fadd_rn(sh, p);          // TwoSum of sh + p
    const float bb = __fsub_rn(s, sh);
    sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb)), q));
    sh = s;
}

}  // namespace mbem
