// dp_ff.cuh — double-float ("float-float") arithmetic for the float64-parity
// pair kernels.
//
// GB300 executes float64 at 1/64 of the float32 rate, so the per-pair
// arithmetic of the parity mode runs on pairs (hi, lo) of floats carrying
// ~48 significant bits (relative error ~1e-14, far inside the 1e-10 parity
// bound), using the error-free transformations of Dekker (1971) and Knuth
// (TAOCP vol. 2): TwoSum, QuickTwoSum and an FMA-based TwoProduct. Functions
// without a double-float form (exp, cos, ...) are evaluated in float64 and
// split back.
#pragma once

struct dpff {
    float hi, lo;
    __device__ __forceinline__ dpff() : hi(0.0f), lo(0.0f) {}
    __device__ __forceinline__ constexpr dpff(float h, float l) : hi(h), lo(l) {}
    // from a double (exact split of its leading 48 bits)
    __device__ __forceinline__ dpff(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __device__ __forceinline__ dpff(int v) : hi((float)v), lo(0.0f) {}
    __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dpff dpff_quick_two_sum(float a, float b) {
    const float s = a + b;
    return dpff(s, b - (s - a));
}

__device__ __forceinline__ dpff dpff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return dpff(s, (a - (s - bb)) + (b - bb));
}

__device__ __forceinline__ dpff operator+(dpff x, dpff y) {
    const dpff s = dpff_two_sum(x.hi, y.hi);
    const dpff t = dpff_two_sum(x.lo, y.lo);
    const dpff u = dpff_quick_two_sum(s.hi, s.lo + t.hi);
    return dpff_quick_two_sum(u.hi, u.lo + t.lo);
}

__device__ __forceinline__ dpff operator-(dpff x) { return dpff(-x.hi, -x.lo); }
__device__ __forceinline__ dpff operator-(dpff x, dpff y) { return x + (-y); }

__device__ __forceinline__ dpff operator*(dpff x, dpff y) {
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    return dpff_quick_two_sum(p, e);
}

__device__ __forceinline__ dpff dpff_mul_f(dpff x, float b) {
    const float p = x.hi * b;
    const float e = fmaf(x.lo, b, fmaf(x.hi, b, -p));
    return dpff_quick_two_sum(p, e);
}

__device__ __forceinline__ dpff operator/(dpff x, dpff y) {
    const float q1 = x.hi / y.hi;
    const dpff r = x - dpff_mul_f(y, q1);
    const float q2 = r.hi / y.hi;
    return dpff_quick_two_sum(q1, q2);
}

__device__ __forceinline__ dpff& operator+=(dpff& x, dpff y) {
    x = x + y;
    return x;
}

__device__ __forceinline__ bool operator<(dpff x, dpff y) { return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo); }
__device__ __forceinline__ bool operator>(dpff x, dpff y) { return y < x; }
__device__ __forceinline__ bool operator<=(dpff x, dpff y) { return !(y < x); }
__device__ __forceinline__ bool operator>=(dpff x, dpff y) { return !(x < y); }

// 1/sqrt(q): float seed refined by one Newton step in double-float.
__device__ __forceinline__ dpff dpff_rsqrt(dpff q) {
    const float y0 = rsqrtf(q.hi);
    // e = 1 - q y0^2
    const dpff qy = dpff_mul_f(q, y0);
    const dpff qyy = dpff_mul_f(qy, y0);
    const dpff e = dpff(1.0f, 0.0f) - qyy;
    return dpff(y0, 0.0f) + dpff_mul_f(e, 0.5f * y0);
}

// Exact int64 -> double-float (hi = nearest float, lo = rounded remainder).
__device__ __forceinline__ dpff dpff_from_ll(long long v) {
    const float hi = __ll2float_rn(v);
    const long long rem = v - __float2ll_rn(hi);
    return dpff(hi, __ll2float_rn(rem));
}

// Functions without a double-float form go through float64.
#define DPFF_VIA_DOUBLE(fn)                                                                    \
    __device__ __forceinline__ dpff fn(dpff x) { return dpff(fn(x.to_double())); }
DPFF_VIA_DOUBLE(exp)
DPFF_VIA_DOUBLE(log)
DPFF_VIA_DOUBLE(sin)
DPFF_VIA_DOUBLE(cos)
DPFF_VIA_DOUBLE(tan)
DPFF_VIA_DOUBLE(sinh)
DPFF_VIA_DOUBLE(cosh)
DPFF_VIA_DOUBLE(tanh)
DPFF_VIA_DOUBLE(erf)
DPFF_VIA_DOUBLE(erfc)
DPFF_VIA_DOUBLE(atan)
DPFF_VIA_DOUBLE(asin)
DPFF_VIA_DOUBLE(acos)
DPFF_VIA_DOUBLE(cbrt)
DPFF_VIA_DOUBLE(sqrt)
#undef DPFF_VIA_DOUBLE
__device__ __forceinline__ dpff fabs(dpff x) { return x.hi < 0.0f ? -x : x; }
__device__ __forceinline__ dpff pow(dpff x, dpff y) { return dpff(pow(x.to_double(), y.to_double())); }
