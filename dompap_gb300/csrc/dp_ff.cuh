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

// Dekker's addition: absolute error below ~2^-47 (|x| + |y|), relative
// 2^-47 for operands of one sign; the pair sums need no more (their float64
// counterparts carry 2^-53 (|x| + |y|)), at about half the instructions of
// the sign-robust form.
__device__ __forceinline__ dpff operator+(dpff x, dpff y) {
    const dpff s = dpff_two_sum(x.hi, y.hi);
    return dpff_quick_two_sum(s.hi, s.lo + (x.lo + y.lo));
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

// 1/sqrt(q): the float estimate y (rsqrtf, then one float Newton step, so
// y is within about an ulp and e below is ~2^-24) refined by one Newton step
// with its second-order term, y (1 + e/2 + 3e^2/8), e = 1 - q y^2. y^2 and
// q.hi y^2 are split exactly by FMA and 1 - p is exact (p is within a few
// ulp of 1); the result is good to ~1.2e-14 relative.
__device__ __forceinline__ dpff dpff_rsqrt(dpff q) {
    const float y0 = rsqrtf(q.hi);
    const float y = fmaf(0.5f * y0, fmaf(-(q.hi * y0), y0, 1.0f), y0);
    const float t = y * y;
    const float tl = fmaf(y, y, -t);   // y^2 = t + tl
    const float p = q.hi * t;
    const float pl = fmaf(q.hi, t, -p);  // q.hi t = p + pl
    const float e = ((1.0f - p) - pl) - fmaf(q.hi, tl, q.lo * t);
    return dpff_quick_two_sum(y, y * e * fmaf(0.375f, e, 0.5f));
}

// x^2 unnormalised: (p, e) with p + e = x^2 to ~2^-48 (for dpff_accumulate).
__device__ __forceinline__ dpff dpff_sqr_unnormalised(dpff x) {
    const float p = x.hi * x.hi;
    return dpff(p, fmaf(x.hi + x.hi, x.lo, fmaf(x.hi, x.hi, -p)));
}

__device__ __forceinline__ dpff dpff_add_f(dpff x, float b) {
    const dpff s = dpff_two_sum(x.hi, b);
    return dpff_quick_two_sum(s.hi, s.lo + x.lo);
}

// int64 -> double-float (rounded to ~48 bits) without 64-bit conversion
// instructions: v = a 2^42 + b 2^20 + c with a in [-2^21, 2^21), b < 2^22,
// c < 2^20, each piece an exact float. fa + fb is a multiple of 2^20 and
// |fa| >= 2^42 > |fb| unless fa = 0, so Fast2Sum (QuickTwoSum) is exact for
// it and again for adding fc (|fc| < 2^20 <= |fa + fb| unless that is 0).
__device__ __forceinline__ dpff dpff_from_ll(long long v) {
    const int a = (int)(v >> 42);
    const int b = (int)(((unsigned long long)v >> 20) & 0x3FFFFFull);
    const int c = (int)((unsigned long long)v & 0xFFFFFull);
    const float fa = dp_small_int(a) * 4398046511104.0f;  // 2^42
    const float fb = dp_small_int(b) * 1048576.0f;        // 2^20
    const dpff ab = dpff_quick_two_sum(fa, fb);
    const dpff t = dpff_quick_two_sum(ab.hi, dp_small_int(c));
    return dpff_quick_two_sum(t.hi, t.lo + ab.lo);
}

// Compensated accumulation s += v (cascaded summation in the manner of
// Neumaier): s.hi carries the running float sum, s.lo collects the exact
// rounding errors of s.hi and the low parts of the addends, unnormalised;
// the value is s.hi + s.lo.
__device__ __forceinline__ void dpff_accumulate(dpff& s, dpff v) {
    const dpff t = dpff_two_sum(s.hi, v.hi);
    s.hi = t.hi;
    s.lo += t.lo + v.lo;
}

// s += x y without normalising the product first: its leading float p and
// the FMA-exact rounding error plus cross terms go to the two parts of s.
__device__ __forceinline__ void dpff_accumulate_prod(dpff& s, dpff x, dpff y) {
    const float p = x.hi * y.hi;
    const float pe = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p)));
    const dpff t = dpff_two_sum(s.hi, p);
    s.hi = t.hi;
    s.lo += t.lo + pe;
}

// Exact float constants of generated expressions (dp_k<dpff>): x c and x + c
// with one float operand.
struct dpff_k {
    float v;
    __device__ __forceinline__ operator dpff() const { return dpff(v, 0.0f); }
};
template <>
struct dp_k_t<dpff> {
    typedef dpff_k type;
    static __device__ __forceinline__ dpff_k make(float v) { return dpff_k{v}; }
};
__device__ __forceinline__ dpff operator*(dpff x, dpff_k k) { return dpff_mul_f(x, k.v); }
__device__ __forceinline__ dpff operator*(dpff_k k, dpff x) { return dpff_mul_f(x, k.v); }
__device__ __forceinline__ dpff operator+(dpff x, dpff_k k) { return dpff_add_f(x, k.v); }
__device__ __forceinline__ dpff operator+(dpff_k k, dpff x) { return dpff_add_f(x, k.v); }
__device__ __forceinline__ dpff operator-(dpff x, dpff_k k) { return dpff_add_f(x, -k.v); }
__device__ __forceinline__ dpff operator-(dpff_k k, dpff x) { return dpff_add_f(-x, k.v); }
__device__ __forceinline__ dpff_k operator-(dpff_k k) { return dpff_k{-k.v}; }

// hi + lo in float64 with the two widenings done on bit patterns.
__device__ __forceinline__ double dpff_to_double(dpff x) { return dp_f2d(x.hi) + dp_f2d(x.lo); }

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
