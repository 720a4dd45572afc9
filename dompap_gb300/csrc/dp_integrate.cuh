// dp_integrate.cuh — one particle's step of the Langevin G-JF or NVE
// leap-frog integrator, the wrap into the box, the fixed-point forms of the
// new position and the neighbour-list skin test. Shared by the statically
// compiled k_integrate (dompap_gpu.cu) and the NVRTC-compiled fused step
// kernel (pair_kernels.cuh), which integrates each particle right after its
// forces; like dp_common.cuh it has no includes.
//
// The new position, shadow and 64-bit fixed point go to *_out buffers: the
// fused kernel writes them into the second set of position buffers while
// other threads still read this step's positions from the first; the
// separate kernel passes the same buffers in and out.
#pragma once

struct dp_int_args {
    const double* pos;      // positions of this step (SoA [k * n + i])
    double* pos_out;        // positions of the next step
    double* vel;            // in place
    double* beta;           // in place (G-JF noise of the previous step)
    const double* force;    // k_integrate only (the fused kernel has F in registers)
    int32_t* img;           // in place
    void* shadow_out;       // 32-bit fixed point of pos_out
    void* pos64_out;        // 64-bit fixed point of pos_out (float64-parity mode)
    const double* pos_ref;  // positions at the last neighbour-list build
    const void* shadow_ref;
    const uint8_t* mclass;  // massmode 1: mass class per particle
    const double* mcoef;    // massmode 1: [class][5]: a, b dt/m, b/(2m), sqrt(2 alpha T dt), dt/m
    const float2* mcoef_f;  // massmode 1: [class]: float32 b/(2m), sqrt(2 alpha T dt)
    const double* mass;     // massmode 2: mass per particle
    const int32_t* order;   // particle id held by each slot: keys its Langevin noise
    dp_dev_status* st;
    long long n;
    double box[DP_MAX_DIM];
    double scale64[DP_MAX_DIM];  // 2^64 / L
    float unit[DP_MAX_DIM];      // L / 2^32
    double thr;                  // (skin/2)^2
    float thr_lo, thr_hi;        // float32 bracket of thr for the shadow test
    double dt;
    double coef[5];              // massmode 0
    float coef_f[2];             // massmode 0: float32 coef[2], coef[3] (the noise terms)
    double temperature;
    double tau;
    unsigned long long seed;
    long long step_offset;       // steps since st->step (within one graph of steps)
    int massmode;                // 0: one mass, 1: mass classes, 2: per-particle masses
    int nve;                     // 1: NVE leap-frog, 0: G-JF
    unsigned long long next_cond;  // fused step in a graph: conditional handle of the next step's rebuild node
    int end_flags;               // fused step: DP_END_* work of its last CTA (0 outside graphs)
    int pad_end;
};

// Work of the last CTA of a fused step captured in a graph: every position
// is wrapped now, so `far` is cleared for the next step; and the next step's
// conditional rebuild node gets its condition (need_rebuild) from here.
#define DP_END_CLEAR_FAR 1
#define DP_END_SET_COND 2

// G-JF coefficients for mass m (dompap/integrator.py:29-36): a, b dt/m,
// b/(2m), sqrt(2 alpha T dt), dt/m.
__device__ __forceinline__ void dp_gjf_coefficients(double m, double dt, double T, double tau, double* c) {
    const double alpha = m / tau;
    const double beta_variance = 2 * alpha * T * dt;
    const double numerator = 1.0 - alpha * dt / 2.0 / m;
    const double denominator = 1.0 + alpha * dt / 2.0 / m;
    const double a = numerator / denominator;
    const double b = 1 / denominator;
    c[0] = a;
    c[1] = b * dt / m;
    c[2] = b / 2 / m;
    c[3] = sqrt(beta_variance);
    c[4] = dt / m;
}

// c: the five float64 coefficients; cf: float32 b/(2m) and sqrt(2 alpha T dt)
// for the noise terms.
template <int MASSMODE>
__device__ __forceinline__ void dp_load_coef(const dp_int_args& a, long long i, double* c, float* cf) {
    if (MASSMODE == 0) {
#pragma unroll
        for (int t = 0; t < 5; ++t) c[t] = a.coef[t];
        cf[0] = a.coef_f[0];
        cf[1] = a.coef_f[1];
    } else if (MASSMODE == 1) {
        const int cl = a.mclass[i];
#pragma unroll
        for (int t = 0; t < 5; ++t) c[t] = __ldg(a.mcoef + cl * 5 + t);
        const float2 f = __ldg(a.mcoef_f + cl);
        cf[0] = f.x;
        cf[1] = f.y;
    } else {
        dp_gjf_coefficients(a.mass[i], a.dt, a.temperature, a.tau, c);
        cf[0] = (float)c[2];
        cf[1] = (float)c[3];
    }
}

// Wrap into [0, L) exactly as wrap_into_box (dompap/positions.py:90-98):
// shift = floor(x / L), image += shift, x -= shift * L. For 0 <= x < L the
// rounded x / L is < 1, so the shift is 0 and the division is skipped.
__device__ __forceinline__ double dp_wrap_axis(double x, double L, int32_t& image) {
    if (!(x >= 0.0 && x < L)) {
        const double s = floor(x / L);
        image += (int32_t)s;
        x -= s * L;
    }
    return x;
}

// neighbor_list_is_old (dompap/neighbor_list.py:183-201) for one particle:
// its min-image displacement^2 since the last build against (skin/2)^2, read
// from the fixed-point shadows in float32 and recomputed in float64 exactly
// as the reference does only within the error bound of the threshold. With
// `exact` (some current or reference position lies far outside the box, where
// the shadows' periodic difference is not the reference's single-shift one)
// always in float64.
template <int D>
__device__ __forceinline__ bool dp_skin_old(const void* shadow_ref, const double* pos_ref, long long n,
                                            const float* unit, const double* box, double thr, float thr_lo,
                                            float thr_hi, long long i, const uint32_t* u, const double* x,
                                            bool exact = false) {
    typedef typename dp_shadow_t<D>::type sh_t;
    if (!exact) {
        uint32_t uref[D];
        dp_shadow_unpack<D>(((const sh_t*)shadow_ref)[i], uref);
        float df[D];
        const float qf = dp_shadow_q<D>(u, uref, unit, df);
        if (qf <= thr_lo) return false;
        if (qf > thr_hi) return true;
    }
    double d[D];
#pragma unroll
    for (int k = 0; k < D; ++k) d[k] = dp_min_image(x[k] - pos_ref[k * n + i], box[k]);
    return dp_sqsum_exact<D>(d) > thr;
}

// Langevin G-JF leap-frog (dompap/integrator.py:17-40, arXiv:1303.7011
// Sec. II.C eqs. 16-17) or NVE leap-frog (:5-14) of particle i with force F,
// then the wrap into the box, the fixed-point forms and the skin test (the
// return value). The deterministic part a v + (b dt / m) F is float64 (two
// fused multiply-adds); the noise terms beta_new = sqrt(2 alpha T dt) z and
// b (beta_old + beta_new) / (2m) are float32, like the float32 normal deviate
// z they scale (relative error ~1e-7 on a random term): this GPU runs float64
// at 1/64 of the float32 rate, and the integrator's float64 work bounds the
// step once the pair loop is cheap. The float64 position is converted to fixed point once: one
// product p = x 2^64 / L gives the wrap test (its bit pattern), the 64-bit
// fixed point and the 32-bit shadow (its upper word). `bad` is set when a
// coordinate is not finite.
template <int D, int MASSMODE, bool NVE, bool WRITE64>
__device__ __forceinline__ bool dp_integrate_one(const dp_int_args& a, long long i, const double* F, bool& bad) {
    const long long n = a.n;
    double c[5];
    float cf[2];
    dp_load_coef<MASSMODE>(a, i, c, cf);
    float z[4];
    // the noise of a particle depends on its id, not on the slot it occupies
    if (!NVE) dp_normals4(a.seed, (unsigned long long)(a.st->step + a.step_offset), (uint32_t)a.order[i], z);
    // every load is issued before the first store (the arrays are not
    // declared non-aliasing, so a store would otherwise order the loads of
    // the next axis behind it)
    double vin[D], xin[D], bin[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const long long o = k * n + i;
        vin[k] = a.vel[o];
        xin[k] = a.pos[o];
        bin[k] = NVE ? 0.0 : a.beta[o];
    }
    uint32_t u[D];
    unsigned long long X[D];
    double xs[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const long long o = k * n + i;
        double v = vin[k];
        double x = xin[k];
        if (NVE) {
            v = v + c[4] * F[k];  // make_one_step_leap_frog (dompap/integrator.py:12)
        } else {
            // separately rounded float32 operations (no contraction)
            const float bn = __fmul_rn(cf[1], z[k]);
            const float noise = __fmul_rn(cf[0], __fadd_rn(dp_d2f_trunc(bin[k]), bn));
            v = fma(c[1], F[k], fma(c[0], v, dp_f2d(noise)));
            a.beta[o] = dp_f2d(bn);
        }
        x = x + v * a.dt;
        double p = x * a.scale64[k];
        const long long pb = __double_as_longlong(p);
        if (!(pb >= 0 && pb < 0x43F0000000000000LL)) {  // p outside [0, 2^64): wrap
            int32_t im = a.img[o];
            x = dp_wrap_axis(x, a.box[k], im);
            a.img[o] = im;
            bad = bad || !isfinite(x);
            p = (x >= 0.0 && x < a.box[k]) ? x * a.scale64[k] : 0.0;
        }
        X[k] = dp_fixed64_of(p);
        u[k] = (uint32_t)(X[k] >> 32);
        a.vel[o] = v;
        a.pos_out[o] = x;
        xs[k] = x;
    }
    ((typename dp_shadow_t<D>::type*)a.shadow_out)[i] = dp_shadow_pack<D>(u);
    if (WRITE64) ((typename dp_fixed64_t<D>::type*)a.pos64_out)[i] = dp_fixed64_pack<D>(X);
    // the new positions are wrapped; the list's reference positions may not be
    return dp_skin_old<D>(a.shadow_ref, a.pos_ref, n, a.unit, a.box, a.thr, a.thr_lo, a.thr_hi, i, u, xs,
                          a.st->ref_far != 0);
}

// Runtime dispatch over the mass mode and the integrator (uniform branches).
template <int D, bool WRITE64>
__device__ __forceinline__ bool dp_integrate_dispatch(const dp_int_args& a, long long i, const double* F, bool& bad) {
    if (a.nve) {
        if (a.massmode == 0) return dp_integrate_one<D, 0, true, WRITE64>(a, i, F, bad);
        if (a.massmode == 1) return dp_integrate_one<D, 1, true, WRITE64>(a, i, F, bad);
        return dp_integrate_one<D, 2, true, WRITE64>(a, i, F, bad);
    }
    if (a.massmode == 0) return dp_integrate_one<D, 0, false, WRITE64>(a, i, F, bad);
    if (a.massmode == 1) return dp_integrate_one<D, 1, false, WRITE64>(a, i, F, bad);
    return dp_integrate_one<D, 2, false, WRITE64>(a, i, F, bad);
}
