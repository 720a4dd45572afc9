// pair_kernels.cuh — pair force / energy / virial / Laplacian kernels.
//
// This file is compiled at run time by NVRTC for sm_103a, once per
// (dimension, pair potential, sigma/epsilon mode, precision). The host
// prepends the DP_* configuration macros, dp_common.cuh and the device
// functions generated from the SymPy pair potential:
//
//   template <typename R> __device__ R dp_pair_u(R s, R inv_s);   // u(s) - u(r_cut)
//   template <typename R> __device__ R dp_pair_f(R s, R inv_s);   // -du/ds
//   template <typename R> __device__ R dp_pair_c(R s, R inv_s);   // d2u/ds2
//
// Semantics follow dompap's neighbour-list kernels:
//   force      dompap/potential.py:163-188  F_n = sum_m eps f(r/sigma) d/r
//   energy     dompap/potential.py:69-100   U = 1/2 sum_n sum_m eps u(r/sigma)
//   virial     dompap/potential.py:253-279  W = 1/D sum_{n<m} eps(n,m) f(r/sigma(n,m)) r (pairs m > n of each list)
//   laplacian  dompap/potential.py:327-364  sum_m eps c(r/sigma) - (D-1) eps f(r/sigma)/r
// with s = r / sigma and every term 0 where s > r_cut (dompap/potential.py:61-65).
// There is no 1/sigma chain-rule factor, exactly as in the reference.
//
// Layout in HBM: positions are SoA float64 pos[k*N + i]; the neighbour list
// is column-major nl[k*N + i] with per-particle counts cnt[i]; the
// fixed-point shadow is one 8- or 16-byte vector per particle.
//
// Configuration macros (set by the host):
//   DP_DIM          spatial dimension (2, 3 or 4)
//   DP_REAL         pair arithmetic type: double (FP64 mode) or float (FP32 mode)
//   DP_PMODE        0 constant sigma/epsilon, 1 per-type table, 2 dense (N, N) matrix
//   DP_SIGMA_ONE    1 when sigma is the constant 1 (the division is skipped)
//   DP_EPS_ONE      1 when epsilon is the constant 1
//   DP_FF           1 in the float64-parity mode: pair arithmetic in double-float
//                   (dp_ff.cuh) on the exact 64-bit fixed-point displacement; the
//                   cut decision within float rounding of r_cut and positions not
//                   yet wrapped into the box take the float64 path
#ifndef DP_FF
#define DP_FF 0
#endif

#ifndef DP_DIM
#error "DP_DIM must be defined"
#endif

// struct dp_pair_args is defined in dp_common.cuh (shared with the host).

typedef DP_REAL real_t;
typedef typename dp_shadow_t<DP_DIM>::type shadow_t;

__device__ __forceinline__ void dp_pair_params(const dp_pair_args& a, long long i, int ti, int j, double& sig,
                                               double& isig, double& eps) {
#if DP_PMODE == 0
    sig = a.sigma;
    isig = a.inv_sigma;
    eps = a.epsilon;
#elif DP_PMODE == 1
    const int tj = __ldg(a.types + j);
    sig = __ldg(a.sig_tab + ti * a.ntypes + tj);
    isig = __ldg(a.isig_tab + ti * a.ntypes + tj);
    eps = __ldg(a.eps_tab + ti * a.ntypes + tj);
#else
    // the dense (N, N) tables are indexed by particle id; with `upper` by
    // (min, max) of the two ids, as dompap's Newton's-third-law double loop
    // (dompap/potential.py:191-214) evaluates every pair once with
    // sigma(n, m), epsilon(n, m), n < m
    long long pi = __ldg(a.order + i), pj = __ldg(a.order + j);
    if (a.upper && pi > pj) {
        const long long t = pi;
        pi = pj;
        pj = t;
    }
    sig = __ldg(a.sig_tab + pi * a.n + pj);
    isig = 1.0 / sig;
    eps = __ldg(a.eps_tab + pi * a.n + pj);
#endif
}

// What one kernel accumulates for a pair; selected at compile time.
// DP_ACC_ENERGY_UPPER: the energy over the partners m of n with m > n (ids).
enum { DP_ACC_FORCE = 0, DP_ACC_ENERGY = 1, DP_ACC_VIRIAL = 2, DP_ACC_LAPLACE = 3, DP_ACC_ENERGY_UPPER = 4 };

// The pair sum of particle (slot) i takes m > n in particle ids: the virial
// (dompap/potential.py:265-278) and the double-loop energies (:103-160).
// Per-type and constant parameters are symmetric, so any one orientation of
// each pair gives the same total and slots are compared; the dense tables may
// not be, so the ids are.
__device__ __forceinline__ bool dp_upper_skip(const dp_pair_args& a, long long i, int j) {
#if DP_PMODE == 2
    return __ldg(a.order + j) <= __ldg(a.order + i);
#else
    return j <= i;
#endif
}

// Per-particle neighbour loop. Returns the scalar sum (energy / virial /
// Laplacian) and, for DP_ACC_FORCE, the force vector in f[].
//
// Float64-parity mode (DP_FF): a pair is evaluated in double-float on the
// exact 64-bit fixed-point displacement, with no float64 instruction in the
// loop (this GPU runs float64 at 1/64 of the float32 rate). Pairs whose
// scaled distance lies within float rounding of r_cut, and every pair while
// some position is far outside the box, take the float64 path of the
// reference instead (its min-image displacement, cut decision and pair
// terms).
//
// LANES > 1 (the fused step for small systems): LANES consecutive lanes share
// particle i, lane `lane` of them taking list entries lane, lane + LANES, ...;
// each returns its partial sums (the caller adds them across the group).
// ALL: no list, every other particle is a candidate partner (dompap's
// double-loop and vectorised force and energy methods,
// dompap/potential.py:103-160,191-250,298-324); lane `lane` takes slots
// lane, lane + LANES, ...
template <int ACC, int LANES = 1, bool ALL = false>
__device__ __forceinline__ double dp_particle_sum(const dp_pair_args& a, long long i, double* f, int lane = 0) {
    constexpr int D = DP_DIM;
    const long long n = a.n;
    const shadow_t* __restrict__ sh = (const shadow_t*)a.shadow;
    uint32_t ui[D];
    double xi[D];
    int ti = 0;
#if DP_PMODE == 1
    ti = a.types[i];
#endif
    real_t acc_v[D];
#pragma unroll
    for (int k = 0; k < D; ++k) acc_v[k] = real_t(0);
    double acc_s = 0.0;
#if DP_FF
    typedef typename dp_fixed64_t<D>::type fx_t;
    const fx_t* __restrict__ p64 = (const fx_t*)a.pos64;
    const bool ff_ok = a.status->far == 0;  // single-shift image == nearest image
    unsigned long long Xi[D];
    dpff U[D];
#pragma unroll
    for (int k = 0; k < D; ++k) U[k] = dpff(a.unit64_hi[k], a.unit64_lo[k]);
    if (ff_ok) {
        // the pre-filter runs on the upper words of the 64-bit fixed point
        dp_fixed64_unpack<D>(p64[i], Xi);
#pragma unroll
        for (int k = 0; k < D; ++k) ui[k] = (uint32_t)(Xi[k] >> 32);
    } else {
        dp_shadow_unpack<D>(sh[i], ui);
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = a.pos[k * n + i];
    }
    const float rcut_f = a.rcut_f;
    const bool rcut_finite = a.rcut_finite != 0;
    dpff facc[D];  // compensated sums (dpff_accumulate)
    dpff sacc;
    bool used64 = false;
#if DP_PMODE == 0
    const dpff sig_c(a.ff_const[0], a.ff_const[1]), isig_c(a.ff_const[2], a.ff_const[3]),
        eps_c(a.ff_const[4], a.ff_const[5]);
#endif
#else
    dp_shadow_unpack<D>(sh[i], ui);
#if !(DP_REAL_IS_FLOAT)
#pragma unroll
    for (int k = 0; k < D; ++k) xi[k] = a.pos[k * n + i];
#endif
#endif
    // Two passes over windows of up to 32 listed neighbours. Pass 1 runs the
    // float32 pre-filter on the shadows and keeps a bit per neighbour that
    // may lie within r_cut * sigma_max; pass 2 evaluates the pair terms of
    // the kept ones only, in list order. A warp then runs the pair arithmetic
    // as often as its busiest lane has kept neighbours, not once per listed
    // one (in a dense liquid with a thin skin most listed neighbours of most
    // lanes are outside r_cut at any step).
    const int c_all = ALL ? (int)n : a.cnt[i];
    const int c = LANES > 1 ? (c_all > lane ? (c_all - lane + LANES - 1) / LANES : 0) : c_all;
    const int32_t* __restrict__ row = ALL ? nullptr : a.nl + i + (LANES > 1 ? (long long)lane * n : 0LL);
    const long long entry_stride = (long long)LANES * n;
    for (int base = 0; base < c; base += 32) {
        const int w = min(32, c - base);
        uint32_t kept = 0;
#pragma unroll 4
        for (int t = 0; t < w; ++t) {
            const int j = ALL ? (base + t) * LANES + lane : __ldg(row + (long long)(base + t) * entry_stride);
            if (ALL && j == i) continue;
            // the virial and the double-loop energy are upper-triangle sums
            // over n < m with sigma(n, m), epsilon(n, m)
            if ((ACC == DP_ACC_VIRIAL || ACC == DP_ACC_ENERGY_UPPER) && dp_upper_skip(a, i, j)) continue;
            uint32_t uj[D];
            dp_shadow_unpack<D>(__ldg(sh + j), uj);
            float df[D];
            if (dp_shadow_q<D>(ui, uj, a.unit, df) <= a.cut2f) kept |= 1u << t;
        }
        while (kept) {
            const int t = __ffs(kept) - 1;
            kept &= kept - 1;
            const int j = ALL ? (base + t) * LANES + lane : __ldg(row + (long long)(base + t) * entry_stride);
            uint32_t uj[D];
#if DP_FF
            unsigned long long Xj[D];
            if (ff_ok) {
                dp_fixed64_unpack<D>(p64[j], Xj);
#pragma unroll
                for (int k = 0; k < D; ++k) uj[k] = (uint32_t)(Xj[k] >> 32);
            } else {
                dp_shadow_unpack<D>(__ldg(sh + j), uj);
            }
#else
            dp_shadow_unpack<D>(__ldg(sh + j), uj);
#endif
            float df[D];
            const float qf = dp_shadow_q<D>(ui, uj, a.unit, df);
#if DP_REAL_IS_FLOAT
            double sig, isig, eps;
            dp_pair_params(a, i, ti, j, sig, isig, eps);
            // FP32 pair arithmetic on the fixed-point displacement.
            const float rinv = rsqrtf(qf);
            const float r = qf * rinv;
#if DP_SIGMA_ONE
            const float s = r, sinv = rinv;
#else
            const float s = r * (float)isig, sinv = rinv * (float)sig;
#endif
            if (s > (float)a.rcut) continue;
            const float e = (float)eps;
            if (ACC == DP_ACC_FORCE) {
#if DP_EPS_ONE
                const float sf = dp_pair_f<float>(s, sinv);
#else
                const float sf = e * dp_pair_f<float>(s, sinv);
#endif
                const float g = sf * rinv;
#pragma unroll
                for (int k = 0; k < D; ++k) acc_v[k] = fmaf(g, df[k], acc_v[k]);
            } else if (ACC == DP_ACC_ENERGY || ACC == DP_ACC_ENERGY_UPPER) {
                acc_s += (double)(e * dp_pair_u<float>(s, sinv));
            } else if (ACC == DP_ACC_VIRIAL) {
                acc_s += (double)(e * dp_pair_f<float>(s, sinv) * r);
            } else {
                acc_s += (double)(e * dp_pair_c<float>(s, sinv) + (float)(D - 1) * (-e * dp_pair_f<float>(s, sinv)) * rinv);
            }
#else
#if DP_FF
            if (ff_ok) {
                // double-float pair arithmetic on the exact fixed-point displacement
                dpff d[D];
#pragma unroll
                for (int k = 0; k < D; ++k) d[k] = dpff_from_ll((long long)(Xi[k] - Xj[k])) * U[k];
                dpff q = dpff_sqr_unnormalised(d[0]);
#pragma unroll
                for (int k = 1; k < D; ++k) dpff_accumulate(q, dpff_sqr_unnormalised(d[k]));
                q = dpff_quick_two_sum(q.hi, q.lo);
                const dpff rinv = dpff_rsqrt(q);
                const dpff r = q * rinv;
#if DP_PMODE == 0
                const dpff fsig = sig_c, fisig = isig_c, feps = eps_c;
#elif DP_PMODE == 1
                const int tj = __ldg(a.types + j);
                const float2* tri = a.ff_tab + 3 * (ti * a.ntypes + tj);
                const float2 t0 = __ldg(tri), t1 = __ldg(tri + 1), t2 = __ldg(tri + 2);
                const dpff fsig(t0.x, t0.y), fisig(t1.x, t1.y), feps(t2.x, t2.y);
#else
                double sig, isig, eps;
                dp_pair_params(a, i, ti, j, sig, isig, eps);
                const dpff fsig(sig), fisig(isig), feps(eps);
#endif
#if DP_SIGMA_ONE
                const dpff s = r, sinv = rinv;
#else
                const dpff s = r * fisig, sinv = rinv * fsig;
#endif
                if (!(rcut_finite && fabsf(s.hi - rcut_f) <= 1e-5f * rcut_f)) {
                    if (s.hi > rcut_f) continue;
                    if (ACC == DP_ACC_FORCE) {
#if DP_EPS_ONE
                        const dpff g = dp_pair_f<dpff>(s, sinv) * rinv;
#else
                        const dpff g = feps * dp_pair_f<dpff>(s, sinv) * rinv;
#endif
#pragma unroll
                        for (int k = 0; k < D; ++k) dpff_accumulate_prod(facc[k], g, d[k]);
                    } else if (ACC == DP_ACC_ENERGY || ACC == DP_ACC_ENERGY_UPPER) {
                        dpff_accumulate(sacc, feps * dp_pair_u<dpff>(s, sinv));
                    } else if (ACC == DP_ACC_VIRIAL) {
                        dpff_accumulate(sacc, feps * dp_pair_f<dpff>(s, sinv) * r);
                    } else {
                        const dpff sf = feps * dp_pair_f<dpff>(s, sinv);
                        dpff_accumulate(sacc, feps * dp_pair_c<dpff>(s, sinv) - dpff(D - 1) * sf * rinv);
                    }
                    continue;
                }
                // within float rounding of r_cut: the float64 path below
#pragma unroll
                for (int k = 0; k < D; ++k) xi[k] = a.pos[k * n + i];
            }
            used64 = true;
#endif
            // FP64 pair arithmetic. d and r^2 follow the reference exactly; 1/r
            // comes from one reciprocal square root (no divisions), and where s
            // lies within a few ulp of r_cut, r = sqrt(r^2) and s = r / sigma are
            // recomputed with IEEE operations so the cut decision is the
            // reference's.
            double sig, isig, eps;
            dp_pair_params(a, i, ti, j, sig, isig, eps);
            double d[D];
#pragma unroll
            for (int k = 0; k < D; ++k) d[k] = dp_min_image(xi[k] - __ldg(a.pos + k * n + j), a.box[k]);
            const double q = dp_sqsum_exact<D>(d);
            const double rinv = rsqrt(q);
            double r = q * rinv;
#if DP_SIGMA_ONE
            double s = r;
            const double sinv = rinv;
#else
            double s = r * isig;
            const double sinv = rinv * sig;
#endif
            if (fabs(s - a.rcut) <= 1e-14 * a.rcut) {
                r = sqrt(q);
#if DP_SIGMA_ONE
                s = r;
#else
                s = r / sig;
#endif
            }
            if (s > a.rcut) continue;
            if (ACC == DP_ACC_FORCE) {
#if DP_EPS_ONE
                const double sf = dp_pair_f<double>(s, sinv);
#else
                const double sf = eps * dp_pair_f<double>(s, sinv);
#endif
                const double g = sf * rinv;
#pragma unroll
                for (int k = 0; k < D; ++k) acc_v[k] = fma(g, d[k], acc_v[k]);
            } else if (ACC == DP_ACC_ENERGY || ACC == DP_ACC_ENERGY_UPPER) {
                acc_s += eps * dp_pair_u<double>(s, sinv);
            } else if (ACC == DP_ACC_VIRIAL) {
                acc_s += eps * dp_pair_f<double>(s, sinv) * r;
            } else {
                const double sf = eps * dp_pair_f<double>(s, sinv);
                acc_s += eps * dp_pair_c<double>(s, sinv) + (double)(D - 1) * (-sf) * rinv;
            }
#endif
        }
    }
#if DP_FF
    // double-float -> float64 by moving bits (one float64 add per value)
    if (ACC == DP_ACC_FORCE) {
#pragma unroll
        for (int k = 0; k < D; ++k) f[k] = used64 ? (double)acc_v[k] + dpff_to_double(facc[k]) : dpff_to_double(facc[k]);
    }
    return used64 ? acc_s + dpff_to_double(sacc) : dpff_to_double(sacc);
#else
    if (ACC == DP_ACC_FORCE) {
#pragma unroll
        for (int k = 0; k < D; ++k) f[k] = (double)acc_v[k];
    }
    return acc_s;
#endif
}

// F (SoA float64) for every particle. One thread per particle; the
// double-float loop is limited to 64 registers (four 256-thread CTAs per SM).
#if DP_FF
#define DP_FORCES_BOUNDS __launch_bounds__(256, 4)
#else
#define DP_FORCES_BOUNDS __launch_bounds__(256)
#endif
extern "C" __global__ void DP_FORCES_BOUNDS dp_forces(dp_pair_args a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double f[DP_DIM];
    dp_particle_sum<DP_ACC_FORCE>(a, i, f);
    bool finite = true;
#pragma unroll
    for (int k = 0; k < DP_DIM; ++k) {
        a.out[k * a.n + i] = f[k];
        finite = finite && dp_isfinite_bits(f[k]);
    }
    if (!finite) atomicExch(&a.status->nonfinite, 1);
}

#if !DP_MLP
// One MD step of particle i in one kernel: its pair forces from this step's
// positions (as dp_forces), then its integration, wrap, fixed-point forms and
// skin test (dp_integrate_one) into the second set of position buffers, which
// no thread of this launch reads. The float64 integrator work runs on the
// float64 pipe beside the pair arithmetic of other warps, and the forces
// never go through memory. `far` must have been cleared by the host-side
// step sequence when the previous step wrapped every position.
#ifndef DP_STEP_MIN_BLOCKS
#define DP_STEP_MIN_BLOCKS 0
#endif

#ifndef DP_STEP_SETS_COND
#define DP_STEP_SETS_COND 1
#endif
#if DP_STEP_SETS_COND
// Device-side condition of a graph's conditional node (CUDA device runtime).
extern "C" __device__ void cudaGraphSetConditional(unsigned long long handle, unsigned int value);
#endif

// End of a fused step in a graph. Each CTA adds 1 and, in the upper word, 1
// if one of its particles moved beyond skin/2, to one 64-bit counter; the
// CTA that brings the count to the grid size is the last one: every other CTA
// has finished (and read `far`), so it clears `far` (all positions are
// wrapped now) and sets the condition of the next step's rebuild node from
// the summed flags, so that node needs no condition kernel of its own. No
// fence is needed: the condition comes from the counter itself. Called by
// every thread of the CTA with its own `old`.
__device__ __forceinline__ void dp_step_end(const dp_int_args& b, bool old) {
    if (b.end_flags == 0) return;  // uniform: launches outside graphs
    const int cta_old = __syncthreads_or(old ? 1 : 0);
    if (threadIdx.x != 0) return;
    const unsigned long long mine = 1ull | ((unsigned long long)(cta_old != 0) << 32);
    const unsigned long long prev = atomicAdd(&b.st->ticket, mine);
    if ((unsigned)(prev & 0xffffffffull) != gridDim.x - 1) return;
    b.st->ticket = 0ull;
    const bool rebuild = ((prev + mine) >> 32) != 0;
    if (b.end_flags & DP_END_CLEAR_FAR) b.st->far = 0;
#if DP_STEP_SETS_COND
    if (b.end_flags & DP_END_SET_COND) cudaGraphSetConditional(b.next_cond, rebuild ? 1u : 0u);
#else
    (void)rebuild;
#endif
}
#if DP_STEP_MIN_BLOCKS > 0
#define DP_STEP_BOUNDS __launch_bounds__(256, DP_STEP_MIN_BLOCKS)
#else
#define DP_STEP_BOUNDS __launch_bounds__(256)
#endif
extern "C" __global__ void DP_STEP_BOUNDS dp_step(dp_pair_args a, dp_int_args b) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool old = false, bad = false;
    if (i < a.n) {
        double f[DP_DIM];
        dp_particle_sum<DP_ACC_FORCE>(a, i, f);
#pragma unroll
        for (int k = 0; k < DP_DIM; ++k) bad = bad || !dp_isfinite_bits(f[k]);
        old = dp_integrate_dispatch<DP_DIM, DP_FF != 0>(b, i, f, bad);
    }
    const bool any_old = __any_sync(0xffffffffu, old);
    const bool any_bad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (any_old) atomicExch(&b.st->need_rebuild, 1);
        if (any_bad) atomicExch(&b.st->nonfinite, 1);
    }
    dp_step_end(b, old);
}

// The fused step for small systems: LANES lanes per particle. The lanes
// split the particle's list (dp_particle_sum<..., LANES>), their partial
// forces are added across the group in a fixed order, and the group's first
// lane integrates. Below a few tens of thousands of particles this spreads the
// pair loops over LANES times more threads than dp_step, whose one thread per
// particle leaves most SMs idle.
template <int LANES, bool ALL = false>
__device__ __forceinline__ void dp_step_split(const dp_pair_args& a, const dp_int_args& b) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long i = t / LANES;
    const int lane = (int)(t % LANES);
    bool old = false, bad = false;
    const bool active = i < a.n;  // uniform across the group, not the warp
    double f[DP_DIM];
#pragma unroll
    for (int k = 0; k < DP_DIM; ++k) f[k] = 0.0;
    if (active) dp_particle_sum<DP_ACC_FORCE, LANES, ALL>(a, i, f, lane);
    // every lane of the warp takes part in the shuffles (groups past the
    // last particle add zeros)
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) {
#pragma unroll
        for (int k = 0; k < DP_DIM; ++k) f[k] += __shfl_down_sync(0xffffffffu, f[k], off, LANES);
    }
    if (active && lane == 0) {
#pragma unroll
        for (int k = 0; k < DP_DIM; ++k) bad = bad || !dp_isfinite_bits(f[k]);
        old = dp_integrate_dispatch<DP_DIM, DP_FF != 0>(b, i, f, bad);
    }
    const bool any_old = __any_sync(0xffffffffu, old);
    const bool any_bad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (any_old) atomicExch(&b.st->need_rebuild, 1);
        if (any_bad) atomicExch(&b.st->nonfinite, 1);
    }
    dp_step_end(b, old);
}

extern "C" __global__ void DP_STEP_BOUNDS dp_step_warp(dp_pair_args a, dp_int_args b) { dp_step_split<32>(a, b); }
extern "C" __global__ void DP_STEP_BOUNDS dp_step_quad(dp_pair_args a, dp_int_args b) { dp_step_split<4>(a, b); }

// ---------------------------------------------------------------------------
// No neighbour list: dompap's double-loop and vectorised methods
// (dompap/potential.py:103-160 energy, :191-250 and :298-324 forces). One
// warp per particle; lane l takes the slots l, l + 32, ... (every other
// particle is a candidate, tested with the same pre-filter and pair arithmetic
// as the list kernels), and the partial sums are added across the warp in a
// fixed order.
extern "C" __global__ void DP_STEP_BOUNDS dp_step_all(dp_pair_args a, dp_int_args b) { dp_step_split<32, true>(a, b); }

extern "C" __global__ void __launch_bounds__(256) dp_forces_all(dp_pair_args a) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long i = t >> 5;
    const int lane = (int)(t & 31);
    const bool active = i < a.n;  // uniform across the warp
    double f[DP_DIM];
#pragma unroll
    for (int k = 0; k < DP_DIM; ++k) f[k] = 0.0;
    if (active) dp_particle_sum<DP_ACC_FORCE, 32, true>(a, i, f, lane);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int k = 0; k < DP_DIM; ++k) f[k] += __shfl_down_sync(0xffffffffu, f[k], off);
    }
    if (!active || lane != 0) return;
    bool finite = true;
#pragma unroll
    for (int k = 0; k < DP_DIM; ++k) {
        a.out[k * a.n + i] = f[k];
        finite = finite && dp_isfinite_bits(f[k]);
    }
    if (!finite) atomicExch(&a.status->nonfinite, 1);
}

// U = sum over n < m of eps u(r / sigma) (no halving), per-block partials.
extern "C" __global__ void __launch_bounds__(256) dp_energy_all(dp_pair_args a) {
    __shared__ double smem[32];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long i = t >> 5;
    double v = 0.0;
    if (i < a.n) v = dp_particle_sum<DP_ACC_ENERGY_UPPER, 32, true>(a, i, nullptr, (int)(t & 31));
    v = dp_block_sum(v, smem);
    if (threadIdx.x == 0) a.partial[blockIdx.x] = v;
}
#endif

// Per-block partial sums of a scalar pair quantity (energy or virial); the
// host-side reduction kernel adds the partials in a fixed order.
template <int ACC>
__device__ __forceinline__ void dp_scalar_partial(const dp_pair_args& a) {
    __shared__ double smem[32];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < a.n) v = dp_particle_sum<ACC>(a, i, nullptr);
    v = dp_block_sum(v, smem);
    if (threadIdx.x == 0) a.partial[blockIdx.x] = v;
}

extern "C" __global__ void __launch_bounds__(256) dp_energy(dp_pair_args a) { dp_scalar_partial<DP_ACC_ENERGY>(a); }

extern "C" __global__ void __launch_bounds__(256) dp_virial(dp_pair_args a) { dp_scalar_partial<DP_ACC_VIRIAL>(a); }

// Per-particle Laplacian of the potential energy (float64 out[i]).
extern "C" __global__ void __launch_bounds__(256) dp_laplacian(dp_pair_args a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    a.out[i] = dp_particle_sum<DP_ACC_LAPLACE>(a, i, nullptr);
}

// u_cut, f_cut, c_cut of the compiled potential at scaled distances s[i]
// (the reference's pair_potential / pair_force / pair_curvature callables).
extern "C" __global__ void dp_eval_pair(const double* s_in, double* u, double* f, double* c, long long n,
                                        double rcut) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = s_in[i];
    if (s > rcut) {
        u[i] = 0.0;
        f[i] = 0.0;
        c[i] = 0.0;
        return;
    }
    const real_t sr = (real_t)s, sinv = real_t(1) / sr;
    u[i] = (double)dp_pair_u<real_t>(sr, sinv);
    f[i] = (double)dp_pair_f<real_t>(sr, sinv);
    c[i] = (double)dp_pair_c<real_t>(sr, sinv);
}

#if DP_MLP
// ---------------------------------------------------------------------------
// Pair surrogate path: the generated dp_pair_* functions hold the cheap
// terms of the potential (in float32), the network of mlp_common.cuh the
// costly ones; sigma = epsilon = 1 in this mode. Each unique pair inside
// r_cut is evaluated once (Newton's third law): a warp owns 32 particles, and
// before each round every lane advances along its particle's neighbour list
// to the next partner it owns (dp_owns_pair) inside r_cut, so a round's 32 network rows are
// all real pairs (two 16-row tensor-core tiles); each row's result goes back
// to the lane owning the pair, which adds
//   f/r = f_cheap(r)/r + (f r)_nn / r^2,   u = u_cheap(r) + u_nn.
// Forces: +F to i in registers, -F to j as a 64-bit fixed-point atomic add
// (integer sums are exact, so the result does not depend on the order of the
// atomics; 2^-32 resolution); dp_mlp_forces_finish converts the sums to float64.
#define DP_MLP_FX_LIMIT 1073741824.0f  // 2^30: larger contributions are flagged

// round(v 2^32) for |v| <= 2^30 from the float's bits (integer shifts, no
// 64-bit conversion instruction); halves round away from zero.
__device__ __forceinline__ long long dp_f2fx32(float v) {
    const uint32_t b = __float_as_uint(v);
    const int e = (int)((b >> 23) & 0xFFu) - 127;  // v = 1.m 2^e
    if (e < -33) return 0;                          // |v 2^32| < 1/2 (zeros and subnormals too)
    const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u);
    const int sh = e + 9;                           // v 2^32 = m 2^(e + 32 - 23)
    const long long r = sh >= 0 ? (m << sh) : ((m + (1LL << (-sh - 1))) >> (-sh));
    return (b >> 31) ? -r : r;
}

__device__ __forceinline__ void dp_mlp_fx_add(unsigned long long* p, float v, bool& bad) {
    bad = bad || !(fabsf(v) < DP_MLP_FX_LIMIT);
    const float c = fminf(fmaxf(v, -DP_MLP_FX_LIMIT), DP_MLP_FX_LIMIT);
    atomicAdd(p, (unsigned long long)dp_f2fx32(c));
}

template <int ACC>
__device__ __forceinline__ void dp_mlp_pass(const dp_pair_args& a, const dp_mlp_dev* mg, unsigned long long* fx) {
    constexpr int D = DP_DIM;
    __shared__ dp_mlp_dev m;
    __shared__ double red[32];
    dp_mlp_load(&m, mg);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2;
    const long long n = a.n;
    const long long i = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * 32 + lane;
    const bool active = i < n;
    const shadow_t* __restrict__ sh = (const shadow_t*)a.shadow;
    uint32_t ui[D];
    if (active) dp_shadow_unpack<D>(sh[i], ui);
    const int c = active ? a.cnt[i] : 0;
    const float rc2 = (float)(a.rcut * a.rcut);
    float f[D];
#pragma unroll
    for (int k = 0; k < D; ++k) f[k] = 0.0f;
    double acc = 0.0;
    bool bad = false;
    int kk = 0;
    while (true) {
        // this lane's next unique pair inside r_cut
        bool valid = false;
        int j = 0;
        float q = m.x_mean, df[D];
        while (kk < c && !valid) {
            j = __ldg(a.nl + (long long)kk * n + i);
            ++kk;
            if (!dp_owns_pair(i, j)) continue;
            uint32_t uj[D];
            dp_shadow_unpack<D>(__ldg(sh + j), uj);
            const float qq = dp_shadow_q<D>(ui, uj, a.unit, df);
            if (qq <= rc2) {
                valid = true;
                q = qq;
            }
        }
        if (!__any_sync(0xffffffffu, valid)) break;
        float nn_u = 0.f, nn_f = 0.f;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const float sg = __shfl_sync(0xffffffffu, q, 16 * t + g);
            const float sg8 = __shfl_sync(0xffffffffu, q, 16 * t + g + 8);
            float y[2][2];
            dp_mlp_tile<false>(m, sg, sg8, y);
            const int o = lane - 16 * t;       // row of this lane's own pair in tile t
            const int src = 4 * (o & 7);        // quad holding that row
            const float r0u = __shfl_sync(0xffffffffu, y[0][0], src), r0f = __shfl_sync(0xffffffffu, y[0][1], src);
            const float r1u = __shfl_sync(0xffffffffu, y[1][0], src), r1f = __shfl_sync(0xffffffffu, y[1][1], src);
            if (o >= 0 && o < 16) {
                nn_u = (o < 8) ? r0u : r1u;
                nn_f = (o < 8) ? r0f : r1f;
            }
        }
        if (valid) {
            const float rinv = rsqrtf(q);
            const float r = q * rinv;
            const float fr = dp_pair_f<float>(r, rinv) * rinv + nn_f * m.f_scale * (rinv * rinv);
            if (ACC == DP_ACC_FORCE) {
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const float fk = fr * df[k];
                    f[k] += fk;
                    dp_mlp_fx_add(fx + (long long)k * n + j, -fk, bad);
                }
            } else if (ACC == DP_ACC_ENERGY) {
                // the host halves the full-list sum: a unique pair counts twice
                acc += 2.0 * (double)(dp_pair_u<float>(r, rinv) + nn_u * m.u_scale);
            } else {
                acc += (double)(fr * q);
            }
        }
    }
    if (ACC == DP_ACC_FORCE) {
        if (active) {
#pragma unroll
            for (int k = 0; k < D; ++k) dp_mlp_fx_add(fx + (long long)k * n + i, f[k], bad);
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(&a.status->nonfinite, 1);
    } else {
        const double v = dp_block_sum(acc, red);
        if (threadIdx.x == 0) a.partial[blockIdx.x] = v;
    }
}

extern "C" __global__ void __launch_bounds__(256, 2) dp_forces_mlp(dp_pair_args a, const dp_mlp_dev* mlp,
                                                                unsigned long long* fx) {
    dp_mlp_pass<DP_ACC_FORCE>(a, mlp, fx);
}
extern "C" __global__ void __launch_bounds__(256, 2) dp_energy_mlp(dp_pair_args a, const dp_mlp_dev* mlp,
                                                                unsigned long long* fx) {
    dp_mlp_pass<DP_ACC_ENERGY>(a, mlp, fx);
}
extern "C" __global__ void __launch_bounds__(256, 2) dp_virial_mlp(dp_pair_args a, const dp_mlp_dev* mlp,
                                                                unsigned long long* fx) {
    dp_mlp_pass<DP_ACC_VIRIAL>(a, mlp, fx);
}

// ---------------------------------------------------------------------------
// The same pass on the fifth-generation tensor cores (dp_umma.cuh): a CTA of
// 128 threads owns 128 particles; per round every thread takes its next unique
// pair inside r_cut and writes that pair's layer-1 activations (bf16 high part
// and remainder) as one row of the 128 x 64 A operand in shared memory; one
// thread issues the 4 K-steps x 2 parts of tcgen05.mma against W2 (bf16, in
// shared memory) into a 128-lane x 64-column fp32 TMEM accumulator; each thread
// then reads its own row back (tcgen05.ld) and finishes layers 2 and 3 for its
// pair, with no exchange between threads.
#define DP_TC_WAIT_LIMIT (1 << 22)

template <int ACC>
__device__ __forceinline__ void dp_mlp_pass_tc(const dp_pair_args& a, const dp_mlp_dev* mg, unsigned long long* fx) {
    constexpr int D = DP_DIM;
    constexpr int ROWS = 128;
    __shared__ __align__(128) unsigned char sA_hi[ROWS * 64 * 2];
    __shared__ __align__(128) unsigned char sA_lo[ROWS * 64 * 2];
    __shared__ __align__(128) unsigned char sB[64 * 64 * 2];
    __shared__ float s_w1[64], s_b1[64], s_b2[64], s_w30[64], s_w31[64], s_misc[6];
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    __shared__ double red[32];
    const int tid = threadIdx.x, warp = tid >> 5;
    // network: scalars, and W2 from its packed B fragments into the canonical layout
    if (tid < 64) {
        s_w1[tid] = mg->w1[tid];
        s_b1[tid] = mg->b1[tid];
        s_b2[tid] = mg->b2[tid];
        s_w30[tid] = mg->w3[0][tid];
        s_w31[tid] = mg->w3[1][tid];
    }
    if (tid == 0) {
        s_misc[0] = mg->b3[0];
        s_misc[1] = mg->b3[1];
        s_misc[2] = mg->x_mean;
        s_misc[3] = mg->x_inv_scale;
        s_misc[4] = mg->u_scale;
        s_misc[5] = mg->f_scale;
        dp_mbar_init(&s_mbar, 1);
    }
    for (int t = tid; t < 4 * 8 * 32; t += ROWS) {
        const int lane = t & 31, nt = (t >> 5) & 7, kt = t >> 8;
        const int nrow = nt * 8 + (lane >> 2), k = kt * 16 + 2 * (lane & 3);
        *(uint32_t*)(sB + dp_umma_offset(nrow, k, 64)) = mg->w2frag[t * 2 + 0];
        *(uint32_t*)(sB + dp_umma_offset(nrow, k + 8, 64)) = mg->w2frag[t * 2 + 1];
    }
    if (warp == 0) dp_tmem_alloc(&s_tmem, 64);
    dp_async_smem_fence();
    dp_tc_fence_before();
    __syncthreads();
    dp_tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = dp_umma_idesc_bf16<ROWS, 64>();
    const float x_mean = s_misc[2], x_inv = s_misc[3], u_scale = s_misc[4], f_scale = s_misc[5];

    const long long n = a.n;
    const long long i = (long long)blockIdx.x * ROWS + tid;
    const bool active = i < n;
    const shadow_t* __restrict__ sh = (const shadow_t*)a.shadow;
    uint32_t ui[D];
    if (active) dp_shadow_unpack<D>(sh[i], ui);
    const int c = active ? a.cnt[i] : 0;
    const float rc2 = (float)(a.rcut * a.rcut);
    float f[D];
#pragma unroll
    for (int k = 0; k < D; ++k) f[k] = 0.0f;
    double acc = 0.0;
    bool bad = false, timed_out = false;
    uint32_t phase = 0;
    int kk = 0;
    // this thread's next unique pair inside r_cut (the search of round r + 1
    // runs while the tensor core computes round r)
    bool nvalid = false;
    int nj = 0;
    float nq = x_mean;
    auto search = [&]() {
        nvalid = false;
        nq = x_mean;
        while (kk < c && !nvalid) {
            const int jj = __ldg(a.nl + (long long)kk * n + i);
            ++kk;
            if (!dp_owns_pair(i, jj)) continue;
            uint32_t uj[D];
            dp_shadow_unpack<D>(__ldg(sh + jj), uj);
            float dd[D];
            const float qq = dp_shadow_q<D>(ui, uj, a.unit, dd);
            if (qq <= rc2) {
                nvalid = true;
                nj = jj;
                nq = qq;
            }
        }
    };
    search();
    while (true) {
        const bool valid = nvalid;
        const int j = nj;
        const float q = nq;
        // previous round's TMEM reads are complete in every thread past this barrier
        dp_tc_fence_before();
        if (!__syncthreads_or(valid)) break;
        dp_tc_fence_after();
        // layer 1 into row tid of the A operand
        const float x = (q - x_mean) * x_inv;
#pragma unroll
        for (int g8 = 0; g8 < 8; ++g8) {
            uint32_t hi[4], lo[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int k = g8 * 8 + 2 * e;
                dp_split2(dp_mlp_act<false>(fmaf(s_w1[k], x, s_b1[k])),
                          dp_mlp_act<false>(fmaf(s_w1[k + 1], x, s_b1[k + 1])), hi[e], lo[e]);
            }
            const int o = dp_umma_offset(tid, g8 * 8, ROWS);
            *(uint4*)(sA_hi + o) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
            *(uint4*)(sA_lo + o) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
        dp_async_smem_fence();
        dp_tc_fence_before();
        __syncthreads();
        dp_tc_fence_after();
        if (tid == 0) {
            const uint32_t a_hi = dp_smem_addr(sA_hi), a_lo = dp_smem_addr(sA_lo), b = dp_smem_addr(sB);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const uint64_t bd = dp_umma_desc(b + ks * (64 * 32));
                dp_umma_bf16(tmem, dp_umma_desc(a_lo + ks * (ROWS * 32)), bd, idesc, ks > 0 ? 1u : 0u);
                dp_umma_bf16(tmem, dp_umma_desc(a_hi + ks * (ROWS * 32)), bd, idesc, 1u);
            }
            dp_umma_commit(&s_mbar);
        }
        search();  // next round's pair, overlapping the MMAs
        const bool ok = dp_mbar_wait(&s_mbar, phase, DP_TC_WAIT_LIMIT);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        dp_tc_fence_after();
        // layers 2 and 3 for this thread's pair: two halves of 32 columns
        float y0 = s_misc[0], y1 = s_misc[1];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            float z[32];
            dp_tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(half * 32), z);
#pragma unroll
            for (int cc = 0; cc < 32; ++cc) {
                const int col = half * 32 + cc;
                const float h = dp_mlp_act<false>(z[cc] + s_b2[col]);
                y0 = fmaf(h, s_w30[col], y0);
                y1 = fmaf(h, s_w31[col], y1);
            }
        }
        if (valid) {
            const float rinv = rsqrtf(q);
            const float r = q * rinv;
            const float fr = dp_pair_f<float>(r, rinv) * rinv + y1 * f_scale * (rinv * rinv);
            if (ACC == DP_ACC_FORCE) {
                // the displacement again from the partner's shadow (cached), not kept across the round
                uint32_t uj[D];
                dp_shadow_unpack<D>(__ldg(sh + j), uj);
                float df[D];
                dp_shadow_q<D>(ui, uj, a.unit, df);
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const float fk = fr * df[k];
                    f[k] += fk;
                    dp_mlp_fx_add(fx + (long long)k * n + j, -fk, bad);
                }
            } else if (ACC == DP_ACC_ENERGY) {
                acc += 2.0 * (double)(dp_pair_u<float>(r, rinv) + y0 * u_scale);
            } else {
                acc += (double)(fr * q);
            }
        }
    }
    if (timed_out) {
        // the MMAs of the abandoned round may still be in flight: wait (bounded) before freeing TMEM
        dp_mbar_wait(&s_mbar, phase ^ 1u, DP_TC_WAIT_LIMIT);
        if (tid == 0) atomicExch(&a.status->device_error, 1);
    }
    dp_tc_fence_before();
    __syncthreads();
    if (warp == 0) dp_tmem_dealloc(tmem, 64);
    if (ACC == DP_ACC_FORCE) {
        if (active) {
#pragma unroll
            for (int k = 0; k < D; ++k) dp_mlp_fx_add(fx + (long long)k * n + i, f[k], bad);
        }
        if (bad) atomicExch(&a.status->nonfinite, 1);
    } else {
        const double v = dp_block_sum(acc, red);
        if (threadIdx.x == 0) a.partial[blockIdx.x] = v;
    }
}

extern "C" __global__ void __launch_bounds__(128, 5) dp_forces_mlp_tc(dp_pair_args a, const dp_mlp_dev* mlp,
                                                                      unsigned long long* fx) {
    dp_mlp_pass_tc<DP_ACC_FORCE>(a, mlp, fx);
}
extern "C" __global__ void __launch_bounds__(128, 5) dp_energy_mlp_tc(dp_pair_args a, const dp_mlp_dev* mlp,
                                                                      unsigned long long* fx) {
    dp_mlp_pass_tc<DP_ACC_ENERGY>(a, mlp, fx);
}
extern "C" __global__ void __launch_bounds__(128, 5) dp_virial_mlp_tc(dp_pair_args a, const dp_mlp_dev* mlp,
                                                                      unsigned long long* fx) {
    dp_mlp_pass_tc<DP_ACC_VIRIAL>(a, mlp, fx);
}

// Fixed-point force sums -> float64 forces (SoA), and clear the sums.
extern "C" __global__ void __launch_bounds__(256) dp_mlp_forces_finish(dp_pair_args a, unsigned long long* fx) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n * DP_DIM) return;
    a.out[t] = (double)(long long)fx[t] * (1.0 / 4294967296.0);
    fx[t] = 0ull;
}
#endif
