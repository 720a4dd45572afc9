// dp_common.cuh — device helpers shared by the statically compiled kernels
// (dompap_gpu.cu) and the NVRTC-compiled pair kernels (pair_kernels.cuh).
//
// Everything here is plain CUDA C++ with no includes, so that the same text is
// compiled by nvcc and embedded verbatim into NVRTC programs.
#pragma once

#ifdef __CUDACC_RTC__
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
#endif

#define DP_MAX_DIM 4

// Device status word shared by every kernel of one simulation handle. The host
// reads it (pinned mirror) after each chunk of steps.
struct dp_dev_status {
    int32_t need_rebuild;     // 1: the next step rebuilds the neighbour list
    int32_t max_neighbors;    // largest neighbour count seen by the last build
    int32_t cell_overflow;    // largest cell occupancy seen when it exceeded capacity
    int32_t nonfinite;        // a force or position became NaN/Inf
    int32_t far;              // some coordinate lies outside [-L/4, 5L/4) (not yet wrapped)
    int32_t device_error;     // a bounded device-side wait gave up: the launch's results are invalid
    int32_t ref_far;          // `far` held when the current list was built (its reference positions)
    int32_t pad;
    int64_t rebuilds;         // neighbour-list builds done on the device
    int64_t step;             // steps integrated (the RNG counter)
    // fused step in a graph: CTAs finished (low 32 bits) and CTAs with a
    // particle beyond skin/2 (high 32 bits); its last CTA resets it
    unsigned long long ticket;
};

// Arguments of the NVRTC-compiled pair kernels (pair_kernels.cuh); the host
// fills the same struct, so the layout is shared by construction.
struct dp_pair_args {
    const double* pos;
    const void* shadow;
    const int32_t* nl;
    const int32_t* cnt;
    const int32_t* types;
    const double* sig_tab;
    const double* eps_tab;
    const double* isig_tab;  // 1 / sigma per type pair (DP_PMODE == 1)
    const float2* ff_tab;    // DP_PMODE == 1: (sigma, 1/sigma, epsilon) as double-float triples
    const void* pos64;       // 64-bit fixed-point positions (X = x 2^64 / L), one vector per particle
    const int32_t* order;    // particle id held by each slot (slots are in cell order after a rebuild)
    double* out;
    double* partial;
    dp_dev_status* status;
    long long n;
    int ntypes;
    int upper;               // DP_PMODE == 2: parameters of (min, max) of the two ids (Newton's-third-law loop)
    double box[DP_MAX_DIM];
    float unit[DP_MAX_DIM];  // L / 2^32 per axis
    float unit64_hi[DP_MAX_DIM];  // L / 2^64 per axis as a double-float
    float unit64_lo[DP_MAX_DIM];
    double sigma;            // DP_PMODE == 0
    double inv_sigma;        // DP_PMODE == 0
    double epsilon;          // DP_PMODE == 0
    double rcut;             // r_cut in units of sigma
    float cut2f;             // pre-filter: skip a pair when its float32 r^2 exceeds this
    float rcut_f;            // (float) rcut
    int rcut_finite;
    float ff_const[6];       // DP_PMODE == 0: sigma, 1/sigma, epsilon as double-float pairs
    int pad1;
};

// Arguments of the batched-replica kernel (batch_kernels.cuh).
struct dp_batch_args {
    double* pos;               // SoA [k * ntot + i]
    double* vel;
    double* beta;
    int32_t* img;
    void* shadow;              // fixed-point positions, one vector per particle
    const long long* offset;   // [n_rep + 1] first particle of each replica
    const int32_t* order;      // replicas in processing order (this launch's bucket)
    const double* box;         // [n_rep * DP_MAX_DIM]
    const double* coef;        // [n_rep * 5] G-JF a, b dt/m, b/(2m), sqrt(2 alpha T dt), dt/m
    const int32_t* ncell;      // [n_rep * DP_MAX_DIM] cells per axis, 0 = all pairs
    double* obs;               // [n_rep * 4] sum U, sum W, sum m v^2, samples
    float* force_out;          // optional SoA float forces of the last step
    int32_t* queue;            // work counter of this launch (zeroed before it)
    dp_dev_status* st;
    long long ntot;
    int n_rep;                 // replicas in `order`
    int steps;
    int sample_every;          // accumulate observables every this many steps (0: never)
    int max_n;                 // shared-memory capacity in particles
    int max_cells;             // shared-memory capacity in cells
    int nve;                   // 1: NVE leap-frog instead of G-JF
    double dt;
    float rc2;                 // r_cut^2 (float32 cut)
    int pad;
    unsigned long long seed;
    // Verlet lists (nlist == nullptr: cell stencil every step)
    uint16_t* nlist;           // [off * kmax + ((k / 8) * n + p) * 8 + k % 8]: k-th listed neighbour of p
    int32_t* ncnt;             // [ntot] list lengths
    void* shadow_ref;          // [ntot] fixed-point positions at the replica's last build
    unsigned long long* list_stats;  // [0]: builds, [1]: replicas whose list overflowed
    int32_t* list_gen;         // [n_rep total] generation each replica's list was built for
    int kmax;
    float rl2;                 // list cutoff^2 = (r_cut + skin)^2
    float skin_thr2;           // (skin / 2)^2: rebuild when some particle moved farther
    int gen;                   // current generation (changes whenever the host changes state or settings)
};

// ---------------------------------------------------------------------------
// Minimum image, single +-L shift per axis, exactly as
// dompap/positions.py:12-16 (box/2 is exact in binary floating point).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dp_min_image(double d, double L) {
    const double half = 0.5 * L;
    if (d > half) {
        d -= L;
    } else if (d < -half) {
        d += L;
    }
    return d;
}

// Sequential d0^2 + d1^2 + ... without FMA contraction, matching the order and
// rounding of NumPy/Numba summing a short float64 vector (bit-exact pair test,
// dompap/neighbor_list.py:32-33).
template <int D>
__device__ __forceinline__ double dp_sqsum_exact(const double* d) {
    double q = __dmul_rn(d[0], d[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) q = __dadd_rn(q, __dmul_rn(d[k], d[k]));
    return q;
}

// ---------------------------------------------------------------------------
// Fixed-point position shadow: u = floor(x * 2^32 / L) mod 2^32 per axis.
// The wrap-around difference (int32)(u_i - u_j) is the nearest-image
// displacement in units of L / 2^32, so the pair pre-filter needs no float64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t dp_fixed(double x, double scale /* 2^32 / L */) {
    const long long t = __double2ll_rd(x * scale);
    return (uint32_t)(unsigned long long)t;
}

// 64-bit fixed point X = floor(x 2^64 / L) for 0 <= x < L (exact product
// rounding aside), the source of the exact nearest-image displacement
// (int64)(X_i - X_j) of the double-float pair arithmetic.
template <int D>
struct dp_fixed64_t {
    typedef ulonglong4 type;
};
template <>
struct dp_fixed64_t<2> {
    typedef ulonglong2 type;
};
template <int D>
__device__ __forceinline__ void dp_fixed64_unpack(const typename dp_fixed64_t<D>::type& v, unsigned long long* X);
template <>
__device__ __forceinline__ void dp_fixed64_unpack<2>(const ulonglong2& v, unsigned long long* X) {
    X[0] = v.x;
    X[1] = v.y;
}
template <>
__device__ __forceinline__ void dp_fixed64_unpack<3>(const ulonglong4& v, unsigned long long* X) {
    X[0] = v.x;
    X[1] = v.y;
    X[2] = v.z;
}
template <>
__device__ __forceinline__ void dp_fixed64_unpack<4>(const ulonglong4& v, unsigned long long* X) {
    X[0] = v.x;
    X[1] = v.y;
    X[2] = v.z;
    X[3] = v.w;
}
template <int D>
__device__ __forceinline__ typename dp_fixed64_t<D>::type dp_fixed64_pack(const unsigned long long* X);
template <>
__device__ __forceinline__ ulonglong2 dp_fixed64_pack<2>(const unsigned long long* X) {
    return make_ulonglong2(X[0], X[1]);
}
template <>
__device__ __forceinline__ ulonglong4 dp_fixed64_pack<3>(const unsigned long long* X) {
    return make_ulonglong4(X[0], X[1], X[2], 0ull);
}
template <>
__device__ __forceinline__ ulonglong4 dp_fixed64_pack<4>(const unsigned long long* X) {
    return make_ulonglong4(X[0], X[1], X[2], X[3]);
}

// Both fixed-point forms of one coordinate from the float64 product
// p = x 2^64 / L: the 64-bit one and its upper 32 bits (the shadow). The
// coordinate must lie in [0, L); a product rounded up to 2^64 saturates.
// floor(p) from the bit pattern (integer shifts, no float64 conversion
// instruction): p < 1 and negative p give 0, p >= 2^64 saturates.
__device__ __forceinline__ unsigned long long dp_fixed64_of(double p) {
    const long long b = __double_as_longlong(p);
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    if (b < 0 || e < 0) return 0ull;
    if (e >= 64) return ~0ull;
    const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    return e >= 52 ? m << (e - 52) : m >> (52 - e);
}

// Half lists (the surrogate mode evaluates each pair once): particle i owns
// the pair {i, j} when the two slots differ in parity and i < j, or share it
// and i > j. Exactly one of the two owns every pair, and each particle owns
// about half of its partners whatever the order of the slots (the cell order
// puts most partners of a particle early in a Morton block above it).
__device__ __forceinline__ bool dp_owns_pair(long long i, long long j) {
    return ((i ^ j) & 1) ? (i < j) : (i > j);
}

// x is neither infinite nor NaN (integer test of the exponent field).
__device__ __forceinline__ bool dp_isfinite_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

// Integer m with |m| < 2^24 as a float, exactly (one 32-bit conversion
// instruction).
__device__ __forceinline__ float dp_small_int(int m) { return __int2float_rn(m); }

// int32 -> float rounded to nearest.
__device__ __forceinline__ float dp_i2f(int n) { return __int2float_rn(n); }

// float -> double by moving the bits (sign, exponent rebiased, mantissa),
// without branches: infinities and NaN keep their class, float subnormals
// become signed zeros (below 1.2e-38; no value that reaches this function
// needs them).
__device__ __forceinline__ double dp_f2d(float z) {
    const uint32_t b = __float_as_uint(z);
    const uint32_t e = (b >> 23) & 0xFFu;
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    const unsigned long long ed = e == 0u ? 0ull : (e == 0xFFu ? 0x7FFull : (unsigned long long)(e + (1023u - 127u)));
    const unsigned long long mant = e == 0u ? 0ull : (unsigned long long)(b & 0x7FFFFFu) << 29;
    return __longlong_as_double((long long)(sign | (ed << 52) | mant));
}

// float64 -> float32 by moving bits, truncating the mantissa (exact for a
// float64 that holds a float32 value; values beyond float32 range become
// infinities, below it zero). No float64 instruction.
__device__ __forceinline__ float dp_d2f_trunc(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FFu) - 1023 + 127;
    const uint32_t sign = (uint32_t)(b >> 63) << 31;
    const uint32_t mant = (uint32_t)((b >> 29) & 0x7FFFFFu);
    const uint32_t body = e <= 0 ? 0u : (e >= 255 ? 0x7F800000u : ((uint32_t)e << 23) | mant);
    return __uint_as_float(sign | body);
}

// A constant of a generated pair potential that float32 holds exactly
// (dp_k<R>(48.0f)): R itself for float and double; the double-float
// arithmetic (dp_ff.cuh) gives it a type whose products and sums take the
// cheaper one-float forms.
template <typename R>
struct dp_k_t {
    typedef R type;
    static __device__ __forceinline__ R make(float v) { return R(v); }
};
template <typename R>
__device__ __forceinline__ typename dp_k_t<R>::type dp_k(float v) {
    return dp_k_t<R>::make(v);
}

template <int D>
struct dp_shadow_t;
template <>
struct dp_shadow_t<2> {
    typedef uint2 type;
};
template <>
struct dp_shadow_t<3> {
    typedef uint4 type;
};
template <>
struct dp_shadow_t<4> {
    typedef uint4 type;
};

template <int D>
__device__ __forceinline__ void dp_shadow_unpack(const typename dp_shadow_t<D>::type& s, uint32_t* u);
template <>
__device__ __forceinline__ void dp_shadow_unpack<2>(const uint2& s, uint32_t* u) {
    u[0] = s.x;
    u[1] = s.y;
}
template <>
__device__ __forceinline__ void dp_shadow_unpack<3>(const uint4& s, uint32_t* u) {
    u[0] = s.x;
    u[1] = s.y;
    u[2] = s.z;
}
template <>
__device__ __forceinline__ void dp_shadow_unpack<4>(const uint4& s, uint32_t* u) {
    u[0] = s.x;
    u[1] = s.y;
    u[2] = s.z;
    u[3] = s.w;
}

template <int D>
__device__ __forceinline__ typename dp_shadow_t<D>::type dp_shadow_pack(const uint32_t* u);
template <>
__device__ __forceinline__ uint2 dp_shadow_pack<2>(const uint32_t* u) {
    return make_uint2(u[0], u[1]);
}
template <>
__device__ __forceinline__ uint4 dp_shadow_pack<3>(const uint32_t* u) {
    return make_uint4(u[0], u[1], u[2], 0u);
}
template <>
__device__ __forceinline__ uint4 dp_shadow_pack<4>(const uint32_t* u) {
    return make_uint4(u[0], u[1], u[2], u[3]);
}

// Float32 squared displacement from two fixed-point shadows.
template <int D>
__device__ __forceinline__ float dp_shadow_q(const uint32_t* ui, const uint32_t* uj, const float* unit,
                                             float* df) {
    float q = 0.0f;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        df[k] = dp_i2f((int)(ui[k] - uj[k])) * unit[k];
        q = fmaf(df[k], df[k], q);
    }
    return q;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11),
// written from the published round function and constants.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 dp_philox4x32_10(uint4 ctr, uint2 key) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        const uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
        const uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
        ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
        key.x += W0;
        key.y += W1;
    }
    return ctr;
}

// Four standard normal deviates for (particle, step) by the Box-Muller
// transform of two Philox outputs pairs.
__device__ __forceinline__ void dp_normals4(uint64_t seed, uint64_t step, uint32_t particle, float* z) {
    const uint4 r = dp_philox4x32_10(make_uint4(particle, (uint32_t)step, (uint32_t)(step >> 32), 0x64706d64u),
                                     make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const float two_pow_m32 = 2.3283064365386963e-10f;
    // u in (0, 1] for the logarithm, v in [0, 1) for the angle
    const float u0 = ((float)r.x + 1.0f) * two_pow_m32;
    const float v0 = (float)r.y * two_pow_m32;
    const float u1 = ((float)r.z + 1.0f) * two_pow_m32;
    const float v1 = (float)r.w * two_pow_m32;
    const float rad0 = sqrtf(-2.0f * logf(fminf(u0, 1.0f)));
    const float rad1 = sqrtf(-2.0f * logf(fminf(u1, 1.0f)));
    float s0, c0, s1, c1;
    sincospif(2.0f * v0, &s0, &c0);
    sincospif(2.0f * v1, &s1, &c1);
    z[0] = rad0 * c0;
    z[1] = rad0 * s0;
    z[2] = rad1 * c1;
    z[3] = rad1 * s1;
}

// Block-wide float64 sum (blockDim.x a multiple of 32, <= 1024); result valid
// in thread 0. Uses warp shuffles, then one warp over the per-warp sums.
__device__ __forceinline__ double dp_block_sum(double v, double* smem /* >= 32 doubles */) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    const int nwarps = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nwarps) ? smem[threadIdx.x] : 0.0;
    if (warp == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}
