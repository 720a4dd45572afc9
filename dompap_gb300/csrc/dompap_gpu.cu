// dompap_gpu.cu — GB300 (sm_103a) implementation of the C ABI in
// include/dompap_gpu.h: device state, the statically compiled kernels (cell
// list, Verlet list, integrators, reductions, layout transposes) and the NVRTC
// pipeline that compiles the SymPy-generated pair potential together with
// pair_kernels.cuh.
//
// Design (one process, one GPU, one stream per handle):
//  * particle state lives in HBM as SoA float64 pos/vel/beta/force[k*N + i]
//    plus int32 images; a fixed-point copy of the positions (uint32 per axis,
//    packed in one 8/16-byte vector per particle) feeds the pair pre-filter;
//  * the neighbour list is column-major nl[k*N + i] with counts cnt[i];
//  * run(steps) replays CUDA graphs of `chunk` steps. Each step is
//    [gated rebuild: cell clear, cell fill, cell sort, Verlet build, done]
//    -> pair forces -> integrate + wrap + skin test (sets need_rebuild).
//    The rebuild kernels return at once unless need_rebuild is set, so the
//    graph needs no host decision. After each chunk the host reads the status
//    word; on a neighbour-list or cell overflow it restores the chunk's start
//    state, grows the capacity and replays the chunk.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <dlfcn.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "dompap_gpu.h"
#include "dp_common.cuh"
#include "dp_integrate.cuh"
#include "dp_umma.cuh"
#include "dp_embedded.h"
#include "mlp_common.cuh"
#include "mlp_train.cuh"  // dp_src_common[], dp_src_pair[] (generated at build time)

// ===========================================================================
// errors
// ===========================================================================
static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(DP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define RET(call)              \
    do {                       \
        int rc_ = (call);      \
        if (rc_ != DP_OK) return rc_; \
    } while (0)

static inline unsigned grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    return (unsigned)std::max<long long>(1, g);
}

// ===========================================================================
// static kernels
// ===========================================================================
namespace {

constexpr int kBlock = 256;

// Host layout (particle id major, (n, dim)) <-> device SoA in slot order:
// element (id, k) lives at k * n + slot_of[id] (slot_of null: slot = id). The
// host side is read or written contiguously (it may be page-locked host memory
// read over the host link); the scattered side is device memory.
template <typename T>
__global__ void k_host_to_slots(const T* __restrict__ in, T* __restrict__ out, const int32_t* __restrict__ slot_of,
                                long long n, int dim) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * dim) return;
    const long long i = t / dim;
    const int k = (int)(t - i * dim);
    out[k * n + (slot_of ? slot_of[i] : i)] = in[t];
}

template <typename T>
__global__ void k_slots_to_host(const T* __restrict__ in, T* __restrict__ out, const int32_t* __restrict__ slot_of,
                                long long n, int dim) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * dim) return;
    const long long i = t / dim;
    const int k = (int)(t - i * dim);
    out[t] = in[k * n + (slot_of ? slot_of[i] : i)];
}

struct ShadowArgs {
    const double* pos;
    void* shadow;
    void* pos64;
    dp_dev_status* st;
    long long n;
    double scale64[DP_MAX_DIM];
    double box[DP_MAX_DIM];
};

// 64-bit fixed point of one coordinate, wrapped into [0, L) first when needed.
__device__ __forceinline__ unsigned long long fixed64_wrapped(double x, double L, double scale64) {
    if (!(x >= 0.0 && x < L)) x -= floor(x / L) * L;
    return dp_fixed64_of(x * scale64);
}

// Fixed-point forms of all positions (the 64-bit X of the position wrapped
// into the box, the shadow its upper word, as the integrators write them);
// flags coordinates outside [-L/4, 5L/4), for which the single-shift image is
// not the nearest one. One float64 product per coordinate in the box: its
// bit pattern is the in-box test.
template <int D>
__global__ void k_shadow(ShadowArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    uint32_t u[D];
    unsigned long long X[D];
    bool far = false;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double x = a.pos[k * a.n + i];
        double p = x * a.scale64[k];
        const long long pb = __double_as_longlong(p);
        if (!(pb >= 0 && pb < 0x43F0000000000000LL)) {  // p outside [0, 2^64): wrap a copy
            far = far || !(x >= -0.25 * a.box[k] && x < 1.25 * a.box[k]);
            const double w = x - floor(x / a.box[k]) * a.box[k];
            p = (w >= 0.0 && w < a.box[k]) ? w * a.scale64[k] : 0.0;
        }
        X[k] = dp_fixed64_of(p);
        u[k] = (uint32_t)(X[k] >> 32);
    }
    ((typename dp_shadow_t<D>::type*)a.shadow)[i] = dp_shadow_pack<D>(u);
    ((typename dp_fixed64_t<D>::type*)a.pos64)[i] = dp_fixed64_pack<D>(X);
    if (far) atomicExch(&a.st->far, 1);
}

// --------------------------- skin test ------------------------------------
// neighbor_list_is_old (dompap/neighbor_list.py:183-201): rebuild when some
// particle's min-image displacement^2 since the last build exceeds (skin/2)^2.
// The displacement since the last build is read from the fixed-point shadows
// in float32; only when it lies within the error bound of (skin/2)^2 is it
// recomputed in float64 exactly as the reference does.
struct SkinArgs {
    const double* pos;
    const double* pos_ref;
    const void* shadow;
    const void* shadow_ref;
    dp_dev_status* st;
    long long n;
    double box[DP_MAX_DIM];
    float unit[DP_MAX_DIM];
    double thr;    // (0.5 * skin)^2
    float thr_lo;  // below: certainly not old
    float thr_hi;  // above: certainly old
};

template <int D>
__global__ void k_skin_check(SkinArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool old = false;
    if (i < a.n) {
        typedef typename dp_shadow_t<D>::type sh_t;
        uint32_t u[D];
        dp_shadow_unpack<D>(((const sh_t*)a.shadow)[i], u);
        double x[D];
#pragma unroll
        for (int k = 0; k < D; ++k) x[k] = a.pos[k * a.n + i];
        old = dp_skin_old<D>(a.shadow_ref, a.pos_ref, a.n, a.unit, a.box, a.thr, a.thr_lo, a.thr_hi, i, u, x,
                             a.st->far != 0 || a.st->ref_far != 0);
    }
    if (__any_sync(0xffffffffu, old) && (threadIdx.x & 31) == 0) atomicExch(&a.st->need_rebuild, 1);
}

// --------------------------- cell binning ---------------------------------
// The cell list of dompap/neighbor_list.py:42-180 as a counting sort. Cells
// are at least `cutoff` wide plus an absolute margin for the rounding of the
// fixed-point shadows (nc = floor(L / w) per axis, >= 3), so every pair
// closer than the cutoff lies in the 3^D stencil of its cell; the reference
// uses cells of width `cutoff` with nc = ceil(L / cutoff) and misses pairs
// when L / cutoff is not an integer. A particle's cell comes from its shadow
// in integer arithmetic, c_k = (u_k nc_k) >> 32, i.e. from its periodic image
// in [0, L). Cells are keyed in Morton (Z) order of their coordinates
// (row-major when the padded Morton range would be too large), counted,
// prefix-summed into contiguous slot ranges, and each particle is given a
// slot in its cell's range, ties ordered by particle id, so that the order is
// a function of the positions alone. The per-particle state then moves into
// that order (k_permute): the partners a step gathers lie close together in
// memory, and each cell of the Verlet build is one contiguous range.
struct BinArgs {
    const void* shadow;    // shadows of the current slots
    const int32_t* order;  // particle id of each current slot
    int32_t* key;          // [n] cell key of each current slot
    int32_t* rank;         // [n] arrival rank within its cell (atomic)
    int32_t* bin_cnt;      // [nbins] particles per cell key
    int32_t* bin_start;    // [nbins + 1] first slot of each cell key
    int32_t* bin_part;     // [ceil(nbins / kScanTile)] scan partial sums
    int32_t* src_of;       // [n] current slot of the particle that new slot t receives
    dp_dev_status* st;
    long long n;
    long long nbins;
    int nc[DP_MAX_DIM];
    int morton;            // 1: Morton keys on the power-of-two padded grid
};

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

// Bit interleaving for Morton keys: bit b of x moves to bit D b.
template <int D>
__device__ __forceinline__ uint32_t dp_spread_bits(uint32_t x);
template <>
__device__ __forceinline__ uint32_t dp_spread_bits<2>(uint32_t x) {
    x &= 0xFFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    return (x | (x << 1)) & 0x55555555u;
}
template <>
__device__ __forceinline__ uint32_t dp_spread_bits<3>(uint32_t x) {
    x &= 0x3FFu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    return (x | (x << 2)) & 0x09249249u;
}
template <>
__device__ __forceinline__ uint32_t dp_spread_bits<4>(uint32_t x) {
    x &= 0xFFu;
    x = (x | (x << 12)) & 0x000F000Fu;
    x = (x | (x << 6)) & 0x03030303u;
    return (x | (x << 3)) & 0x11111111u;
}

// Cell coordinates of a shadow (fixed-point position in [0, 2^32) per axis).
template <int D>
__device__ __forceinline__ void shadow_cell(const uint32_t* u, const int* nc, int* c) {
#pragma unroll
    for (int k = 0; k < D; ++k) c[k] = (int)(((unsigned long long)u[k] * (unsigned)nc[k]) >> 32);
}

template <int D>
__device__ __forceinline__ int cell_key(const int* c, const int* nc, int morton) {
    if (morton) {
        uint32_t key = 0;
#pragma unroll
        for (int k = 0; k < D; ++k) key |= dp_spread_bits<D>((uint32_t)c[k]) << (D - 1 - k);
        return (int)key;
    }
    int l = c[0];
#pragma unroll
    for (int k = 1; k < D; ++k) l = l * nc[k] + c[k];
    return l;
}

__global__ void k_bin_clear(BinArgs a) {
    if (!a.st->need_rebuild) return;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < a.nbins;
         c += (long long)gridDim.x * blockDim.x)
        a.bin_cnt[c] = 0;
}

template <int D>
__global__ void k_bin_count(BinArgs a) {
    if (!a.st->need_rebuild) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    typedef typename dp_shadow_t<D>::type sh_t;
    uint32_t u[D];
    dp_shadow_unpack<D>(((const sh_t*)a.shadow)[i], u);
    int c[D];
    shadow_cell<D>(u, a.nc, c);
    const int key = cell_key<D>(c, a.nc, a.morton);
    a.key[i] = key;
    a.rank[i] = atomicAdd(a.bin_cnt + key, 1);
}

// Exclusive scan of one value per thread over a block of kScanThreads.
__device__ __forceinline__ int block_exclusive_scan(int v, int* smem, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nwarps ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        smem[lane] = w;
    }
    __syncthreads();
    const int before = warp ? smem[warp - 1] : 0;
    *total = smem[nwarps - 1];
    __syncthreads();
    return before + x - v;
}

// Scan of the cell counts: per-tile sums, a one-block scan of those, then
// each tile's exclusive scan plus its offset (bin_start[nbins] = n).
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(BinArgs a) {
    if (!a.st->need_rebuild) return;
    __shared__ int smem[32];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPer;
    int v = 0;
#pragma unroll
    for (int t = 0; t < kScanPer; ++t)
        if (base + t < a.nbins) v += a.bin_cnt[base + t];
    int total = 0;
    block_exclusive_scan(v, smem, &total);
    if (threadIdx.x == 0) a.bin_part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_top(BinArgs a, int parts) {
    if (!a.st->need_rebuild) return;
    __shared__ int smem[32];
    const int per = (parts + kScanThreads - 1) / kScanThreads;
    const int b = threadIdx.x * per;
    int v = 0;
    for (int t = 0; t < per; ++t)
        if (b + t < parts) v += a.bin_part[b + t];
    int total = 0;
    int run = block_exclusive_scan(v, smem, &total);
    for (int t = 0; t < per; ++t)
        if (b + t < parts) {
            const int x = a.bin_part[b + t];
            a.bin_part[b + t] = run;
            run += x;
        }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(BinArgs a) {
    if (!a.st->need_rebuild) return;
    __shared__ int smem[32];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPer;
    int c[kScanPer];
    int v = 0;
#pragma unroll
    for (int t = 0; t < kScanPer; ++t) {
        c[t] = base + t < a.nbins ? a.bin_cnt[base + t] : 0;
        v += c[t];
    }
    int total = 0;
    int run = a.bin_part[blockIdx.x] + block_exclusive_scan(v, smem, &total);
#pragma unroll
    for (int t = 0; t < kScanPer; ++t)
        if (base + t < a.nbins) {
            a.bin_start[base + t] = run;
            run += c[t];
        }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.bin_start[a.nbins] = (int)a.n;
}

__global__ void k_bin_scatter(BinArgs a) {
    if (!a.st->need_rebuild) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    a.src_of[a.bin_start[a.key[i]] + a.rank[i]] = (int32_t)i;
}

// Each cell's range ordered by particle id (the atomic ranks are not
// deterministic; the result is).
__global__ void k_bin_sort(BinArgs a) {
    if (!a.st->need_rebuild) return;
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.nbins) return;
    const int lo = a.bin_start[b], hi = a.bin_start[b + 1];
    for (int t = lo + 1; t < hi; ++t) {
        const int32_t v = a.src_of[t];
        const int32_t id = a.order[v];
        int u = t - 1;
        while (u >= lo && a.order[a.src_of[u]] > id) {
            a.src_of[u + 1] = a.src_of[u];
            --u;
        }
        a.src_of[u + 1] = v;
    }
}

// --------------------------- permutation of the state ----------------------
// Arrays that move with their particle: element `esize` bytes, `comps`
// components at a stride of n elements (SoA), or one vector per particle.
struct PermArray {
    void* data;     // the state array
    void* scratch;  // same shape, receives the permuted copy
    int esize;      // 1, 4, 8, 16 or 32
    int comps;
};

constexpr int kMaxPermArrays = 12;

struct PermArgs {
    PermArray arr[kMaxPermArrays];
    int count;
    const int32_t* src_of;  // new slot t <- current slot src_of[t] (null: copy back)
    const int32_t* order;   // particle id of each current slot
    int32_t* slot_of;       // [n] slot of each particle id (updated)
    dp_dev_status* st;
    long long n;
};

// Copy the components of one particle's entry: every load is issued before
// the first store (independent loads in flight), element type by size.
template <typename T>
__device__ __forceinline__ void copy_comps(const void* src, void* dst, long long from, long long to, long long n,
                                           int comps) {
    T v[DP_MAX_DIM];
#pragma unroll
    for (int k = 0; k < DP_MAX_DIM; ++k)
        if (k < comps) v[k] = ((const T*)src)[k * n + from];
#pragma unroll
    for (int k = 0; k < DP_MAX_DIM; ++k)
        if (k < comps) ((T*)dst)[k * n + to] = v[k];
}

__device__ __forceinline__ void copy_entry(const PermArray& a, const void* src, void* dst, long long from,
                                           long long to, long long n) {
    switch (a.esize) {
        case 1: copy_comps<uint8_t>(src, dst, from, to, n, a.comps); break;
        case 4: copy_comps<uint32_t>(src, dst, from, to, n, a.comps); break;
        case 8: copy_comps<uint2>(src, dst, from, to, n, a.comps); break;
        case 16: copy_comps<uint4>(src, dst, from, to, n, 1); break;
        default: {  // 32 bytes: two 16-byte halves
            const uint4 lo = ((const uint4*)src)[2 * from], hi = ((const uint4*)src)[2 * from + 1];
            ((uint4*)dst)[2 * to] = lo;
            ((uint4*)dst)[2 * to + 1] = hi;
        }
    }
}

// Gather every state array into cell order (into the scratch arrays) and
// record the new slot of each particle id. One array per blockIdx.y, so the
// arrays are copied side by side rather than one after another per thread.
__global__ void k_permute(PermArgs p) {
    if (!p.st->need_rebuild) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const long long o = p.src_of[t];
    const PermArray a = p.arr[blockIdx.y];
    copy_entry(a, a.data, a.scratch, o, t, p.n);
    if (blockIdx.y == 0) p.slot_of[p.order[o]] = (int32_t)t;
}

// The permuted copies back into the state arrays (the kernels captured after
// a rebuild read the state at fixed addresses).
__global__ void k_permute_back(PermArgs p) {
    if (!p.st->need_rebuild) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const PermArray a = p.arr[blockIdx.y];
    copy_entry(a, a.scratch, a.data, t, t, p.n);
}

__global__ void k_iota(int32_t* a, int32_t* b, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = (int32_t)i;
    b[i] = (int32_t)i;
}

// slot_of from order (after a restore of the backed-up order).
__global__ void k_invert_order(const int32_t* order, int32_t* slot_of, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    slot_of[order[i]] = (int32_t)i;
}

// --------------------------- Verlet list ----------------------------------
// get_neighbor_list_double_loop (dompap/neighbor_list.py:7-39): m is a
// neighbour of n when sqrt(sum d^2) < cutoff with the single-shift minimum
// image, tested in float64 without FMA (bit-identical pair set).
struct NlArgs {
    const double* pos;
    double* pos_ref;
    const void* shadow;
    void* shadow_ref;
    int32_t* nl;
    int32_t* cnt;
    const int32_t* bin_start;  // cell ranges of the cell build
    const int32_t* src_of;     // slot of each entry of the ranges (null: the entries are the slots)
    dp_dev_status* st;
    long long n;
    int kcap;
    int morton;
    int nc[DP_MAX_DIM];
    double box[DP_MAX_DIM];
    float unit[DP_MAX_DIM];
    double cutoff;
    float lo2;  // float32 r^2 below this: certainly inside the cutoff
    float hi2;  // float32 r^2 above this: certainly outside
    int half;   // 1: only the partners particle i owns (dp_owns_pair; the surrogate mode uses each pair once)
};

template <int D>
__global__ void __launch_bounds__(kBlock) k_nl_build_cells(NlArgs a) {
    if (!a.st->need_rebuild) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    typedef typename dp_shadow_t<D>::type sh_t;
    const sh_t* sh = (const sh_t*)a.shadow;
    const bool far = a.st->far != 0;
    const long long n = a.n;
    double xi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) xi[k] = a.pos[k * n + i];
    const sh_t shi = sh[i];
    uint32_t ui[D];
    dp_shadow_unpack<D>(shi, ui);
    int ci[D];
    shadow_cell<D>(ui, a.nc, ci);
    // each axis' share of the key for the cells at offsets -1, 0, +1 (periodic);
    // a stencil cell's key is the sum of one share per axis (Morton: disjoint
    // bits; row-major: coordinate times the axis stride)
    int part[D][3];
    {
        int stride = 1;
#pragma unroll
        for (int k = D - 1; k >= 0; --k) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                int c = ci[k] + d - 1;
                if (c < 0) c += a.nc[k];
                if (c >= a.nc[k]) c -= a.nc[k];
                part[k][d] = a.morton ? (int)(dp_spread_bits<D>((uint32_t)c) << (D - 1 - k)) : c * stride;
            }
            stride *= a.nc[k];
        }
    }
    int count = 0;
    int stencil = 1;
#pragma unroll
    for (int k = 0; k < D; ++k) stencil *= 3;
    for (int s = 0; s < stencil; ++s) {
        int key = 0;
        int rem = s;
#pragma unroll
        for (int k = D - 1; k >= 0; --k) {
            const int d = rem % 3;
            rem /= 3;
            key += d == 0 ? part[k][0] : (d == 1 ? part[k][1] : part[k][2]);
        }
        const int lo = __ldg(a.bin_start + key), hi = __ldg(a.bin_start + key + 1);
        for (int t = lo; t < hi; ++t) {
            const int j = a.src_of ? __ldg(a.src_of + t) : t;
            if (a.half ? !dp_owns_pair(i, j) : j == i) continue;
            // float32 pre-test on the fixed-point displacement (nearest image,
            // never longer than the single-shift one); float64 only near the cutoff
            uint32_t uj[D];
            dp_shadow_unpack<D>(__ldg(sh + j), uj);
            float df[D];
            const float qf = dp_shadow_q<D>(ui, uj, a.unit, df);
            if (qf > a.hi2) continue;
            bool inside = qf < a.lo2 && !far;
            if (!inside) {
                double d[D];
#pragma unroll
                for (int k = 0; k < D; ++k) d[k] = dp_min_image(xi[k] - a.pos[k * n + j], a.box[k]);
                inside = sqrt(dp_sqsum_exact<D>(d)) < a.cutoff;
            }
            if (inside) {
                if (count < a.kcap) a.nl[(long long)count * n + i] = j;
                ++count;
            }
        }
    }
    a.cnt[i] = min(count, a.kcap);
    atomicMax(&a.st->max_neighbors, count);
#pragma unroll
    for (int k = 0; k < D; ++k) a.pos_ref[k * n + i] = xi[k];
    ((sh_t*)a.shadow_ref)[i] = shi;
}

// All-pairs build for boxes with fewer than 3 cells per axis; rows come out in
// ascending index order, exactly the reference's double loop. As in the cell
// build, the float32 shadow test decides every pair outside its error bracket
// and float64 (the reference's test) only the rest.
template <int D>
__global__ void __launch_bounds__(kBlock) k_nl_build_allpairs(NlArgs a) {
    if (!a.st->need_rebuild) return;
    typedef typename dp_shadow_t<D>::type sh_t;
    __shared__ double tile[D][kBlock];
    __shared__ sh_t tsh[kBlock];
    const long long n = a.n;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    const bool far = a.st->far != 0;
    const sh_t* sh = (const sh_t*)a.shadow;
    double xi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) xi[k] = active ? a.pos[k * n + i] : 0.0;
    uint32_t ui[D];
    dp_shadow_unpack<D>(active ? sh[i] : sh_t{}, ui);
    int count = 0;
    for (long long base = 0; base < n; base += kBlock) {
        const long long jl = base + threadIdx.x;
#pragma unroll
        for (int k = 0; k < D; ++k) tile[k][threadIdx.x] = (jl < n) ? a.pos[k * n + jl] : 0.0;
        tsh[threadIdx.x] = (jl < n) ? sh[jl] : sh_t{};
        __syncthreads();
        if (active) {
            const int lim = (int)min((long long)kBlock, n - base);
            for (int t = 0; t < lim; ++t) {
                const long long j = base + t;
                if (a.half ? !dp_owns_pair(i, j) : j == i) continue;
                uint32_t uj[D];
                dp_shadow_unpack<D>(tsh[t], uj);
                float df[D];
                const float qf = dp_shadow_q<D>(ui, uj, a.unit, df);
                if (qf > a.hi2) continue;
                bool inside = qf < a.lo2 && !far;
                if (!inside) {
                    double d[D];
#pragma unroll
                    for (int k = 0; k < D; ++k) d[k] = dp_min_image(xi[k] - tile[k][t], a.box[k]);
                    inside = sqrt(dp_sqsum_exact<D>(d)) < a.cutoff;
                }
                if (inside) {
                    if (count < a.kcap) a.nl[(long long)count * n + i] = (int32_t)j;
                    ++count;
                }
            }
        }
        __syncthreads();
    }
    if (!active) return;
    a.cnt[i] = min(count, a.kcap);
    atomicMax(&a.st->max_neighbors, count);
#pragma unroll
    for (int k = 0; k < D; ++k) a.pos_ref[k * n + i] = xi[k];
    ((sh_t*)a.shadow_ref)[i] = sh[i];
}

// Self-test of the bounded device-side waits, without a GPU fault: one CTA
// allocates tensor memory as the surrogate pass does, waits on an mbarrier
// that nothing arrives at, gives up after `limit` tries, frees the tensor
// memory and records device_error (the host then reports DP_ERR_TIMEOUT).
__global__ void __launch_bounds__(128) k_selftest_bounded_wait(dp_dev_status* st, int limit) {
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t s_tmem;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) dp_mbar_init(&mbar, 1);
    if (warp == 0) dp_tmem_alloc(&s_tmem, 64);
    dp_tc_fence_before();
    __syncthreads();
    dp_tc_fence_after();
    const bool arrived = dp_mbar_wait(&mbar, 0u, limit);
    if (!arrived && threadIdx.x == 0) atomicExch(&st->device_error, 1);
    dp_tc_fence_before();
    __syncthreads();
    if (warp == 0) dp_tmem_dealloc(s_tmem, 64);
}

__global__ void k_rebuild_done(dp_dev_status* st) {
    if (st->need_rebuild) {
        st->need_rebuild = 0;
        st->rebuilds += 1;
        st->ref_far = st->far;  // the list's reference positions are the current ones
    }
}

__global__ void k_set_rebuild(dp_dev_status* st) { st->need_rebuild = 1; }

// Condition of the graph's rebuild node: the sequence runs only when some
// particle moved more than skin/2 (or a rebuild was requested).
// reset_far: the previous (fused) step wrapped every position.
__global__ void k_rebuild_cond(dp_dev_status* st, cudaGraphConditionalHandle h, int reset_far) {
    if (reset_far) st->far = 0;
    cudaGraphSetConditional(h, st->need_rebuild ? 1u : 0u);
}


// End of a graph of steps; clear_far: its last (fused) step wrapped every position.
__global__ void k_advance_step(dp_dev_status* st, long long steps, int clear_far) {
    st->step += steps;
    if (clear_far) st->far = 0;
}

// Rows of the column-major list (in slots) -> row-major (N, kout) by particle
// id, entries as particle ids, each row sorted ascending and -1 padded
// (dompap's neighbor_list layout).
__global__ void k_nl_export(const int32_t* __restrict__ nl, const int32_t* __restrict__ cnt, int32_t* out,
                            const int32_t* __restrict__ order, const int32_t* __restrict__ slot_of, long long n,
                            int kout) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long r = slot_of[i];
    const int c = cnt[r];
    int32_t* row = out + i * kout;
    int m = 0;  // entries kept so far (<= kout), the kout smallest in ascending order
    for (int k = 0; k < c; ++k) {
        const int32_t v = order[nl[(long long)k * n + r]];
        int u;
        if (m < kout) {
            u = m - 1;
            ++m;
        } else if (v < row[kout - 1]) {
            u = kout - 2;
        } else {
            continue;
        }
        while (u >= 0 && row[u] > v) {
            row[u + 1] = row[u];
            --u;
        }
        row[u + 1] = v;
    }
    for (int k = m; k < kout; ++k) row[k] = -1;
}

// A half list (each pair in the row of the particle that owns it,
// dp_owns_pair) closed into the full one: row i gets its own entries and i
// from every row j that holds it. The distance test is
// symmetric (the min-image displacement of j - i is the negated one of i - j
// and the sum of squares is the same), so the closure is the list a full
// build at the same reference positions makes. Count pass, then scatter into
// an unsorted column-major list that k_nl_export sorts.
__global__ void k_nl_half_count(const int32_t* __restrict__ nl, const int32_t* __restrict__ cnt, int32_t* fcnt,
                                int32_t* fmax, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) atomicAdd(fcnt + nl[(long long)k * n + i], 1);
    const int mine = atomicAdd(fcnt + i, c) + c;
    atomicMax(fmax, mine);
}

__global__ void k_nl_half_scatter(const int32_t* __restrict__ nl, const int32_t* __restrict__ cnt, int32_t* fill,
                                  int32_t* full, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) {
        const int32_t j = nl[(long long)k * n + i];
        full[(long long)atomicAdd(fill + i, 1) * n + i] = j;
        full[(long long)atomicAdd(fill + j, 1) * n + j] = (int32_t)i;
    }
}

// --------------------------- integrators ----------------------------------
// Mass handling: MASSMODE 0 one mass for all particles (coefficients as
// arguments), 1 per-particle class index into a coefficient table, 2
// per-particle masses (coefficients computed in the kernel).
// The per-particle step is dp_integrate_one (dp_integrate.cuh). This kernel
// integrates in place after a separate force kernel (the surrogate mode, and
// the timing of the integrator alone); the other modes fuse it into the pair
// kernel.
template <int D, int MASSMODE, bool NVE, bool WRITE64>
__global__ void __launch_bounds__(kBlock) k_integrate(dp_int_args a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->far = 0;  // every position is wrapped below
    bool old = false, bad = false;
    if (i < a.n) {
        double F[D];
#pragma unroll
        for (int k = 0; k < D; ++k) F[k] = a.force[k * a.n + i];
        old = dp_integrate_one<D, MASSMODE, NVE, WRITE64>(a, i, F, bad);
    }
    const bool any_old = __any_sync(0xffffffffu, old);
    const bool any_bad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (any_old) atomicExch(&a.st->need_rebuild, 1);
        if (any_bad) atomicExch(&a.st->nonfinite, 1);
    }
}

// sum_n m_n |v_n|^2, per-block partials.
template <int D, int MASSMODE>
__global__ void __launch_bounds__(kBlock) k_sum_mv2(dp_int_args a, const double* class_mass, double* partial) {
    __shared__ double smem[32];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < a.n) {
        double m;
        if (MASSMODE == 0) m = class_mass[0];
        else if (MASSMODE == 1) m = class_mass[a.mclass[i]];
        else m = a.mass[i];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double vk = a.vel[k * a.n + i];
            s += vk * vk;
        }
        v = m * s;
    }
    v = dp_block_sum(v, smem);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

// Fixed-order sum of per-block partials (one block): deterministic totals.
__global__ void __launch_bounds__(1024) k_reduce(const double* __restrict__ partial, long long m, double* out) {
    __shared__ double smem[32];
    double v = 0.0;
    for (long long t = threadIdx.x; t < m; t += blockDim.x) v += partial[t];
    v = dp_block_sum(v, smem);
    if (threadIdx.x == 0) out[0] = v;
}

template <int D>
__global__ void k_normals(unsigned long long seed, long long step, double* out, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float z[4];
    dp_normals4(seed, (unsigned long long)step, (uint32_t)i, z);
#pragma unroll
    for (int k = 0; k < D; ++k) out[i * D + k] = (double)z[k];
}

// wrap_into_box on demand (dompap/positions.py:90-98), with the shadow update.
template <int D>
__global__ void k_wrap(dp_int_args a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->far = 0;
    if (i >= a.n) return;
    uint32_t u[D];
    unsigned long long X[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const long long o = k * a.n + i;
        int32_t im = a.img[o];
        const int32_t im0 = im;
        const double x = dp_wrap_axis(a.pos[o], a.box[k], im);
        a.pos_out[o] = x;
        if (im != im0) a.img[o] = im;
        X[k] = fixed64_wrapped(x, a.box[k], a.scale64[k]);
        u[k] = (uint32_t)(X[k] >> 32);
    }
    ((typename dp_shadow_t<D>::type*)a.shadow_out)[i] = dp_shadow_pack<D>(u);
    ((typename dp_fixed64_t<D>::type*)a.pos64_out)[i] = dp_fixed64_pack<D>(X);
}

// Pair-distance histogram for g(r) (dompap/positions.py:58-87): all ordered
// pairs (i in A, j in B, self pairs included), np.round minimum image,
// np.histogram bins (half-open, the last one closed). The distance comes from
// the fixed-point shadow in float32; within 1e-5 of a bin edge it is
// recomputed in float64 exactly as NumPy does.
struct RdfArgs {
    const double* pos;
    const void* shadow;
    const int32_t* types;
    const double* edges;
    unsigned long long* counts;
    long long n;
    int nbins;
    int type_a, type_b;  // -1: all particles
    double box[DP_MAX_DIM];
    float unit[DP_MAX_DIM];
};

template <int D>
__device__ __forceinline__ int rdf_bin(double r, const double* e, int nb) {
    if (!(r >= e[0]) || !(r <= e[nb])) return -1;
    if (r == e[nb]) return nb - 1;
    int lo = 0, hi = nb;  // e[lo] <= r < e[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (r >= e[mid]) lo = mid; else hi = mid;
    }
    return lo;
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_rdf(RdfArgs a) {
    extern __shared__ unsigned char smem_raw[];
    double* edges = (double*)smem_raw;
    unsigned int* hist = (unsigned int*)(edges + a.nbins + 1);
    for (int t = threadIdx.x; t <= a.nbins; t += blockDim.x) edges[t] = a.edges[t];
    for (int t = threadIdx.x; t < a.nbins; t += blockDim.x) hist[t] = 0u;
    __syncthreads();
    typedef typename dp_shadow_t<D>::type sh_t;
    const sh_t* sh = (const sh_t*)a.shadow;
    const long long total = a.n * a.n;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        const long long i = p / a.n, j = p - (p / a.n) * a.n;
        if (a.type_a >= 0 && a.types[i] != a.type_a) continue;
        if (a.type_b >= 0 && a.types[j] != a.type_b) continue;
        uint32_t ui[D], uj[D];
        dp_shadow_unpack<D>(sh[i], ui);
        dp_shadow_unpack<D>(sh[j], uj);
        float df[D];
        const float rf = sqrtf(dp_shadow_q<D>(ui, uj, a.unit, df));
        int b = rdf_bin<D>((double)rf, edges, a.nbins);
        bool near_edge = false;
        const double tol = 1e-5 * (double)rf + 1e-9;
        if (b >= 0) {
            near_edge = ((double)rf - edges[b] < tol) || (edges[b + 1] - (double)rf < tol);
        } else {
            near_edge = fabs((double)rf - edges[0]) < tol || fabs((double)rf - edges[a.nbins]) < tol;
        }
        if (near_edge) {
            double q = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const double L = a.box[k];
                double d = a.pos[k * a.n + i] - a.pos[k * a.n + j];
                d -= L * rint(d / L);
                q = (k == 0) ? __dmul_rn(d, d) : __dadd_rn(q, __dmul_rn(d, d));
            }
            b = rdf_bin<D>(sqrt(q), edges, a.nbins);
        }
        if (b >= 0) atomicAdd(hist + b, 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < a.nbins; t += blockDim.x)
        if (hist[t]) atomicAdd(a.counts + t, (unsigned long long)hist[t]);
}

}  // namespace

// ===========================================================================
// allocation-free kinetic sum (see dp_sum_mv2_noalloc in dompap_gpu.h)
// ===========================================================================
// Scratch for the per-block partial sums, one double per block of kBlock
// particles: 16384 blocks = 128 KiB, i.e. at most 4,194,304 particles per
// call. It lives in every GPU that loads this library until the process
// exits. Every call shares it and overwrites exactly the partials it reads,
// so nothing carries over between calls; calls that overlap on the GPU (two
// streams at once) race on it.
#define DP_NOALLOC_MAX_BLOCKS 16384
static __device__ __align__(256) double g_noalloc_partial[DP_NOALLOC_MAX_BLOCKS];

namespace {
__global__ void __launch_bounds__(kBlock) k_mv2_rowmajor(const double* __restrict__ vel,
                                                          const double* __restrict__ mass, long long n, int dim,
                                                          double* __restrict__ partial) {
    __shared__ double smem[32];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        double s = 0.0;
        for (int k = 0; k < dim; ++k) {
            const double vk = vel[i * dim + k];
            s += vk * vk;
        }
        v = mass[i] * s;
    }
    v = dp_block_sum(v, smem);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
}
}  // namespace

// Device address of g_noalloc_partial, looked up once per device (host code
// cannot use the symbol itself: on the host it only names a stand-in). The
// cached address belongs to the device's primary context; cudaDeviceReset
// ends that context, and the header tells callers not to call again after it.
static std::mutex g_noalloc_mutex;
static double* g_noalloc_addr[64] = {nullptr};

// ===========================================================================
// NVRTC pair-kernel libraries
// ===========================================================================
struct PairLib {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t forces = nullptr, energy = nullptr, virial = nullptr, laplacian = nullptr, eval = nullptr;
    cudaKernel_t step = nullptr;  // fused forces + integrate (not in the surrogate program)
    cudaKernel_t step_warp = nullptr;  // the same, one warp per particle (small systems)
    cudaKernel_t step_quad = nullptr;  // the same, four lanes per particle
    // no neighbour list (dompap's double-loop methods): fused step, forces, energy
    cudaKernel_t step_all = nullptr, forces_all = nullptr, energy_all = nullptr;
    cudaKernel_t batch[4] = {nullptr, nullptr, nullptr, nullptr};  // 128, 256, 512, 1024 threads
    cudaKernel_t forces_mlp = nullptr, energy_mlp = nullptr, virial_mlp = nullptr, mlp_finish = nullptr;
    cudaKernel_t forces_mlp_tc = nullptr, energy_mlp_tc = nullptr, virial_mlp_tc = nullptr;  // tcgen05
};

static std::mutex g_lib_mutex;
static std::unordered_map<std::string, PairLib> g_libs;

// --------------------------- on-disk cubin cache ------------------------
// A pair program takes seconds to compile; its CUBIN is kept on disk under a
// key of the program text and the NVRTC version, in DOMPAP_NVRTC_CACHE (empty
// or "0": off) or else in _build/nvrtc_cache beside the library. A file holds
// the program text it was compiled from and is used only when that text
// matches exactly; unreadable or foreign files are ignored and rewritten.
static std::string cubin_cache_dir(bool explicit_only) {
    if (const char* env = std::getenv("DOMPAP_NVRTC_CACHE")) {
        if (!*env || std::strcmp(env, "0") == 0) return "";
        return env;
    }
    if (explicit_only) return "";
    Dl_info info;
    if (dladdr((void*)&cubin_cache_dir, &info) && info.dli_fname) {
        const std::string lib = info.dli_fname;
        const size_t k = lib.rfind('/');
        if (k != std::string::npos) return lib.substr(0, k) + "/_build/nvrtc_cache";
    }
    return "";
}

static std::string cubin_cache_path(const std::string& dir, const std::string& src) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a
    auto mix = [&h](const void* data, size_t len) {
        const unsigned char* b = (const unsigned char*)data;
        for (size_t i = 0; i < len; ++i) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    mix(src.data(), src.size());
    int major = 0, minor = 0;
    nvrtcVersion(&major, &minor);
    mix(&major, sizeof(major));
    mix(&minor, sizeof(minor));
    char name[64];
    snprintf(name, sizeof(name), "/%016llx.dpcubin", (unsigned long long)h);
    return dir + name;
}

static const char kCacheMagic[8] = {'D', 'P', 'C', 'U', 'B', 'I', 'N', '1'};

static bool cubin_cache_read(const std::string& path, const std::string& src, std::vector<char>* cubin) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    bool ok = false;
    char magic[8];
    uint64_t src_len = 0, bin_len = 0;
    if (std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCacheMagic, 8) == 0 &&
        std::fread(&src_len, sizeof(src_len), 1, f) == 1 && src_len == src.size()) {
        std::string text(src_len, '\0');
        if (std::fread(&text[0], 1, src_len, f) == src_len && text == src &&
            std::fread(&bin_len, sizeof(bin_len), 1, f) == 1 && bin_len > 0 && bin_len < (1ull << 30)) {
            cubin->resize(bin_len);
            ok = std::fread(cubin->data(), 1, bin_len, f) == bin_len;
        }
    }
    std::fclose(f);
    return ok;
}

static void cubin_cache_write(const std::string& dir, const std::string& path, const std::string& src,
                              const std::vector<char>& cubin) {
    // create the directory and its parent (the library's _build) if needed
    const size_t k = dir.rfind('/');
    if (k != std::string::npos && k > 0) mkdir(dir.substr(0, k).c_str(), 0755);
    mkdir(dir.c_str(), 0755);
    const std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    const uint64_t src_len = src.size(), bin_len = cubin.size();
    bool ok = std::fwrite(kCacheMagic, 1, 8, f) == 8 && std::fwrite(&src_len, sizeof(src_len), 1, f) == 1 &&
              std::fwrite(src.data(), 1, src_len, f) == src_len && std::fwrite(&bin_len, sizeof(bin_len), 1, f) == 1 &&
              std::fwrite(cubin.data(), 1, bin_len, f) == bin_len;
    ok = (std::fclose(f) == 0) && ok;
    if (ok)
        std::rename(tmp.c_str(), path.c_str());  // atomic: readers see a whole file or none
    else
        std::remove(tmp.c_str());
}

// NVRTC: program text -> sm_103a CUBIN (host only; no GPU needed).
// resource_log (optional): compile with the assembler's verbose report
// (registers, spill bytes, shared memory per kernel) and return that log.
static int nvrtc_compile(const std::string& src, std::vector<char>* cubin, std::string* resource_log);

// cache: use the on-disk cubin cache (explicit_only: only when
// DOMPAP_NVRTC_CACHE names a directory).
static int nvrtc_cubin(const std::string& src, std::vector<char>* cubin, std::string* resource_log = nullptr,
                       bool cache = false, bool explicit_only = false) {
    const std::string dir = cache && !resource_log ? cubin_cache_dir(explicit_only) : std::string();
    if (!dir.empty()) {
        const std::string path = cubin_cache_path(dir, src);
        if (cubin_cache_read(path, src, cubin)) return DP_OK;
        RET(nvrtc_compile(src, cubin, nullptr));
        cubin_cache_write(dir, path, src, *cubin);
        return DP_OK;
    }
    return nvrtc_compile(src, cubin, resource_log);
}

static int nvrtc_compile(const std::string& src, std::vector<char>* cubin, std::string* resource_log) {
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "dompap_pair.cu", 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) return fail(DP_ERR_NVRTC, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "--fmad=true",
                          "-DDP_NVRTC=1", "--ptxas-options=-v"};
    const int nopt = (int)(sizeof(opts) / sizeof(opts[0])) - (resource_log ? 0 : 1);
    r = nvrtcCompileProgram(prog, nopt, opts);
    if (r != NVRTC_SUCCESS) {
        size_t log_size = 0;
        nvrtcGetProgramLogSize(prog, &log_size);
        std::string log(log_size, '\0');
        if (log_size) nvrtcGetProgramLog(prog, &log[0]);
        nvrtcDestroyProgram(&prog);
        return fail(DP_ERR_NVRTC, std::string("NVRTC compile of the pair potential failed: ") + log);
    }
    if (resource_log) {
        size_t log_size = 0;
        nvrtcGetProgramLogSize(prog, &log_size);
        resource_log->assign(log_size, '\0');
        if (log_size) nvrtcGetProgramLog(prog, &(*resource_log)[0]);
    }
    size_t cubin_size = 0;
    nvrtcGetCUBINSize(prog, &cubin_size);
    cubin->resize(cubin_size);
    nvrtcGetCUBIN(prog, cubin->data());
    nvrtcDestroyProgram(&prog);
    return DP_OK;
}

static int compile_pair_lib(const std::string& src, PairLib* out) {
    std::lock_guard<std::mutex> lock(g_lib_mutex);
    auto it = g_libs.find(src);
    if (it != g_libs.end()) {
        *out = it->second;
        return DP_OK;
    }
    std::vector<char> cubin;
    RET(nvrtc_cubin(src, &cubin, nullptr, true));
    PairLib pl;
    CK(cudaLibraryLoadData(&pl.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    CK(cudaLibraryGetKernel(&pl.forces, pl.lib, "dp_forces"));
    CK(cudaLibraryGetKernel(&pl.energy, pl.lib, "dp_energy"));
    CK(cudaLibraryGetKernel(&pl.virial, pl.lib, "dp_virial"));
    CK(cudaLibraryGetKernel(&pl.laplacian, pl.lib, "dp_laplacian"));
    CK(cudaLibraryGetKernel(&pl.eval, pl.lib, "dp_eval_pair"));
    if (src.find("#define DP_MLP 1") == std::string::npos) {
        CK(cudaLibraryGetKernel(&pl.step, pl.lib, "dp_step"));
        CK(cudaLibraryGetKernel(&pl.step_warp, pl.lib, "dp_step_warp"));
        CK(cudaLibraryGetKernel(&pl.step_quad, pl.lib, "dp_step_quad"));
        CK(cudaLibraryGetKernel(&pl.step_all, pl.lib, "dp_step_all"));
        CK(cudaLibraryGetKernel(&pl.forces_all, pl.lib, "dp_forces_all"));
        CK(cudaLibraryGetKernel(&pl.energy_all, pl.lib, "dp_energy_all"));
    }
    if (src.find("#define DP_MLP 1") != std::string::npos) {
        CK(cudaLibraryGetKernel(&pl.forces_mlp, pl.lib, "dp_forces_mlp"));
        CK(cudaLibraryGetKernel(&pl.mlp_finish, pl.lib, "dp_mlp_forces_finish"));
        CK(cudaLibraryGetKernel(&pl.forces_mlp_tc, pl.lib, "dp_forces_mlp_tc"));
        CK(cudaLibraryGetKernel(&pl.energy_mlp_tc, pl.lib, "dp_energy_mlp_tc"));
        CK(cudaLibraryGetKernel(&pl.virial_mlp_tc, pl.lib, "dp_virial_mlp_tc"));
        CK(cudaLibraryGetKernel(&pl.energy_mlp, pl.lib, "dp_energy_mlp"));
        CK(cudaLibraryGetKernel(&pl.virial_mlp, pl.lib, "dp_virial_mlp"));
    }
    if (src.find("dp_batch_steps_128") != std::string::npos) {
        CK(cudaLibraryGetKernel(&pl.batch[0], pl.lib, "dp_batch_steps_128"));
        CK(cudaLibraryGetKernel(&pl.batch[1], pl.lib, "dp_batch_steps_256"));
        CK(cudaLibraryGetKernel(&pl.batch[2], pl.lib, "dp_batch_steps_512"));
        CK(cudaLibraryGetKernel(&pl.batch[3], pl.lib, "dp_batch_steps_1024"));
    }
    g_libs.emplace(src, pl);
    *out = pl;
    return DP_OK;
}

// ===========================================================================
// handle
// ===========================================================================
struct GraphEntry {
    long long steps;
    int kind;
    unsigned long long version;
    cudaGraphExec_t exec;
    long long launches;          // launched every time the graph runs
    long long rebuild_launches;  // launched per executed rebuild node (0: gated kernels, counted above)
    bool fused = false;          // dp_step graph: each step moves the positions to the other buffer set
    const double* pos_key = nullptr;  // current position buffer when the graph was captured
};

struct dp_sim {
    int dim = 3;
    long long n = 0;
    int precision = DP_PREC_FP64;
    cudaStream_t stream = nullptr;
    cudaStream_t cstream = nullptr;  // captures the bodies of conditional graph nodes
    bool conditional_graphs = true;  // cleared if the CUDA driver rejects conditional nodes
    bool fused_step = true;          // run() uses dp_step (DOMPAP_FUSED_STEP=0: separate kernels)
    // up to warp_step_max particles the fused step runs one warp per particle
    // (dp_step_warp), up to quad_step_max four lanes per particle
    // (dp_step_quad); DOMPAP_WARP_STEP / DOMPAP_QUAD_STEP set them (0: never)
    long long warp_step_max = 8192;
    long long quad_step_max = 65536;
    // launch shape set by the autotuner (dp_set_step_launch): lanes per
    // particle of the fused step (0: the size thresholds above) and resident
    // CTAs per SM it is compiled for (0: the measured default per mode)
    int step_lanes = 0;
    int step_blocks = 0;
    // force and energy methods (dompap's method strings): DP_METHOD_LIST or
    // the all-pairs kernels (DP_METHOD_ALLPAIRS; DP_METHOD_ALLPAIRS_NEWTON for
    // forces: parameters of each pair by (min, max) id). Not in the surrogate
    // mode, whose kernels are list kernels.
    int force_method = DP_METHOD_LIST;
    int energy_method = DP_METHOD_LIST;
    // surrogate pass: 0 = tcgen05 from 65,536 particles (the 128-particle CTAs
    // fill the GPU; on par with mma.sync there), mma.sync below; 1 = tcgen05;
    // 2 = mma.sync (DOMPAP_MLP_TENSOR=tcgen05 | mma)
    int mlp_tensor = 0;
    // neighbour lists hold only the partners a particle owns (dp_owns_pair)
    // in the surrogate mode (its kernels use each pair once); an export
    // builds a full one for the moment
    bool nl_half = false;         // kind of the list currently built
    // second set of position buffers: a fused step reads pos/shadow/pos64 and
    // writes these, then the two sets change roles
    double* pos_alt = nullptr;
    void* shadow_alt = nullptr;
    void* pos64_alt = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    double *pos = nullptr, *vel = nullptr, *beta = nullptr, *force = nullptr, *pos_ref = nullptr;
    int32_t* img = nullptr;
    void* shadow = nullptr;
    void* shadow_ref = nullptr;
    void* pos64 = nullptr;
    size_t shadow_bytes = 0;
    double *bk_pos = nullptr, *bk_vel = nullptr, *bk_beta = nullptr;
    int32_t* bk_img = nullptr;

    // masses
    int mass_mode = 0;
    std::vector<double> class_mass{1.0};
    uint8_t* mclass = nullptr;
    double* mcoef = nullptr;      // [nclass][5]
    float2* mcoef_f = nullptr;    // [nclass]: float32 b/(2m), sqrt(2 alpha T dt)
    double* class_mass_dev = nullptr;
    double* mass = nullptr;       // per particle (mode 2)

    int32_t* types = nullptr;
    bool have_types = false;
    int min_type = 0, max_type = 0;
    double box[DP_MAX_DIM] = {0, 0, 0, 0};
    bool have_box = false;

    // potential
    bool have_pot = false;
    std::string pot_src;
    double r_cut = 1.0;
    PairLib lib;
    bool lib_valid = false;

    // pair surrogate (DP_PREC_MLP)
    const dp_mlp_dev* mlp_dev = nullptr;
    unsigned long long* mlp_fx = nullptr;  // surrogate mode: fixed-point force sums (zero between launches)

    // pair parameters
    int pmode = DP_PAIR_CONST;
    int ntypes = 1;
    double sigma = 1.0, epsilon = 1.0, sig_max = 1.0;
    double *sig_tab = nullptr, *eps_tab = nullptr, *isig_tab = nullptr;
    float2* ff_tab = nullptr;  // (sigma, 1/sigma, epsilon) double-float triples per type pair

    // neighbour list
    double skin = 1.0;
    int kcap = 512;
    int method = DP_NL_CELL;
    bool use_cells = false;
    double cutoff = 0.0;
    int nc[DP_MAX_DIM] = {0, 0, 0, 0};
    long long ncell = 0;
    int32_t *nl = nullptr, *cnt = nullptr;
    long long nl_alloc = 0;
    // cell binning (counting sort): cell keys, Morton or row-major
    bool morton = false;
    long long nbins = 0, bins_alloc = 0;
    int32_t *bin_cnt = nullptr, *bin_start = nullptr, *bin_part = nullptr;
    int32_t *bin_key = nullptr, *bin_rank = nullptr, *src_of = nullptr;
    // slots: after each cell-list rebuild the per-particle state is stored in
    // cell order; order[slot] = particle id, slot_of[id] = slot
    bool reorder = true;  // DOMPAP_REORDER=0: the state keeps its order, the build reads through src_of
    int32_t *order = nullptr, *slot_of = nullptr;
    // scratch of the permutation (vel, beta, img, order, types, mass classes, masses)
    double *sc_vel = nullptr, *sc_beta = nullptr, *sc_mass = nullptr;
    int32_t *sc_img = nullptr, *sc_order = nullptr, *sc_types = nullptr;
    uint8_t* sc_mclass = nullptr;
    // backup of the permutation-dependent arrays for an overflow replay
    int32_t *bk_order = nullptr, *bk_types = nullptr;
    uint8_t* bk_mclass = nullptr;
    double* bk_mass = nullptr;
    bool nl_config_dirty = true;
    bool nl_built = false;

    // integrator
    double dt = 0.01, temperature = 1.0, tau = 0.1;
    unsigned long long seed = 0;

    dp_dev_status* dstat = nullptr;
    dp_dev_status* hstat = nullptr;  // pinned
    double* partial = nullptr;
    long long partial_alloc = 0;
    double* dsum = nullptr;
    double* hsum = nullptr;  // pinned

    unsigned long long version = 1;
    std::vector<GraphEntry> graphs;
    long long launches_last = 0;
};

// ---------------------------------------------------------------------------
static void free_graphs(dp_sim* s) {
    for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
}

static int dalloc(void** p, size_t bytes) {
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    if (bytes == 0) return DP_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(DP_ERR_CUDA, std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
    }
    return DP_OK;
}

template <typename T>
static int dalloc_t(T** p, size_t count) {
    return dalloc((void**)p, count * sizeof(T));
}

static int ensure_partial(dp_sim* s, long long blocks) {
    if (blocks <= s->partial_alloc) return DP_OK;
    RET(dalloc_t(&s->partial, (size_t)blocks));
    s->partial_alloc = blocks;
    s->version++;
    return DP_OK;
}

static void fill_scale(const dp_sim* s, double* scale, float* unit) {
    for (int k = 0; k < DP_MAX_DIM; ++k) {
        const double L = (k < s->dim) ? s->box[k] : 1.0;
        if (scale) scale[k] = 4294967296.0 / L;
        if (unit) unit[k] = (float)(L / 4294967296.0);
    }
}

// Largest fixed-point unit L / 2^32 over the axes times sqrt(D): the absolute
// error bound (with a factor 4 margin) of a float32 distance from the shadows.
static double shadow_abs_error(const dp_sim* s) {
    double lmax = 0.0;
    for (int k = 0; k < s->dim; ++k) lmax = std::max(lmax, s->box[k]);
    return 4.0 * lmax / 4294967296.0 * std::sqrt((double)s->dim);
}

// float32 squared-distance thresholds bracketing a float64 distance `r`:
// below lo the distance is certainly < r, above hi certainly > r.
static void bracket(const dp_sim* s, double r, float* lo2, float* hi2) {
    const double e = shadow_abs_error(s);
    const double lo = (r - e) * (1.0 - 1e-5);
    const double hi = (r + e) * (1.0 + 1e-5);
    *lo2 = lo > 0.0 ? (float)(lo * lo) * (1.0f - 1e-6f) : -1.0f;
    *hi2 = std::isfinite(hi) ? (float)(hi * hi) * (1.0f + 1e-6f) : INFINITY;
}

static int launch_shadow(dp_sim* s) {
    ShadowArgs a{};
    a.pos = s->pos;
    a.shadow = s->shadow;
    a.pos64 = s->pos64;
    a.st = s->dstat;
    a.n = s->n;
    for (int k = 0; k < DP_MAX_DIM; ++k) a.scale64[k] = 18446744073709551616.0 / ((k < s->dim) ? s->box[k] : 1.0);
    for (int k = 0; k < DP_MAX_DIM; ++k) a.box[k] = (k < s->dim) ? s->box[k] : 1.0;
    CK(cudaMemsetAsync(&s->dstat->far, 0, sizeof(int32_t), s->stream));
    const unsigned g = grid_for(s->n, kBlock);
    switch (s->dim) {
        case 2: k_shadow<2><<<g, kBlock, 0, s->stream>>>(a); break;
        case 3: k_shadow<3><<<g, kBlock, 0, s->stream>>>(a); break;
        default: k_shadow<4><<<g, kBlock, 0, s->stream>>>(a); break;
    }
    CK(cudaGetLastError());
    return DP_OK;
}

// --------------------------- mass classes ---------------------------------
static int upload_mass_coefficients(dp_sim* s) {
    const int nclass = (int)s->class_mass.size();
    std::vector<double> coef((size_t)nclass * 5);
    for (int c = 0; c < nclass; ++c) {
        const double m = s->class_mass[c];
        const double alpha = m / s->tau;
        const double beta_variance = 2 * alpha * s->temperature * s->dt;
        const double numerator = 1.0 - alpha * s->dt / 2.0 / m;
        const double denominator = 1.0 + alpha * s->dt / 2.0 / m;
        const double a = numerator / denominator;
        const double b = 1 / denominator;
        coef[c * 5 + 0] = a;
        coef[c * 5 + 1] = b * s->dt / m;
        coef[c * 5 + 2] = b / 2 / m;
        coef[c * 5 + 3] = std::sqrt(beta_variance);
        coef[c * 5 + 4] = s->dt / m;
    }
    RET(dalloc_t(&s->mcoef, coef.size()));
    CK(cudaMemcpy(s->mcoef, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float2> coef_f((size_t)nclass);
    for (int c = 0; c < nclass; ++c) coef_f[c] = make_float2((float)coef[c * 5 + 2], (float)coef[c * 5 + 3]);
    RET(dalloc_t(&s->mcoef_f, coef_f.size()));
    CK(cudaMemcpy(s->mcoef_f, coef_f.data(), coef_f.size() * sizeof(float2), cudaMemcpyHostToDevice));
    RET(dalloc_t(&s->class_mass_dev, (size_t)nclass));
    CK(cudaMemcpy(s->class_mass_dev, s->class_mass.data(), nclass * sizeof(double), cudaMemcpyHostToDevice));
    s->version++;
    return DP_OK;
}

// --------------------------- neighbour-list configuration -----------------
static int configure_nl(dp_sim* s) {
    if (!s->nl_config_dirty) return DP_OK;
    if (!s->have_box) return fail(DP_ERR_ARG, "box not set");
    const double reach = s->sig_max * s->r_cut;
    s->cutoff = reach + s->skin;  // dompap/Simulation.py:353-356
    bool cells = s->method == DP_NL_CELL && std::isfinite(s->cutoff) && s->cutoff > 0;
    long long ncell = 1;
    int pmax = 1;  // power of two covering the largest cell count
    for (int k = 0; k < s->dim && cells; ++k) {
        // cells strictly wider than the cutoff plus the shadow's rounding
        // (a few L / 2^32): a pair closer than the cutoff is never more than
        // one cell apart when the cells come from the shadows
        const double w = s->cutoff * (1.0 + 1e-10) + 8.0 * s->box[k] / 4294967296.0;
        const double ncd = std::floor(s->box[k] / w);
        if (!(ncd >= 3.0) || ncd > 65536.0) {
            cells = false;
            break;
        }
        s->nc[k] = (int)ncd;
        ncell *= s->nc[k];
        while (pmax < s->nc[k]) pmax <<= 1;
        if (ncell > (1LL << 30)) cells = false;
    }
    s->use_cells = cells;
    if (!cells) {
        for (int k = 0; k < DP_MAX_DIM; ++k) s->nc[k] = 0;
        s->ncell = 0;
        s->nbins = 0;
    } else {
        for (int k = s->dim; k < DP_MAX_DIM; ++k) s->nc[k] = 1;
        s->ncell = ncell;
        // Morton keys on the padded grid while it stays within 2^26 keys and
        // the bit interleaving's width (16 bits per axis in 2-D, 10 in 3-D, 8 in 4-D)
        long long padded = 1;
        for (int k = 0; k < s->dim; ++k) padded *= pmax;
        const int bits_per_axis = s->dim == 2 ? 16 : (s->dim == 3 ? 10 : 8);
        s->morton = padded <= (1LL << 26) && pmax <= (1 << bits_per_axis);
        s->nbins = s->morton ? padded : ncell;
        if (s->nbins > s->bins_alloc) {
            RET(dalloc_t(&s->bin_cnt, (size_t)s->nbins));
            RET(dalloc_t(&s->bin_start, (size_t)s->nbins + 1));
            RET(dalloc_t(&s->bin_part, (size_t)((s->nbins + kScanTile - 1) / kScanTile)));
            s->bins_alloc = s->nbins;
        }
        if (!s->bin_key) {
            const size_t n = (size_t)s->n, nd = n * s->dim;
            RET(dalloc_t(&s->bin_key, n));
            RET(dalloc_t(&s->bin_rank, n));
            RET(dalloc_t(&s->src_of, n));
            RET(dalloc_t(&s->sc_vel, nd));
            RET(dalloc_t(&s->sc_beta, nd));
            RET(dalloc_t(&s->sc_img, nd));
            RET(dalloc_t(&s->sc_order, n));
            RET(dalloc_t(&s->bk_order, n));
        }
    }
    const long long need = (long long)s->kcap * s->n;
    if (need > s->nl_alloc) {
        RET(dalloc_t(&s->nl, (size_t)need));
        s->nl_alloc = need;
    }
    s->nl_config_dirty = false;
    s->nl_built = false;
    s->version++;
    return DP_OK;
}

// Scratch and backup arrays of the optional per-particle arrays (types, mass
// classes, masses), allocated once those exist.
static int ensure_perm_extras(dp_sim* s) {
    const size_t n = (size_t)s->n;
    if (s->types && !s->sc_types) {
        RET(dalloc_t(&s->sc_types, n));
        RET(dalloc_t(&s->bk_types, n));
    }
    if (s->mclass && !s->sc_mclass) {
        RET(dalloc_t(&s->sc_mclass, n));
        RET(dalloc_t(&s->bk_mclass, n));
    }
    if (s->mass && !s->sc_mass) {
        RET(dalloc_t(&s->sc_mass, n));
        RET(dalloc_t(&s->bk_mass, n));
    }
    return DP_OK;
}

// The state arrays that move with their particle, with their scratch: the
// positions use the second position set (free during a rebuild: a fused step
// writes it after the rebuild, the separate integrator does not use it).
static void fill_perm_args(const dp_sim* s, PermArgs& p) {
    memset(&p, 0, sizeof(p));
    const int sh = s->dim == 2 ? 8 : 16;
    const int p64 = s->dim == 2 ? 16 : 32;
    auto add = [&](void* data, void* scratch, int esize, int comps) {
        if (data && scratch) p.arr[p.count++] = PermArray{data, scratch, esize, comps};
    };
    add(s->pos, s->pos_alt, 8, s->dim);
    add(s->shadow, s->shadow_alt, sh, 1);
    add(s->pos64, s->pos64_alt, p64, 1);
    add(s->vel, s->sc_vel, 8, s->dim);
    add(s->beta, s->sc_beta, 8, s->dim);
    add(s->img, s->sc_img, 4, s->dim);
    add(s->order, s->sc_order, 4, 1);
    add(s->types, s->sc_types, 4, 1);
    add(s->mclass, s->sc_mclass, 1, 1);
    add(s->mass, s->sc_mass, 8, 1);
    p.src_of = s->src_of;
    p.order = s->order;
    p.slot_of = s->slot_of;
    p.st = s->dstat;
    p.n = s->n;
}

// The gated rebuild sequence (no effect unless need_rebuild is set).
// The surrogate mode uses each pair once: its lists hold only the partners a particle owns (dp_owns_pair).
static bool list_half(const dp_sim* s) { return s->precision == DP_PREC_MLP; }

static int launch_rebuild(dp_sim* s, long long* launches) {
    const unsigned gp = grid_for(s->n, kBlock);
    NlArgs na{};
    na.half = list_half(s) ? 1 : 0;
    na.pos = s->pos;
    na.pos_ref = s->pos_ref;
    na.shadow = s->shadow;
    na.shadow_ref = s->shadow_ref;
    na.nl = s->nl;
    na.cnt = s->cnt;
    na.st = s->dstat;
    na.n = s->n;
    na.kcap = s->kcap;
    na.cutoff = s->cutoff;
    bracket(s, s->cutoff, &na.lo2, &na.hi2);
    fill_scale(s, nullptr, na.unit);
    for (int k = 0; k < DP_MAX_DIM; ++k) na.box[k] = (k < s->dim) ? s->box[k] : 1.0;
    long long nl_launches = 0;
    if (s->use_cells) {
        // counting sort of the slots by cell key
        BinArgs ba{};
        ba.shadow = s->shadow;
        ba.order = s->order;
        ba.key = s->bin_key;
        ba.rank = s->bin_rank;
        ba.bin_cnt = s->bin_cnt;
        ba.bin_start = s->bin_start;
        ba.bin_part = s->bin_part;
        ba.src_of = s->src_of;
        ba.st = s->dstat;
        ba.n = s->n;
        ba.nbins = s->nbins;
        ba.morton = s->morton ? 1 : 0;
        for (int k = 0; k < DP_MAX_DIM; ++k) ba.nc[k] = s->nc[k];
        const int parts = (int)((s->nbins + kScanTile - 1) / kScanTile);
        k_bin_clear<<<(unsigned)std::min<long long>(grid_for(s->nbins, kBlock), 8192), kBlock, 0, s->stream>>>(ba);
        switch (s->dim) {
            case 2: k_bin_count<2><<<gp, kBlock, 0, s->stream>>>(ba); break;
            case 3: k_bin_count<3><<<gp, kBlock, 0, s->stream>>>(ba); break;
            default: k_bin_count<4><<<gp, kBlock, 0, s->stream>>>(ba); break;
        }
        k_scan_reduce<<<parts, kScanThreads, 0, s->stream>>>(ba);
        k_scan_top<<<1, kScanThreads, 0, s->stream>>>(ba, parts);
        k_scan_down<<<parts, kScanThreads, 0, s->stream>>>(ba);
        k_bin_scatter<<<gp, kBlock, 0, s->stream>>>(ba);
        k_bin_sort<<<grid_for(s->nbins, kBlock), kBlock, 0, s->stream>>>(ba);
        nl_launches = 7;
        if (s->reorder) {
            // the state into cell order: slot t <- slot src_of[t]
            PermArgs pa;
            fill_perm_args(s, pa);
            const dim3 gpa(gp, (unsigned)pa.count);
            k_permute<<<gpa, kBlock, 0, s->stream>>>(pa);
            k_permute_back<<<gpa, kBlock, 0, s->stream>>>(pa);
            nl_launches += 2;
        }
        na.bin_start = s->bin_start;
        na.src_of = s->reorder ? nullptr : s->src_of;
        na.morton = ba.morton;
        for (int k = 0; k < DP_MAX_DIM; ++k) na.nc[k] = s->nc[k];
        switch (s->dim) {
            case 2: k_nl_build_cells<2><<<gp, kBlock, 0, s->stream>>>(na); break;
            case 3: k_nl_build_cells<3><<<gp, kBlock, 0, s->stream>>>(na); break;
            default: k_nl_build_cells<4><<<gp, kBlock, 0, s->stream>>>(na); break;
        }
        nl_launches += 1;
    } else {
        switch (s->dim) {
            case 2: k_nl_build_allpairs<2><<<gp, kBlock, 0, s->stream>>>(na); break;
            case 3: k_nl_build_allpairs<3><<<gp, kBlock, 0, s->stream>>>(na); break;
            default: k_nl_build_allpairs<4><<<gp, kBlock, 0, s->stream>>>(na); break;
        }
        nl_launches = 1;
    }
    k_rebuild_done<<<1, 1, 0, s->stream>>>(s->dstat);
    CK(cudaGetLastError());
    if (launches) *launches += nl_launches + 1;
    return DP_OK;
}

static void fill_pair_args(const dp_sim* s, dp_pair_args& a, double* out) {
    memset(&a, 0, sizeof(a));
    a.pos = s->pos;
    a.shadow = s->shadow;
    a.nl = s->nl;
    a.cnt = s->cnt;
    a.types = s->types;
    a.sig_tab = s->sig_tab;
    a.eps_tab = s->eps_tab;
    a.isig_tab = s->isig_tab;
    a.ff_tab = s->ff_tab;
    a.pos64 = s->pos64;
    a.order = s->order;
    a.out = out;
    a.partial = s->partial;
    a.status = s->dstat;
    a.n = s->n;
    a.ntypes = s->ntypes;
    for (int k = 0; k < DP_MAX_DIM; ++k) a.box[k] = (k < s->dim) ? s->box[k] : 1.0;
    fill_scale(s, nullptr, a.unit);
    for (int k = 0; k < DP_MAX_DIM; ++k) {
        const double u64 = ((k < s->dim) ? s->box[k] : 1.0) / 18446744073709551616.0;
        a.unit64_hi[k] = (float)u64;
        a.unit64_lo[k] = (float)(u64 - (double)(float)u64);
    }
    a.sigma = s->sigma;
    a.inv_sigma = 1.0 / s->sigma;
    a.epsilon = s->epsilon;
    a.rcut = s->r_cut;
    a.rcut_f = (float)s->r_cut;
    a.rcut_finite = std::isfinite(s->r_cut) ? 1 : 0;
    {
        const double c3[3] = {a.sigma, a.inv_sigma, a.epsilon};
        for (int t = 0; t < 3; ++t) {
            a.ff_const[2 * t] = (float)c3[t];
            a.ff_const[2 * t + 1] = (float)(c3[t] - (double)(float)c3[t]);
        }
    }
    // Pre-filter threshold: a pair is skipped only when its float32 distance,
    // whose error is < 1e-6 relative plus a few L / 2^32, certainly exceeds
    // r_cut * sigma_max.
    double lmax = 0.0;
    for (int k = 0; k < s->dim; ++k) lmax = std::max(lmax, s->box[k]);
    const double reach = s->r_cut * s->sig_max;
    if (std::isfinite(reach)) {
        const double rr = reach * (1.0 + 1e-5) + 8.0 * lmax / 4294967296.0 * std::sqrt((double)s->dim) + 1e-30;
        a.cut2f = (float)(rr * rr * (1.0 + 1e-6));
    } else {
        a.cut2f = INFINITY;
    }
}

static bool use_mlp_tcgen05(const dp_sim* s) {
    return s->mlp_tensor == 1 || (s->mlp_tensor == 0 && s->n >= 65536);
}

// Fixed-point force sums of the surrogate pass (allocated outside any graph
// capture: run() calls this before capturing).
static int ensure_mlp_fx(dp_sim* s) {
    if (s->mlp_fx) return DP_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) return fail(DP_ERR_CUDA, "surrogate force sums not allocated before capture");
    RET(dalloc_t(&s->mlp_fx, (size_t)s->n * s->dim));
    CK(cudaMemsetAsync(s->mlp_fx, 0, (size_t)s->n * s->dim * sizeof(unsigned long long), s->stream));
    return DP_OK;
}

static int launch_pair(dp_sim* s, cudaKernel_t k, double* out, long long* launches) {
    dp_pair_args a;
    fill_pair_args(s, a, out);
    if (s->precision == DP_PREC_MLP) {
        cudaKernel_t km = nullptr;
        if (k == s->lib.forces) km = s->lib.forces_mlp;
        else if (k == s->lib.energy) km = s->lib.energy_mlp;
        else if (k == s->lib.virial) km = s->lib.virial_mlp;
        if (!km) return fail(DP_ERR_ARG, "this quantity is not available with the pair surrogate");
        const dp_mlp_dev* mp = s->mlp_dev;
        unsigned long long* fx = nullptr;
        if (km == s->lib.forces_mlp) {
            RET(ensure_mlp_fx(s));
            fx = s->mlp_fx;
        }
        void* args[] = {&a, &mp, &fx};
        if (use_mlp_tcgen05(s)) {
            // the tcgen05 pass: 128 particles (rows of the tensor-core tile) per CTA
            cudaKernel_t kt = km == s->lib.forces_mlp ? s->lib.forces_mlp_tc
                            : (km == s->lib.energy_mlp ? s->lib.energy_mlp_tc : s->lib.virial_mlp_tc);
            CK(cudaLaunchKernel((const void*)kt, dim3(grid_for(s->n, 128)), dim3(128), args, 0, s->stream));
        } else {
            CK(cudaLaunchKernel((const void*)km, dim3(grid_for(s->n, kBlock)), dim3(kBlock), args, 0, s->stream));
        }
        if (fx) {
            void* fargs[] = {&a, &fx};
            CK(cudaLaunchKernel((const void*)s->lib.mlp_finish, dim3(grid_for(s->n * s->dim, kBlock)), dim3(kBlock),
                                fargs, 0, s->stream));
            if (launches) *launches += 1;
        }
    } else if (k == s->lib.forces && s->force_method != DP_METHOD_LIST && s->lib.forces_all) {
        a.upper = s->force_method == DP_METHOD_ALLPAIRS_NEWTON ? 1 : 0;
        void* args[] = {&a};
        CK(cudaLaunchKernel((const void*)s->lib.forces_all, dim3(grid_for(s->n * 32, kBlock)), dim3(kBlock), args, 0,
                            s->stream));
    } else if (k == s->lib.energy && s->energy_method != DP_METHOD_LIST && s->lib.energy_all) {
        void* args[] = {&a};
        CK(cudaLaunchKernel((const void*)s->lib.energy_all, dim3(grid_for(s->n * 32, kBlock)), dim3(kBlock), args, 0,
                            s->stream));
    } else {
        void* args[] = {&a};
        CK(cudaLaunchKernel((const void*)k, dim3(grid_for(s->n, kBlock)), dim3(kBlock), args, 0, s->stream));
    }
    if (launches) *launches += 1;
    return DP_OK;
}

// Integrator arguments; the outputs default to the current buffers (in place).
static void fill_int_args(const dp_sim* s, dp_int_args& a, long long step_offset, int kind = DP_INT_GJF) {
    memset(&a, 0, sizeof(a));
    a.pos = s->pos;
    a.pos_out = s->pos;
    a.vel = s->vel;
    a.beta = s->beta;
    a.force = s->force;
    a.img = s->img;
    a.shadow_out = s->shadow;
    a.pos64_out = s->pos64;
    a.pos_ref = s->pos_ref;
    a.shadow_ref = s->shadow_ref;
    a.mclass = s->mclass;
    a.mcoef = s->mcoef;
    a.mcoef_f = s->mcoef_f;
    a.mass = s->mass;
    a.order = s->order;
    a.st = s->dstat;
    a.n = s->n;
    for (int k = 0; k < DP_MAX_DIM; ++k) a.box[k] = (k < s->dim) ? s->box[k] : 1.0;
    fill_scale(s, nullptr, a.unit);
    for (int k = 0; k < DP_MAX_DIM; ++k) a.scale64[k] = 18446744073709551616.0 / ((k < s->dim) ? s->box[k] : 1.0);
    a.thr = (0.5 * s->skin) * (0.5 * s->skin);
    bracket(s, 0.5 * s->skin, &a.thr_lo, &a.thr_hi);
    a.dt = s->dt;
    {
        const double m = s->class_mass[0];
        const double alpha = m / s->tau;
        const double beta_variance = 2 * alpha * s->temperature * s->dt;
        const double numerator = 1.0 - alpha * s->dt / 2.0 / m;
        const double denominator = 1.0 + alpha * s->dt / 2.0 / m;
        const double aa = numerator / denominator;
        const double b = 1 / denominator;
        a.coef[0] = aa;
        a.coef[1] = b * s->dt / m;
        a.coef[2] = b / 2 / m;
        a.coef[3] = std::sqrt(beta_variance);
        a.coef[4] = s->dt / m;
        a.coef_f[0] = (float)a.coef[2];
        a.coef_f[1] = (float)a.coef[3];
    }
    a.temperature = s->temperature;
    a.tau = s->tau;
    a.seed = s->seed;
    a.step_offset = step_offset;
    a.massmode = s->mass_mode;
    a.nve = kind == DP_INT_NVE ? 1 : 0;
}

template <int D, bool NVE, bool W64>
static void launch_integrate_dw(dp_sim* s, const dp_int_args& a) {
    const unsigned g = grid_for(s->n, kBlock);
    switch (s->mass_mode) {
        case 0: k_integrate<D, 0, NVE, W64><<<g, kBlock, 0, s->stream>>>(a); break;
        case 1: k_integrate<D, 1, NVE, W64><<<g, kBlock, 0, s->stream>>>(a); break;
        default: k_integrate<D, 2, NVE, W64><<<g, kBlock, 0, s->stream>>>(a); break;
    }
}

// The 64-bit fixed point is only read by the float64-parity pair kernels.
template <int D, bool NVE>
static void launch_integrate_d(dp_sim* s, const dp_int_args& a) {
    if (s->precision == DP_PREC_FP64)
        launch_integrate_dw<D, NVE, true>(s, a);
    else
        launch_integrate_dw<D, NVE, false>(s, a);
}

static int launch_integrate(dp_sim* s, int kind, long long step_offset, long long* launches) {
    dp_int_args a;
    fill_int_args(s, a, step_offset, kind);
    const bool nve = kind == DP_INT_NVE;
    switch (s->dim) {
        case 2: nve ? launch_integrate_d<2, true>(s, a) : launch_integrate_d<2, false>(s, a); break;
        case 3: nve ? launch_integrate_d<3, true>(s, a) : launch_integrate_d<3, false>(s, a); break;
        default: nve ? launch_integrate_d<4, true>(s, a) : launch_integrate_d<4, false>(s, a); break;
    }
    CK(cudaGetLastError());
    if (launches) *launches += 1;
    return DP_OK;
}

static int launch_skin_check(dp_sim* s) {
    SkinArgs a{};
    a.pos = s->pos;
    a.pos_ref = s->pos_ref;
    a.shadow = s->shadow;
    a.shadow_ref = s->shadow_ref;
    a.st = s->dstat;
    a.n = s->n;
    for (int k = 0; k < DP_MAX_DIM; ++k) a.box[k] = (k < s->dim) ? s->box[k] : 1.0;
    fill_scale(s, nullptr, a.unit);
    a.thr = (0.5 * s->skin) * (0.5 * s->skin);
    bracket(s, 0.5 * s->skin, &a.thr_lo, &a.thr_hi);
    const unsigned g = grid_for(s->n, kBlock);
    switch (s->dim) {
        case 2: k_skin_check<2><<<g, kBlock, 0, s->stream>>>(a); break;
        case 3: k_skin_check<3><<<g, kBlock, 0, s->stream>>>(a); break;
        default: k_skin_check<4><<<g, kBlock, 0, s->stream>>>(a); break;
    }
    CK(cudaGetLastError());
    return DP_OK;
}

static int read_status(dp_sim* s) {
    CK(cudaMemcpyAsync(s->hstat, s->dstat, sizeof(dp_dev_status), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

// A bounded device-side wait gave up (the tensor-core surrogate pass): the
// launch's results are invalid; report it and clear the flag.
static int write_status(dp_sim* s);
static int check_device_error(dp_sim* s) {
    if (!s->hstat->device_error) return DP_OK;
    s->hstat->device_error = 0;
    RET(write_status(s));
    return fail(DP_ERR_TIMEOUT, "a bounded device-side wait gave up (tensor-core surrogate pass); the launch's "
                                "results are discarded");
}

static int write_status(dp_sim* s) {
    CK(cudaMemcpyAsync(s->dstat, s->hstat, sizeof(dp_dev_status), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

static int require_ready(dp_sim* s) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (!s->have_box) return fail(DP_ERR_ARG, "box not set");
    if (!s->have_pot || !s->lib_valid) return fail(DP_ERR_NOPOT, "no pair potential set");
    return DP_OK;
}

// Grow capacities after an overflow reported in hstat; returns 1 if grown.
static int grow_after_overflow(dp_sim* s, bool* grown) {
    *grown = false;
    if (s->hstat->max_neighbors > s->kcap) {
        const int want = ((int)(s->hstat->max_neighbors * 1.25) + 32 + 31) & ~31;
        s->kcap = want;
        const long long need = (long long)s->kcap * s->n;
        if (need > s->nl_alloc) {
            RET(dalloc_t(&s->nl, (size_t)need));
            s->nl_alloc = need;
        }
        *grown = true;
    }
    if (*grown) {
        s->version++;
        s->hstat->max_neighbors = 0;
    }
    return DP_OK;
}

// Rebuild now if needed (check) or unconditionally; handles overflow growth.
static int update_nl(dp_sim* s, bool check, int* rebuilt) {
    RET(configure_nl(s));
    if (s->use_cells) RET(ensure_perm_extras(s));
    RET(read_status(s));
    const long long before = s->hstat->rebuilds;
    if (!s->nl_built || !check || s->nl_half != list_half(s)) {
        s->hstat->need_rebuild = 1;
        RET(write_status(s));
    } else {
        RET(launch_skin_check(s));
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        RET(read_status(s));
        const bool was_needed = s->hstat->need_rebuild != 0;
        if (!was_needed) break;
        s->hstat->max_neighbors = 0;
        s->hstat->cell_overflow = 0;
        RET(write_status(s));
        RET(launch_rebuild(s, nullptr));
        RET(read_status(s));
        bool grown = false;
        RET(grow_after_overflow(s, &grown));
        if (!grown) break;
        s->hstat->need_rebuild = 1;
        RET(write_status(s));
    }
    s->nl_built = true;
    s->nl_half = list_half(s);
    if (rebuilt) *rebuilt = (s->hstat->rebuilds != before) ? 1 : 0;
    return DP_OK;
}

// --------------------------- graphs ---------------------------------------
// The rebuild sequence as an IF node of the graph being captured on
// s->stream: a one-thread kernel sets the condition from need_rebuild, and the
// body (captured on s->cstream) runs the cell and list kernels, so steps
// without a rebuild launch none of them.
// h: this step's handle (one per conditional node). With `set_cond` a
// one-thread kernel sets its condition first; otherwise the previous fused
// step's last CTA has set it (dp_step_end).
static int capture_conditional_rebuild(dp_sim* s, cudaGraph_t graph, cudaGraphConditionalHandle h, bool set_cond,
                                       bool reset_far, long long* launches, long long* body_launches) {
    if (set_cond) {
        k_rebuild_cond<<<1, 1, 0, s->stream>>>(s->dstat, h, reset_far ? 1 : 0);
        CK(cudaGetLastError());
        *launches += 1;
    }
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(s->stream, &cs, nullptr, nullptr, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, graph, deps, nullptr, nd, &p));
    CK(cudaStreamUpdateCaptureDependencies(s->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    CK(cudaStreamBeginCaptureToGraph(s->cstream, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                     cudaStreamCaptureModeThreadLocal));
    std::swap(s->stream, s->cstream);
    long long body = 0;
    const int rc = launch_rebuild(s, &body);
    std::swap(s->stream, s->cstream);
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->cstream, &out);
    RET(rc);
    if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("conditional body capture: ") + cudaGetErrorString(e));
    *body_launches = body;
    return DP_OK;
}

static bool use_fused_step(const dp_sim* s) {
    return s->fused_step && s->precision != DP_PREC_MLP && s->lib.step != nullptr;
}

// run() without a neighbour list: the all-pairs fused step
static bool use_allpairs_step(const dp_sim* s) {
    return use_fused_step(s) && s->force_method != DP_METHOD_LIST && s->lib.step_all != nullptr;
}

// The two position buffer sets change roles (host pointers only).
static void swap_position_buffers(dp_sim* s) {
    std::swap(s->pos, s->pos_alt);
    std::swap(s->shadow, s->shadow_alt);
    std::swap(s->pos64, s->pos64_alt);
}

// Fused step: forces from the current buffers, integration into the others.
// end_flags / next_cond: DP_END_* work of the kernel's last CTA (graphs only).
static int launch_step(dp_sim* s, int kind, long long step_offset, long long* launches, int end_flags = 0,
                       cudaGraphConditionalHandle next_cond = 0) {
    dp_pair_args pa;
    fill_pair_args(s, pa, nullptr);
    dp_int_args ia;
    fill_int_args(s, ia, step_offset, kind);
    ia.end_flags = end_flags;
    ia.next_cond = next_cond;
    ia.force = nullptr;
    ia.pos_out = s->pos_alt;
    ia.shadow_out = s->shadow_alt;
    ia.pos64_out = s->pos64_alt;
    void* args[] = {&pa, &ia};
    if (use_allpairs_step(s)) {
        pa.upper = s->force_method == DP_METHOD_ALLPAIRS_NEWTON ? 1 : 0;
        CK(cudaLaunchKernel((const void*)s->lib.step_all, dim3(grid_for(s->n * 32, kBlock)), dim3(kBlock), args, 0,
                            s->stream));
        if (launches) *launches += 1;
        return DP_OK;
    }
    const int lanes = s->step_lanes ? s->step_lanes
                                    : (s->n <= s->warp_step_max ? 32 : (s->n <= s->quad_step_max ? 4 : 1));
    if (lanes == 32 && s->lib.step_warp) {
        // small system: one warp per particle (32 n threads)
        CK(cudaLaunchKernel((const void*)s->lib.step_warp, dim3(grid_for(s->n * 32, kBlock)), dim3(kBlock), args, 0,
                            s->stream));
    } else if (lanes == 4 && s->lib.step_quad) {
        CK(cudaLaunchKernel((const void*)s->lib.step_quad, dim3(grid_for(s->n * 4, kBlock)), dim3(kBlock), args, 0,
                            s->stream));
    } else {
        CK(cudaLaunchKernel((const void*)s->lib.step, dim3(grid_for(s->n, kBlock)), dim3(kBlock), args, 0,
                            s->stream));
    }
    if (launches) *launches += 1;
    return DP_OK;
}

// One chunk of steps into the graph being captured on s->stream; with
// `conditional` the rebuild sequence goes into IF nodes, otherwise the gated
// kernels are launched every step. A fused chunk swaps the host's position
// pointers once per captured step (the caller undoes that until the graph
// has run).
static int record_steps(dp_sim* s, long long steps, int kind, cudaGraph_t graph, bool conditional, bool fused,
                        long long* launches, long long* rebuild_launches) {
    *rebuild_launches = 0;
    const bool no_list = use_allpairs_step(s);
    cudaGraphConditionalHandle h = 0;  // this step's rebuild node
    if (conditional && !no_list) CK(cudaGraphConditionalHandleCreate(&h, graph, 0, 0));
    for (long long t = 0; t < steps; ++t) {
        // after a fused step every position is wrapped and `far` is clear (the
        // step's last CTA clears it); the non-fused kernels clear it in
        // k_integrate, before the next step's list check and pair loop
        if (no_list) {
            // no list to keep: the step reads every particle's position
        } else if (conditional) {
            // the condition of step t > 0 was set by the fused step t - 1
            RET(capture_conditional_rebuild(s, graph, h, !fused || t == 0, false, launches, rebuild_launches));
        } else {
            RET(launch_rebuild(s, launches));
        }
        if (fused) {
            cudaGraphConditionalHandle next = 0;
            int flags = DP_END_CLEAR_FAR;
            if (conditional && !no_list && t + 1 < steps) {
                CK(cudaGraphConditionalHandleCreate(&next, graph, 0, 0));
                flags |= DP_END_SET_COND;
            }
            RET(launch_step(s, kind, t, launches, flags, next));
            swap_position_buffers(s);
            h = next;
        } else {
            RET(launch_pair(s, s->lib.forces, s->force, launches));
            RET(launch_integrate(s, kind, t, launches));
            if (conditional && t + 1 < steps) CK(cudaGraphConditionalHandleCreate(&h, graph, 0, 0));
        }
    }
    k_advance_step<<<1, 1, 0, s->stream>>>(s->dstat, steps, fused && steps > 0 ? 1 : 0);
    CK(cudaGetLastError());
    *launches += 1;
    return DP_OK;
}

// Capture a chunk graph (conditional rebuild nodes when the CUDA driver takes
// them) and instantiate it.
static int build_graph(dp_sim* s, long long steps, int kind, bool conditional, GraphEntry* g) {
    cudaGraph_t graph = nullptr;
    CK(cudaGraphCreate(&graph, 0));
    cudaError_t e = cudaStreamBeginCaptureToGraph(s->stream, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return fail(DP_ERR_CUDA, std::string("cudaStreamBeginCaptureToGraph: ") + cudaGetErrorString(e));
    }
    long long launches = 0, rebuild_launches = 0;
    const bool fused = use_fused_step(s);
    const double* pos_key = s->pos;
    const int rc = record_steps(s, steps, kind, graph, conditional, fused, &launches, &rebuild_launches);
    // the graph has not run yet: put the position pointers back
    while (s->pos != pos_key) swap_position_buffers(s);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(s->stream, &captured);
    if (rc != DP_OK || e != cudaSuccess) {
        cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc != DP_OK ? rc : fail(DP_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    }
    g->steps = steps;
    g->kind = kind;
    g->version = s->version;
    g->launches = launches;
    g->rebuild_launches = rebuild_launches;
    g->fused = fused;
    g->pos_key = pos_key;
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(DP_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    return DP_OK;
}

static int get_graph(dp_sim* s, long long steps, int kind, GraphEntry** out) {
    for (auto& g : s->graphs) {
        if (g.steps == steps && g.kind == kind && g.version == s->version && g.pos_key == s->pos &&
            g.fused == use_fused_step(s)) {
            *out = &g;
            return DP_OK;
        }
    }
    // drop stale graphs
    for (auto it = s->graphs.begin(); it != s->graphs.end();) {
        if (it->version != s->version) {
            cudaGraphExecDestroy(it->exec);
            it = s->graphs.erase(it);
        } else {
            ++it;
        }
    }
    GraphEntry g;
    int rc = DP_ERR_CUDA;
    if (s->conditional_graphs && s->cstream) {
        rc = build_graph(s, steps, kind, true, &g);
        // a driver without conditional nodes: the gated kernels from now on
        if (rc != DP_OK) s->conditional_graphs = false;
    }
    if (rc != DP_OK) RET(build_graph(s, steps, kind, false, &g));
    s->graphs.push_back(g);
    *out = &s->graphs.back();
    return DP_OK;
}

// The state a chunk of steps starts from, for its replay after a list
// overflow. A rebuild inside the chunk may reorder the slots, so the slot
// order and the per-particle parameters it moves are saved with the state.
static int backup_state(dp_sim* s) {
    const size_t n = (size_t)s->n, bd = n * s->dim * sizeof(double), bi = n * s->dim * sizeof(int32_t);
    CK(cudaMemcpyAsync(s->bk_pos, s->pos, bd, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->bk_vel, s->vel, bd, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->bk_beta, s->beta, bd, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->bk_img, s->img, bi, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_order) CK(cudaMemcpyAsync(s->bk_order, s->order, n * 4, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_types && s->types) CK(cudaMemcpyAsync(s->bk_types, s->types, n * 4, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_mclass && s->mclass) CK(cudaMemcpyAsync(s->bk_mclass, s->mclass, n, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_mass && s->mass) CK(cudaMemcpyAsync(s->bk_mass, s->mass, n * 8, cudaMemcpyDeviceToDevice, s->stream));
    return DP_OK;
}

static int restore_state(dp_sim* s) {
    const size_t n = (size_t)s->n, bd = n * s->dim * sizeof(double), bi = n * s->dim * sizeof(int32_t);
    CK(cudaMemcpyAsync(s->pos, s->bk_pos, bd, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->vel, s->bk_vel, bd, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->beta, s->bk_beta, bd, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->img, s->bk_img, bi, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_order) {
        CK(cudaMemcpyAsync(s->order, s->bk_order, n * 4, cudaMemcpyDeviceToDevice, s->stream));
        k_invert_order<<<grid_for(s->n, kBlock), kBlock, 0, s->stream>>>(s->order, s->slot_of, s->n);
        CK(cudaGetLastError());
    }
    if (s->bk_types && s->types) CK(cudaMemcpyAsync(s->types, s->bk_types, n * 4, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_mclass && s->mclass) CK(cudaMemcpyAsync(s->mclass, s->bk_mclass, n, cudaMemcpyDeviceToDevice, s->stream));
    if (s->bk_mass && s->mass) CK(cudaMemcpyAsync(s->mass, s->bk_mass, n * 8, cudaMemcpyDeviceToDevice, s->stream));
    return launch_shadow(s);
}

static long long chunk_steps(const dp_sim* s) {
    long long c = (4LL << 20) / std::max<long long>(1, s->n);
    c = std::max<long long>(32, std::min<long long>(1024, c));
    return c;
}

// Capture and instantiate, before any step runs, every chunk graph a run of
// `steps` steps will launch: the chunk lengths, each keyed by the position
// buffer set that is current when it starts (a fused chunk of odd length
// leaves the other set current). A timed run then measures launches only.
static int prepare_one(dp_sim* s, long long c, int kind, bool other_set) {
    if (other_set) swap_position_buffers(s);
    GraphEntry* g = nullptr;
    const int rc = get_graph(s, c, kind, &g);
    if (other_set) swap_position_buffers(s);
    return rc;
}

static int prepare_graphs(dp_sim* s, long long steps, int kind) {
    if (steps <= 0) return DP_OK;
    const long long chunk = chunk_steps(s);
    const bool odd = use_fused_step(s) && (chunk & 1);  // each full chunk flips the sets
    const long long full = steps / chunk, rem = steps % chunk;
    if (full >= 1) RET(prepare_one(s, chunk, kind, false));
    if (full >= 2 && odd) RET(prepare_one(s, chunk, kind, true));
    if (rem > 0) RET(prepare_one(s, rem, kind, odd && (full & 1)));
    return DP_OK;
}

static int run_impl(dp_sim* s, long long steps, int kind, float* ms) {
    RET(require_ready(s));
    if (kind != DP_INT_GJF && kind != DP_INT_NVE) return fail(DP_ERR_ARG, "unknown integrator kind");
    if (steps < 0) return fail(DP_ERR_ARG, "steps must be >= 0");
    // make the list current (the reference checks it at the start of every step)
    RET(update_nl(s, true, nullptr));
    RET(ensure_partial(s, grid_for(s->n, kBlock)));
    if (s->precision == DP_PREC_MLP) RET(ensure_mlp_fx(s));
    s->launches_last = 0;
    RET(prepare_graphs(s, steps, kind));
    if (ms) CK(cudaEventRecord(s->ev0, s->stream));
    const long long chunk = chunk_steps(s);
    long long done = 0;
    int retries = 0;
    while (done < steps) {
        const long long c = std::min(chunk, steps - done);
        const long long step0 = s->hstat->step;  // hstat is current: every path here ends in read_status
        const long long rebuilds0 = s->hstat->rebuilds;
        // a chunk needs the backup only if a list build inside it can
        // overflow: at a later step, or at its first step when a rebuild is
        // pending (hstat is current here)
        const bool backed_up = !use_allpairs_step(s) && (c > 1 || s->hstat->need_rebuild != 0);
        if (backed_up) RET(backup_state(s));
        GraphEntry* g = nullptr;
        RET(get_graph(s, c, kind, &g));
        CK(cudaGraphLaunch(g->exec, s->stream));
        // a fused chunk of odd length leaves the positions in the other buffer set
        if (g->fused && (c & 1)) swap_position_buffers(s);
        RET(read_status(s));
        RET(check_device_error(s));
        if (s->hstat->nonfinite) {
            s->hstat->nonfinite = 0;
            RET(write_status(s));
            return fail(DP_ERR_NONFINITE, "a force or position became NaN/Inf during run()");
        }
        bool grown = false;
        RET(grow_after_overflow(s, &grown));
        if (grown) {
            if (!backed_up) return fail(DP_ERR_OVERFLOW, "neighbour list overflow without a pending build");
            if (++retries > 8) return fail(DP_ERR_OVERFLOW, "neighbour list keeps overflowing");
            RET(restore_state(s));
            s->hstat->step = step0;
            s->hstat->need_rebuild = 1;
            RET(write_status(s));
            continue;  // replay the chunk with the larger capacity
        }
        s->launches_last += g->launches + (s->hstat->rebuilds - rebuilds0) * g->rebuild_launches;
        done += c;
    }
    if (ms) {
        CK(cudaEventRecord(s->ev1, s->stream));
        CK(cudaEventSynchronize(s->ev1));
        CK(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    }
    return DP_OK;
}

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* dp_last_error(void) { return g_err.c_str(); }

int dp_version(void) { return 100; }

int dp_create(int dim, int64_t n, int precision, dp_sim** out) {
    if (!out) return fail(DP_ERR_ARG, "out is null");
    *out = nullptr;
    if (dim < 2 || dim > 4) return fail(DP_ERR_ARG, "dimension must be 2, 3 or 4");
    if (n < 1 || n > 2147483647LL) return fail(DP_ERR_ARG, "number of particles must be in [1, 2^31)");
    if (precision != DP_PREC_FP64 && precision != DP_PREC_FP32) return fail(DP_ERR_ARG, "unknown precision");
    dp_sim* s = new dp_sim();
    s->dim = dim;
    s->n = n;
    s->precision = precision;
    // DOMPAP_CONDITIONAL_GRAPHS=0 selects the gated rebuild kernels (profilers
    // that do not follow conditional graph nodes see every launch then)
    if (const char* env = std::getenv("DOMPAP_CONDITIONAL_GRAPHS")) s->conditional_graphs = std::atoi(env) != 0;
    if (const char* env = std::getenv("DOMPAP_FUSED_STEP")) s->fused_step = std::atoi(env) != 0;
    if (const char* env = std::getenv("DOMPAP_WARP_STEP")) s->warp_step_max = std::atoll(env);
    if (const char* env = std::getenv("DOMPAP_QUAD_STEP")) s->quad_step_max = std::atoll(env);
    if (const char* env = std::getenv("DOMPAP_REORDER")) s->reorder = std::atoi(env) != 0;
    if (const char* env = std::getenv("DOMPAP_MLP_TENSOR"))
        s->mlp_tensor = std::strcmp(env, "tcgen05") == 0 ? 1 : (std::strcmp(env, "mma") == 0 ? 2 : 0);
    int rc = DP_OK;
    auto cleanup = [&]() {
        dp_destroy(s);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->cstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, std::string("stream/event creation: ") + cudaGetErrorString(cudaGetLastError()));
        return cleanup();
    }
    const size_t nd = (size_t)n * dim;
    if ((rc = dalloc_t(&s->pos, nd)) || (rc = dalloc_t(&s->vel, nd)) || (rc = dalloc_t(&s->beta, nd)) ||
        (rc = dalloc_t(&s->force, nd)) || (rc = dalloc_t(&s->pos_ref, nd)) || (rc = dalloc_t(&s->img, nd)) ||
        (rc = dalloc_t(&s->bk_pos, nd)) || (rc = dalloc_t(&s->bk_vel, nd)) || (rc = dalloc_t(&s->bk_beta, nd)) ||
        (rc = dalloc_t(&s->bk_img, nd)) || (rc = dalloc_t(&s->cnt, (size_t)n)) ||
        (rc = dalloc_t(&s->order, (size_t)n)) || (rc = dalloc_t(&s->slot_of, (size_t)n)))
        return cleanup();
    k_iota<<<grid_for(n, kBlock), kBlock, 0, s->stream>>>(s->order, s->slot_of, n);  // slot = particle id
    s->shadow_bytes = (size_t)n * (dim == 2 ? 8 : 16);
    if ((rc = dalloc(&s->shadow, s->shadow_bytes)) || (rc = dalloc(&s->shadow_ref, s->shadow_bytes)) ||
        (rc = dalloc(&s->pos64, (size_t)n * (dim == 2 ? 16 : 32))) || (rc = dalloc_t(&s->pos_alt, nd)) ||
        (rc = dalloc(&s->shadow_alt, s->shadow_bytes)) || (rc = dalloc(&s->pos64_alt, (size_t)n * (dim == 2 ? 16 : 32))))
        return cleanup();
    if (cudaMemset(s->shadow, 0, s->shadow_bytes) != cudaSuccess ||
        cudaMemset(s->shadow_ref, 0, s->shadow_bytes) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "cudaMemset failed");
        return cleanup();
    }
    if (cudaMemset(s->pos, 0, nd * 8) != cudaSuccess || cudaMemset(s->vel, 0, nd * 8) != cudaSuccess ||
        cudaMemset(s->beta, 0, nd * 8) != cudaSuccess || cudaMemset(s->force, 0, nd * 8) != cudaSuccess ||
        cudaMemset(s->pos_ref, 0, nd * 8) != cudaSuccess || cudaMemset(s->img, 0, nd * 4) != cudaSuccess ||
        cudaMemset(s->cnt, 0, (size_t)n * 4) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "cudaMemset failed");
        return cleanup();
    }
    if (cudaMalloc(&s->dstat, sizeof(dp_dev_status)) != cudaSuccess ||
        cudaMallocHost(&s->hstat, sizeof(dp_dev_status)) != cudaSuccess ||
        cudaMalloc(&s->dsum, sizeof(double)) != cudaSuccess || cudaMallocHost(&s->hsum, sizeof(double)) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "status allocation failed");
        return cleanup();
    }
    memset(s->hstat, 0, sizeof(dp_dev_status));
    if (cudaMemcpy(s->dstat, s->hstat, sizeof(dp_dev_status), cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "status init failed");
        return cleanup();
    }
    if ((rc = upload_mass_coefficients(s))) return cleanup();
    *out = s;
    return DP_OK;
}

int dp_destroy(dp_sim* s) {
    if (!s) return DP_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_graphs(s);
    void* bufs[] = {s->pos, s->vel, s->beta, s->force, s->pos_ref, s->img, s->shadow, s->shadow_ref, s->pos64,
                    s->pos_alt, s->shadow_alt, s->pos64_alt, s->mlp_fx,
                    s->ff_tab, s->bk_pos,
                    s->bk_vel, s->bk_beta, s->bk_img, s->mclass, s->mcoef, s->mcoef_f, s->class_mass_dev, s->mass, s->types,
                    s->sig_tab, s->eps_tab, s->isig_tab, s->nl, s->cnt, s->bin_cnt, s->bin_start, s->bin_part,
                    s->bin_key, s->bin_rank, s->src_of, s->order, s->slot_of, s->sc_vel, s->sc_beta, s->sc_mass,
                    s->sc_img, s->sc_order, s->sc_types, s->sc_mclass, s->bk_order, s->bk_types, s->bk_mclass,
                    s->bk_mass, s->dstat,
                    s->partial, s->dsum};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (s->hstat) cudaFreeHost(s->hstat);
    if (s->hsum) cudaFreeHost(s->hsum);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->cstream) cudaStreamDestroy(s->cstream);
    delete s;
    return DP_OK;
}

static int rebuild_pair_lib(dp_sim* s);

int dp_set_precision(dp_sim* s, int precision) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (precision != DP_PREC_FP64 && precision != DP_PREC_FP32 && precision != DP_PREC_MLP)
        return fail(DP_ERR_ARG, "unknown precision");
    if (precision == DP_PREC_MLP && !s->mlp_dev) return fail(DP_ERR_ARG, "no pair surrogate attached (dp_set_mlp)");
    if (precision == DP_PREC_MLP && s->pmode != DP_PAIR_CONST)
        return fail(DP_ERR_ARG, "the pair surrogate needs constant sigma = epsilon = 1");
    if (precision == DP_PREC_FP64 && s->have_box) RET(launch_shadow(s));  // refresh the 64-bit fixed point
    if (precision == s->precision) return DP_OK;
    s->precision = precision;
    if (s->have_pot) RET(rebuild_pair_lib(s));
    return DP_OK;
}

// --------------------------- state ----------------------------------------
// The device's view of a page-locked host array (cudaHostAlloc / registered),
// or nullptr for pageable memory. The transposing kernels then read or write
// the host array directly over the host link: one pass, no staging copy.
static const void* mapped_view(const void* host) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

// host (n, comps) in particle-id order -> device SoA in slot order; the
// caller synchronises (the host array must not change before that).
static int upload_f64_async(dp_sim* s, const double* host, double* dev_soa, int comps) {
    if (!host) return fail(DP_ERR_ARG, "null array");
    const unsigned g = grid_for(s->n * comps, kBlock);
    if (const double* view = (const double*)mapped_view(host)) {
        k_host_to_slots<double><<<g, kBlock, 0, s->stream>>>(view, dev_soa, s->slot_of, s->n, comps);
    } else {
        // stage through the backup buffer to transpose on the device
        CK(cudaMemcpyAsync(s->bk_pos, host, (size_t)s->n * comps * sizeof(double), cudaMemcpyHostToDevice,
                           s->stream));
        k_host_to_slots<double><<<g, kBlock, 0, s->stream>>>(s->bk_pos, dev_soa, s->slot_of, s->n, comps);
    }
    CK(cudaGetLastError());
    return DP_OK;
}

static int upload_aos_f64_async(dp_sim* s, const double* host, double* dev_soa) {
    return upload_f64_async(s, host, dev_soa, s->dim);
}

static int upload_aos_f64(dp_sim* s, const double* host, double* dev_soa) {
    RET(upload_aos_f64_async(s, host, dev_soa));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

// device SoA in slot order -> host (n, comps) in particle-id order; the
// caller synchronises before reading it.
static int download_f64_async(dp_sim* s, const double* dev_soa, double* host, int comps) {
    if (!host) return fail(DP_ERR_ARG, "null array");
    const unsigned g = grid_for(s->n * comps, kBlock);
    if (double* view = (double*)mapped_view(host)) {
        k_slots_to_host<double><<<g, kBlock, 0, s->stream>>>(dev_soa, view, s->slot_of, s->n, comps);
        CK(cudaGetLastError());
    } else {
        k_slots_to_host<double><<<g, kBlock, 0, s->stream>>>(dev_soa, s->bk_vel, s->slot_of, s->n, comps);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(host, s->bk_vel, (size_t)s->n * comps * sizeof(double), cudaMemcpyDeviceToHost,
                           s->stream));
    }
    return DP_OK;
}

static int download_aos_f64_async(dp_sim* s, const double* dev_soa, double* host) {
    return download_f64_async(s, dev_soa, host, s->dim);
}

static int download_aos_f64(dp_sim* s, const double* dev_soa, double* host) {
    RET(download_aos_f64_async(s, dev_soa, host));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

// host int32 (n, comps) in id order -> device SoA in slot order, staged
// through bk_img (n * dim int32, comps <= dim).
static int upload_i32(dp_sim* s, const int32_t* host, int32_t* dev_soa, int comps) {
    const size_t bytes = (size_t)s->n * comps * sizeof(int32_t);
    CK(cudaMemcpyAsync(s->bk_img, host, bytes, cudaMemcpyHostToDevice, s->stream));
    k_host_to_slots<int32_t><<<grid_for(s->n * comps, kBlock), kBlock, 0, s->stream>>>(s->bk_img, dev_soa, s->slot_of,
                                                                                         s->n, comps);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

int dp_set_positions(dp_sim* s, const double* p) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    RET(upload_aos_f64_async(s, p, s->pos));
    if (s->have_box) RET(launch_shadow(s));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}
int dp_get_positions(dp_sim* s, double* p) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    return download_aos_f64(s, s->pos, p);
}
int dp_get_reference_positions(dp_sim* s, double* p) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    return download_aos_f64(s, s->pos_ref, p);
}
int dp_set_velocities(dp_sim* s, const double* v) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    return upload_aos_f64(s, v, s->vel);
}
int dp_get_velocities(dp_sim* s, double* v) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    return download_aos_f64(s, s->vel, v);
}
int dp_set_betas(dp_sim* s, const double* b) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    return upload_aos_f64(s, b, s->beta);
}
int dp_get_betas(dp_sim* s, double* b) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    return download_aos_f64(s, s->beta, b);
}
int dp_set_images(dp_sim* s, const int32_t* im) {
    if (!s || !im) return fail(DP_ERR_ARG, "null argument");
    return upload_i32(s, im, s->img, s->dim);
}
int dp_get_images(dp_sim* s, int32_t* im) {
    if (!s || !im) return fail(DP_ERR_ARG, "null argument");
    const size_t bytes = (size_t)s->n * s->dim * sizeof(int32_t);
    k_slots_to_host<int32_t><<<grid_for(s->n * s->dim, kBlock), kBlock, 0, s->stream>>>(s->img, s->bk_img,
                                                                                         s->slot_of, s->n, s->dim);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(im, s->bk_img, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

int dp_set_masses(dp_sim* s, const double* m) {
    if (!s || !m) return fail(DP_ERR_ARG, "null argument");
    std::map<double, int> classes;
    for (long long i = 0; i < s->n && classes.size() <= 256; ++i) classes.emplace(m[i], 0);
    if (classes.size() == 1) {
        s->mass_mode = 0;
        s->class_mass.assign(1, m[0]);
    } else if (classes.size() <= 256) {
        s->mass_mode = 1;
        s->class_mass.clear();
        int c = 0;
        for (auto& kv : classes) {
            kv.second = c++;
            s->class_mass.push_back(kv.first);
        }
        std::vector<uint8_t> cls((size_t)s->n);
        for (long long i = 0; i < s->n; ++i) cls[i] = (uint8_t)classes[m[i]];
        if (!s->mclass) RET(dalloc_t(&s->mclass, (size_t)s->n));
        // by particle id into the slot order (staged through bk_img)
        CK(cudaMemcpyAsync(s->bk_img, cls.data(), (size_t)s->n, cudaMemcpyHostToDevice, s->stream));
        k_host_to_slots<uint8_t><<<grid_for(s->n, kBlock), kBlock, 0, s->stream>>>(
            (const uint8_t*)s->bk_img, s->mclass, s->slot_of, s->n, 1);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s->stream));
    } else {
        s->mass_mode = 2;
        s->class_mass.assign(1, m[0]);
        if (!s->mass) RET(dalloc_t(&s->mass, (size_t)s->n));
        RET(upload_f64_async(s, m, s->mass, 1));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (s->mass_mode == 2) {
        // the reduction kernels read per-particle masses
        RET(dalloc_t(&s->class_mass_dev, 1));
        CK(cudaMemcpy(s->class_mass_dev, s->class_mass.data(), sizeof(double), cudaMemcpyHostToDevice));
    }
    return upload_mass_coefficients(s);
}

int dp_set_types(dp_sim* s, const int32_t* t) {
    if (!s || !t) return fail(DP_ERR_ARG, "null argument");
    int lo = t[0], hi = t[0];
    for (long long i = 1; i < s->n; ++i) {
        lo = std::min(lo, (int)t[i]);
        hi = std::max(hi, (int)t[i]);
    }
    if (lo < 0) return fail(DP_ERR_ARG, "particle types must be >= 0");
    if (s->pmode == DP_PAIR_TYPES && hi >= s->ntypes)
        return fail(DP_ERR_ARG, "a particle type exceeds the per-type parameter table");
    s->min_type = lo;
    s->max_type = hi;
    if (!s->types) RET(dalloc_t(&s->types, (size_t)s->n));
    RET(upload_i32(s, t, s->types, 1));
    s->have_types = true;
    s->version++;
    return DP_OK;
}

int dp_set_box(dp_sim* s, const double* box) {
    if (!s || !box) return fail(DP_ERR_ARG, "null argument");
    for (int k = 0; k < s->dim; ++k) {
        if (!(box[k] > 0.0) || !std::isfinite(box[k])) return fail(DP_ERR_ARG, "box sides must be positive and finite");
        s->box[k] = box[k];
    }
    s->have_box = true;
    s->nl_config_dirty = true;
    s->version++;
    return launch_shadow(s);
}

// --------------------------- potential ------------------------------------
static std::string hexd(double v) {
    if (std::isinf(v)) return v > 0 ? "(1.0/0.0)" : "(-1.0/0.0)";
    char buf[64];
    snprintf(buf, sizeof(buf), "%a", v);
    return buf;
}

// step_sets_cond: the fused step may set the next step's graph condition
// (device-side cudaGraphSetConditional); off for systems that run the gated
// rebuild kernels instead of conditional nodes, whose step kernels profilers
// can then follow inside graphs.
static std::string pair_program(int dim, int precision, int pmode, bool sig_one, bool eps_one,
                                const std::string& pot_src, bool with_batch, int step_blocks_hint = 6,
                                bool step_sets_cond = true) {
    std::string src;
    src += std::string("#define DP_STEP_SETS_COND ") + (step_sets_cond ? "1" : "0") + "\n";
    src += "#define DP_DIM " + std::to_string(dim) + "\n";
    if (precision == DP_PREC_MLP) src += "#define DP_MLP 1\n";
    if (precision == DP_PREC_FP64) src += "#define DP_FF 1\n";
    if (precision == DP_PREC_FP32 || precision == DP_PREC_MLP) {
        src += "#define DP_REAL float\n#define DP_REAL_IS_FLOAT 1\n";
    } else {
        src += "#define DP_REAL double\n#define DP_REAL_IS_FLOAT 0\n";
    }
    src += "#define DP_PMODE " + std::to_string(pmode) + "\n";
    src += std::string("#define DP_SIGMA_ONE ") + (sig_one ? "1" : "0") + "\n";
    src += std::string("#define DP_EPS_ONE ") + (eps_one ? "1" : "0") + "\n";
    // resident 256-thread CTAs per SM the fused step kernel is compiled for
    // (register cap 65536 / (256 n)); DOMPAP_STEP_MIN_BLOCKS overrides
    int step_blocks = step_blocks_hint;
    if (const char* env = std::getenv("DOMPAP_STEP_MIN_BLOCKS")) step_blocks = std::atoi(env);
    src += "#define DP_STEP_MIN_BLOCKS " + std::to_string(std::max(0, std::min(8, step_blocks))) + "\n";
    src += dp_src_common;
    src += dp_src_integrate;
    if (precision == DP_PREC_MLP) src += dp_src_mlp;
    if (precision == DP_PREC_MLP) src += dp_src_umma;
    if (precision == DP_PREC_FP64) src += dp_src_ff;
    src += "\n// ---- generated pair potential ----\n";
    src += pot_src;
    src += "\n// ---- pair kernels ----\n";
    src += dp_src_pair;
    if (with_batch) {
        src += "\n// ---- batched replicas ----\n";
        src += dp_src_batch;
    }
    return src;
}

// Resident 256-thread CTAs per SM the fused step kernel is compiled for
// (measured on GB300 against 4, 5, 6, 7 and 8): 4 (64 registers) for the
// double-float pair loop in 3 and 4 dimensions, whose pair terms spill under
// a tighter cap (1M LJ particles: 0.99 ms per step against 1.10 with 6; 1M
// harmonic: 3 % faster) and for per-type or per-pair tables (~600 bytes of
// spills under 40 registers; the Wahnstrom mixture ran 17 % slower with 6);
// 6 (40 registers) for the float32 pair loop and in 2 dimensions, where the
// occupancy is worth more (7-8 % faster than with 4).
static int step_blocks_for(int dim, int precision, int pmode) {
    if (pmode != DP_PAIR_CONST) return 4;
    return precision == DP_PREC_FP64 && dim >= 3 ? 4 : 6;
}

static int rebuild_pair_lib(dp_sim* s) {
    const bool sig_one = s->pmode == DP_PAIR_CONST && s->sigma == 1.0;
    const bool eps_one = s->pmode == DP_PAIR_CONST && s->epsilon == 1.0;
    const int step_blocks = s->step_blocks ? s->step_blocks : step_blocks_for(s->dim, s->precision, s->pmode);
    const std::string src =
        pair_program(s->dim, s->precision, s->pmode, sig_one, eps_one, s->pot_src, false, step_blocks,
                     s->conditional_graphs);
    PairLib pl;
    RET(compile_pair_lib(src, &pl));
    s->lib = pl;
    s->lib_valid = true;
    s->version++;
    return DP_OK;
}

int dp_set_pair_methods(dp_sim* s, int force_method, int energy_method) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (force_method < DP_METHOD_LIST || force_method > DP_METHOD_ALLPAIRS_NEWTON)
        return fail(DP_ERR_ARG, "unknown force method");
    if (energy_method != DP_METHOD_LIST && energy_method != DP_METHOD_ALLPAIRS)
        return fail(DP_ERR_ARG, "unknown energy method");
    if (force_method != s->force_method || energy_method != s->energy_method) {
        s->force_method = force_method;
        s->energy_method = energy_method;
        s->version++;
    }
    return DP_OK;
}

int dp_set_step_launch(dp_sim* s, int lanes, int blocks_per_sm) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (lanes != 0 && lanes != 1 && lanes != 4 && lanes != 32) return fail(DP_ERR_ARG, "lanes must be 0, 1, 4 or 32");
    if (blocks_per_sm < 0 || blocks_per_sm > 8) return fail(DP_ERR_ARG, "blocks_per_sm must be in [0, 8]");
    if (lanes != s->step_lanes) {
        s->step_lanes = lanes;
        s->version++;
    }
    if (blocks_per_sm != s->step_blocks) {
        s->step_blocks = blocks_per_sm;
        if (s->have_pot) RET(rebuild_pair_lib(s));
    }
    return DP_OK;
}

int dp_get_step_launch(dp_sim* s, int* lanes, int* blocks_per_sm) {
    if (!s || !lanes || !blocks_per_sm) return fail(DP_ERR_ARG, "null argument");
    *lanes = s->step_lanes ? s->step_lanes
                           : (s->n <= s->warp_step_max ? 32 : (s->n <= s->quad_step_max ? 4 : 1));
    *blocks_per_sm = s->step_blocks ? s->step_blocks : step_blocks_for(s->dim, s->precision, s->pmode);
    return DP_OK;
}

int dp_set_potential(dp_sim* s, const char* device_source, double r_cut) {
    if (!s || !device_source) return fail(DP_ERR_ARG, "null argument");
    if (!(r_cut > 0.0)) return fail(DP_ERR_ARG, "r_cut must be positive");
    s->pot_src = device_source;
    s->r_cut = r_cut;
    s->have_pot = true;
    s->lib_valid = false;
    RET(rebuild_pair_lib(s));
    s->nl_config_dirty = true;
    return DP_OK;
}

int dp_set_pair_params(dp_sim* s, int mode, int ntypes, const double* sigma, const double* epsilon) {
    if (!s || !sigma || !epsilon) return fail(DP_ERR_ARG, "null argument");
    double smax = 0.0;
    if (mode == DP_PAIR_CONST) {
        s->sigma = sigma[0];
        s->epsilon = epsilon[0];
        smax = sigma[0];
        s->ntypes = 1;
    } else if (mode == DP_PAIR_TYPES) {
        if (ntypes < 1 || ntypes > 4096) return fail(DP_ERR_ARG, "ntypes must be in [1, 4096]");
        if (!s->have_types) return fail(DP_ERR_ARG, "per-type parameters need particle types (dp_set_types)");
        if (s->max_type >= ntypes) return fail(DP_ERR_ARG, "a particle type exceeds the per-type parameter table");
        const size_t m = (size_t)ntypes * ntypes;
        for (size_t t = 0; t < m; ++t) smax = std::max(smax, sigma[t]);
        std::vector<double> inv(m);
        for (size_t t = 0; t < m; ++t) inv[t] = 1.0 / sigma[t];
        RET(dalloc_t(&s->sig_tab, m));
        RET(dalloc_t(&s->eps_tab, m));
        RET(dalloc_t(&s->isig_tab, m));
        CK(cudaMemcpy(s->sig_tab, sigma, m * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(s->eps_tab, epsilon, m * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(s->isig_tab, inv.data(), m * sizeof(double), cudaMemcpyHostToDevice));
        std::vector<float2> ff(3 * m);
        auto split = [](double v) { return make_float2((float)v, (float)(v - (double)(float)v)); };
        for (size_t t = 0; t < m; ++t) {
            ff[3 * t + 0] = split(sigma[t]);
            ff[3 * t + 1] = split(inv[t]);
            ff[3 * t + 2] = split(epsilon[t]);
        }
        RET(dalloc_t(&s->ff_tab, ff.size()));
        CK(cudaMemcpy(s->ff_tab, ff.data(), ff.size() * sizeof(float2), cudaMemcpyHostToDevice));
        s->ntypes = ntypes;
    } else if (mode == DP_PAIR_DENSE) {
        const size_t m = (size_t)s->n * s->n;
        for (size_t t = 0; t < m; ++t) smax = std::max(smax, sigma[t]);
        RET(dalloc_t(&s->sig_tab, m));
        RET(dalloc_t(&s->eps_tab, m));
        CK(cudaMemcpy(s->sig_tab, sigma, m * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(s->eps_tab, epsilon, m * sizeof(double), cudaMemcpyHostToDevice));
        s->ntypes = 1;
    } else {
        return fail(DP_ERR_ARG, "unknown pair-parameter mode");
    }
    if (!(smax > 0.0)) return fail(DP_ERR_ARG, "the largest sigma must be positive");
    s->pmode = mode;
    s->sig_max = smax;  // largest sigma (dompap/Simulation.py:346-351)
    s->nl_config_dirty = true;
    s->version++;
    if (s->have_pot) RET(rebuild_pair_lib(s));
    return DP_OK;
}

int dp_set_neighbor_list(dp_sim* s, double skin, int max_neighbors, int method) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (!(skin >= 0.0)) return fail(DP_ERR_ARG, "skin must be >= 0");
    if (max_neighbors < 1) return fail(DP_ERR_ARG, "max_number_of_neighbors must be >= 1");
    if (method != DP_NL_CELL && method != DP_NL_ALLPAIRS) return fail(DP_ERR_ARG, "unknown neighbour-list method");
    s->skin = skin;
    s->kcap = max_neighbors;
    s->method = method;
    s->nl_config_dirty = true;
    s->version++;
    return DP_OK;
}

int dp_update_neighbor_list(dp_sim* s, int check, int* rebuilt) {
    RET(require_ready(s));
    return update_nl(s, check != 0, rebuilt);
}

int dp_get_neighbor_list(dp_sim* s, int32_t* out, int kmax, int32_t* max_count) {
    RET(require_ready(s));
    if (!out || kmax < 1) return fail(DP_ERR_ARG, "bad output");
    RET(update_nl(s, true, nullptr));
    const unsigned g = grid_for(s->n, kBlock);
    const int32_t* rows = s->nl;
    const int32_t* counts = s->cnt;
    int32_t* full = nullptr;  // half lists: the full list, unsorted, column-major
    int32_t* fcnt = nullptr;  // its counts (n) and their maximum
    int32_t fmax = s->hstat->max_neighbors;
    cudaError_t e = cudaSuccess;
    if (s->nl_half) {
        // the reference's list is the full one (every partner of every particle)
        RET(dalloc_t(&fcnt, (size_t)s->n + 1));
        e = cudaMemsetAsync(fcnt, 0, ((size_t)s->n + 1) * sizeof(int32_t), s->stream);
        if (e == cudaSuccess) {
            k_nl_half_count<<<g, kBlock, 0, s->stream>>>(s->nl, s->cnt, fcnt, fcnt + s->n, s->n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&fmax, fcnt + s->n, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e == cudaSuccess && dalloc_t(&full, (size_t)s->n * std::max(fmax, 1)) != DP_OK)
            e = cudaErrorMemoryAllocation;
        if (e == cudaSuccess) e = cudaMemsetAsync(fcnt, 0, (size_t)s->n * sizeof(int32_t), s->stream);
        if (e == cudaSuccess) {
            k_nl_half_scatter<<<g, kBlock, 0, s->stream>>>(s->nl, s->cnt, fcnt, full, s->n);
            e = cudaGetLastError();
        }
        rows = full;
        counts = fcnt;
    }
    int32_t* dout = nullptr;
    if (e == cudaSuccess && dalloc_t(&dout, (size_t)s->n * kmax) != DP_OK) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
        k_nl_export<<<g, kBlock, 0, s->stream>>>(rows, counts, dout, s->order, s->slot_of, s->n, kmax);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, dout, (size_t)s->n * kmax * sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(dout);
    cudaFree(full);
    cudaFree(fcnt);
    if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("neighbour-list export: ") + cudaGetErrorString(e));
    if (max_count) *max_count = fmax;
    return DP_OK;
}

int dp_set_integrator(dp_sim* s, double time_step, double temperature, double damping_time, uint64_t seed) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    s->dt = time_step;
    s->temperature = temperature;
    s->tau = damping_time;
    s->seed = seed;
    s->version++;
    return upload_mass_coefficients(s);
}

int dp_run(dp_sim* s, int64_t steps, int kind) { return run_impl(s, steps, kind, nullptr); }

int dp_selftest_bounded_wait(dp_sim* s, int32_t limit) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (limit < 1 || limit > (1 << 20)) return fail(DP_ERR_ARG, "limit must be in [1, 2^20]");
    k_selftest_bounded_wait<<<1, 128, 0, s->stream>>>(s->dstat, limit);
    CK(cudaGetLastError());
    RET(read_status(s));
    return check_device_error(s);
}

int dp_run_timed(dp_sim* s, int64_t steps, int kind, float* ms) {
    if (!ms) return fail(DP_ERR_ARG, "ms is null");
    return run_impl(s, steps, kind, ms);
}

int dp_run_host(dp_sim* s, const double* positions, const double* velocities, const double* betas, int64_t steps,
                int kind, double* positions_out, double* velocities_out, double* betas_out) {
    RET(require_ready(s));
    // uploads, run and downloads are ordered on the stream; the host waits
    // inside run() (its status reads) and once after the downloads
    if (positions) {
        RET(upload_aos_f64_async(s, positions, s->pos));
        RET(launch_shadow(s));
    }
    if (velocities) RET(upload_aos_f64_async(s, velocities, s->vel));
    if (betas) RET(upload_aos_f64_async(s, betas, s->beta));
    RET(run_impl(s, steps, kind, nullptr));
    if (positions_out) RET(download_aos_f64_async(s, s->pos, positions_out));
    if (velocities_out) RET(download_aos_f64_async(s, s->vel, velocities_out));
    if (betas_out) RET(download_aos_f64_async(s, s->beta, betas_out));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

// --------------------------- observables ----------------------------------
int dp_forces(dp_sim* s, double* forces) {
    RET(require_ready(s));
    RET(update_nl(s, true, nullptr));
    RET(launch_pair(s, s->lib.forces, s->force, nullptr));
    RET(read_status(s));
    RET(check_device_error(s));
    if (s->hstat->nonfinite) {
        s->hstat->nonfinite = 0;
        RET(write_status(s));
    }
    return download_aos_f64(s, s->force, forces);
}

static int scalar_pair(dp_sim* s, cudaKernel_t k, double* out) {
    RET(require_ready(s));
    if (!out) return fail(DP_ERR_ARG, "null output");
    RET(update_nl(s, true, nullptr));
    // one partial sum per block of the kernel launch_pair uses
    const bool tc = s->precision == DP_PREC_MLP && use_mlp_tcgen05(s);
    const bool all = k == s->lib.energy && s->energy_method != DP_METHOD_LIST && s->lib.energy_all;
    const long long blocks = all ? grid_for(s->n * 32, kBlock) : grid_for(s->n, tc ? 128 : kBlock);
    RET(ensure_partial(s, blocks));
    RET(launch_pair(s, k, nullptr, nullptr));
    k_reduce<<<1, 1024, 0, s->stream>>>(s->partial, blocks, s->dsum);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(s->hsum, s->dsum, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *out = *s->hsum;
    if (tc) {
        RET(read_status(s));
        RET(check_device_error(s));
    }
    return DP_OK;
}

int dp_potential_energy(dp_sim* s, double* energy) {
    double e = 0.0;
    RET(scalar_pair(s, s ? s->lib.energy : nullptr, &e));
    // the list kernel sums every pair twice (dompap/potential.py:69-100 halves
    // it); the double-loop kernel sums each pair once (:103-160)
    const bool all = s->energy_method != DP_METHOD_LIST && s->lib.energy_all;
    *energy = all ? e : e / 2;
    return DP_OK;
}

int dp_virial(dp_sim* s, double* virial) {
    double w = 0.0;
    RET(scalar_pair(s, s ? s->lib.virial : nullptr, &w));
    *virial = w / s->dim;
    return DP_OK;
}

int dp_laplacian(dp_sim* s, double* lap) {
    RET(require_ready(s));
    if (!lap) return fail(DP_ERR_ARG, "null output");
    RET(update_nl(s, true, nullptr));
    RET(launch_pair(s, s->lib.laplacian, s->bk_beta, nullptr));
    RET(download_f64_async(s, s->bk_beta, lap, 1));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

int dp_sum_mv2(dp_sim* s, double* out) {
    if (!s || !out) return fail(DP_ERR_ARG, "null argument");
    const long long blocks = grid_for(s->n, kBlock);
    RET(ensure_partial(s, blocks));
    dp_int_args a;
    fill_int_args(s, a, 0);
    const unsigned g = (unsigned)blocks;
#define DP_MV2(D)                                                                                               \
    switch (s->mass_mode) {                                                                                     \
        case 0: k_sum_mv2<D, 0><<<g, kBlock, 0, s->stream>>>(a, s->class_mass_dev, s->partial); break;          \
        case 1: k_sum_mv2<D, 1><<<g, kBlock, 0, s->stream>>>(a, s->class_mass_dev, s->partial); break;          \
        default: k_sum_mv2<D, 2><<<g, kBlock, 0, s->stream>>>(a, s->class_mass_dev, s->partial); break;         \
    }
    switch (s->dim) {
        case 2: DP_MV2(2); break;
        case 3: DP_MV2(3); break;
        default: DP_MV2(4); break;
    }
#undef DP_MV2
    k_reduce<<<1, 1024, 0, s->stream>>>(s->partial, blocks, s->dsum);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(s->hsum, s->dsum, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *out = *s->hsum;
    return DP_OK;
}

int dp_eval_potential(dp_sim* s, const double* sv, int64_t n, double* u, double* f, double* c) {
    if (!s || !sv || !u || !f || !c) return fail(DP_ERR_ARG, "null argument");
    if (!s->have_pot || !s->lib_valid) return fail(DP_ERR_NOPOT, "no pair potential set");
    if (n <= 0) return DP_OK;
    double* buf = nullptr;
    RET(dalloc_t(&buf, (size_t)n * 4));
    const size_t b = (size_t)n * sizeof(double);
    cudaError_t e = cudaMemcpyAsync(buf, sv, b, cudaMemcpyHostToDevice, s->stream);
    double* du = buf + n;
    double* df = buf + 2 * n;
    double* dc = buf + 3 * n;
    long long nn = n;
    double rc = s->r_cut;
    void* args[] = {&buf, &du, &df, &dc, &nn, &rc};
    if (e == cudaSuccess)
        e = cudaLaunchKernel((const void*)s->lib.eval, dim3(grid_for(n, kBlock)), dim3(kBlock), args, 0, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(u, du, b, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(f, df, b, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c, dc, b, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("dp_eval_potential: ") + cudaGetErrorString(e));
    return DP_OK;
}

int dp_get_normals(dp_sim* s, int64_t step, double* out) {
    if (!s || !out) return fail(DP_ERR_ARG, "null argument");
    const unsigned g = grid_for(s->n, kBlock);
    switch (s->dim) {
        case 2: k_normals<2><<<g, kBlock, 0, s->stream>>>(s->seed, step, s->bk_vel, s->n); break;
        case 3: k_normals<3><<<g, kBlock, 0, s->stream>>>(s->seed, step, s->bk_vel, s->n); break;
        default: k_normals<4><<<g, kBlock, 0, s->stream>>>(s->seed, step, s->bk_vel, s->n); break;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, s->bk_vel, (size_t)s->n * s->dim * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

int dp_get_stats(dp_sim* s, dp_stats* st) {
    if (!s || !st) return fail(DP_ERR_ARG, "null argument");
    RET(read_status(s));
    memset(st, 0, sizeof(*st));
    st->steps = s->hstat->step;
    st->rebuilds = s->hstat->rebuilds;
    st->max_neighbors = s->hstat->max_neighbors;
    st->neighbor_capacity = s->kcap;
    for (int k = 0; k < 4; ++k) st->cells[k] = s->use_cells ? s->nc[k] : 0;
    st->cell_capacity = 0;  // cells are contiguous slot ranges: no capacity
    st->method_used = s->use_cells ? DP_NL_CELL : DP_NL_ALLPAIRS;
    st->nl_cutoff = s->cutoff;
    st->conditional_graphs = s->conditional_graphs ? 1 : 0;
    return DP_OK;
}

int dp_time_kernel(dp_sim* s, int which, int reps, float* ms) {
    RET(require_ready(s));
    if (!ms || reps < 1) return fail(DP_ERR_ARG, "bad arguments");
    RET(update_nl(s, true, nullptr));
    RET(ensure_partial(s, grid_for(s->n, kBlock)));
    auto once = [&]() -> int {
        switch (which) {
            case DP_KERNEL_FORCES: return launch_pair(s, s->lib.forces, s->force, nullptr);
            case DP_KERNEL_GJF: return launch_integrate(s, DP_INT_GJF, 0, nullptr);
            case DP_KERNEL_NVE: return launch_integrate(s, DP_INT_NVE, 0, nullptr);
            case DP_KERNEL_REBUILD:
                k_set_rebuild<<<1, 1, 0, s->stream>>>(s->dstat);
                return launch_rebuild(s, nullptr);
            case DP_KERNEL_SKIN: return launch_skin_check(s);
            case DP_KERNEL_STEP:
                if (!use_fused_step(s)) return fail(DP_ERR_ARG, "no fused step kernel in this mode");
                return launch_step(s, DP_INT_GJF, 0, nullptr);
            default: return fail(DP_ERR_ARG, "unknown kernel");
        }
    };
    const bool moves = which == DP_KERNEL_GJF || which == DP_KERNEL_NVE || which == DP_KERNEL_STEP;
    if (moves) RET(backup_state(s));
    RET(once());  // warm-up
    CK(cudaEventRecord(s->ev0, s->stream));
    for (int r = 0; r < reps; ++r) RET(once());
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, s->ev0, s->ev1));
    *ms = t / reps;
    // the integrator kernels moved the particles: put the state back and
    // leave a consistent list behind
    if (moves) RET(restore_state(s));
    RET(read_status(s));
    s->hstat->need_rebuild = 1;
    RET(write_status(s));
    RET(update_nl(s, true, nullptr));
    return DP_OK;
}


int dp_wrap(dp_sim* s) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (!s->have_box) return fail(DP_ERR_ARG, "box not set");
    dp_int_args a;
    fill_int_args(s, a, 0);
    const unsigned g = grid_for(s->n, kBlock);
    switch (s->dim) {
        case 2: k_wrap<2><<<g, kBlock, 0, s->stream>>>(a); break;
        case 3: k_wrap<3><<<g, kBlock, 0, s->stream>>>(a); break;
        default: k_wrap<4><<<g, kBlock, 0, s->stream>>>(a); break;
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    return DP_OK;
}

int dp_rdf_counts(dp_sim* s, int type_a, int type_b, const double* edges, int nbins, uint64_t* counts) {
    if (!s || !edges || !counts) return fail(DP_ERR_ARG, "null argument");
    if (!s->have_box) return fail(DP_ERR_ARG, "box not set");
    if (nbins < 1 || nbins > 8192) return fail(DP_ERR_ARG, "nbins must be in [1, 8192]");
    if ((type_a >= 0 || type_b >= 0) && !s->have_types) return fail(DP_ERR_ARG, "particle types not set");
    for (int b = 0; b < nbins; ++b)
        if (!(edges[b] <= edges[b + 1])) return fail(DP_ERR_ARG, "r_bins array must be sorted in ascending order.");
    double* dedges = nullptr;
    unsigned long long* dcounts = nullptr;
    RET(dalloc_t(&dedges, (size_t)nbins + 1));
    int rc = dalloc_t(&dcounts, (size_t)nbins);
    if (rc) {
        cudaFree(dedges);
        return rc;
    }
    RdfArgs a{};
    a.pos = s->pos;
    a.shadow = s->shadow;
    a.types = s->types;
    a.edges = dedges;
    a.counts = dcounts;
    a.n = s->n;
    a.nbins = nbins;
    a.type_a = type_a;
    a.type_b = type_b;
    for (int k = 0; k < DP_MAX_DIM; ++k) a.box[k] = (k < s->dim) ? s->box[k] : 1.0;
    fill_scale(s, nullptr, a.unit);
    const size_t smem = (size_t)(nbins + 1) * sizeof(double) + (size_t)nbins * sizeof(unsigned int);
    const long long pairs = s->n * s->n;
    const unsigned g = (unsigned)std::min<long long>(grid_for(pairs, kBlock), 152LL * 8);
    cudaError_t e = cudaMemcpyAsync(dedges, edges, (nbins + 1) * sizeof(double), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(dcounts, 0, nbins * sizeof(unsigned long long), s->stream);
    if (e == cudaSuccess && smem > 48 * 1024) {
        switch (s->dim) {
            case 2: e = cudaFuncSetAttribute(k_rdf<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); break;
            case 3: e = cudaFuncSetAttribute(k_rdf<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); break;
            default: e = cudaFuncSetAttribute(k_rdf<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); break;
        }
    }
    if (e == cudaSuccess) {
        switch (s->dim) {
            case 2: k_rdf<2><<<g, kBlock, smem, s->stream>>>(a); break;
            case 3: k_rdf<3><<<g, kBlock, smem, s->stream>>>(a); break;
            default: k_rdf<4><<<g, kBlock, smem, s->stream>>>(a); break;
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(counts, dcounts, nbins * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(dedges);
    cudaFree(dcounts);
    if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("dp_rdf_counts: ") + cudaGetErrorString(e));
    return DP_OK;
}

int dp_sum_mv2_noalloc(const double* velocities, const double* masses, int64_t n, int dim, double* out,
                       void* stream) {
    if (!velocities || !masses || !out) return fail(DP_ERR_ARG, "null device pointer");
    if (dim < 1 || dim > DP_MAX_DIM) return fail(DP_ERR_ARG, "dimension must be in [1, 4]");
    if (n < 1) return fail(DP_ERR_ARG, "number of particles must be >= 1");
    const long long blocks = (n - 1) / kBlock + 1;  // n >= 1: no overflow near INT64_MAX
    if (blocks > DP_NOALLOC_MAX_BLOCKS)
        return fail(DP_ERR_ARG, "dp_sum_mv2_noalloc: " + std::to_string(n) + " particles exceed its fixed scratch (at most " +
                                    std::to_string((long long)DP_NOALLOC_MAX_BLOCKS * kBlock) + ")");
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(DP_ERR_ARG, "device ordinal out of range");
    double* partial = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_addr[dev]) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
            if (e != cudaSuccess || !p)
                return fail(DP_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_partial): ") + cudaGetErrorString(e));
            g_noalloc_addr[dev] = (double*)p;
        }
        partial = g_noalloc_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    k_mv2_rowmajor<<<(unsigned)blocks, kBlock, 0, st>>>(velocities, masses, n, dim, partial);
    k_reduce<<<1, 1024, 0, st>>>(partial, blocks, out);
    CK(cudaGetLastError());
    return DP_OK;
}

int64_t dp_kernel_launches(dp_sim* s) { return s ? s->launches_last : 0; }

}  // extern "C"

// ===========================================================================
// batched replicas (many independent small systems, one persistent kernel)
// ===========================================================================
namespace {

// Fixed-point shadow of every particle of every replica (each with its box).
__global__ void k_batch_shadow(const double* pos, void* shadow, const int32_t* rep_of, const double* box, int dim,
                               long long ntot) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntot) return;
    const int r = rep_of[i];
    uint32_t u[DP_MAX_DIM] = {0, 0, 0, 0};
    for (int k = 0; k < dim; ++k) u[k] = dp_fixed(pos[k * ntot + i], 4294967296.0 / box[r * DP_MAX_DIM + k]);
    if (dim == 2)
        ((uint2*)shadow)[i] = make_uint2(u[0], u[1]);
    else
        ((uint4*)shadow)[i] = make_uint4(u[0], u[1], u[2], u[3]);
}

}  // namespace

struct BatchGraph {
    long long steps;
    int sample_every, nve, record;
    unsigned long long version;
    cudaGraphExec_t exec;
};

struct dp_batch {
    int dim = 3;
    int n_rep = 0;
    long long ntot = 0;
    cudaStream_t stream = nullptr, stream2 = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr, join = nullptr;
    double *pos = nullptr, *vel = nullptr, *beta = nullptr, *stage = nullptr;
    int32_t *img = nullptr, *rep_of = nullptr, *order = nullptr, *ncell = nullptr, *queue = nullptr;
    void* shadow = nullptr;
    long long* offset = nullptr;
    double *box = nullptr, *coef = nullptr, *obs = nullptr;
    float* force_out = nullptr;
    dp_dev_status* dstat = nullptr;
    dp_dev_status* hstat = nullptr;
    // Verlet lists (skin < 0: cell stencil every step); skin 0.45 was the
    // fastest of 0.2 - 0.8 for LJ replicas at T 0.7 - 2.0, dt 0.005
    double skin = 0.45;
    int kmax_req = 0;  // 0: from the densest replica
    int kmax = 0;      // capacity of the allocated lists
    uint16_t* nlist = nullptr;
    int32_t* ncnt = nullptr;
    void* shadow_ref = nullptr;
    unsigned long long* list_stats = nullptr;
    int32_t* list_gen = nullptr;  // per replica: the generation its list was built for
    std::vector<long long> h_offset;
    std::vector<double> h_box, h_temp;
    std::vector<int> h_ncell, h_order;
    bool have_state = false, have_pot = false;
    std::string pot_src;
    double r_cut = 2.5;
    PairLib lib;
    double dt = 0.005, tau = 0.1, mass = 1.0;
    unsigned long long seed = 0;
    int split_n = 1024, threads_small = 256, threads_large = 1024;
    unsigned long long version = 1;
    std::vector<BatchGraph> graphs;
};

static int batch_kernel_index(int threads) {
    switch (threads) {
        case 128: return 0;
        case 256: return 1;
        case 512: return 2;
        case 1024: return 3;
        default: return -1;
    }
}

static int batch_upload_coef(dp_batch* b) {
    std::vector<double> coef((size_t)b->n_rep * 5);
    const double m = b->mass;
    for (int r = 0; r < b->n_rep; ++r) {
        const double T = b->h_temp.empty() ? 1.0 : b->h_temp[r];
        const double alpha = m / b->tau;  // dompap/integrator.py:29-36
        const double beta_variance = 2 * alpha * T * b->dt;
        const double numerator = 1.0 - alpha * b->dt / 2.0 / m;
        const double denominator = 1.0 + alpha * b->dt / 2.0 / m;
        const double bb = 1 / denominator;
        coef[r * 5 + 0] = numerator / denominator;
        coef[r * 5 + 1] = bb * b->dt / m;
        coef[r * 5 + 2] = bb / 2 / m;
        coef[r * 5 + 3] = std::sqrt(beta_variance);
        coef[r * 5 + 4] = b->dt / m;
    }
    CK(cudaMemcpy(b->coef, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice));
    b->version++;
    return DP_OK;
}

// Cells for the replica's binning, with the cutoff c = r_cut + skin (lists)
// or r_cut (no lists). With lists (binning only for builds) c/2 wide with a
// 5^D stencil where every axis has at least 5 of them (stored negated): fewer
// candidates per build; otherwise, and without lists (binning every step,
// where the loop over many sparse cells costs more), c wide with a 3^D stencil
// (at least 3 per axis); else all pairs inside the replica.
static int batch_configure_cells(dp_batch* b) {
    b->h_ncell.assign((size_t)b->n_rep * DP_MAX_DIM, 0);
    const double width = b->r_cut + std::max(0.0, b->skin);
    const int first_reach = b->skin >= 0.0 ? 2 : 1;
    for (int r = 0; r < b->n_rep; ++r) {
        for (int reach = first_reach; reach >= 1; --reach) {
            bool ok = true;
            int nc[DP_MAX_DIM] = {0, 0, 0, 0};
            for (int k = 0; k < b->dim; ++k) {
                nc[k] = (int)std::floor(b->h_box[r * DP_MAX_DIM + k] * reach / (width * (1.0 + 1e-6)));
                ok = ok && nc[k] >= 2 * reach + 1;
            }
            long long cells = 1;
            for (int k = 0; k < b->dim; ++k) cells *= std::max(nc[k], 1);
            if (!ok || cells > 32768) continue;
            for (int k = 0; k < b->dim; ++k) b->h_ncell[r * DP_MAX_DIM + k] = reach == 2 ? -nc[k] : nc[k];
            break;
        }
    }
    CK(cudaMemcpy(b->ncell, b->h_ncell.data(), b->h_ncell.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    b->version++;
    return DP_OK;
}

// Replicas sorted by size (largest first) and split into a small and a large
// bucket, each run by its own persistent launch.
struct BatchBucket {
    int first, count, threads, max_n, max_cells;
};

static void batch_buckets(const dp_batch* b, BatchBucket* out, int* nb) {
    *nb = 0;
    int large = 0;
    while (large < b->n_rep) {
        const int r = b->h_order[large];
        if (b->h_offset[r + 1] - b->h_offset[r] <= b->split_n) break;
        ++large;
    }
    auto fill = [&](int first, int count, int threads) {
        BatchBucket bk{first, count, threads, 0, 1};
        for (int q = first; q < first + count; ++q) {
            const int r = b->h_order[q];
            bk.max_n = std::max(bk.max_n, (int)(b->h_offset[r + 1] - b->h_offset[r]));
            int cells = 1;
            for (int k = 0; k < b->dim; ++k) cells *= std::max(std::abs(b->h_ncell[r * DP_MAX_DIM + k]), 1);
            bk.max_cells = std::max(bk.max_cells, cells);
        }
        out[(*nb)++] = bk;
    };
    if (large > 0) fill(0, large, b->threads_large);
    if (large < b->n_rep) fill(large, b->n_rep - large, b->threads_small);
}

static size_t batch_smem(int dim, int max_n, int max_cells) {
    const size_t sh = (dim == 2 ? 8 : 16);
    return (size_t)max_n * sh + (size_t)((max_n + 7) & ~7) * 2 + (size_t)(2 * max_cells + 1) * 4;
}

static int batch_record(dp_batch* b, long long steps, int sample_every, int nve, int record) {
    BatchBucket bk[2];
    int nb = 0;
    batch_buckets(b, bk, &nb);
    CK(cudaMemsetAsync(b->queue, 0, 2 * sizeof(int32_t), b->stream));
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (nb == 2) {
        CK(cudaEventRecord(b->fork, b->stream));
        CK(cudaStreamWaitEvent(b->stream2, b->fork, 0));
    }
    for (int q = 0; q < nb; ++q) {
        const BatchBucket& k = bk[q];
        const int ki = batch_kernel_index(k.threads);
        if (ki < 0) return fail(DP_ERR_ARG, "threads per replica must be 128, 256, 512 or 1024");
        if (k.max_n > 65535) return fail(DP_ERR_ARG, "a replica has more than 65535 particles");
        const size_t smem = batch_smem(b->dim, k.max_n, k.max_cells);
        if (smem > 227 * 1024)
            return fail(DP_ERR_ARG, "a replica does not fit in shared memory (" + std::to_string(smem) + " bytes)");
        CK(cudaKernelSetAttributeForDevice(b->lib.batch[ki], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem,
                                           dev));
        dp_batch_args a;
        memset(&a, 0, sizeof(a));
        a.pos = b->pos;
        a.vel = b->vel;
        a.beta = b->beta;
        a.img = b->img;
        a.shadow = b->shadow;
        a.offset = b->offset;
        a.order = b->order + k.first;
        a.box = b->box;
        a.coef = b->coef;
        a.ncell = b->ncell;
        a.obs = b->obs;
        a.force_out = record ? b->force_out : nullptr;
        a.queue = b->queue + q;
        a.st = b->dstat;
        a.ntot = b->ntot;
        a.n_rep = k.count;
        a.steps = (int)steps;
        a.sample_every = sample_every;
        a.max_n = k.max_n;
        a.max_cells = k.max_cells;
        a.nve = nve;
        a.dt = b->dt;
        a.rc2 = (float)(b->r_cut * b->r_cut);
        a.seed = b->seed;
        if (b->skin >= 0.0 && b->nlist) {
            const double rl = b->r_cut + b->skin;
            a.nlist = b->nlist;
            a.ncnt = b->ncnt;
            a.shadow_ref = b->shadow_ref;
            a.list_stats = b->list_stats;
            a.list_gen = b->list_gen;
            a.gen = (int)(b->version & 0x3FFFFFFF);  // a graph is captured per version
            a.kmax = b->kmax;
            // conservative in float32: the list reaches a little past r_cut + skin
            // and a build comes a little before skin/2
            a.rl2 = (float)(rl * rl * (1.0 + 1e-5));
            a.skin_thr2 = (float)(0.25 * b->skin * b->skin * (1.0 - 1e-5));
        }
        const int per_sm = std::max(1, std::min(2048 / k.threads, (int)((228 * 1024) / (smem + 1024))));
        const unsigned grid = (unsigned)std::max(1, std::min(k.count, sms * per_sm));
        void* args[] = {&a};
        cudaStream_t st = (q == 0) ? b->stream : b->stream2;
        CK(cudaLaunchKernel((const void*)b->lib.batch[ki], dim3(grid), dim3(k.threads), args, smem, st));
    }
    if (nb == 2) {
        CK(cudaEventRecord(b->join, b->stream2));
        CK(cudaStreamWaitEvent(b->stream, b->join, 0));
    }
    k_advance_step<<<1, 1, 0, b->stream>>>(b->dstat, steps, 0);
    CK(cudaGetLastError());
    return DP_OK;
}

extern "C" {

int dp_batch_create(int dim, int n_rep, const int32_t* counts, dp_batch** out) {
    if (!out || !counts) return fail(DP_ERR_ARG, "null argument");
    *out = nullptr;
    if (dim < 2 || dim > 4) return fail(DP_ERR_ARG, "dimension must be 2, 3 or 4");
    if (n_rep < 1) return fail(DP_ERR_ARG, "need at least one replica");
    dp_batch* b = new dp_batch();
    b->dim = dim;
    b->n_rep = n_rep;
    b->h_offset.assign((size_t)n_rep + 1, 0);
    for (int r = 0; r < n_rep; ++r) {
        if (counts[r] < 2 || counts[r] > 65535) {
            delete b;
            return fail(DP_ERR_ARG, "replica sizes must be in [2, 65535]");
        }
        b->h_offset[r + 1] = b->h_offset[r] + counts[r];
    }
    b->ntot = b->h_offset[n_rep];
    b->h_order.resize(n_rep);
    for (int r = 0; r < n_rep; ++r) b->h_order[r] = r;
    std::stable_sort(b->h_order.begin(), b->h_order.end(), [&](int x, int y) { return counts[x] > counts[y]; });
    int rc = DP_OK;
    auto cleanup = [&]() {
        dp_batch_destroy(b);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "stream/event creation failed");
        return cleanup();
    }
    const size_t nd = (size_t)b->ntot * dim;
    if ((rc = dalloc_t(&b->pos, nd)) || (rc = dalloc_t(&b->vel, nd)) || (rc = dalloc_t(&b->beta, nd)) ||
        (rc = dalloc_t(&b->stage, nd)) || (rc = dalloc_t(&b->img, nd)) || (rc = dalloc_t(&b->rep_of, b->ntot)) ||
        (rc = dalloc_t(&b->order, (size_t)n_rep)) || (rc = dalloc_t(&b->ncell, (size_t)n_rep * DP_MAX_DIM)) ||
        (rc = dalloc_t(&b->queue, 2)) || (rc = dalloc_t(&b->offset, (size_t)n_rep + 1)) ||
        (rc = dalloc_t(&b->box, (size_t)n_rep * DP_MAX_DIM)) || (rc = dalloc_t(&b->coef, (size_t)n_rep * 5)) ||
        (rc = dalloc_t(&b->obs, (size_t)n_rep * 4)) || (rc = dalloc(&b->shadow, (size_t)b->ntot * (dim == 2 ? 8 : 16))))
        return cleanup();
    if (cudaMalloc(&b->dstat, sizeof(dp_dev_status)) != cudaSuccess ||
        cudaMallocHost(&b->hstat, sizeof(dp_dev_status)) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "status allocation failed");
        return cleanup();
    }
    memset(b->hstat, 0, sizeof(dp_dev_status));
    std::vector<int32_t> rep_of((size_t)b->ntot);
    for (int r = 0; r < n_rep; ++r)
        for (long long i = b->h_offset[r]; i < b->h_offset[r + 1]; ++i) rep_of[i] = r;
    if (cudaMemcpy(b->dstat, b->hstat, sizeof(dp_dev_status), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->rep_of, rep_of.data(), rep_of.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->offset, b->h_offset.data(), b->h_offset.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->order, b->h_order.data(), (size_t)n_rep * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(b->obs, 0, (size_t)n_rep * 4 * 8) != cudaSuccess || cudaMemset(b->img, 0, nd * 4) != cudaSuccess ||
        cudaMemset(b->beta, 0, nd * 8) != cudaSuccess) {
        rc = fail(DP_ERR_CUDA, "batch initialisation failed");
        return cleanup();
    }
    *out = b;
    return DP_OK;
}

int dp_batch_destroy(dp_batch* b) {
    if (!b) return DP_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->stream2) cudaStreamSynchronize(b->stream2);
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    void* bufs[] = {b->pos, b->vel, b->beta, b->stage, b->img, b->rep_of, b->order, b->ncell, b->queue, b->shadow,
                    b->offset, b->box, b->coef, b->obs, b->force_out, b->dstat, b->nlist, b->ncnt, b->shadow_ref,
                    b->list_stats, b->list_gen};
    for (void* p : bufs)
        if (p) cudaFree(p);
    if (b->hstat) cudaFreeHost(b->hstat);
    cudaEvent_t evs[] = {b->ev0, b->ev1, b->fork, b->join};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->stream2) cudaStreamDestroy(b->stream2);
    delete b;
    return DP_OK;
}

int dp_batch_set_state(dp_batch* b, const double* positions, const double* velocities, const double* boxes,
                       const double* temperatures) {
    if (!b || !positions || !velocities || !boxes || !temperatures) return fail(DP_ERR_ARG, "null argument");
    b->h_box.assign((size_t)b->n_rep * DP_MAX_DIM, 1.0);
    b->h_temp.assign(temperatures, temperatures + b->n_rep);
    for (int r = 0; r < b->n_rep; ++r)
        for (int k = 0; k < b->dim; ++k) {
            const double L = boxes[r * b->dim + k];
            if (!(L > 0.0) || !std::isfinite(L)) return fail(DP_ERR_ARG, "box sides must be positive");
            b->h_box[r * DP_MAX_DIM + k] = L;
        }
    const size_t bytes = (size_t)b->ntot * b->dim * sizeof(double);
    CK(cudaMemcpy(b->box, b->h_box.data(), b->h_box.size() * 8, cudaMemcpyHostToDevice));
    const unsigned g = grid_for(b->ntot * b->dim, kBlock);
    CK(cudaMemcpyAsync(b->stage, positions, bytes, cudaMemcpyHostToDevice, b->stream));
    k_host_to_slots<double><<<g, kBlock, 0, b->stream>>>(b->stage, b->pos, nullptr, b->ntot, b->dim);
    CK(cudaMemcpyAsync(b->stage, velocities, bytes, cudaMemcpyHostToDevice, b->stream));
    k_host_to_slots<double><<<g, kBlock, 0, b->stream>>>(b->stage, b->vel, nullptr, b->ntot, b->dim);
    k_batch_shadow<<<grid_for(b->ntot, kBlock), kBlock, 0, b->stream>>>(b->pos, b->shadow, b->rep_of, b->box, b->dim,
                                                                        b->ntot);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(b->stream));
    b->have_state = true;
    if (b->have_pot) RET(batch_configure_cells(b));
    return batch_upload_coef(b);
}

int dp_batch_get_state(dp_batch* b, double* positions, double* velocities, int32_t* images) {
    if (!b) return fail(DP_ERR_ARG, "null handle");
    const size_t bytes = (size_t)b->ntot * b->dim * sizeof(double);
    const unsigned g = grid_for(b->ntot * b->dim, kBlock);
    if (positions) {
        k_slots_to_host<double><<<g, kBlock, 0, b->stream>>>(b->pos, b->stage, nullptr, b->ntot, b->dim);
        CK(cudaMemcpyAsync(positions, b->stage, bytes, cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
    }
    if (velocities) {
        k_slots_to_host<double><<<g, kBlock, 0, b->stream>>>(b->vel, b->stage, nullptr, b->ntot, b->dim);
        CK(cudaMemcpyAsync(velocities, b->stage, bytes, cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
    }
    if (images) {
        int32_t* st = (int32_t*)b->stage;
        k_slots_to_host<int32_t><<<g, kBlock, 0, b->stream>>>(b->img, st, nullptr, b->ntot, b->dim);
        CK(cudaMemcpyAsync(images, st, (size_t)b->ntot * b->dim * 4, cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
    }
    CK(cudaGetLastError());
    return DP_OK;
}

int dp_batch_set_potential(dp_batch* b, const char* device_source, double r_cut) {
    if (!b || !device_source) return fail(DP_ERR_ARG, "null argument");
    if (!(r_cut > 0.0) || !std::isfinite(r_cut)) return fail(DP_ERR_ARG, "r_cut must be positive and finite");
    const std::string src = pair_program(b->dim, DP_PREC_FP32, DP_PAIR_CONST, true, true, device_source, true);
    PairLib pl;
    RET(compile_pair_lib(src, &pl));
    if (!pl.batch[0]) return fail(DP_ERR_NVRTC, "batch kernels missing from the compiled program");
    b->lib = pl;
    b->pot_src = device_source;
    b->r_cut = r_cut;
    b->have_pot = true;
    b->version++;
    if (b->have_state) RET(batch_configure_cells(b));
    return DP_OK;
}

int dp_batch_set_integrator(dp_batch* b, double time_step, double damping_time, double mass, uint64_t seed) {
    if (!b) return fail(DP_ERR_ARG, "null handle");
    if (!(mass > 0.0)) return fail(DP_ERR_ARG, "mass must be positive");
    b->dt = time_step;
    b->tau = damping_time;
    b->mass = mass;
    b->seed = seed;
    return batch_upload_coef(b);
}

int dp_batch_set_launch(dp_batch* b, int split_n, int threads_small, int threads_large) {
    if (!b) return fail(DP_ERR_ARG, "null handle");
    if (batch_kernel_index(threads_small) < 0 || batch_kernel_index(threads_large) < 0)
        return fail(DP_ERR_ARG, "threads per replica must be 128, 256, 512 or 1024");
    b->split_n = std::max(0, split_n);
    b->threads_small = threads_small;
    b->threads_large = threads_large;
    b->version++;
    return DP_OK;
}

// List capacity: 1.3 x the pair count of the densest replica's list sphere +
// 16, or the requested one; a multiple of 8 (the lists are stored in 8-entry
// chunks of 16 bytes).
static int batch_list_capacity(const dp_batch* b) {
    if (b->kmax_req > 0) return std::min((b->kmax_req + 7) & ~7, 65528);
    const double rl = b->r_cut + std::max(0.0, b->skin);
    const double pi = 3.141592653589793;
    const double sphere = b->dim == 2 ? pi * rl * rl : (b->dim == 3 ? 4.0 / 3.0 * pi * rl * rl * rl : 0.5 * pi * pi * rl * rl * rl * rl);
    double rho = 0.0;
    for (int r = 0; r < b->n_rep; ++r) {
        double vol = 1.0;
        for (int k = 0; k < b->dim; ++k) vol *= b->h_box[r * DP_MAX_DIM + k];
        rho = std::max(rho, (double)(b->h_offset[r + 1] - b->h_offset[r]) / vol);
    }
    const long long k = ((long long)std::ceil(1.3 * sphere * rho) + 16 + 7) & ~7LL;
    return (int)std::min<long long>(std::max<long long>(k, 8), 65528);
}

static int batch_ensure_lists(dp_batch* b) {
    if (b->skin < 0.0) return DP_OK;
    const int k = batch_list_capacity(b);
    if (b->nlist && k == b->kmax) return DP_OK;
    if (b->nlist) cudaFree(b->nlist);
    b->nlist = nullptr;
    RET(dalloc_t(&b->nlist, (size_t)b->ntot * (size_t)k));
    if (!b->ncnt) RET(dalloc_t(&b->ncnt, (size_t)b->ntot));
    if (!b->shadow_ref) RET(dalloc(&b->shadow_ref, (size_t)b->ntot * (b->dim == 2 ? 8 : 16)));
    if (!b->list_stats) {
        RET(dalloc_t(&b->list_stats, 2));
        CK(cudaMemset(b->list_stats, 0, 2 * sizeof(unsigned long long)));
    }
    if (!b->list_gen) {
        RET(dalloc_t(&b->list_gen, (size_t)b->n_rep));
        CK(cudaMemset(b->list_gen, 0xFF, (size_t)b->n_rep * sizeof(int32_t)));  // -1: never built
    }
    b->kmax = k;
    b->version++;
    return DP_OK;
}

int dp_batch_run(dp_batch* b, int64_t steps, int sample_every, int nve, int record_forces, float* ms) {
    if (!b) return fail(DP_ERR_ARG, "null handle");
    if (!b->have_state || !b->have_pot) return fail(DP_ERR_NOPOT, "batch state or potential not set");
    if (steps < 0 || steps > (1LL << 30)) return fail(DP_ERR_ARG, "bad step count");
    if (steps == 0) return DP_OK;
    if (record_forces && !b->force_out) RET(dalloc_t(&b->force_out, (size_t)b->ntot * b->dim));
    RET(batch_ensure_lists(b));
    BatchGraph* g = nullptr;
    for (auto& x : b->graphs)
        if (x.steps == steps && x.sample_every == sample_every && x.nve == nve && x.record == record_forces &&
            x.version == b->version)
            g = &x;
    if (!g) {
        for (auto& x : b->graphs) cudaGraphExecDestroy(x.exec);
        b->graphs.clear();
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = batch_record(b, steps, sample_every, nve, record_forces);
        const cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
        if (rc != DP_OK) return rc;
        if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        BatchGraph bg{steps, sample_every, nve, record_forces, b->version, nullptr};
        const cudaError_t ei = cudaGraphInstantiate(&bg.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(DP_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ei));
        b->graphs.push_back(bg);
        g = &b->graphs.back();
    }
    if (ms) CK(cudaEventRecord(b->ev0, b->stream));
    CK(cudaGraphLaunch(g->exec, b->stream));
    if (ms) CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaMemcpyAsync(b->hstat, b->dstat, sizeof(dp_dev_status), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    if (ms) CK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    if (b->hstat->nonfinite) {
        b->hstat->nonfinite = 0;
        CK(cudaMemcpy(b->dstat, b->hstat, sizeof(dp_dev_status), cudaMemcpyHostToDevice));
        return fail(DP_ERR_NONFINITE, "a position became NaN/Inf in a replica");
    }
    return DP_OK;
}

static int nvrtc_check_impl(int dim, int precision, int pair_mode, int with_batch, const char* device_source,
                            int64_t* cubin_bytes, std::string* resource_log) {
    if (!device_source) return fail(DP_ERR_ARG, "null source");
    if (dim < 2 || dim > 4) return fail(DP_ERR_ARG, "dimension must be 2, 3 or 4");
    if (precision != DP_PREC_FP64 && precision != DP_PREC_FP32 && precision != DP_PREC_MLP)
        return fail(DP_ERR_ARG, "unknown precision");
    if (pair_mode < DP_PAIR_CONST || pair_mode > DP_PAIR_DENSE) return fail(DP_ERR_ARG, "unknown pair mode");
    const bool one = pair_mode == DP_PAIR_CONST;
    const std::string src = pair_program(dim, precision, pair_mode, one, one, device_source, with_batch != 0,
                                         step_blocks_for(dim, precision, pair_mode));
    std::vector<char> cubin;
    RET(nvrtc_cubin(src, &cubin, resource_log, true, true));
    if (cubin_bytes) *cubin_bytes = (int64_t)cubin.size();
    return DP_OK;
}

int dp_nvrtc_check(int dim, int precision, int pair_mode, int with_batch, const char* device_source,
                   int64_t* cubin_bytes) {
    return nvrtc_check_impl(dim, precision, pair_mode, with_batch, device_source, cubin_bytes, nullptr);
}

int dp_nvrtc_resources(int dim, int precision, int pair_mode, int with_batch, const char* device_source, char* log,
                       int64_t log_capacity, int64_t* log_bytes) {
    if (!log || log_capacity < 1) return fail(DP_ERR_ARG, "bad log buffer");
    std::string text;
    RET(nvrtc_check_impl(dim, precision, pair_mode, with_batch, device_source, nullptr, &text));
    const size_t len = strnlen(text.c_str(), text.size());
    const size_t k = std::min(len, (size_t)(log_capacity - 1));
    memcpy(log, text.data(), k);
    log[k] = '\0';
    if (log_bytes) *log_bytes = (int64_t)len;
    return DP_OK;
}

int dp_batch_set_neighbor_list(dp_batch* b, double skin, int kmax) {
    if (!b) return fail(DP_ERR_ARG, "null handle");
    if (!std::isfinite(skin)) return fail(DP_ERR_ARG, "skin must be finite");
    if (kmax < 0 || kmax > 65535) return fail(DP_ERR_ARG, "kmax must be in [0, 65535]");
    b->skin = skin < 0.0 ? -1.0 : skin;
    b->kmax_req = kmax;
    b->version++;
    if (b->have_state && b->have_pot) RET(batch_configure_cells(b));
    return DP_OK;
}

int dp_batch_list_stats(dp_batch* b, int64_t* builds, int64_t* overflowed, int32_t* kmax) {
    if (!b) return fail(DP_ERR_ARG, "null handle");
    unsigned long long h[2] = {0, 0};
    if (b->list_stats) CK(cudaMemcpy(h, b->list_stats, sizeof(h), cudaMemcpyDeviceToHost));
    if (builds) *builds = (int64_t)h[0];
    if (overflowed) *overflowed = (int64_t)h[1];
    if (kmax) *kmax = b->skin < 0.0 ? 0 : b->kmax;
    return DP_OK;
}

int dp_batch_observables(dp_batch* b, double* out, int reset) {
    if (!b || !out) return fail(DP_ERR_ARG, "null argument");
    CK(cudaMemcpy(out, b->obs, (size_t)b->n_rep * 4 * sizeof(double), cudaMemcpyDeviceToHost));
    if (reset) CK(cudaMemset(b->obs, 0, (size_t)b->n_rep * 4 * sizeof(double)));
    return DP_OK;
}

int dp_batch_last_forces(dp_batch* b, double* forces) {
    if (!b || !forces) return fail(DP_ERR_ARG, "null argument");
    if (!b->force_out) return fail(DP_ERR_ARG, "no step was run with record_forces");
    std::vector<float> f((size_t)b->ntot * b->dim);
    CK(cudaMemcpy(f.data(), b->force_out, f.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (long long i = 0; i < b->ntot; ++i)
        for (int k = 0; k < b->dim; ++k) forces[i * b->dim + k] = (double)f[(size_t)k * b->ntot + i];
    return DP_OK;
}

}  // extern "C"

// ===========================================================================
// pair surrogate network (training, evaluation)
// ===========================================================================
struct dp_mlp {
    float *master = nullptr, *mo = nullptr, *ve = nullptr, *grad = nullptr, *norm = nullptr, *loss = nullptr;
    unsigned long long* gradfx = nullptr;  // DP_MLP_NPARAM + 1 (the loss last)
    dp_mlp_dev* dev = nullptr;
    float* s = nullptr;
    float2* t = nullptr;
    long long n = 0;
    long long* idx = nullptr;
    long long idx_cap = 0;
    float* losses = nullptr;
    long long losses_cap = 0;
    long long step = 0;
    cudaStream_t stream = nullptr;
};

static int mlp_pack(dp_mlp* m) {
    k_mlp_pack<<<4, 256, 0, m->stream>>>(m->master, m->norm, m->dev);
    CK(cudaGetLastError());
    return DP_OK;
}

static int mlp_grad_launch(dp_mlp* m, const float* s, const float2* t, const long long* idx, long long batch,
                           float wf, bool accurate) {
    MlpTrainArgs a;
    a.s = s;
    a.t = t;
    a.idx = idx;
    a.batch = batch;
    a.mdev = m->dev;
    a.master = m->master;
    a.gradfx = m->gradfx;
    a.lossfx = m->gradfx + DP_MLP_NPARAM;
    a.wf = wf;
    a.inv_batch = 1.0f / (float)batch;
    CK(cudaMemsetAsync(m->gradfx, 0, (DP_MLP_NPARAM + 1) * sizeof(unsigned long long), m->stream));
    const long long tiles = (batch + 15) / 16;
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((tiles + 7) / 8, 152LL * 4));
    if (accurate)
        k_mlp_grad<true><<<grid, 256, DP_MLP_GRAD_SMEM, m->stream>>>(a);
    else
        k_mlp_grad<false><<<grid, 256, DP_MLP_GRAD_SMEM, m->stream>>>(a);
    k_mlp_grad_finish<<<grid_for(DP_MLP_NPARAM, kBlock), kBlock, 0, m->stream>>>(a.gradfx, a.lossfx, m->grad,
                                                                                   m->loss);
    CK(cudaGetLastError());
    return DP_OK;
}

extern "C" {

int dp_mlp_create(dp_mlp** out) {
    if (!out) return fail(DP_ERR_ARG, "null argument");
    *out = nullptr;
    dp_mlp* m = new dp_mlp();
    int rc = DP_OK;
    if ((rc = dalloc_t(&m->master, DP_MLP_NPARAM)) || (rc = dalloc_t(&m->mo, DP_MLP_NPARAM)) ||
        (rc = dalloc_t(&m->ve, DP_MLP_NPARAM)) || (rc = dalloc_t(&m->grad, DP_MLP_NPARAM)) ||
        (rc = dalloc_t(&m->norm, 4)) || (rc = dalloc_t(&m->loss, 1)) || (rc = dalloc_t(&m->dev, 1)) ||
        (rc = dalloc_t(&m->gradfx, DP_MLP_NPARAM + 1))) {
        dp_mlp_destroy(m);
        return rc;
    }
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
        dp_mlp_destroy(m);
        return fail(DP_ERR_CUDA, "stream creation failed");
    }
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, DP_MLP_GRAD_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_grad<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, DP_MLP_GRAD_SMEM);
    if (e != cudaSuccess) {
        dp_mlp_destroy(m);
        return fail(DP_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    }
    *out = m;
    return DP_OK;
}

int dp_mlp_destroy(dp_mlp* m) {
    if (!m) return DP_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    void* bufs[] = {m->master, m->mo, m->ve, m->grad, m->norm, m->loss, m->dev, m->s, m->t, m->idx, m->losses,
                    m->gradfx};
    for (void* p : bufs)
        if (p) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return DP_OK;
}

int dp_mlp_param_count(void) { return DP_MLP_NPARAM; }

int dp_set_mlp(dp_sim* s, dp_mlp* m) {
    if (!s) return fail(DP_ERR_ARG, "null handle");
    if (!m && s->precision == DP_PREC_MLP) return fail(DP_ERR_ARG, "switch precision before detaching the surrogate");
    s->mlp_dev = m ? m->dev : nullptr;
    s->version++;
    return DP_OK;
}

int dp_mlp_set_params(dp_mlp* m, const float* params, const float* norm) {
    if (!m || !params || !norm) return fail(DP_ERR_ARG, "null argument");
    CK(cudaMemcpyAsync(m->master, params, DP_MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemcpyAsync(m->norm, norm, 4 * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemsetAsync(m->mo, 0, DP_MLP_NPARAM * sizeof(float), m->stream));
    CK(cudaMemsetAsync(m->ve, 0, DP_MLP_NPARAM * sizeof(float), m->stream));
    m->step = 0;
    RET(mlp_pack(m));
    CK(cudaStreamSynchronize(m->stream));
    return DP_OK;
}

int dp_mlp_get_params(dp_mlp* m, float* params) {
    if (!m || !params) return fail(DP_ERR_ARG, "null argument");
    CK(cudaMemcpyAsync(params, m->master, DP_MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return DP_OK;
}

int dp_mlp_set_data(dp_mlp* m, const float* s, const float* targets, int64_t n) {
    if (!m || !s || !targets || n < 1) return fail(DP_ERR_ARG, "bad training data");
    RET(dalloc_t(&m->s, (size_t)n));
    RET(dalloc_t(&m->t, (size_t)n));
    CK(cudaMemcpy(m->s, s, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->t, targets, (size_t)n * 2 * sizeof(float), cudaMemcpyHostToDevice));
    m->n = n;
    return DP_OK;
}

int dp_mlp_train(dp_mlp* m, int64_t steps, int batch, float lr0, float lr1, float wf, uint64_t seed, int accurate,
                 float* losses) {
    if (!m || !m->s) return fail(DP_ERR_ARG, "no training data");
    if (steps < 1 || batch < 16) return fail(DP_ERR_ARG, "bad steps / batch");
    if (batch > m->idx_cap) {
        RET(dalloc_t(&m->idx, (size_t)batch));
        m->idx_cap = batch;
    }
    if (steps > m->losses_cap) {
        RET(dalloc_t(&m->losses, (size_t)steps));
        m->losses_cap = steps;
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (long long k = 0; k < steps; ++k) {
        // cosine decay from lr0 to lr1
        const double frac = steps > 1 ? (double)k / (double)(steps - 1) : 1.0;
        const float lr = (float)(lr1 + 0.5 * (lr0 - lr1) * (1.0 + std::cos(3.141592653589793 * frac)));
        k_mlp_sample<<<grid_for(batch, kBlock), kBlock, 0, m->stream>>>(m->idx, batch, m->n, seed, m->step);
        RET(mlp_grad_launch(m, m->s, m->t, m->idx, batch, wf, accurate != 0));
        CK(cudaMemcpyAsync(m->losses + k, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, m->stream));
        ++m->step;
        const float c1 = 1.0f / (1.0f - std::pow(b1, (float)m->step));
        const float c2 = 1.0f / (1.0f - std::pow(b2, (float)m->step));
        k_mlp_adam<<<grid_for(DP_MLP_NPARAM, kBlock), kBlock, 0, m->stream>>>(m->master, m->mo, m->ve, m->grad, lr,
                                                                               b1, b2, eps, c1, c2);
        RET(mlp_pack(m));
    }
    CK(cudaGetLastError());
    if (losses) CK(cudaMemcpyAsync(losses, m->losses, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return DP_OK;
}

int dp_mlp_eval(dp_mlp* m, const float* s, int64_t n, float* y, int accurate) {
    if (!m || !s || !y || n < 1) return fail(DP_ERR_ARG, "bad arguments");
    float* buf = nullptr;
    RET(dalloc_t(&buf, (size_t)n * 3));
    cudaError_t e = cudaMemcpyAsync(buf, s, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream);
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>(((n + 15) / 16 + 7) / 8, 152LL * 8));
    if (e == cudaSuccess) {
        if (accurate)
            k_mlp_eval<true><<<grid, 256, 0, m->stream>>>(buf, n, m->dev, buf + n);
        else
            k_mlp_eval<false><<<grid, 256, 0, m->stream>>>(buf, n, m->dev, buf + n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, buf + n, (size_t)n * 2 * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("dp_mlp_eval: ") + cudaGetErrorString(e));
    return DP_OK;
}

int dp_mlp_gradients(dp_mlp* m, const float* s, const float* targets, int64_t n, float wf, int accurate, float* grad,
                     float* loss) {
    if (!m || !s || !targets || !grad || n < 1) return fail(DP_ERR_ARG, "bad arguments");
    // targets are read as float2: start them on an 8-byte boundary
    const long long toff = (n + 1) & ~1LL;
    float* buf = nullptr;
    RET(dalloc_t(&buf, (size_t)(toff + 2 * n)));
    cudaError_t e = cudaMemcpyAsync(buf, s, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(buf + toff, targets, (size_t)n * 2 * sizeof(float), cudaMemcpyHostToDevice, m->stream);
    int rc = DP_OK;
    if (e == cudaSuccess) rc = mlp_grad_launch(m, buf, (const float2*)(buf + toff), nullptr, n, wf, accurate != 0);
    if (e == cudaSuccess && rc == DP_OK)
        e = cudaMemcpyAsync(grad, m->grad, DP_MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    float l = 0.f;
    if (e == cudaSuccess && rc == DP_OK) e = cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(buf);
    if (rc != DP_OK) return rc;
    if (e != cudaSuccess) return fail(DP_ERR_CUDA, std::string("dp_mlp_gradients: ") + cudaGetErrorString(e));
    if (loss) *loss = l / (float)n;
    return DP_OK;
}

}  // extern "C"
