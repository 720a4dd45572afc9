// batch_kernels.cuh — thousands of independent replicas in one persistent
// kernel (compiled by NVRTC together with pair_kernels.cuh and the generated
// pair potential).
//
// Each CTA takes a replica from a work queue (largest first) and runs all
// `steps` steps of it before taking the next, so replicas never wait on one
// another. Per step, inside the CTA:
//   0. skin test against the positions of the replica's last list build;
//   1. when a build is due (or the host changed anything since): cell
//      binning in shared memory — the fixed-point positions counting-sorted
//      into cells at least r_cut + skin wide, or kept in index order when a
//      box has fewer than 3 cells per axis (all pairs) — and a Verlet list per
//      particle (16-bit local indices in 16-byte chunks of 8, the chunks
//      column-major in HBM); a replica whose
//      list would overflow its capacity uses the 27-cell stencil for the rest
//      of the launch (binning every step), so no pair is ever missed;
//   2. pair forces in float32 from the fixed-point displacements of the
//      listed partners, the replica's positions read from shared memory;
//   3. G-JF (or NVE) leap-frog as dompap/integrator.py:17-40 (deterministic
//      part float64, noise terms float32 as in dp_integrate.cuh), wrap
//      as dompap/positions.py:90-98, new fixed-point position to HBM.
// Every `sample_every` steps the CTA adds U, W and sum m v^2 of the replica to
// its observable slots (float64).

__device__ __forceinline__ int dp_batch_block_scan(int* cnt, int nc, int* warp_tot) {
    // exclusive scan of cnt[0..nc) in place, blockDim.x threads; returns the total
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int carry = 0;
    for (int base = 0; base < nc; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int v = c < nc ? cnt[c] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < nw) warp_tot[lane] = w;  // inclusive warp totals
        }
        __syncthreads();
        const int before = (warp > 0 ? warp_tot[warp - 1] : 0) + carry;
        if (c < nc) cnt[c] = before + x - v;
        carry += warp_tot[nw - 1];
        __syncthreads();
    }
    return carry;
}

// visit(q) for every binned slot q != slot of the (2 R + 1)^D cells around
// the particle in `slot`. Cells are numbered with the last axis fastest, so the
// 2 R + 1 cells of a stencil row along it hold consecutive slots: the walk
// takes (2 R + 1)^(D-1) rows, each one slot range (two where the row wraps
// around the box). The stencil width is a compile-time constant, so the digits
// of the row index are taken by multiplications, not divisions; a box has at
// least 2 R + 1 cells per axis, so one conditional subtraction wraps a cell.
template <int D, int R, typename Visit>
__device__ __forceinline__ void dp_batch_stencil_cells(int slot, const uint32_t* up, const int* nc, const int* s_start,
                                                       Visit& visit) {
    constexpr int span = 2 * R + 1;
    int rows = 1;
#pragma unroll
    for (int k = 0; k + 1 < D; ++k) rows *= span;
    int lo[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const int c = (int)__umulhi(up[k], (uint32_t)nc[k]) - R;
        lo[k] = c < 0 ? c + nc[k] : c;
    }
    const int nl = nc[D - 1];
    const int a = lo[D - 1];         // first cell of a row along the last axis
    const int b = a + 2 * R;         // last one, before the wrap
    for (int s = 0; s < rows; ++s) {
        int rem = s, base = 0;
#pragma unroll
        for (int k = 0; k + 1 < D; ++k) {
            int cc = lo[k] + rem % span;
            rem /= span;
            cc -= (cc >= nc[k]) ? nc[k] : 0;
            base = base * nc[k] + cc;
        }
        base *= nl;
        // cells a..b of the row (b < nl) or a..nl-1 and 0..b-nl
        const int e1 = s_start[base + min(b, nl - 1) + 1];
        for (int q = s_start[base + a]; q < e1; ++q)
            if (q != slot) visit(q);
        if (b >= nl) {
            const int e2 = s_start[base + (b - nl) + 1];
            for (int q = s_start[base]; q < e2; ++q)
                if (q != slot) visit(q);
        }
    }
}

// visit(q) for every binned slot q != slot of the (2 reach + 1)^D cells
// around the particle in `slot` (all slots when the box has no cells). Cells
// are at least cutoff / reach wide, so the stencil covers the cutoff sphere.
template <int D, typename Visit>
__device__ __forceinline__ void dp_batch_stencil(bool cells, int reach, int slot, const uint32_t* up, const int* nc,
                                                 const int* s_start, int n, Visit& visit) {
    if (cells) {
        if (reach == 2)
            dp_batch_stencil_cells<D, 2>(slot, up, nc, s_start, visit);
        else
            dp_batch_stencil_cells<D, 1>(slot, up, nc, s_start, visit);
    } else {
        for (int q = 0; q < n; ++q)
            if (q != slot) visit(q);
    }
}

template <int THREADS>
__device__ __forceinline__ void dp_batch_steps(const dp_batch_args& a) {
    constexpr int D = DP_DIM;
    typedef typename dp_shadow_t<D>::type sh_t;
    extern __shared__ __align__(16) unsigned char dp_smem[];
    sh_t* s_sh = (sh_t*)dp_smem;                                  // [max_n] positions (by cell while binned)
    unsigned short* s_idx = (unsigned short*)(s_sh + a.max_n);     // [max_n] local index of each binned slot
    int* s_start = (int*)(s_idx + ((a.max_n + 7) & ~7));           // [max_cells + 1]
    int* s_cur = s_start + a.max_cells + 1;                        // [max_cells]
    __shared__ int s_rep;
    __shared__ int s_warp[32];
    __shared__ double s_red[32];
    sh_t* gsh = (sh_t*)a.shadow;
    sh_t* gref = (sh_t*)a.shadow_ref;
    const long long ntot = a.ntot;

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_rep = atomicAdd(a.queue, 1);
        __syncthreads();
        if (s_rep >= a.n_rep) return;
        const int r = a.order[s_rep];
        const long long off = a.offset[r];
        const int n = (int)(a.offset[r + 1] - off);
        double L[D], scale[D];
        float unit[D];
        int nc[D];
        bool cells = true;
        int ncell = 1;
        // ncell < 0: cells cutoff/2 wide (5^D stencil), > 0: cutoff wide (3^D)
        const int reach = a.ncell[r * DP_MAX_DIM] < 0 ? 2 : 1;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            L[k] = a.box[r * DP_MAX_DIM + k];
            scale[k] = 4294967296.0 / L[k];
            unit[k] = (float)(L[k] / 4294967296.0);
            nc[k] = abs(a.ncell[r * DP_MAX_DIM + k]);
            cells = cells && nc[k] >= 2 * reach + 1;
            ncell *= max(nc[k], 1);
        }
        double c[5];
#pragma unroll
        for (int t = 0; t < 5; ++t) c[t] = a.coef[r * 5 + t];
        // the noise terms in float32, as the single-system integrator
        const float c2f = (float)c[2], c3f = (float)c[3];
        // list of this replica: chunk c of particle p at [(c n + p) 8]
        uint16_t* __restrict__ nl = a.nlist ? a.nlist + off * (long long)a.kmax : nullptr;
        bool use_list = nl != nullptr;  // cleared for the rest of the launch if the list overflows

        const long long step0 = a.st->step;  // advanced by the host-side graph after this launch
        for (int step = 0; step < a.steps; ++step) {
            const long long gstep = step0 + step;
            const bool sample = a.sample_every > 0 && ((gstep + 1) % a.sample_every) == 0;
            // ---- 0. list check: a build when the list is of an older
            // generation (the host changed state or settings since) or some
            // particle moved more than skin/2 since the build
            bool build = false;
            if (use_list) {
                int moved = a.list_gen[r] != a.gen;
                for (int p = threadIdx.x; p < n && !moved; p += THREADS) {
                    uint32_t u[D], u0[D];
                    dp_shadow_unpack<D>(gsh[off + p], u);
                    dp_shadow_unpack<D>(gref[off + p], u0);
                    float df[D];
                    moved = dp_shadow_q<D>(u, u0, unit, df) > a.skin_thr2;
                }
                build = __syncthreads_or(moved);
            }
            // ---- 1. binning (every step without a list, else for a build)
            if (!use_list || build) {
                if (cells) {
                    for (int q = threadIdx.x; q < ncell; q += THREADS) s_start[q] = 0;
                    __syncthreads();
                    for (int p = threadIdx.x; p < n; p += THREADS) {
                        uint32_t u[D];
                        dp_shadow_unpack<D>(gsh[off + p], u);
                        int l = 0;
#pragma unroll
                        for (int k = 0; k < D; ++k) l = l * nc[k] + (int)__umulhi(u[k], (uint32_t)nc[k]);
                        atomicAdd(s_start + l, 1);
                    }
                    __syncthreads();
                    dp_batch_block_scan(s_start, ncell, s_warp);
                    for (int q = threadIdx.x; q < ncell; q += THREADS) s_cur[q] = s_start[q];
                    if (threadIdx.x == 0) s_start[ncell] = n;
                    __syncthreads();
                    for (int p = threadIdx.x; p < n; p += THREADS) {
                        const sh_t v = gsh[off + p];
                        uint32_t u[D];
                        dp_shadow_unpack<D>(v, u);
                        int l = 0;
#pragma unroll
                        for (int k = 0; k < D; ++k) l = l * nc[k] + (int)__umulhi(u[k], (uint32_t)nc[k]);
                        const int slot = atomicAdd(s_cur + l, 1);
                        s_sh[slot] = v;
                        s_idx[slot] = (unsigned short)p;
                    }
                } else {
                    for (int p = threadIdx.x; p < n; p += THREADS) {
                        s_sh[p] = gsh[off + p];
                        s_idx[p] = (unsigned short)p;
                    }
                }
                __syncthreads();
            }
            // ---- 1b. list build from the binned positions
            if (use_list && build) {
                bool overflow = false;
                for (int slot = threadIdx.x; slot < n; slot += THREADS) {
                    uint32_t up[D];
                    dp_shadow_unpack<D>(s_sh[slot], up);
                    const int p = s_idx[slot];
                    int cnt = 0;
                    auto add = [&](int q) {
                        uint32_t uq[D];
                        dp_shadow_unpack<D>(s_sh[q], uq);
                        float df[D];
                        if (dp_shadow_q<D>(up, uq, unit, df) <= a.rl2) {
                            // 8-entry chunks: chunk c of particle p at [(c n + p) 8]
                            if (cnt < a.kmax) nl[((long long)(cnt >> 3) * n + p) * 8 + (cnt & 7)] = s_idx[q];
                            ++cnt;
                        }
                    };
                    dp_batch_stencil<D>(cells, reach, slot, up, nc, s_start, n, add);
                    overflow = overflow || cnt > a.kmax;
                    a.ncnt[off + p] = min(cnt, a.kmax);
                    gref[off + p] = s_sh[slot];
                }
                if (__syncthreads_or(overflow)) {
                    use_list = false;  // the binning is in place: this step uses the stencil
                    if (threadIdx.x == 0) atomicAdd(a.list_stats + 1, 1ull);
                } else if (threadIdx.x == 0) {
                    atomicAdd(a.list_stats, 1ull);
                    a.list_gen[r] = a.gen;
                }
                if (use_list) {
                    // positions back in local order for the list loop
                    for (int p = threadIdx.x; p < n; p += THREADS) s_sh[p] = gsh[off + p];
                    __syncthreads();
                }
            } else if (use_list) {
                for (int p = threadIdx.x; p < n; p += THREADS) s_sh[p] = gsh[off + p];
                __syncthreads();
            }
            // ---- 2. forces (float32) and 3. integration (float64)
            double accU = 0.0, accW = 0.0, accK = 0.0;
            for (int slot = threadIdx.x; slot < n; slot += THREADS) {
                // list mode: slot = local index; stencil mode: binned slot
                uint32_t up[D];
                dp_shadow_unpack<D>(s_sh[slot], up);
                float f[D];
#pragma unroll
                for (int k = 0; k < D; ++k) f[k] = 0.0f;
                float eu = 0.0f, ew = 0.0f;
                auto pair = [&](int q) {
                    uint32_t uq[D];
                    dp_shadow_unpack<D>(s_sh[q], uq);
                    float df[D];
                    const float q2 = dp_shadow_q<D>(up, uq, unit, df);
                    if (q2 <= a.rc2) {
                        const float rinv = rsqrtf(q2);
                        const float rr = q2 * rinv;
                        const float sf = dp_pair_f<float>(rr, rinv);
                        const float g = sf * rinv;
#pragma unroll
                        for (int k = 0; k < D; ++k) f[k] = fmaf(g, df[k], f[k]);
                        if (sample) {
                            eu += dp_pair_u<float>(rr, rinv);
                            ew += sf * rr;
                        }
                    }
                };
                int p;
                if (use_list) {
                    p = slot;
                    const int cnt = a.ncnt[off + p];
                    // one 16-byte load per 8 entries, two chunks ahead of the
                    // pairs being evaluated
                    const uint4* __restrict__ rowc = (const uint4*)nl + p;
                    const int nch = (cnt + 7) >> 3;
                    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
                    uint4 c1 = nch > 0 ? __ldg(rowc) : zero;
                    uint4 c2 = nch > 1 ? __ldg(rowc + n) : zero;
                    for (int ch = 0; ch < nch; ++ch) {
                        const uint4 cur = c1;
                        c1 = c2;
                        c2 = ch + 2 < nch ? __ldg(rowc + (long long)(ch + 2) * n) : zero;
                        const int m = cnt - 8 * ch;
                        const uint32_t w[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                            if (e < m) pair((int)((w[e >> 1] >> (16 * (e & 1))) & 0xFFFFu));
                    }
                } else {
                    p = s_idx[slot];
                    dp_batch_stencil<D>(cells, reach, slot, up, nc, s_start, n, pair);
                }
                // integrate particle i (float64)
                const long long i = off + p;
                float z[4];
                if (!a.nve) dp_normals4(a.seed, (unsigned long long)gstep, (uint32_t)i, z);
                uint32_t un[D];
                double ke = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const long long o = k * ntot + i;
                    double v = a.vel[o];
                    double x = a.pos[o];
                    const double F = (double)f[k];
                    if (a.nve) {
                        v = v + c[4] * F;
                    } else {
                        const float bn = __fmul_rn(c3f, z[k]);
                        const float noise = __fmul_rn(c2f, __fadd_rn(dp_d2f_trunc(a.beta[o]), bn));
                        v = fma(c[1], F, fma(c[0], v, dp_f2d(noise)));
                        a.beta[o] = dp_f2d(bn);
                    }
                    x = x + v * a.dt;
                    const long long t = __double2ll_rd(x * scale[k]);
                    if (t < 0 || t >= 4294967296LL) {
                        if (!(x >= 0.0 && x < L[k])) {
                            const double sh = floor(x / L[k]);
                            a.img[o] += (int32_t)sh;
                            x -= sh * L[k];
                        }
                        un[k] = dp_fixed(x, scale[k]);
                        if (!isfinite(x)) atomicExch(&a.st->nonfinite, 1);
                    } else {
                        un[k] = (uint32_t)t;
                    }
                    a.vel[o] = v;
                    a.pos[o] = x;
                    ke += v * v;
                    if (a.force_out) a.force_out[o] = f[k];
                }
                gsh[i] = dp_shadow_pack<D>(un);
                if (sample) {
                    accU += (double)eu;
                    accW += (double)ew;
                    accK += ke / c[4] * a.dt;  // m |v|^2 with m = dt / (dt/m)
                }
            }
            __syncthreads();
            if (sample) {
                const double U = dp_block_sum(accU, s_red);
                __syncthreads();
                const double W = dp_block_sum(accW, s_red);
                __syncthreads();
                const double K = dp_block_sum(accK, s_red);
                if (threadIdx.x == 0) {
                    a.obs[r * 4 + 0] += 0.5 * U;
                    a.obs[r * 4 + 1] += 0.5 * W / D;
                    a.obs[r * 4 + 2] += K;
                    a.obs[r * 4 + 3] += 1.0;
                }
                __syncthreads();
            }
        }
    }
}

extern "C" __global__ void __launch_bounds__(128) dp_batch_steps_128(dp_batch_args a) { dp_batch_steps<128>(a); }
extern "C" __global__ void __launch_bounds__(256) dp_batch_steps_256(dp_batch_args a) { dp_batch_steps<256>(a); }
extern "C" __global__ void __launch_bounds__(512) dp_batch_steps_512(dp_batch_args a) { dp_batch_steps<512>(a); }
extern "C" __global__ void __launch_bounds__(1024) dp_batch_steps_1024(dp_batch_args a) { dp_batch_steps<1024>(a); }
