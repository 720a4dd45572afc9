// mlp_train.cuh — training and batch evaluation of the pair surrogate
// (statically compiled; included by dompap_gpu.cu after mlp_common.cuh).
//
// Parameters (fp32 masters, flat, DP_MLP_NPARAM): w1[64], b1[64],
// W2[64][64] (row = output unit), b2[64], W3[2][64], b3[2]. The forward pass
// uses bf16-rounded W2 (the tensor-core operand; quantisation-aware
// training) and fp32 biases; w1 and W3 feed float32 FMAs and stay fp32 unless
// DP_MLP_SCALAR_BF16 is 1. Loss per sample: (y0 - t0)^2 + wf (y1 - t1)^2,
// averaged over the batch.
#pragma once

#ifndef DP_MLP_SCALAR_BF16
#define DP_MLP_SCALAR_BF16 0
#endif

#define DP_MLP_NPARAM (64 + 64 + 64 * 64 + 64 + 2 * 64 + 2)
#define DP_MLP_OFF_W1 0
#define DP_MLP_OFF_B1 64
#define DP_MLP_OFF_W2 128
#define DP_MLP_OFF_B2 (128 + 4096)
#define DP_MLP_OFF_W3 (128 + 4096 + 64)
#define DP_MLP_OFF_B3 (128 + 4096 + 64 + 128)

__device__ __forceinline__ float dp_round_bf16(float v) {
    const uint32_t p = dp_pack_bf16(v, 0.0f);
    return dp_bf16_lo_as_float(p);
}

// masters + normalisation -> the device struct used by every forward pass
__global__ void k_mlp_pack(const float* __restrict__ p, const float* __restrict__ norm, dp_mlp_dev* m) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 64) {
        const float w1 = p[DP_MLP_OFF_W1 + t], w30 = p[DP_MLP_OFF_W3 + t], w31 = p[DP_MLP_OFF_W3 + 64 + t];
        m->w1[t] = DP_MLP_SCALAR_BF16 ? dp_round_bf16(w1) : w1;
        m->b1[t] = p[DP_MLP_OFF_B1 + t];
        m->b2[t] = p[DP_MLP_OFF_B2 + t];
        m->w3[0][t] = DP_MLP_SCALAR_BF16 ? dp_round_bf16(w30) : w30;
        m->w3[1][t] = DP_MLP_SCALAR_BF16 ? dp_round_bf16(w31) : w31;
    }
    if (t < 2) m->b3[t] = p[DP_MLP_OFF_B3 + t];
    if (t == 0) {
        m->x_mean = norm[0];
        m->x_inv_scale = norm[1];
        m->u_scale = norm[2];
        m->f_scale = norm[3];
    }
    // B fragments of W2: [kt][nt][lane][2]; B[k][n] = W2[n][k]
    if (t < 4 * 8 * 32) {
        const int lane = t & 31, nt = (t >> 5) & 7, kt = t >> 8;
        const int n = nt * 8 + (lane >> 2), k = kt * 16 + 2 * (lane & 3);
        const float* w = p + DP_MLP_OFF_W2 + n * 64;
        m->w2frag[t * 2 + 0] = dp_pack_bf16(w[k], w[k + 1]);
        m->w2frag[t * 2 + 1] = dp_pack_bf16(w[k + 8], w[k + 9]);
    }
}

// y (n x 2) for inputs s (n); 8 warps per block, 16 samples per warp tile.
template <bool ACCURATE>
__global__ void __launch_bounds__(256) k_mlp_eval(const float* __restrict__ s, long long n, const dp_mlp_dev* mdev,
                                                   float* __restrict__ y) {
    __shared__ dp_mlp_dev m;
    dp_mlp_load(&m, mdev);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2;
    const long long tiles = (n + 15) / 16;
    for (long long tile = (long long)blockIdx.x * 8 + (threadIdx.x >> 5); tile < tiles; tile += (long long)gridDim.x * 8) {
        const long long r0 = tile * 16 + g, r1 = r0 + 8;
        const float sg = r0 < n ? s[r0] : m.x_mean;
        const float sg8 = r1 < n ? s[r1] : m.x_mean;
        float out[2][2];
        dp_mlp_tile<ACCURATE>(m, sg, sg8, out);
        if ((lane & 3) == 0) {
            if (r0 < n) {
                y[2 * r0] = out[0][0];
                y[2 * r0 + 1] = out[0][1];
            }
            if (r1 < n) {
                y[2 * r1] = out[1][0];
                y[2 * r1 + 1] = out[1][1];
            }
        }
    }
}

// Gradient of the batch loss: forward on tensor cores (as inference), the
// backward GEMMs dW2 = dZ2^T H1 and dH1 = dZ2 W2 as bf16 mma.sync with fp32
// accumulation. Every sum across warps and CTAs is taken in 64-bit fixed
// point (integer adds are exact, so the result does not depend on the order
// of the atomics and training is reproducible for a seed): per-CTA sums in
// shared memory, then one atomic per parameter into gradfx[];
// k_mlp_grad_finish turns them into float. Samples: s[idx[b]] (idx null: b)
// for b < batch.
struct MlpTrainArgs {
    const float* s;
    const float2* t;
    const long long* idx;
    long long batch;
    const dp_mlp_dev* mdev;
    const float* master;               // fp32 W2 for the backward product
    unsigned long long* gradfx;        // DP_MLP_NPARAM, fixed point 2^DP_MLP_GRAD_FX_BITS
    unsigned long long* lossfx;        // sum of per-sample losses, fixed point 2^DP_MLP_LOSS_FX_BITS
    float wf;
    float inv_batch;
};

#define DP_MLP_GRAD_FX_BITS 36
#define DP_MLP_LOSS_FX_BITS 32

// v as a two's-complement fixed-point integer 2^BITS v (saturating; a
// gradient beyond 2^(63-BITS) means the training has diverged anyway).
template <int BITS>
__device__ __forceinline__ unsigned long long dp_fx(float v) {
    return (unsigned long long)__float2ll_rn(v * (float)(1ull << BITS));
}

template <int BITS>
__device__ __forceinline__ void dp_fx_add(unsigned long long* p, float v) {
    atomicAdd(p, dp_fx<BITS>(v));
}

// dynamic shared memory of k_mlp_grad (bytes)
#define DP_MLP_GRAD_SMEM (64 * 64 * 8 + 64 * 64 * 2 + 8 * 2 * 16 * 64 * 2)

template <bool ACCURATE>
__global__ void __launch_bounds__(256) k_mlp_grad(MlpTrainArgs a) {
    __shared__ dp_mlp_dev m;
    __shared__ unsigned long long gsmall[64 * 4 + 128 + 2 + 1];  // gw1, gb1, gb2, (unused), gw3, gb3, loss
    extern __shared__ __align__(16) unsigned char dp_grad_smem[];
    unsigned long long* gW2 = (unsigned long long*)dp_grad_smem;            // [n][k] fixed point
    __nv_bfloat16* w2s = (__nv_bfloat16*)(gW2 + 64 * 64);                   // [n][k]
    __nv_bfloat16* stage = w2s + 64 * 64;                                    // [warp][2][16 * 64]
    dp_mlp_load(&m, a.mdev);
    for (int t = threadIdx.x; t < 64 * 64; t += blockDim.x) {
        gW2[t] = 0ull;
        w2s[t] = __float2bfloat16_rn(a.master[DP_MLP_OFF_W2 + t]);
    }
    for (int t = threadIdx.x; t < 64 * 4 + 128 + 3; t += blockDim.x) gsmall[t] = 0ull;
    __syncthreads();
    constexpr int GB = DP_MLP_GRAD_FX_BITS;
    unsigned long long* gw1 = gsmall;
    unsigned long long* gb1 = gsmall + 64;
    unsigned long long* gb2 = gsmall + 128;
    unsigned long long* gw3 = gsmall + 256;
    unsigned long long* gb3 = gsmall + 256 + 128;
    unsigned long long* gloss = gsmall + 256 + 130;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, c = 2 * (lane & 3);
    __nv_bfloat16* sdz = stage + (warp * 2 + 0) * 16 * 64;
    __nv_bfloat16* sh1 = stage + (warp * 2 + 1) * 16 * 64;
    const long long tiles = (a.batch + 15) / 16;
    for (long long tile = (long long)blockIdx.x * 8 + warp; tile < tiles; tile += (long long)gridDim.x * 8) {
        const long long b0 = tile * 16 + g, b1 = b0 + 8;
        const bool v0 = b0 < a.batch, v1 = b1 < a.batch;
        const long long i0 = v0 ? (a.idx ? a.idx[b0] : b0) : 0, i1 = v1 ? (a.idx ? a.idx[b1] : b1) : 0;
        const float sg = v0 ? a.s[i0] : m.x_mean, sg8 = v1 ? a.s[i1] : m.x_mean;
        const float xg = (sg - m.x_mean) * m.x_inv_scale, xg8 = (sg8 - m.x_mean) * m.x_inv_scale;
        uint32_t ahi[4][4], alo[4][4];
        dp_mlp_layer1<ACCURATE>(m, xg, xg8, ahi, alo);
        float z2[8][4];
        dp_mlp_layer2(m, ahi, alo, z2);
        float h2[8][4];
        float p00 = 0.f, p01 = 0.f, p10 = 0.f, p11 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) h2[nt][e] = dp_mlp_act<ACCURATE>(z2[nt][e]);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int col = nt * 8 + c + e;
                p00 = fmaf(h2[nt][e], m.w3[0][col], p00);
                p01 = fmaf(h2[nt][e], m.w3[1][col], p01);
                p10 = fmaf(h2[nt][2 + e], m.w3[0][col], p10);
                p11 = fmaf(h2[nt][2 + e], m.w3[1][col], p11);
            }
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
            p00 += __shfl_xor_sync(0xffffffffu, p00, o);
            p01 += __shfl_xor_sync(0xffffffffu, p01, o);
            p10 += __shfl_xor_sync(0xffffffffu, p10, o);
            p11 += __shfl_xor_sync(0xffffffffu, p11, o);
        }
        const float2 t0 = v0 ? a.t[i0] : make_float2(0.f, 0.f), t1 = v1 ? a.t[i1] : make_float2(0.f, 0.f);
        const float e00 = v0 ? p00 + m.b3[0] - t0.x : 0.f, e01 = v0 ? p01 + m.b3[1] - t0.y : 0.f;
        const float e10 = v1 ? p10 + m.b3[0] - t1.x : 0.f, e11 = v1 ? p11 + m.b3[1] - t1.y : 0.f;
        if ((lane & 3) == 0)
            dp_fx_add<DP_MLP_LOSS_FX_BITS>(gloss, e00 * e00 + a.wf * e01 * e01 + e10 * e10 + a.wf * e11 * e11);
        // dL/dy (mean over the batch)
        const float d00 = 2.f * e00 * a.inv_batch, d01 = 2.f * a.wf * e01 * a.inv_batch;
        const float d10 = 2.f * e10 * a.inv_batch, d11 = 2.f * a.wf * e11 * a.inv_batch;
        // gb3: sum over the 16 rows (one quad lane per group contributes)
        float sb30 = (lane & 3) == 0 ? d00 + d10 : 0.f, sb31 = (lane & 3) == 0 ? d01 + d11 : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sb30 += __shfl_xor_sync(0xffffffffu, sb30, o);
            sb31 += __shfl_xor_sync(0xffffffffu, sb31, o);
        }
        if (lane == 0) {
            dp_fx_add<GB>(gb3, sb30);
            dp_fx_add<GB>(gb3 + 1, sb31);
        }
        // dz2 = (dy0 w3[0] + dy1 w3[1]) * act'(z2); gw3, gb2 partial sums
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int col = nt * 8 + c + e;
                const float hg = h2[nt][e], hg8 = h2[nt][2 + e];
                float gw30 = d00 * hg + d10 * hg8, gw31 = d01 * hg + d11 * hg8;
                const float dzg = (d00 * m.w3[0][col] + d01 * m.w3[1][col]) * (1.f - hg * hg);
                const float dzg8 = (d10 * m.w3[0][col] + d11 * m.w3[1][col]) * (1.f - hg8 * hg8);
                float gbb = dzg + dzg8;
                // sum over the 8 groups (lanes with equal lane & 3)
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) {
                    gw30 += __shfl_xor_sync(0xffffffffu, gw30, o);
                    gw31 += __shfl_xor_sync(0xffffffffu, gw31, o);
                    gbb += __shfl_xor_sync(0xffffffffu, gbb, o);
                }
                if (g == 0) {
                    dp_fx_add<GB>(gw3 + col, gw30);
                    dp_fx_add<GB>(gw3 + 64 + col, gw31);
                    dp_fx_add<GB>(gb2 + col, gbb);
                }
                sdz[g * 64 + col] = __float2bfloat16_rn(dzg);
                sdz[(g + 8) * 64 + col] = __float2bfloat16_rn(dzg8);
            }
        // h1 (fp32 recomputed, stored bf16) in [row][k]
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int half = 0; half < 2; ++half)
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int k = kt * 16 + c + 8 * half + e;
                    sh1[g * 64 + k] = __float2bfloat16_rn(dp_mlp_act<ACCURATE>(fmaf(m.w1[k], xg, m.b1[k])));
                    sh1[(g + 8) * 64 + k] = __float2bfloat16_rn(dp_mlp_act<ACCURATE>(fmaf(m.w1[k], xg8, m.b1[k])));
                }
        __syncwarp();
        // dW2[n][k] += sum_rows dz2[row][n] h1[row][k]: M = n (4 tiles), N = k (8 tiles), K = 16 rows
        const uint16_t* dz16 = (const uint16_t*)sdz;
        const uint16_t* h116 = (const uint16_t*)sh1;
#pragma unroll
        for (int mt = 0; mt < 4; ++mt) {
            uint32_t af[4];
            const int n0 = mt * 16 + g;
            af[0] = (uint32_t)dz16[c * 64 + n0] | ((uint32_t)dz16[(c + 1) * 64 + n0] << 16);
            af[1] = (uint32_t)dz16[c * 64 + n0 + 8] | ((uint32_t)dz16[(c + 1) * 64 + n0 + 8] << 16);
            af[2] = (uint32_t)dz16[(c + 8) * 64 + n0] | ((uint32_t)dz16[(c + 9) * 64 + n0] << 16);
            af[3] = (uint32_t)dz16[(c + 8) * 64 + n0 + 8] | ((uint32_t)dz16[(c + 9) * 64 + n0 + 8] << 16);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int k0 = nt * 8 + g;
                const uint32_t bb0 = (uint32_t)h116[c * 64 + k0] | ((uint32_t)h116[(c + 1) * 64 + k0] << 16);
                const uint32_t bb1 = (uint32_t)h116[(c + 8) * 64 + k0] | ((uint32_t)h116[(c + 9) * 64 + k0] << 16);
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                dp_mma_bf16(acc, af, bb0, bb1);
                const int row = mt * 16 + g, col = nt * 8 + c;
                dp_fx_add<GB>(gW2 + row * 64 + col, acc[0]);
                dp_fx_add<GB>(gW2 + row * 64 + col + 1, acc[1]);
                dp_fx_add<GB>(gW2 + (row + 8) * 64 + col, acc[2]);
                dp_fx_add<GB>(gW2 + (row + 8) * 64 + col + 1, acc[3]);
            }
        }
        // dh1[row][k] = sum_n dz2[row][n] W2[n][k]: M = rows, N = k, K = n (4 k-steps)
        const uint16_t* w216 = (const uint16_t*)w2s;
        float dh1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            dh1[nt][0] = dh1[nt][1] = dh1[nt][2] = dh1[nt][3] = 0.f;
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                uint32_t af[4];
                const int nn = kt * 16 + c;
                af[0] = (uint32_t)dz16[g * 64 + nn] | ((uint32_t)dz16[g * 64 + nn + 1] << 16);
                af[1] = (uint32_t)dz16[(g + 8) * 64 + nn] | ((uint32_t)dz16[(g + 8) * 64 + nn + 1] << 16);
                af[2] = (uint32_t)dz16[g * 64 + nn + 8] | ((uint32_t)dz16[g * 64 + nn + 9] << 16);
                af[3] = (uint32_t)dz16[(g + 8) * 64 + nn + 8] | ((uint32_t)dz16[(g + 8) * 64 + nn + 9] << 16);
                const int k = nt * 8 + g;
                const uint32_t bb0 = (uint32_t)w216[nn * 64 + k] | ((uint32_t)w216[(nn + 1) * 64 + k] << 16);
                const uint32_t bb1 = (uint32_t)w216[(nn + 8) * 64 + k] | ((uint32_t)w216[(nn + 9) * 64 + k] << 16);
                dp_mma_bf16(dh1[nt], af, bb0, bb1);
            }
        }
        // dz1 = dh1 act'(h1); gw1 += dz1 x, gb1 += dz1 (rows g, g+8; columns nt*8 + c + e)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int k = nt * 8 + c + e;
                const float hg = dp_mlp_act<ACCURATE>(fmaf(m.w1[k], xg, m.b1[k]));
                const float hg8 = dp_mlp_act<ACCURATE>(fmaf(m.w1[k], xg8, m.b1[k]));
                const float zg = v0 ? dh1[nt][e] * (1.f - hg * hg) : 0.f;
                const float zg8 = v1 ? dh1[nt][2 + e] * (1.f - hg8 * hg8) : 0.f;
                float gw = zg * xg + zg8 * xg8, gb = zg + zg8;
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) {
                    gw += __shfl_xor_sync(0xffffffffu, gw, o);
                    gb += __shfl_xor_sync(0xffffffffu, gb, o);
                }
                if (g == 0) {
                    dp_fx_add<GB>(gw1 + k, gw);
                    dp_fx_add<GB>(gb1 + k, gb);
                }
            }
        __syncwarp();
    }
    __syncthreads();
    unsigned long long* G = a.gradfx;
    for (int t = threadIdx.x; t < 64 * 64; t += blockDim.x) atomicAdd(G + DP_MLP_OFF_W2 + t, gW2[t]);
    for (int t = threadIdx.x; t < 64; t += blockDim.x) {
        atomicAdd(G + DP_MLP_OFF_W1 + t, gw1[t]);
        atomicAdd(G + DP_MLP_OFF_B1 + t, gb1[t]);
        atomicAdd(G + DP_MLP_OFF_B2 + t, gb2[t]);
        atomicAdd(G + DP_MLP_OFF_W3 + t, gw3[t]);
        atomicAdd(G + DP_MLP_OFF_W3 + 64 + t, gw3[64 + t]);
    }
    if (threadIdx.x < 2) atomicAdd(G + DP_MLP_OFF_B3 + threadIdx.x, gb3[threadIdx.x]);
    if (threadIdx.x == 0) atomicAdd(a.lossfx, *gloss);
}

// Fixed-point sums -> float gradient and loss.
__global__ void k_mlp_grad_finish(const unsigned long long* __restrict__ gradfx,
                                  const unsigned long long* __restrict__ lossfx, float* grad, float* loss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < DP_MLP_NPARAM) grad[t] = (float)((double)(long long)gradfx[t] * (1.0 / (double)(1ull << DP_MLP_GRAD_FX_BITS)));
    if (t == 0) *loss = (float)((double)(long long)*lossfx * (1.0 / (double)(1ull << DP_MLP_LOSS_FX_BITS)));
}

// Adam (Kingma & Ba 2015) on the fp32 masters.
__global__ void k_mlp_adam(float* p, float* mo, float* ve, const float* grad, float lr, float b1, float b2,
                           float eps, float c1, float c2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= DP_MLP_NPARAM) return;
    const float gr = grad[t];
    const float m1 = b1 * mo[t] + (1.f - b1) * gr;
    const float v1 = b2 * ve[t] + (1.f - b2) * gr * gr;
    mo[t] = m1;
    ve[t] = v1;
    p[t] -= lr * (m1 * c1) / (sqrtf(v1 * c2) + eps);
}

// Random minibatch indices (Philox) for one training step.
__global__ void k_mlp_sample(long long* idx, long long batch, long long n, unsigned long long seed, long long step) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    const uint4 r = dp_philox4x32_10(make_uint4((uint32_t)b, (uint32_t)step, (uint32_t)(step >> 32), 0x6d6c7031u),
                                     make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const unsigned long long v = ((unsigned long long)r.x << 32) | r.y;
    idx[b] = (long long)(v % (unsigned long long)n);
}
