// mlp_common.cuh — the 1 -> 64 -> 64 -> 2 pair surrogate on tensor cores.
//
// Network (per pair, input s = r^2):
//   x  = (s - x_mean) * x_inv_scale
//   h1 = tanh(w1 * x + b1)                 64 units (bf16 weights)
//   h2 = tanh(W2 h1 + b2)                  64 x 64 bf16 weights, fp32 accumulate (mma)
//   y  = W3 h2 + b3                        2 outputs (bf16 weights)
//   u_nn = y0 * u_scale,  (f r)_nn = y1 * f_scale,  (f/r)_nn = (f r)_nn / s
// A warp evaluates 16 pairs per call ("tile"): the 16 x 64 layer-1
// activations are produced directly in the A-fragment layout of
// mma.sync.m16n8k16 (row = pair, column = unit), split into a bf16 high part
// and a bf16 remainder so the activations keep ~16 bits (the weights are
// bf16 by construction); layer 2 is 4 k-steps x 8 n-tiles x 2 parts of bf16
// MMAs with fp32 accumulators initialised to b2, and layer 3 is a float32 dot
// product over each lane's 16 columns reduced across the quad.
//
// Fragment layout of m16n8k16 (lane L, g = L / 4, c = 2 (L % 4)):
//   A (16x16, row-major): a0 = A[g][c..c+1], a1 = A[g+8][c..c+1],
//                         a2 = A[g][c+8..c+9], a3 = A[g+8][c+8..c+9]
//   B (16x8, col-major):  b0 = B[c..c+1][g],   b1 = B[c+8..c+9][g]
//   C (16x8, fp32):       c0,c1 = C[g][c..c+1], c2,c3 = C[g+8][c..c+1]
// (the lower 16 bits of a packed pair hold the lower column / row index).
#pragma once

#define DP_MLP_H 64

struct dp_mlp_dev {
    float w1[DP_MLP_H];
    float b1[DP_MLP_H];
    float b2[DP_MLP_H];
    float w3[2][DP_MLP_H];
    float b3[2];
    float x_mean, x_inv_scale, u_scale, f_scale;  // f_scale scales f r
    float pad[2];
    // W2 as ready-made B fragments: [k-step 4][n-tile 8][lane 32][2 regs]
    uint32_t w2frag[4 * 8 * 32 * 2];
};

__device__ __forceinline__ uint32_t dp_pack_bf16(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ float dp_tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void dp_mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float dp_bf16_lo_as_float(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float dp_bf16_hi_as_float(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

template <bool ACCURATE>
__device__ __forceinline__ float dp_mlp_act(float x) {
    return ACCURATE ? tanhf(x) : dp_tanh_approx(x);
}

// Split two fp32 values into a packed bf16 high part and a packed bf16 remainder.
__device__ __forceinline__ void dp_split2(float v0, float v1, uint32_t& hi, uint32_t& lo) {
    hi = dp_pack_bf16(v0, v1);
    lo = dp_pack_bf16(v0 - dp_bf16_lo_as_float(hi), v1 - dp_bf16_hi_as_float(hi));
}

// Layer-1 activations h1 = act(w1 x + b1) for rows g (input xg) and g+8
// (xg8) as A fragments (high and remainder parts).
template <bool ACCURATE>
__device__ __forceinline__ void dp_mlp_layer1(const dp_mlp_dev& m, float xg, float xg8, uint32_t ahi[4][4],
                                              uint32_t alo[4][4]) {
    const int c = 2 * (threadIdx.x & 3);
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int col = kt * 16 + c + 8 * half;
            const float w0 = m.w1[col], w1 = m.w1[col + 1], bb0 = m.b1[col], bb1 = m.b1[col + 1];
            dp_split2(dp_mlp_act<ACCURATE>(fmaf(w0, xg, bb0)), dp_mlp_act<ACCURATE>(fmaf(w1, xg, bb1)),
                      ahi[kt][2 * half + 0], alo[kt][2 * half + 0]);
            dp_split2(dp_mlp_act<ACCURATE>(fmaf(w0, xg8, bb0)), dp_mlp_act<ACCURATE>(fmaf(w1, xg8, bb1)),
                      ahi[kt][2 * half + 1], alo[kt][2 * half + 1]);
        }
    }
}

// Layer-2 pre-activations z2 (fp32, C layout: acc[nt][0..3]).
__device__ __forceinline__ void dp_mlp_layer2(const dp_mlp_dev& m, const uint32_t ahi[4][4], const uint32_t alo[4][4],
                                              float acc[8][4]) {
    const int lane = threadIdx.x & 31;
    const int c = 2 * (lane & 3);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float b0 = m.b2[nt * 8 + c], b1 = m.b2[nt * 8 + c + 1];
        acc[nt][0] = b0;
        acc[nt][1] = b1;
        acc[nt][2] = b0;
        acc[nt][3] = b1;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint32_t* bf = m.w2frag + ((kt * 8 + nt) * 32 + lane) * 2;
            const uint32_t b0f = bf[0], b1f = bf[1];
            dp_mma_bf16(acc[nt], alo[kt], b0f, b1f);
            dp_mma_bf16(acc[nt], ahi[kt], b0f, b1f);
        }
    }
}

// Full tile: y[row][out] for rows g (row 0) and g+8 (row 1), valid in every
// lane of the quad.
template <bool ACCURATE>
__device__ __forceinline__ void dp_mlp_tile(const dp_mlp_dev& m, float sg, float sg8, float y[2][2]) {
    const int c = 2 * (threadIdx.x & 3);
    const float xg = (sg - m.x_mean) * m.x_inv_scale;
    const float xg8 = (sg8 - m.x_mean) * m.x_inv_scale;
    uint32_t ahi[4][4], alo[4][4];
    dp_mlp_layer1<ACCURATE>(m, xg, xg8, ahi, alo);
    float acc[8][4];
    dp_mlp_layer2(m, ahi, alo, acc);
    float p00 = 0.f, p01 = 0.f, p10 = 0.f, p11 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int col = nt * 8 + c + e;
            const float h_g = dp_mlp_act<ACCURATE>(acc[nt][e]);
            const float h_g8 = dp_mlp_act<ACCURATE>(acc[nt][2 + e]);
            p00 = fmaf(h_g, m.w3[0][col], p00);
            p01 = fmaf(h_g, m.w3[1][col], p01);
            p10 = fmaf(h_g8, m.w3[0][col], p10);
            p11 = fmaf(h_g8, m.w3[1][col], p11);
        }
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
        p00 += __shfl_xor_sync(0xffffffffu, p00, o);
        p01 += __shfl_xor_sync(0xffffffffu, p01, o);
        p10 += __shfl_xor_sync(0xffffffffu, p10, o);
        p11 += __shfl_xor_sync(0xffffffffu, p11, o);
    }
    y[0][0] = p00 + m.b3[0];
    y[0][1] = p01 + m.b3[1];
    y[1][0] = p10 + m.b3[0];
    y[1][1] = p11 + m.b3[1];
}

// Copy the network into shared memory (blockDim-strided).
__device__ __forceinline__ void dp_mlp_load(dp_mlp_dev* dst, const dp_mlp_dev* src) {
    const uint32_t* s = (const uint32_t*)src;
    uint32_t* d = (uint32_t*)dst;
    for (int t = threadIdx.x; t < (int)(sizeof(dp_mlp_dev) / 4); t += blockDim.x) d[t] = s[t];
}
