// dp_umma.cuh — fifth-generation tensor-core (tcgen05) building blocks for
// the pair surrogate's 128 x 64 x 64 layer (inline PTX; sm_100-family only).
//
//   * TMEM: a CTA allocates 64 columns (one fp32 64-wide row per lane, 128
//     lanes = the M = 128 rows of the accumulator);
//   * operands in shared memory in the K-major, no-swizzle canonical layout:
//     "core matrices" of 8 rows x 16 bytes, per 16-wide K step the row blocks
//     256 bytes apart (stride byte offset) and the two K halves 128 bytes
//     apart (leading byte offset);
//   * one thread issues tcgen05.mma (kind::f16: bf16 x bf16 -> fp32) and
//     commits to an mbarrier, every thread waits on it with an iteration
//     limit, and each warp reads its 32 accumulator lanes with tcgen05.ld.
// Like dp_common.cuh it has no includes (it is embedded in NVRTC programs).
#pragma once

__device__ __forceinline__ uint32_t dp_smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (row, k) of a rows x 64 bf16 operand in the
// canonical layout (K steps of 16 columns are rows * 32 bytes apart).
__device__ __forceinline__ int dp_umma_offset(int row, int k, int rows) {
    return (k >> 4) * (rows * 32) + (row >> 3) * 256 + ((k >> 3) & 1) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, leading byte offset (K
// direction), stride byte offset (M/N direction), descriptor version 1,
// no swizzle.
__device__ __forceinline__ uint64_t dp_umma_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
template <int M, int N>
__device__ __forceinline__ uint32_t dp_umma_idesc_bf16() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void dp_tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dp_smem_addr(dst_smem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void dp_tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void dp_umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void dp_umma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(dp_smem_addr(mbar)));
}

__device__ __forceinline__ void dp_mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(dp_smem_addr(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Wait for the given phase parity of the mbarrier; false after `limit` tries.
__device__ __forceinline__ bool dp_mbar_wait(uint64_t* mbar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; ++it) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(dp_smem_addr(mbar)), "r"(parity));
    }
    return done != 0;
}

__device__ __forceinline__ void dp_tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void dp_tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }
__device__ __forceinline__ void dp_async_smem_fence() { asm volatile("fence.proxy.async.shared::cta;"); }

// 32 consecutive fp32 columns of this thread's TMEM lane (warp w reads lanes
// 32 w .. 32 w + 31; taddr holds the warp's lane base and the first column).
__device__ __forceinline__ void dp_tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = __uint_as_float(r[c]);
}
