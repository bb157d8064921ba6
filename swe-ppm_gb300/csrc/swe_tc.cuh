// Fifth-generation tensor-core primitives (tcgen05, sm_103a) used by the MLP
// surrogate: TMEM allocation, BF16 x BF16 -> FP32 MMAs with operands in
// shared memory, completion through an mbarrier, TMEM -> register loads.
//
// Operand layout: K-major, no swizzle.  A matrix of R rows (M or N) and K
// columns (K a multiple of 16) is stored as 8 x 8 "core matrices" (8 rows of
// 16 bytes, 128 contiguous bytes each), core matrix (r/8, k/8) at byte
// ((r/8) * (K/8) + k/8) * 128.  Core matrices adjacent in K are 128 bytes
// apart (leading byte offset), adjacent in R (K/8) * 128 bytes apart (stride
// byte offset).  One MMA consumes a K slice of 16: its descriptor starts
// 256 bytes further per slice.
//
// The same bytes read as an MN-major operand (instruction-descriptor
// transpose bit set): a matrix stored K-major with W columns serves as an
// operand whose K runs over the stored ROWS and whose M or N runs over the
// stored columns.  A core matrix is then 8 K-rows of 8 consecutive M/N
// elements -- the same 128 bytes -- with M/N blocks 128 bytes apart and K
// blocks (W/8) * 128 bytes apart.  So a buffer of activations [edge][neuron]
// is both the A operand of the next layer's GEMM and, transposed for free, an
// operand of the weight-gradient GEMM (K = edges).
//
// Accumulators: M = 128 rows, row r in TMEM lane r, column j in TMEM column
// base + j (FP32).  Warp w of the CTA reads lanes 32w .. 32w+31.
#pragma once

#include <cstdint>

namespace swegb {
namespace tc {

__device__ __forceinline__ uint32_t smemAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

/// byte offset of element (r, k) in the core-matrix layout of a matrix with K columns
__device__ __forceinline__ uint32_t coreOffset(int r, int k, int K) {
    return uint32_t((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

/// shared-memory matrix descriptor (no swizzle, K-major) of the K slice
/// starting at column k0 of a matrix with K columns stored at `base`
__device__ __forceinline__ uint64_t smemDesc(const void *base, int k0, int K) {
    const uint32_t addr = smemAddr(base) + uint32_t(k0 >> 3) * 128u;
    const uint32_t lbo = 128u, sbo = uint32_t(K >> 3) * 128u;
    return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // descriptor version of sm_100 family
}

/// MN-major descriptor of the K slice starting at stored row k0 of a matrix
/// stored K-major with W columns (see the layout note above)
__device__ __forceinline__ uint64_t smemDescMN(const void *base, int k0, int W) {
    const uint32_t kblock = uint32_t(W >> 3) * 128u;
    const uint32_t addr = smemAddr(base) + uint32_t(k0 >> 3) * kblock;
    const uint32_t lbo = kblock, sbo = 128u;
    return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/// instruction descriptor: BF16 A and B, FP32 D, M x N; aMN / bMN select
/// the MN-major (transposed) reading of A / B
__host__ __device__ constexpr uint32_t idescBf16(int M, int N, bool aMN = false, bool bMN = false) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(aMN) << 15) | (uint32_t(bMN) << 16) |
           (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

/// TMEM columns for the CTA (warp-wide; a power of two >= 32); the address lands in *slot
__device__ __forceinline__ void tmemAlloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(slot)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmemFree(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

/// D (+)= A * B^T for one K slice of 16 (single issuing thread)
__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1 : 0));
}
/// the MMAs issued so far by this thread arrive on the mbarrier when done
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(mbar)));
}

__device__ __forceinline__ void mbarInit(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
/// bounded wait for phase `parity` of the mbarrier; false when the limit ran out
__device__ __forceinline__ bool mbarWait(uint64_t *mbar, uint32_t parity, int limit = 1 << 22) {
    for (int i = 0; i < limit; i++) {
        uint32_t ok;
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok)
                     : "r"(smemAddr(mbar)), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/// generic-proxy shared-memory writes become visible to the tensor cores
__device__ __forceinline__ void fenceSmemForMma() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/// 16 FP32 columns of this thread's TMEM lane, starting at column `col`
__device__ __forceinline__ void load16(uint32_t tbase, int col, float (&v)[16]) {
    const uint32_t lane = (threadIdx.x >> 5) * 32u;
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(tbase + (lane << 16) + uint32_t(col)));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

} // namespace tc
} // namespace swegb
