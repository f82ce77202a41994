// Shared-memory stage ring fed by the bulk-copy engine, for the kernels that
// stream the block-CSR stiffness (the difference-form product in k_solve.cu,
// the multigrid level-0 smoother in k_amg.cu).  A persistent CTA walks tiles
// of consecutive rows (16 or 8), whose row offsets, column indices and
// values are contiguous in the block-CSR arrays; one thread copies a tile
// into a stage with cp.async.bulk, completing on the stage's "full" mbarrier
// by byte count, up to stages - 1 tiles ahead, and the warps release a stage
// through its "empty" mbarrier once they have computed its rows.  Every wait
// is bounded by STREAM_WAIT_CYCLES (about a second).
#pragma once
#include <cuda_runtime.h>

namespace lpm {

constexpr long long STREAM_WAIT_CYCLES = 2000000000LL;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// wait for the completion of the barrier's phase of the given parity;
// false after STREAM_WAIT_CYCLES
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    const unsigned a = smem_u32(bar);
    const long long t0 = clock64();
    for (;;) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok)
            return true;
        if (clock64() - t0 > STREAM_WAIT_CYCLES)
            return false;
    }
}

// mbar_wait by every lane of a warp, with one outcome for the warp (a lane
// that ran out makes the whole warp give up)
__device__ __forceinline__ bool warp_mbar_wait(unsigned long long *bar, unsigned parity)
{
    const bool ok = mbar_wait(bar, parity);
    return __all_sync(0xffffffffu, ok);
}

// global -> shared copy by the bulk-copy engine, completing on bar (both
// addresses 16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// A stage: the tile's ROWS + 2 row offsets (rows r0 .. r0 + ROWS + 1, a
// multiple of 16 bytes; the row-offset array is padded so the last tile's
// copy stays inside it), its column indices at cols_off and its values at
// vals_off.
struct StreamLayout {
    int stages, stage_bytes, cols_off, vals_off;
};

}  // namespace lpm
