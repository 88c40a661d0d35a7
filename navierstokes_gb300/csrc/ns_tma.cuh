// ns_tma.cuh -- TMA tile loads into shared memory, counted by an mbarrier.
//
// One elected thread of a block issues cp.async.bulk.tensor for the block's
// halo tile; the mbarrier's transaction count covers its bytes.  Every wait
// on the barrier is bounded: a thread that gives up sets the context's error
// word, drains the copy for a second bounded period and its block returns
// (the host reports NS_ERR_TIMEOUT).
#pragma once

#include "ns_internal.cuh"

namespace ns {

constexpr long long kTmaSpinLimit = 1LL << 24;

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier at most `limit` polls.
// False: the wait gave up and `err` is set.  A copy the barrier counts may
// still be in flight when the wait gives up, and a block that exits while it
// is would leave it landing in shared memory the SM may have handed to the
// next block; so after giving up the thread keeps polling for up to `limit`
// more polls before it returns.  Only a copy that never completes at all
// outlives its block.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity,
                                                  int *err, long long limit = kTmaSpinLimit)
{
    long long spins = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (++spins > limit) {
            atomicCAS(err, 0, 1);  // the first failure recorded wins
            for (long long k = 0; k < limit && !mbar_try_wait(bar, parity); k++) {
            }
            return false;
        }
    }
    return true;
}

// Box of a 3-D tensor map at (x, y, z) into shared memory; the caller keeps
// x times the element size a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
        "r"(smem_addr(bar))
        : "memory");
}

}  // namespace ns
