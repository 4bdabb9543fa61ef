// TMA (cp.async.bulk.tensor) tile loads and mbarrier waits, inline PTX for
// sm_100-class GPUs.  Every wait is bounded: after kMaxPolls failed polls the
// caller gets `false`, records an error and skips its tile instead of hanging.
#pragma once
#include <cuda.h>
#include <cstdint>

namespace hg {

// A poll of a phase that has not completed returns after about 3.8 us on a
// GB300 (measured by hg_selftest_bounded_wait), so a lost tile is given up
// after about 1 s; a tile's copy completes within microseconds.
constexpr uint32_t kMaxPolls = 1u << 18;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// true once the barrier's phase `parity` has completed; false after `polls` polls
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, uint32_t parity, uint32_t polls) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// the kernels' wait: true once phase `parity` has completed; false after kMaxPolls polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) { return mbar_wait_n(bar, parity, kMaxPolls); }

// 2-D tiled load of the box at element coordinates (x, y) into shared memory;
// completion is counted on `bar` in bytes.  x * 4 bytes must be a multiple of 16.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace hg
