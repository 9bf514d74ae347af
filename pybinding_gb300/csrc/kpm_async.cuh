// Shared-memory mbarriers and bulk (TMA) copies for the sm_103a kernels, as inline PTX.
//
// Every wait is bounded: after kWaitCycles (about two seconds) it records an error in
// *err and returns false, and it also returns false early once *err is set by another
// block, so that a kernel whose producer or consumer has given up winds down instead of
// hanging the GPU. The caller reports the error to the host.
#pragma once

#include <cstdint>

namespace kpm {
namespace async {

constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(void const* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase with this parity to complete (bounded; see the file comment).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int* err) {
    uint32_t const a = smem_u32(b);
    long long const t0 = clock64();
    for (unsigned spin = 1;; ++spin) {
        if (mbar_try(a, parity)) return true;
        if ((spin & 63u) == 0 && *reinterpret_cast<int volatile*>(err) != 0) return false;
        if (clock64() - t0 > kWaitCycles) {
            atomicExch(err, 1);
            return false;
        }
    }
}

// Warp-wide wait: lane 0 polls (bounded), then every lane checks the completed phase once
// for its own acquire. Polling with all 32 lanes issues 32 shared-memory barrier operations
// per poll, which serialise like same-address atomics and steal shared-memory bandwidth.
// The phase cannot advance again before this warp arrives, so the parity stays valid.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* b, uint32_t parity, int* err) {
    bool ok = true;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait(b, parity, err);
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    if (ok) {
        uint32_t const a = smem_u32(b);
        long long const t0 = clock64();
        while (!mbar_try(a, parity))
            if (clock64() - t0 > kWaitCycles) {  // not expected: the phase is complete
                atomicExch(err, 3);
                ok = false;
                break;
            }
    }
    return __all_sync(0xffffffffu, ok);
}

// Wait for this block's own asynchronous work (copies, MMAs) before it exits, also after
// an error elsewhere; still bounded.
__device__ __forceinline__ void mbar_drain(uint64_t* b, uint32_t parity, int* err) {
    uint32_t const a = smem_u32(b);
    long long const t0 = clock64();
    while (!mbar_try(a, parity))
        if (clock64() - t0 > kWaitCycles) {
            atomicExch(err, 2);
            return;
        }
}

// Bulk copy of `bytes` (a multiple of 16) from global to shared memory, both 16-byte
// aligned; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_load(void* dst, void const* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace async
}  // namespace kpm
