// Device-side helpers shared by the scoring kernels: 1-D bulk copies
// (cp.async.bulk) completed on an mbarrier, bounded waits, cache-hinted
// loads/stores and the device error word.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_status.hpp"

namespace idash {

// splitmix64 finaliser (Steele, Lea, Flood 2014): the counter-based mixer of
// every synthetic generator in the library.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The serving digest, in 32-bit arithmetic.  Output words are taken by
// aligned quads of the output layout (word indices 4Q .. 4Q+3).  A quad's
// hash starts at its key hash_index_key(Q), takes h = h * kHashMul + w for
// each of its words present, in index order, and ends with hash_finish (xor-
// shifts around an odd multiply).  The digest is the sum mod 2^64 of the
// quads' hashes: order-independent across launches, and changed by any word,
// by moving a word within its quad or to another quad.  The key of quad Q + d,
// when the low word of Q does not wrap on adding d, is hash_index_key(Q) +
// d * kHashLo: keys along a row follow by addition.
constexpr uint32_t kHashLo = 0x85EBCA77u, kHashHi = 0xC2B2AE3Du, kHashMul = 0x9E3779B1u;

__host__ __device__ __forceinline__ uint32_t hash_index_key(uint64_t index) {
    return uint32_t(index) * kHashLo + uint32_t(index >> 32) * kHashHi;
}

__host__ __device__ __forceinline__ uint32_t hash_finish(uint32_t x) {
    x ^= x >> 15;
    x *= 0x2C1B3C6Du;
    x ^= x >> 12;
    return x;
}

__host__ __device__ __forceinline__ uint32_t hash_step(uint32_t h, uint32_t w) { return h * kHashMul + w; }

// ~1 s at the GB300's 2.07 GHz maximum SM clock.
constexpr long long kWaitLimitCycles = 2000000000ll;

__device__ __forceinline__ void report_error(uint32_t *err, uint32_t code) {
    if (err) atomicCAS(err, 0u, code);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// As mbar_try_wait, but the thread may be suspended for up to `ns`
// nanoseconds waiting for the phase (it resumes when the phase completes), so
// a waiting warp does not spin through issue slots.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity, uint32_t ns) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity), "r"(ns)
        : "memory");
    return done != 0;
}

// Waits for the barrier phase `parity` to complete, for at most
// kWaitLimitCycles.  Returns false (and records kDevTimeout) on expiry.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *err) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait_sleep(bar, parity, 1000000u)) {
        if (clock64() - t0 > kWaitLimitCycles) {
            report_error(err, kDevTimeout);
            return false;
        }
    }
    return true;
}

// Global -> shared bulk copy (no tensor map).  dst/src 16-byte aligned,
// bytes a multiple of 16; completion is counted on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// 16-byte shared-memory load at a 32-bit shared address.  Volatile: never
// moved above the mbarrier wait that makes the data visible.
__device__ __forceinline__ uint4 lds_v4(uint32_t addr) {
    uint4 v;
    asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(addr));
    return v;
}

__device__ __forceinline__ int4 ldg_nc_v4(const void *p) {
    int4 v;
    asm volatile("ld.global.nc.v4.s32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// Streaming (evict-first) 16-byte store: outputs are written once.
__device__ __forceinline__ void stg_cs_v4(void *p, int4 v) {
    asm volatile("st.global.cs.v4.s32 [%0], {%1,%2,%3,%4};" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}

}  // namespace idash
