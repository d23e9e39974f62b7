// Negacyclic product of a TRLWE mask with a binary key, mod (X^N + 1, 2^32),
// shared by the encryption and decryption kernels (tLweSymEncryptZero and
// tLwePhase, eval/idash.cpp:625 and :714).
//
// With ext[N + t] = a[t] and ext[t] = -a[t] (t < N), the product is
//   (a*s)[j] = sum over the key's set positions i of ext[N + j - i].
// A thread owns kNegCols consecutive coefficients j0 .. j0 + kNegCols - 1 and
// walks the key in chunks of 32 positions.  For chunk c the words it needs
// lie in the 32 + kNegCols words from N + j0 - 32c - 32, which are loaded
// into registers once and then serve every set bit of the chunk.  The key is
// the same for all threads, so each bit test is a uniform branch.
//
// ext is stored with 4 words of padding after every 32 (neg_padded), so the
// windows of neighbouring threads, kNegCols words apart, start in different
// shared-memory banks.  Requires N a multiple of 32 and j0 a multiple of
// kNegCols with j0 + kNegCols <= N.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace idash {

constexpr uint32_t kNegCols = 16;

__host__ __device__ constexpr uint32_t neg_padded(uint32_t i) { return i + ((i >> 5) << 2); }

// Words of one padded extension of length 2N.
__host__ __device__ constexpr uint32_t neg_ext_words(uint32_t N) { return neg_padded(2 * N); }

// Words in front of the extensions: the key's N / 32 bit masks, rounded up to 16 bytes.
__host__ __device__ constexpr uint32_t neg_mask_words(uint32_t N) { return (N / 32 + 3) / 4 * 4; }

// key_mask[w] bit b = 1 when key position 32w + b is set.  Every thread of
// the CTA calls it; the caller synchronises before the masks are read.
__device__ __forceinline__ void neg_build_mask(uint32_t *key_mask, uint32_t N, const uint32_t *key_idx, uint32_t n_nz) {
    for (uint32_t w = threadIdx.x; w < N / 32; w += blockDim.x) key_mask[w] = 0;
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < n_nz; q += blockDim.x)
        atomicOr(&key_mask[key_idx[q] / 32], 1u << (key_idx[q] % 32));
}

// ext entries for mask word t of a row.
__device__ __forceinline__ void neg_store(uint32_t *ext, uint32_t N, uint32_t t, uint32_t v) {
    ext[neg_padded(N + t)] = v;
    ext[neg_padded(t)] = 0u - v;
}

// acc[r] = (a*s)[j0 + r], r < kNegCols.
__device__ __forceinline__ void neg_product(const uint32_t *ext, uint32_t N, uint32_t j0, const uint32_t *key_mask,
                                            uint32_t (&acc)[kNegCols]) {
#pragma unroll
    for (uint32_t r = 0; r < kNegCols; ++r) acc[r] = 0;
    const uint32_t base = smem_addr(ext);
    for (uint32_t c = 0; c < N / 32; ++c) {
        const uint32_t m = key_mask[c];
        if (m == 0) continue;
        // volatile 16-byte loads: the window stays in registers (the compiler
        // may not re-issue them inside the bit tests)
        const uint32_t w0 = N + j0 - 32 * c - 32;
        uint32_t win[32 + kNegCols];
#pragma unroll
        for (uint32_t k = 0; k < (32 + kNegCols) / 4; ++k) {
            const uint4 v = lds_v4(base + 4 * neg_padded(w0 + 4 * k));
            win[4 * k] = v.x;
            win[4 * k + 1] = v.y;
            win[4 * k + 2] = v.z;
            win[4 * k + 3] = v.w;
        }
        // key position 32c + p contributes win[32 + r - p] to coefficient j0 + r
#pragma unroll
        for (uint32_t p = 0; p < 32; ++p)
            if (m & (1u << p)) {
#pragma unroll
                for (uint32_t r = 0; r < kNegCols; ++r) acc[r] += win[32 + r - p];
            }
    }
}

}  // namespace idash
