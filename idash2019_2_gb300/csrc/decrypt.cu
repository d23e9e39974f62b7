// Party A's decryption of the output TRLWE on the GPU: decrypt_predictions
// (eval/idash.cpp:682-761) computes, per output ciphertext, the phase
// b - a*s (tLwePhase: a negacyclic polynomial product mod X^N + 1 over
// Z/2^32 with the integer key s) and reads its coefficients
// [0, NUM_SAMPLES) as t32tod(phase[j]) = phase[j] / 2^32, stored as float.
//
// The product is exact: only the key's nonzero coefficients are visited (a
// TFHE key is binary, so about N/2 of them), and each of the NUM_SAMPLES
// coefficients is a sum of N/2 words mod 2^32.  The float conversion
// float(phase / 2^32) equals float(phase) * 2^-32 exactly (scaling by a power
// of two commutes with round-to-nearest for these magnitudes).
#include <algorithm>

#include "capi_internal.hpp"
#include "common.cuh"
#include "negacyclic.cuh"

namespace idash {
namespace {

constexpr uint32_t kDecryptThreads = 256;
constexpr uint32_t kDecryptCols = 4;  // coefficients per thread, kDecryptThreads apart

// One CTA per row (grid-stride over rows).  Shared memory: ext[2N], the
// negacyclic extension of the mask a (ext[N + t] = a[t], ext[t] = -a[t]) so
// that (a*s)[j] = sum_i s_i * ext[N + j - i]; then the key's nonzero
// positions (and values, for a non-binary key).  Thread t owns coefficients
// t + 256c: a warp's loads of one key position are consecutive words.
template <bool kBinary>
__global__ void __launch_bounds__(kDecryptThreads) k_decrypt_phase(const uint8_t *in, uint64_t in_stride,
                                                                   uint32_t N, uint32_t num_samples,
                                                                   const uint32_t *key_idx, const int32_t *key_val,
                                                                   uint32_t n_nz, uint64_t n_rows, float *out) {
    extern __shared__ __align__(16) uint32_t sh[];
    uint32_t *ext = sh;
    uint32_t *idx = sh + 2 * N;
    int32_t *val = reinterpret_cast<int32_t *>(idx + n_nz);
    for (uint32_t q = threadIdx.x; q < n_nz; q += blockDim.x) {
        idx[q] = key_idx[q];
        if (!kBinary) val[q] = key_val[q];
    }
    for (uint64_t row = blockIdx.x; row < n_rows; row += gridDim.x) {
        const uint32_t *a = reinterpret_cast<const uint32_t *>(in + row * in_stride);
        __syncthreads();  // the previous row is done with ext
        for (uint32_t t = threadIdx.x; t < N; t += blockDim.x) {
            const uint32_t v = a[t];
            ext[N + t] = v;
            ext[t] = 0u - v;
        }
        __syncthreads();
        for (uint32_t j0 = threadIdx.x; j0 < num_samples; j0 += kDecryptThreads * kDecryptCols) {
            uint32_t acc[kDecryptCols];
#pragma unroll
            for (uint32_t c = 0; c < kDecryptCols; ++c) acc[c] = 0;
            // coefficient j = j0 + 256c is read only when j < N (N >= 4 may be
            // smaller than 1024), so ext[N + j - i] stays inside [1, 2N)
            const uint32_t *e = ext + N + j0;
#pragma unroll 4
            for (uint32_t q = 0; q < n_nz; ++q) {
                const uint32_t *p = e - idx[q];
                const uint32_t s = kBinary ? 1u : uint32_t(val[q]);
#pragma unroll
                for (uint32_t c = 0; c < kDecryptCols; ++c)
                    if (j0 + c * kDecryptThreads < N) acc[c] += kBinary ? p[c * kDecryptThreads] : s * p[c * kDecryptThreads];
            }
#pragma unroll
            for (uint32_t c = 0; c < kDecryptCols; ++c) {
                const uint32_t j = j0 + c * kDecryptThreads;
                if (j < num_samples) {
                    const uint32_t phase = a[N + j] - acc[c];
                    out[row * num_samples + j] = __int2float_rn(int32_t(phase)) * 0x1p-32f;
                }
            }
        }
    }
}

// Binary keys, N a multiple of 32: the register-windowed product of
// negacyclic.cuh, kNegCols consecutive coefficients per thread, kRowsPerCta
// rows per CTA, each with its own padded extension.  Measured on the
// 242,646 x 1,000 decryption: 8 columns per thread 8.4 ms, 16 columns 7.0 ms,
// 32 columns 8.1 ms (k_decrypt_phase: 15.2 ms); testing the key bits in
// pairs (one three-input add for two set bits) was slower at every width.
template <uint32_t kRowThreads>
__global__ void __launch_bounds__(kDecryptThreads) k_decrypt_binary(const uint8_t *in, uint64_t in_stride, uint32_t N,
                                                                    uint32_t num_samples, const uint32_t *key_idx,
                                                                    uint32_t n_nz, uint64_t n_rows, float *out) {
    constexpr uint32_t kRowsPerCta = kDecryptThreads / kRowThreads;
    extern __shared__ __align__(16) uint32_t sh[];
    uint32_t *key_mask = sh;
    uint32_t *ext_all = sh + neg_mask_words(N);  // kRowsPerCta padded extensions
    neg_build_mask(key_mask, N, key_idx, n_nz);
    const uint32_t sub = threadIdx.x / kRowThreads, x = threadIdx.x % kRowThreads;
    const uint32_t j0 = kNegCols * x;
    const uint32_t ext_words = neg_ext_words(N);
    for (uint64_t row0 = uint64_t(blockIdx.x) * kRowsPerCta; row0 < n_rows; row0 += uint64_t(gridDim.x) * kRowsPerCta) {
        __syncthreads();  // the previous rows are done with ext (and the key mask is complete)
        for (uint32_t t = threadIdx.x; t < kRowsPerCta * N; t += blockDim.x) {
            const uint32_t s = t / N, k = t % N;
            if (row0 + s >= n_rows) break;
            neg_store(ext_all + s * ext_words, N, k, reinterpret_cast<const uint32_t *>(in + (row0 + s) * in_stride)[k]);
        }
        __syncthreads();
        const uint64_t row = row0 + sub;
        if (row >= n_rows || j0 >= num_samples) continue;
        uint32_t acc[kNegCols];
        neg_product(ext_all + sub * ext_words, N, j0, key_mask, acc);
        const uint32_t *b = reinterpret_cast<const uint32_t *>(in + row * in_stride) + N;
        float *o = out + row * num_samples;
#pragma unroll
        for (uint32_t r = 0; r < kNegCols; ++r) {
            const uint32_t j = j0 + r;
            if (j < num_samples) o[j] = __int2float_rn(int32_t(b[j] - acc[r])) * 0x1p-32f;
        }
    }
}

}  // namespace
}  // namespace idash

using namespace idash;

extern "C" idash_status idash_decrypt_trlwe_device(idash_ctx *ctx, const int32_t *key, uint32_t N, const void *d_in,
                                                   const idash_row_layout *in_layout, uint64_t n_rows,
                                                   uint32_t num_samples, float *d_out, void *stream) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    if (!key || !d_in || !in_layout || !d_out || N < 4 || N > 2048 || (N & (N - 1)) || num_samples == 0 ||
        num_samples > N)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "idash_decrypt_trlwe_device: bad arguments");
    if (in_layout->row_stride < uint64_t(2) * N * 4 || in_layout->payload_offset % 4 || in_layout->row_stride % 4)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "idash_decrypt_trlwe_device: bad row layout");
    if (n_rows == 0) return IDASH_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    StagedKey k;
    idash_status st = ctx->check_cuda(stage_key(key, N, s, &k), "key upload");
    if (st != IDASH_OK) return st;
    const uint8_t *in = static_cast<const uint8_t *>(d_in) + in_layout->payload_offset;
    if (k.binary && N % 32 == 0) {
        // threads per row: kNegCols coefficients each, rounded up to whole warps
        const uint32_t need = (num_samples + kNegCols - 1) / kNegCols;
        const uint32_t row_threads = need <= 32 ? 32 : need <= 64 ? 64 : 128;  // need <= 2048 / kNegCols
        const uint32_t rows_per_cta = kDecryptThreads / row_threads;
        const size_t smem = (size_t(neg_mask_words(N)) + size_t(rows_per_cta) * neg_ext_words(N)) * 4;
        auto launch = [&](auto kernel) {
            // up to 8 rows of 2.25N words (144 KiB at N = 2048): above the default 48 KiB
            const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kDecryptThreads, smem) != cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
            const uint64_t ctas = (n_rows + rows_per_cta - 1) / rows_per_cta;
            const uint32_t blocks = uint32_t(std::min<uint64_t>(ctas, uint64_t(ctx->sm_count) * per_sm));
            kernel<<<blocks, kDecryptThreads, smem, s>>>(in, in_layout->row_stride, N, num_samples, k.idx, k.n_nz,
                                                         n_rows, d_out);
            return cudaGetLastError();
        };
        const cudaError_t le = row_threads == 32   ? launch(k_decrypt_binary<32>)
                               : row_threads == 64 ? launch(k_decrypt_binary<64>)
                                                   : launch(k_decrypt_binary<128>);
        st = ctx->check_cuda(le, "k_decrypt_binary launch");
        release_key(&k, s);
        if (st == IDASH_OK) ctx->stats.kernel_launches++;
        return st;
    }
    const size_t smem = size_t(2) * N * 4 + size_t(k.n_nz) * (k.binary ? 4 : 8);
    const uint32_t blocks = uint32_t(std::min<uint64_t>(n_rows, uint64_t(ctx->sm_count) * 8));
    if (k.binary)
        k_decrypt_phase<true><<<blocks, kDecryptThreads, smem, s>>>(in, in_layout->row_stride, N, num_samples, k.idx,
                                                                   k.val, k.n_nz, n_rows, d_out);
    else
        k_decrypt_phase<false><<<blocks, kDecryptThreads, smem, s>>>(in, in_layout->row_stride, N, num_samples,
                                                                    k.idx, k.val, k.n_nz, n_rows, d_out);
    st = ctx->check_cuda(cudaGetLastError(), "k_decrypt_phase launch");
    release_key(&k, s);
    if (st == IDASH_OK) ctx->stats.kernel_launches++;
    return st;
}
