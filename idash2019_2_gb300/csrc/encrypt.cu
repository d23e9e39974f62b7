// Party A's encryption on the GPU: encrypt_data_ph1 / ph2
// (eval/idash.cpp:615-679).  Each row is a fresh TRLWE encryption of zero
// (tLweSymEncryptZero, :625: mask a uniform, noise e Gaussian with standard
// deviation alpha on the torus, b = a*s + e), to which the one-hot genotype
// messages are added at b[sample + region * REGION_SIZE] (setScore,
// eval/idash.h:152-156, called from :649-676).
//
// Randomness is counter-based (splitmix64 over seed, stream, index), so rows
// are independent of the launch shape.  Streams: 21 mask words, 22 noise.
// Noise: Box-Muller on two 24-bit uniforms, scaled by alpha * 2^32 and
// truncated toward zero as dtot32 truncates.  The product a*s visits the
// key's nonzero coefficients only (exact mod 2^32).
#include <algorithm>

#include "capi_internal.hpp"
#include "common.cuh"
#include "negacyclic.cuh"

namespace idash {
namespace {

constexpr uint32_t kEncThreads = 256;
constexpr uint32_t kEncCols = 4;  // coefficients per thread, kEncThreads apart
constexpr uint32_t kNoSource = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t enc_hash(uint64_t key, uint64_t index) {
    return uint32_t(mix64(key ^ index) >> 32);
}

struct EncArgs {
    uint32_t N, num_samples, num_regions, region_size;
    int32_t one, nan[3], tag;
    float noise_scale;  // alpha * 2^32
    double variance;    // alpha^2
    uint64_t key_a, key_e;
    uint64_t n_rows;
    const uint32_t *key_idx;
    const int32_t *key_val;
    uint32_t n_nz;
    const uint32_t *slot_src;   // [n_rows * num_regions]: 3p + v or kNoSource
    const int8_t *geno;         // [p * geno_stride + s]
    uint32_t geno_stride;
    const uint32_t *row_index;  // header index per row (may be null: row number)
    const uint32_t *row_out;    // output row per row (may be null: same row)
    uint8_t *out;
    uint64_t out_stride, payload_off;
    int64_t var_off, hdr_off;
    int32_t *noise;  // optional [n_rows * N]
};

// Noise and message of coefficient j of row r, and the body word b[j].
__device__ __forceinline__ void enc_finish(const EncArgs &a, uint64_t r, uint32_t j, uint32_t as_j, uint32_t *body) {
    // noise: dtot32(alpha * z), z standard normal (Box-Muller)
    const uint64_t ni = (r * a.N + j) * 2;
    const float u1 = (float(enc_hash(a.key_e, ni) >> 8) + 0.5f) * 0x1p-24f;
    const float u2 = float(enc_hash(a.key_e, ni + 1) >> 8) * 0x1p-24f;
    const float z = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    const int32_t e_j = int32_t(truncf(a.noise_scale * z));
    // message: the one-hot value of the feature in this slot
    uint32_t m = 0;
    const uint32_t g = j / a.region_size, smp = j % a.region_size;
    if (g < a.num_regions && smp < a.num_samples) {
        const uint32_t src = a.slot_src[r * a.num_regions + g];
        if (src != kNoSource) {
            const uint32_t pi = src / 3, v = src % 3;
            const int32_t gv = a.geno[uint64_t(pi) * a.geno_stride + smp];
            if (gv == int32_t(v)) m = uint32_t(a.one);
            else if (gv < 0 || gv > 2) m = uint32_t(a.nan[v]);
        }
    }
    body[j] = as_j + uint32_t(e_j) + m;
    if (a.noise) a.noise[r * a.N + j] = e_j;
}

// One CTA per row (grid-stride).  Shared memory: ext[2N], the negacyclic
// extension of the fresh mask (ext[N + t] = a[t], ext[t] = -a[t]), then the
// key's nonzero positions and values.  Thread t owns coefficients t + 256c.
template <bool kBinary>
__global__ void __launch_bounds__(kEncThreads) k_encrypt_rows(const EncArgs a) {
    extern __shared__ __align__(16) uint32_t sh[];
    const uint32_t N = a.N;
    uint32_t *ext = sh;
    uint32_t *idx = sh + 2 * N;
    int32_t *val = reinterpret_cast<int32_t *>(idx + a.n_nz);
    for (uint32_t q = threadIdx.x; q < a.n_nz; q += blockDim.x) {
        idx[q] = a.key_idx[q];
        val[q] = a.key_val[q];
    }
    for (uint64_t r = blockIdx.x; r < a.n_rows; r += gridDim.x) {
        const uint64_t orow = a.row_out ? a.row_out[r] : r;
        uint8_t *rec = a.out + orow * a.out_stride;
        uint32_t *mask = reinterpret_cast<uint32_t *>(rec + a.payload_off);
        uint32_t *body = mask + N;
        __syncthreads();  // the previous row is done with ext
        for (uint32_t t = threadIdx.x; t < N; t += blockDim.x) {
            const uint32_t v = enc_hash(a.key_a, r * N + t);
            ext[N + t] = v;
            ext[t] = 0u - v;
            mask[t] = v;
        }
        __syncthreads();
        for (uint32_t j0 = threadIdx.x; j0 < N; j0 += kEncThreads * kEncCols) {
            uint32_t acc[kEncCols] = {0, 0, 0, 0};
            // j = j0 + 256c is used only when j < N, so ext[N + j - i] stays
            // inside [1, 2N) for every key position i < N
            const uint32_t *e = ext + N + j0;
            for (uint32_t q = 0; q < a.n_nz; ++q) {
                const uint32_t *p = e - idx[q];
                const uint32_t s = kBinary ? 1u : uint32_t(val[q]);
#pragma unroll
                for (uint32_t c = 0; c < kEncCols; ++c)
                    if (j0 + c * kEncThreads < N) acc[c] += kBinary ? p[c * kEncThreads] : s * p[c * kEncThreads];
            }
#pragma unroll
            for (uint32_t c = 0; c < kEncCols; ++c) {
                const uint32_t j = j0 + c * kEncThreads;
                if (j >= N) continue;
                enc_finish(a, r, j, acc[c], body);
            }
        }
        if (threadIdx.x == 0) {
            if (a.hdr_off >= 0) {
                *reinterpret_cast<uint32_t *>(rec + a.hdr_off) = a.row_index ? a.row_index[r] : uint32_t(r);
                *reinterpret_cast<int32_t *>(rec + a.hdr_off + 4) = a.tag;
            }
            if (a.var_off >= 0) *reinterpret_cast<double *>(rec + a.var_off) = a.variance;
        }
    }
}

// Binary keys, N a multiple of 32: the register-windowed product of
// negacyclic.cuh, kNegCols consecutive coefficients per thread, kRowsPerCta
// rows per CTA, each with its own padded extension of its fresh mask.
template <uint32_t kRowThreads>
__global__ void __launch_bounds__(kEncThreads) k_encrypt_binary(const EncArgs a) {
    constexpr uint32_t kRowsPerCta = kEncThreads / kRowThreads;
    extern __shared__ __align__(16) uint32_t sh[];
    const uint32_t N = a.N;
    uint32_t *key_mask = sh;
    uint32_t *ext_all = sh + neg_mask_words(N);  // kRowsPerCta padded extensions
    neg_build_mask(key_mask, N, a.key_idx, a.n_nz);
    const uint32_t sub = threadIdx.x / kRowThreads, x = threadIdx.x % kRowThreads;
    const uint32_t j0 = kNegCols * x;
    const uint32_t ext_words = neg_ext_words(N);
    for (uint64_t r0 = uint64_t(blockIdx.x) * kRowsPerCta; r0 < a.n_rows; r0 += uint64_t(gridDim.x) * kRowsPerCta) {
        __syncthreads();  // the previous rows are done with ext (and the key mask is complete)
        for (uint32_t t = threadIdx.x; t < kRowsPerCta * N; t += blockDim.x) {
            const uint32_t s = t / N, k = t % N;
            const uint64_t r = r0 + s;
            if (r >= a.n_rows) break;
            const uint32_t v = enc_hash(a.key_a, r * N + k);
            neg_store(ext_all + s * ext_words, N, k, v);
            const uint64_t orow = a.row_out ? a.row_out[r] : r;
            reinterpret_cast<uint32_t *>(a.out + orow * a.out_stride + a.payload_off)[k] = v;
        }
        __syncthreads();
        const uint64_t r = r0 + sub;
        if (r >= a.n_rows || j0 >= N) continue;
        uint32_t acc[kNegCols];
        neg_product(ext_all + sub * ext_words, N, j0, key_mask, acc);
        const uint64_t orow = a.row_out ? a.row_out[r] : r;
        uint8_t *rec = a.out + orow * a.out_stride;
        uint32_t *body = reinterpret_cast<uint32_t *>(rec + a.payload_off) + N;
#pragma unroll 4
        for (uint32_t q = 0; q < kNegCols; ++q) enc_finish(a, r, j0 + q, acc[q], body);
        if (x == 0) {
            if (a.hdr_off >= 0) {
                *reinterpret_cast<uint32_t *>(rec + a.hdr_off) = a.row_index ? a.row_index[r] : uint32_t(r);
                *reinterpret_cast<int32_t *>(rec + a.hdr_off + 4) = a.tag;
            }
            if (a.var_off >= 0) *reinterpret_cast<double *>(rec + a.var_off) = a.variance;
        }
    }
}

}  // namespace
}  // namespace idash

using namespace idash;

extern "C" idash_status idash_encrypt_trlwe_device(idash_ctx *ctx, const idash_encrypt_params *p, const int32_t *key,
                                                   uint64_t seed, uint64_t n_rows, const uint32_t *d_slot_src,
                                                   const int8_t *d_geno, uint32_t geno_stride,
                                                   const uint32_t *d_row_index, const uint32_t *d_row_out,
                                                   void *d_out, const idash_row_layout *out_layout, int32_t *d_noise,
                                                   void *stream) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    if (!p || !key || !d_out || !out_layout || p->k != 1 || p->N < 4 || p->N > 2048 || (p->N & (p->N - 1)) ||
        p->num_regions == 0 || p->region_size == 0 || uint64_t(p->num_regions) * p->region_size > p->N ||
        p->num_samples > p->region_size || !(p->alpha >= 0.0 && p->alpha < 0.5))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "idash_encrypt_trlwe_device: bad parameters");
    if ((p->num_samples > 0 && (!d_slot_src || !d_geno || geno_stride < p->num_samples)) ||
        out_layout->row_stride < uint64_t(2) * p->N * 4 || out_layout->payload_offset % 4 ||
        out_layout->row_stride % 4)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "idash_encrypt_trlwe_device: bad buffers or layout");
    if (n_rows == 0) return IDASH_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    StagedKey k;
    idash_status st = ctx->check_cuda(stage_key(key, p->N, s, &k), "key upload");
    if (st != IDASH_OK) return st;
    EncArgs a{};
    a.N = p->N;
    a.num_samples = p->num_samples;
    a.num_regions = p->num_regions;
    a.region_size = p->region_size;
    a.one = p->one_t32;
    for (int v = 0; v < 3; ++v) a.nan[v] = p->nan_t32[v];
    a.tag = p->record_tag;
    a.noise_scale = float(p->alpha * 4294967296.0);
    a.variance = p->alpha * p->alpha;
    a.key_a = mix64(seed + mix64(21));
    a.key_e = mix64(seed + mix64(22));
    a.n_rows = n_rows;
    a.key_idx = k.idx;
    a.key_val = k.val;
    a.n_nz = k.n_nz;
    a.slot_src = d_slot_src;
    a.geno = d_geno;
    a.geno_stride = geno_stride;
    a.row_index = d_row_index;
    a.row_out = d_row_out;
    a.out = static_cast<uint8_t *>(d_out);
    a.out_stride = out_layout->row_stride;
    a.payload_off = out_layout->payload_offset;
    a.var_off = out_layout->variance_offset;
    a.hdr_off = out_layout->header_offset;
    a.noise = d_noise;
    if (k.binary && p->N % 32 == 0) {
        // threads per row: kNegCols coefficients each, rounded up to whole warps
        const uint32_t need = p->N / kNegCols;
        const uint32_t row_threads = need <= 32 ? 32 : need <= 64 ? 64 : 128;  // N <= 2048
        const uint32_t rows_per_cta = kEncThreads / row_threads;
        const size_t smem = (size_t(neg_mask_words(p->N)) + size_t(rows_per_cta) * neg_ext_words(p->N)) * 4;
        auto launch = [&](auto kernel) {
            // up to 8 rows of 2.25N words (144 KiB at N = 2048): above the default 48 KiB
            const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kEncThreads, smem) != cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
            const uint64_t ctas = (n_rows + rows_per_cta - 1) / rows_per_cta;
            const uint32_t blocks = uint32_t(std::min<uint64_t>(ctas, uint64_t(ctx->sm_count) * per_sm));
            kernel<<<blocks, kEncThreads, smem, s>>>(a);
            return cudaGetLastError();
        };
        const cudaError_t le = row_threads == 32   ? launch(k_encrypt_binary<32>)
                               : row_threads == 64 ? launch(k_encrypt_binary<64>)
                                                   : launch(k_encrypt_binary<128>);
        st = ctx->check_cuda(le, "k_encrypt_binary launch");
        release_key(&k, s);
        if (st == IDASH_OK) ctx->stats.kernel_launches++;
        return st;
    }
    const size_t smem = size_t(2) * p->N * 4 + size_t(a.n_nz) * 8;
    const uint32_t blocks = uint32_t(std::min<uint64_t>(n_rows, uint64_t(ctx->sm_count) * 8));
    if (k.binary)
        k_encrypt_rows<true><<<blocks, kEncThreads, smem, s>>>(a);
    else
        k_encrypt_rows<false><<<blocks, kEncThreads, smem, s>>>(a);
    st = ctx->check_cuda(cudaGetLastError(), "k_encrypt_rows launch");
    release_key(&k, s);
    if (st == IDASH_OK) ctx->stats.kernel_launches++;
    return st;
}
