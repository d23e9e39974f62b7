// Seeded synthetic workloads with the reference's shapes.
//
// Host: idash_synth_model builds tag/target positions, nearest-k neighbour
// windows (the rule of train/to_vw.py:33-34) and integer models (coefficients
// uniform in [-8192, 8191] with zeros dropped as train/test_vw_hr.py:44 does;
// one integer bias per output), numbered like the reference's keygen
// (eval/idash.cpp:337-339, :388-390).
//
// Device: valid encryptions under a seeded binary key of the one-hot
// genotype bits, message 2^18 (= ONE_IN_T32, eval/idash.cpp:39) per set bit,
// noise approximately Gaussian with sd ~128 (= 2^-25 * 2^32, the reference's
// alpha, eval/idash.cpp:20).
//
// All randomness is the counter-based hash h(seed, stream, index) below, so
// any tile can be regenerated independently.  Streams:
//   1 key bits, 2 genotypes, 3 LWE masks, 4 LWE noise, 5 TRLWE masks,
//   6 TRLWE noise, 10 tag positions, 11 target positions, 12 neighbour
//   counts, 13 coefficients, 14 biases.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "capi_internal.hpp"
#include "common.cuh"

namespace idash {

__host__ __device__ __forceinline__ uint64_t stream_key(uint64_t seed, uint64_t stream) {
    return mix64(seed + mix64(stream));
}

__host__ __device__ __forceinline__ uint32_t hash32k(uint64_t key, uint64_t index) {
    return uint32_t(mix64(key ^ index) >> 32);
}

__host__ __device__ __forceinline__ uint32_t hash32(uint64_t seed, uint64_t stream, uint64_t index) {
    return hash32k(stream_key(seed, stream), index);
}

namespace {

// One warp per LWE sample (feature f, individual i): mask words from stream 3,
// body = <a, s> + noise + bit * one.
__global__ void k_synth_lwe(uint64_t seed, uint32_t n, uint32_t n_indiv, uint64_t n_samples, uint32_t *out,
                            uint64_t row_stride, int32_t one) {
    const uint64_t key_s = stream_key(seed, 1), key_g = stream_key(seed, 2), key_a = stream_key(seed, 3),
                   key_e = stream_key(seed, 4);
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = uint64_t(gridDim.x) * (blockDim.x / 32);
    for (uint64_t sample = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; sample < n_samples;
         sample += warps) {
        const uint64_t f = sample / n_indiv, i = sample % n_indiv;
        uint32_t *dst = out + f * row_stride + i * (n + 1);
        uint32_t dot = 0;
        for (uint32_t j = lane; j < n; j += 32) {
            const uint32_t aj = hash32k(key_a, sample * n + j);
            dst[j] = aj;
            if (hash32k(key_s, j) & 1u) dot += aj;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) dot += __shfl_xor_sync(0xFFFFFFFFu, dot, off);
        if (lane == 0) {
            uint32_t b = dot;
            for (uint32_t k = 0; k < 4; ++k) b += hash32k(key_e, sample * 4 + k) % 221u;
            b -= 440u;
            const uint64_t p = f / 3, v = f % 3;
            if (hash32k(key_g, p * n_indiv + i) % 3u == v) b += uint32_t(one);
            dst[n] = b;
        }
    }
}

// One CTA per TRLWE row: a uniform, b = a*s + e + m mod X^N+1 where m holds
// the one-hot bit of feature row*R + r for individual s at slot r*RS + s.
__global__ void k_synth_trlwe(uint64_t seed, uint32_t N, uint32_t num_samples, uint32_t num_regions,
                              uint32_t region_size, uint32_t n_features, uint64_t row_begin, uint8_t *base,
                              uint64_t stride, uint64_t payload_off, int64_t var_off, int64_t hdr_off, int32_t tag,
                              int32_t one, double variance) {
    extern __shared__ uint32_t sh[];
    uint32_t *a = sh;          // N words
    uint32_t *key = sh + N;    // N words (0/1)
    const uint64_t row = row_begin + blockIdx.x;  // global row; stored at blockIdx.x
    const uint64_t key_s = stream_key(seed, 1), key_g = stream_key(seed, 2), key_a = stream_key(seed, 5),
                   key_e = stream_key(seed, 6);
    uint8_t *rec = base + uint64_t(blockIdx.x) * stride;
    uint32_t *out = reinterpret_cast<uint32_t *>(rec + payload_off);
    for (uint32_t j = threadIdx.x; j < N; j += blockDim.x) {
        a[j] = hash32k(key_a, row * N + j);
        key[j] = hash32k(key_s, j) & 1u;
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < N; j += blockDim.x) {
        // (a*s)[j] = sum_{i<=j} s_i a_{j-i} - sum_{i>j} s_i a_{N+j-i}
        uint32_t acc = 0;
        for (uint32_t i = 0; i <= j; ++i) acc += key[i] * a[j - i];
        for (uint32_t i = j + 1; i < N; ++i) acc -= key[i] * a[N + j - i];
        for (uint32_t k = 0; k < 4; ++k) acc += hash32k(key_e, (row * N + j) * 4 + k) % 221u;
        acc -= 440u;
        const uint32_t r = j / region_size, s = j % region_size;
        if (r < num_regions && s < num_samples) {
            const uint64_t feat = row * num_regions + r;
            if (feat < n_features) {
                const uint64_t p = feat / 3, v = feat % 3;
                if (hash32k(key_g, p * num_samples + s) % 3u == v) acc += uint32_t(one);
            }
        }
        out[j] = a[j];
        out[N + j] = acc;
    }
    if (threadIdx.x == 0) {
        if (hdr_off >= 0) {
            *reinterpret_cast<uint32_t *>(rec + hdr_off) = uint32_t(row);
            *reinterpret_cast<int32_t *>(rec + hdr_off + 4) = tag;
        }
        if (var_off >= 0) *reinterpret_cast<double *>(rec + var_off) = variance;
    }
}

// Order-independent digest of a request's output words (the quad hashes of
// common.cuh, global word indices index_base + i), accumulated into *digest.
// A pass over the outputs, for scoring kernels that do not take the digest
// as they store (the warp-specialised one does).  One thread per quad; a
// whole quad at a 16-byte aligned address is one 16-byte load.
__global__ void k_digest(const uint32_t *words, uint64_t n_words, uint64_t index_base,
                         unsigned long long *digest) {
    uint64_t acc = 0;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uint64_t first = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t end = index_base + n_words, q0 = index_base >> 2, q_end = (end + 3) >> 2;
    for (uint64_t q = q0 + first; q < q_end; q += stride) {
        const uint64_t lo = q * 4 > index_base ? q * 4 : index_base, hi = q * 4 + 4 < end ? q * 4 + 4 : end;
        const uint32_t *w = words + (lo - index_base);
        uint32_t h = hash_index_key(q);
        if (hi - lo == 4 && (reinterpret_cast<uintptr_t>(w) & 15u) == 0) {
            const uint4 v = *reinterpret_cast<const uint4 *>(w);
            h = hash_step(hash_step(hash_step(hash_step(h, v.x), v.y), v.z), v.w);
        } else {
            for (uint64_t i = lo; i < hi; ++i) h = hash_step(h, w[i - lo]);
        }
        acc += hash_finish(h);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(digest, (unsigned long long)acc);
}

// Uniformly random ciphertext rows (stream 7): word j of global row r is
// hash(seed, 7, r * row_words + j).  Statistically the same as encryptions,
// without their cost; used for serving requests.
__global__ void k_fill_uniform(uint64_t seed, uint64_t row_begin, uint64_t n_rows, uint32_t row_words,
                               uint8_t *base, uint64_t stride) {
    const uint64_t key = stream_key(seed, 7);
    // 16-byte stores of 4 words when every row starts 16-byte aligned
    const bool quads = ((reinterpret_cast<uintptr_t>(base) | stride) & 15u) == 0 && row_words % 4 == 0;
    // a row per block (grid-stride), its words across the threads: no division
    for (uint64_t r = blockIdx.x; r < n_rows; r += gridDim.x) {
        uint32_t *out = reinterpret_cast<uint32_t *>(base + r * stride);
        const uint64_t w0 = (row_begin + r) * row_words;
        if (quads) {
            for (uint32_t j = 4 * threadIdx.x; j < row_words; j += 4 * blockDim.x)
                *reinterpret_cast<uint4 *>(out + j) = make_uint4(hash32k(key, w0 + j), hash32k(key, w0 + j + 1),
                                                                 hash32k(key, w0 + j + 2), hash32k(key, w0 + j + 3));
        } else {
            for (uint32_t j = threadIdx.x; j < row_words; j += blockDim.x) out[j] = hash32k(key, w0 + j);
        }
    }
}

}  // namespace

cudaError_t fill_uniform_rows(uint64_t seed, uint64_t row_begin, uint64_t n_rows, uint32_t row_words, uint8_t *d_out,
                              uint64_t row_stride, int sm_count, cudaStream_t s) {
    if (n_rows == 0) return cudaSuccess;
    const uint32_t blocks = uint32_t(std::min<uint64_t>(n_rows, uint64_t(sm_count) * 16));
    k_fill_uniform<<<blocks, 256, 0, s>>>(seed, row_begin, n_rows, row_words, d_out, row_stride);
    return cudaGetLastError();
}

cudaError_t synth_trlwe_rows(uint64_t seed, const idash_trlwe_params &p, uint64_t n_features, uint64_t row_begin,
                             uint64_t row_end, uint8_t *d_out, const idash_row_layout &layout, cudaStream_t s) {
    if (row_end <= row_begin) return cudaSuccess;
    const size_t smem = size_t(2) * p.N * sizeof(uint32_t);
    k_synth_trlwe<<<uint32_t(row_end - row_begin), 256, smem, s>>>(
        seed, p.N, p.num_samples, p.num_regions, p.region_size, uint32_t(n_features), row_begin, d_out,
        layout.row_stride, layout.payload_offset, layout.variance_offset, layout.header_offset, p.record_tag,
        p.one_t32, 0x1p-50);
    return cudaGetLastError();
}

cudaError_t digest_words(const uint32_t *words, uint64_t n_words, uint64_t index_base, uint64_t *d_digest,
                         int sm_count, cudaStream_t s) {
    if (n_words == 0) return cudaSuccess;
    const uint64_t want = (n_words + 255) / 256;
    const uint32_t blocks = uint32_t(std::min<uint64_t>(want, uint64_t(sm_count) * 8));
    k_digest<<<blocks, 256, 0, s>>>(words, n_words, index_base, reinterpret_cast<unsigned long long *>(d_digest));
    return cudaGetLastError();
}

uint64_t digest_host(const uint32_t *words, uint64_t n_words, uint64_t index_base) {
    uint64_t acc = 0;
    for (uint64_t i = 0; i < n_words;) {
        uint32_t h = hash_index_key((index_base + i) >> 2);
        do {
            h = hash_step(h, words[i]);
            ++i;
        } while (i < n_words && ((index_base + i) & 3u) != 0);
        acc += hash_finish(h);
    }
    return acc;
}

}  // namespace idash

using namespace idash;

extern "C" idash_status idash_synth_model(const idash_synth_spec *spec, idash_synth_model_t *out) {
    if (!spec || !out) return IDASH_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    const uint32_t P = spec->n_tags, T = spec->n_targets;
    if (P == 0 || (spec->neighbours == 0 && (spec->n_choices == 0 || spec->n_choices > 8)))
        return IDASH_ERR_INVALID_ARGUMENT;
    const uint64_t seed = spec->seed;
    std::vector<uint64_t> tag(P), tgt(T);
    for (uint32_t p = 0; p < P; ++p) tag[p] = 100 + 16ull * p + hash32(seed, 10, p) % 16u;
    const uint64_t lo = tag.front(), span = tag.back() - tag.front() + 1;
    for (uint32_t t = 0; t < T; ++t) tgt[t] = lo + mix64(stream_key(seed, 11) ^ t) % span;
    std::sort(tgt.begin(), tgt.end());

    std::vector<uint32_t> wstart(T), wlen(T);
    uint64_t est_terms = 0;
    for (uint32_t t = 0; t < T; ++t) {
        uint32_t k = spec->neighbours ? spec->neighbours : spec->choices[hash32(seed, 12, t) % spec->n_choices];
        k = std::min(k, P);
        // nearest-k tags by |position difference|, ties to the left
        int64_t r = std::lower_bound(tag.begin(), tag.end(), tgt[t]) - tag.begin();
        int64_t l = r - 1;
        uint32_t got = 0;
        while (got < k) {
            const bool take_left =
                r >= int64_t(P) || (l >= 0 && tgt[t] - tag[l] <= tag[r] - tgt[t]);
            if (take_left) --l;
            else ++r;
            ++got;
        }
        wstart[t] = uint32_t(l + 1);
        wlen[t] = uint32_t(r - (l + 1));
        est_terms += 3ull * (3ull * wlen[t] + 1);
    }
    const uint64_t n_out = 3ull * T;
    out->term_ptr = static_cast<uint64_t *>(std::malloc(sizeof(uint64_t) * (n_out + 1)));
    out->term_feat = static_cast<uint32_t *>(std::malloc(sizeof(uint32_t) * (est_terms + 1)));
    out->term_coef = static_cast<int32_t *>(std::malloc(sizeof(int32_t) * (est_terms + 1)));
    out->tag_pos = static_cast<uint64_t *>(std::malloc(sizeof(uint64_t) * P));
    out->target_pos = static_cast<uint64_t *>(std::malloc(sizeof(uint64_t) * (T + 1)));
    out->window_start = static_cast<uint32_t *>(std::malloc(sizeof(uint32_t) * (T + 1)));
    out->window_len = static_cast<uint32_t *>(std::malloc(sizeof(uint32_t) * (T + 1)));
    if (!out->term_ptr || !out->term_feat || !out->term_coef || !out->tag_pos || !out->target_pos ||
        !out->window_start || !out->window_len) {
        idash_synth_model_free(out);
        return IDASH_ERR_OUT_OF_MEMORY;
    }
    std::memcpy(out->tag_pos, tag.data(), sizeof(uint64_t) * P);
    if (T) {
        std::memcpy(out->target_pos, tgt.data(), sizeof(uint64_t) * T);
        std::memcpy(out->window_start, wstart.data(), sizeof(uint32_t) * T);
        std::memcpy(out->window_len, wlen.data(), sizeof(uint32_t) * T);
    }
    const uint64_t kc = stream_key(seed, 13), kb = stream_key(seed, 14);
    uint64_t nt = 0;
    out->term_ptr[0] = 0;
    for (uint64_t o = 0; o < n_out; ++o) {
        const uint32_t t = uint32_t(o / 3);
        for (uint32_t q = 0; q < wlen[t]; ++q) {
            const uint32_t p = wstart[t] + q;
            for (uint32_t u = 0; u < 3; ++u) {
                const int32_t c = int32_t(hash32k(kc, o * 192 + q * 3 + u) % 16384u) - 8192;
                if (c == 0) continue;
                out->term_feat[nt] = 3 * p + u;
                out->term_coef[nt] = c;
                ++nt;
            }
        }
        out->term_feat[nt] = IDASH_CONSTANT_FEATURE;
        out->term_coef[nt] = int32_t(hash32k(kb, o) % 16384u) - 8192;
        ++nt;
        out->term_ptr[o + 1] = nt;
    }
    out->n_out = n_out;
    out->n_terms = nt;
    return IDASH_OK;
}

extern "C" void idash_synth_model_free(idash_synth_model_t *m) {
    if (!m) return;
    std::free(m->term_ptr);
    std::free(m->term_feat);
    std::free(m->term_coef);
    std::free(m->tag_pos);
    std::free(m->target_pos);
    std::free(m->window_start);
    std::free(m->window_len);
    std::memset(m, 0, sizeof(*m));
}

extern "C" idash_status idash_synth_lwe_device(idash_ctx *ctx, uint64_t seed, uint32_t n, uint32_t n_indiv,
                                               uint64_t n_feat_rows, int32_t *d_out, uint64_t row_stride,
                                               void *stream) {
    if (!ctx || !d_out || n == 0 || n_indiv == 0 || row_stride < uint64_t(n_indiv) * (n + 1))
        return IDASH_ERR_INVALID_ARGUMENT;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const uint64_t samples = n_feat_rows * n_indiv;
    if (samples == 0) return IDASH_OK;
    const uint32_t threads = 256;
    const uint64_t want = (samples + 7) / 8;
    const uint32_t blocks = uint32_t(std::min<uint64_t>(want, uint64_t(ctx->sm_count) * 64));
    k_synth_lwe<<<blocks, threads, 0, s>>>(seed, n, n_indiv, samples, reinterpret_cast<uint32_t *>(d_out),
                                           row_stride, 1 << 18);
    return ctx->check_cuda(cudaGetLastError(), "k_synth_lwe launch");
}

extern "C" idash_status idash_synth_trlwe_device(idash_ctx *ctx, uint64_t seed, const idash_trlwe_params *p,
                                                 uint32_t n_tags, void *d_out, const idash_row_layout *layout,
                                                 void *stream) {
    if (!ctx || !p || !d_out || !layout) return IDASH_ERR_INVALID_ARGUMENT;
    if (p->k != 1 || p->N == 0 || p->N > 4096 || p->num_regions == 0 ||
        uint64_t(p->num_regions) * p->region_size > p->N || p->num_samples > p->region_size)
        return IDASH_ERR_INVALID_ARGUMENT;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const uint64_t n_features = 3ull * n_tags;
    const uint64_t rows = (n_features + p->num_regions - 1) / p->num_regions;
    if (rows == 0) return IDASH_OK;
    if (rows >= (1ull << 31)) return IDASH_ERR_INVALID_ARGUMENT;
    return ctx->check_cuda(synth_trlwe_rows(seed, *p, n_features, 0, rows, static_cast<uint8_t *>(d_out), *layout, s),
                           "k_synth_trlwe launch");
}

extern "C" void idash_synth_key(uint64_t seed, uint32_t N, int32_t *out) {
    if (!out) return;
    for (uint32_t j = 0; j < N; ++j) out[j] = int32_t(hash32(seed, 1, j) & 1u);
}

extern "C" idash_status idash_synth_uniform_device(idash_ctx *ctx, uint64_t seed, uint64_t row_begin, uint64_t n_rows,
                                                   uint32_t row_words, void *d_out, uint64_t row_stride,
                                                   void *stream) {
    if (!ctx || !d_out || row_words == 0 || row_stride < uint64_t(row_words) * 4 || row_stride % 4)
        return IDASH_ERR_INVALID_ARGUMENT;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    return ctx->check_cuda(fill_uniform_rows(seed, row_begin, n_rows, row_words, static_cast<uint8_t *>(d_out),
                                             row_stride, ctx->sm_count, s),
                           "k_fill_uniform launch");
}
