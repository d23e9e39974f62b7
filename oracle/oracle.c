/*
 * oracle.c — TEST INFRASTRUCTURE ONLY (see oracle.h).  Plain C + OpenMP.
 *
 * oracle_trlwe_score restates cloud_compute_score (eval/idash.cpp:763-848)
 * step by step on flat arrays; the TFHE primitives it calls there are
 * restated inline from their definitions:
 *   tLweClear (idash.cpp:796)       -> zero a and b, variance = 0
 *   tLweAddMulTo (idash.cpp:817)    -> a,b += coef * C; variance += coef^2 var
 *   tLweCopy (idash.cpp:825)        -> copy coefficients and variance
 *   torusPolynomialMulByXai (:832)  -> negacyclic rotation by X^e, e in [0,2N)
 *   tLweAddTo (idash.cpp:835)       -> a,b += rotated; variance += 0
 */
#include "oracle.h"

#include <omp.h>
#include <stdlib.h>
#include <string.h>

uint64_t oracle_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t oracle_hash32(uint64_t seed, uint64_t stream, uint64_t index) {
    const uint64_t key = oracle_mix64(seed + oracle_mix64(stream));
    return (uint32_t)(oracle_mix64(key ^ index) >> 32);
}

static inline void rotate_add(uint32_t *acc, const uint32_t *src, uint32_t N, uint32_t e) {
    /* acc += X^e * src mod X^N+1, e in [0, 2N) */
    for (uint32_t j = 0; j < N; ++j) {
        uint32_t t = j + e;
        int neg = 0;
        if (t >= 2 * N) t -= 2 * N;
        if (t >= N) { t -= N; neg = 1; }
        acc[t] += neg ? 0u - src[j] : src[j];
    }
}

int oracle_trlwe_score(uint32_t N, uint32_t num_samples, uint32_t num_regions, uint32_t region_size,
                       int32_t one_t32, uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                       const int32_t *term_coef, const uint32_t *row_of_index, uint64_t n_index,
                       uint64_t n_rows, const int32_t *in_rows, const double *in_var,
                       int32_t *out_rows, double *out_var, int n_threads) {
    if (N == 0 || num_regions == 0 || region_size == 0 || num_samples > region_size ||
        (uint64_t)num_regions * region_size > N)
        return -1;
    const uint64_t W = 2ull * N; /* k = 1: a then b */
    int bad = 0;
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel num_threads(n_threads) reduction(| : bad)
    {
        uint32_t *tmp = (uint32_t *)calloc((size_t)num_regions * W, sizeof(uint32_t));
        double *tvar = (double *)calloc(num_regions, sizeof(double));
#pragma omp for schedule(dynamic, 64)
        for (int64_t o = 0; o < (int64_t)n_out; ++o) {
            memset(tmp, 0, sizeof(uint32_t) * num_regions * W);
            memset(tvar, 0, sizeof(double) * num_regions);
            for (uint64_t t = term_ptr[o]; t < term_ptr[o + 1]; ++t) {
                const uint32_t feat = term_feat[t];
                const uint32_t coef = (uint32_t)term_coef[t];
                if (feat == ORACLE_CONSTANT_FEATURE) {
                    const uint32_t scaled = coef * (uint32_t)one_t32;
                    for (uint32_t s = 0; s < num_samples; ++s) tmp[N + s] += scaled;
                    continue;
                }
                const uint32_t region = feat % num_regions;
                const uint64_t index = feat / num_regions;
                uint64_t row = index;
                if (row_of_index) {
                    if (index >= n_index) { bad = 1; continue; }
                    row = row_of_index[index];
                }
                if (row >= n_rows) { bad = 1; continue; }
                const uint32_t *src = (const uint32_t *)(in_rows + row * W);
                uint32_t *dst = tmp + (uint64_t)region * W;
                for (uint64_t j = 0; j < W; ++j) dst[j] += coef * src[j];
                if (in_var) tvar[region] += (double)((int64_t)term_coef[t] * term_coef[t]) * in_var[row];
            }
            uint32_t *out = (uint32_t *)(out_rows + (uint64_t)o * W);
            memcpy(out, tmp, sizeof(uint32_t) * W);
            for (uint32_t r = 1; r < num_regions; ++r) {
                const uint32_t e = 2 * N - r * region_size;
                rotate_add(out, tmp + (uint64_t)r * W, N, e);          /* mask a */
                rotate_add(out + N, tmp + (uint64_t)r * W + N, N, e);  /* body b */
            }
            for (uint32_t j = region_size; j < N; ++j) out[N + j] = 0;
            if (out_var) out_var[o] = tvar[0];
        }
        free(tmp);
        free(tvar);
    }
    return bad ? -2 : 0;
}

int oracle_lwe_score(uint32_t n, uint32_t n_indiv, int32_t one_t32, uint64_t n_out,
                     const uint64_t *term_ptr, const uint32_t *term_feat, const int32_t *term_coef,
                     uint64_t n_feat_rows, const int32_t *in, uint64_t in_row_stride,
                     uint64_t out_begin, uint64_t out_end, int32_t *out, uint64_t out_row_stride,
                     int n_threads) {
    if (out_end > n_out || out_begin > out_end) return -1;
    const uint64_t L = (uint64_t)n_indiv * (n + 1);
    int bad = 0;
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for num_threads(n_threads) schedule(dynamic, 4) reduction(| : bad)
    for (int64_t o = (int64_t)out_begin; o < (int64_t)out_end; ++o) {
        uint32_t *dst = (uint32_t *)(out + (uint64_t)(o - (int64_t)out_begin) * out_row_stride);
        memset(dst, 0, sizeof(uint32_t) * L);
        for (uint64_t t = term_ptr[o]; t < term_ptr[o + 1]; ++t) {
            const uint32_t feat = term_feat[t];
            const uint32_t coef = (uint32_t)term_coef[t];
            if (feat == ORACLE_CONSTANT_FEATURE) {
                const uint32_t scaled = coef * (uint32_t)one_t32;
                for (uint32_t i = 0; i < n_indiv; ++i) dst[(uint64_t)i * (n + 1) + n] += scaled;
                continue;
            }
            if (feat >= n_feat_rows) { bad = 1; continue; }
            const uint32_t *src = (const uint32_t *)(in + (uint64_t)feat * in_row_stride);
            for (uint64_t j = 0; j < L; ++j) dst[j] += coef * src[j];
        }
    }
    return bad ? -2 : 0;
}

int oracle_intpoly_score(uint32_t N, uint32_t num_samples, uint32_t region_size, int32_t one_t32,
                         uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                         const int16_t *term_poly, const int32_t *bias, uint64_t n_rows,
                         const int32_t *in_rows, uint64_t out_begin, uint64_t out_end,
                         int32_t *out_rows, int n_threads) {
    if (out_end > n_out || out_begin > out_end || num_samples > region_size || region_size > N) return -1;
    const uint64_t W = 2ull * N;
    int bad = 0;
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for num_threads(n_threads) schedule(dynamic, 1) reduction(| : bad)
    for (int64_t o = (int64_t)out_begin; o < (int64_t)out_end; ++o) {
        uint32_t *dst = (uint32_t *)(out_rows + (uint64_t)(o - (int64_t)out_begin) * W);
        memset(dst, 0, sizeof(uint32_t) * W);
        for (uint64_t t = term_ptr[o]; t < term_ptr[o + 1]; ++t) {
            const uint32_t feat = term_feat[t];
            if (feat >= n_rows) { bad = 1; continue; }
            const int16_t *w = term_poly + t * N;
            for (uint32_t p = 0; p < 2; ++p) {
                const uint32_t *c = (const uint32_t *)(in_rows + (uint64_t)feat * W + (uint64_t)p * N);
                uint32_t *d = dst + (uint64_t)p * N;
                for (uint32_t i = 0; i < N; ++i) {
                    const uint32_t wi = (uint32_t)(int32_t)w[i];
                    if (wi == 0) continue;
                    for (uint32_t j = 0; j < N; ++j) {
                        const uint32_t prod = wi * c[j];
                        const uint32_t k = i + j;
                        if (k < N) d[k] += prod;
                        else d[k - N] -= prod; /* X^N = -1 */
                    }
                }
            }
        }
        const uint32_t scaled = (uint32_t)bias[o] * (uint32_t)one_t32;
        for (uint32_t s = 0; s < num_samples; ++s) dst[N + s] += scaled;
        for (uint32_t j = region_size; j < N; ++j) dst[N + j] = 0;
    }
    return bad ? -2 : 0;
}

void oracle_sample_extract(uint32_t N, const int32_t *trlwe, uint32_t slot, int32_t *out) {
    const uint32_t *a = (const uint32_t *)trlwe;
    for (uint32_t j = 0; j < N; ++j) {
        if (j <= slot) out[j] = (int32_t)a[slot - j];
        else out[j] = (int32_t)(0u - a[N + slot - j]);
    }
    out[N] = trlwe[N + slot];
}

void oracle_trlwe_decrypt(uint32_t N, const int32_t *key, uint64_t n_rows, uint64_t stride_words,
                          const int32_t *rows, uint32_t num_samples, float *out, int n_threads) {
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 16)
    for (int64_t r = 0; r < (int64_t)n_rows; ++r) {
        const uint32_t *a = (const uint32_t *)(rows + (uint64_t)r * stride_words);
        const uint32_t *b = a + N;
        for (uint32_t j = 0; j < num_samples; ++j) {
            /* (a*s)[j] = sum_{i<=j} s_i a_{j-i} - sum_{i>j} s_i a_{N+j-i} */
            uint32_t acc = 0;
            for (uint32_t i = 0; i < N; ++i) {
                const uint32_t s = (uint32_t)key[i];
                if (s == 0) continue;
                acc += i <= j ? s * a[j - i] : 0u - s * a[N + j - i];
            }
            const int32_t phase = (int32_t)(b[j] - acc);
            out[(uint64_t)r * num_samples + j] = (float)((double)phase / 4294967296.0);
        }
    }
}

/* Synthetic per-individual LWE inputs (streams as in the product generator):
 *   key bit s_j      = hash(seed, 1, j) & 1
 *   genotype g(p,i)  = hash(seed, 2, p*n_indiv + i) % 3, feature f = 3p+v has bit (g == v)
 *   mask a_j(f,i)    = hash(seed, 3, (f*n_indiv + i)*n + j)
 *   noise e(f,i)     = sum_{k<4} (hash(seed, 4, (f*n_indiv+i)*4+k) % 221) - 440
 *   body b(f,i)      = sum_j a_j s_j + e + bit * 2^18   (mod 2^32)
 * Word w of row f is individual w/(n+1), position w%(n+1) (n = body). */
void oracle_synth_lwe_words(uint64_t seed, uint32_t n, uint32_t n_indiv, uint64_t feature,
                            uint64_t w0, uint64_t count, int32_t *out) {
    for (uint64_t w = w0; w < w0 + count; ++w) {
        const uint64_t i = w / (n + 1), j = w % (n + 1);
        const uint64_t sample = feature * n_indiv + i;
        if (j < n) {
            out[w - w0] = (int32_t)oracle_hash32(seed, 3, sample * n + j);
            continue;
        }
        uint32_t b = 0;
        for (uint32_t k = 0; k < n; ++k)
            if (oracle_hash32(seed, 1, k) & 1u) b += oracle_hash32(seed, 3, sample * n + k);
        for (uint32_t k = 0; k < 4; ++k) b += (oracle_hash32(seed, 4, sample * 4 + k) % 221u);
        b -= 440u;
        const uint64_t p = feature / 3, v = feature % 3;
        const uint32_t g = oracle_hash32(seed, 2, p * n_indiv + i) % 3u;
        if (g == v) b += 1u << 18;
        out[w - w0] = (int32_t)b;
    }
}

/* ------------------------------------------------------------------ synth */
static uint64_t synth_key(uint64_t seed, uint64_t stream) { return oracle_mix64(seed + oracle_mix64(stream)); }
static uint32_t synth_h(uint64_t key, uint64_t index) { return (uint32_t)(oracle_mix64(key ^ index) >> 32); }

static int cmp_u64(const void *a, const void *b) {
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

void oracle_synth_model_free(oracle_synth_model_t *m) {
    if (!m) return;
    free(m->term_ptr);
    free(m->term_feat);
    free(m->term_coef);
    free(m->window_start);
    free(m->window_len);
    memset(m, 0, sizeof(*m));
}

int oracle_synth_model(uint64_t seed, uint32_t n_tags, uint32_t n_targets, uint32_t neighbours, uint32_t n_choices,
                       const uint32_t *choices, oracle_synth_model_t *out) {
    memset(out, 0, sizeof(*out));
    if (n_tags == 0 || (neighbours == 0 && (n_choices == 0 || !choices))) return -1;
    const uint32_t P = n_tags, T = n_targets;
    uint64_t *tag = (uint64_t *)malloc(sizeof(uint64_t) * P);
    uint64_t *tgt = (uint64_t *)malloc(sizeof(uint64_t) * (T + 1));
    out->window_start = (uint32_t *)malloc(sizeof(uint32_t) * (T + 1));
    out->window_len = (uint32_t *)malloc(sizeof(uint32_t) * (T + 1));
    if (!tag || !tgt || !out->window_start || !out->window_len) {
        free(tag);
        free(tgt);
        oracle_synth_model_free(out);
        return -1;
    }
    const uint64_t k10 = synth_key(seed, 10), k11 = synth_key(seed, 11), k12 = synth_key(seed, 12);
    for (uint32_t p = 0; p < P; ++p) tag[p] = 100 + 16ull * p + synth_h(k10, p) % 16u;
    const uint64_t lo = tag[0], span = tag[P - 1] - tag[0] + 1;
    for (uint32_t t = 0; t < T; ++t) tgt[t] = lo + oracle_mix64(k11 ^ t) % span;
    qsort(tgt, T, sizeof(uint64_t), cmp_u64);
    uint64_t est = 0;
    for (uint32_t t = 0; t < T; ++t) {
        uint32_t k = neighbours ? neighbours : choices[synth_h(k12, t) % n_choices];
        if (k > P) k = P;
        /* first tag at or after the target, then grow the window to k tags,
           taking the left one on ties */
        int64_t r = 0, hi = P;
        while (r < hi) {
            const int64_t mid = (r + hi) / 2;
            if (tag[mid] < tgt[t]) r = mid + 1;
            else hi = mid;
        }
        int64_t l = r - 1;
        for (uint32_t got = 0; got < k; ++got) {
            const int take_left = r >= (int64_t)P || (l >= 0 && tgt[t] - tag[l] <= tag[r] - tgt[t]);
            if (take_left) --l;
            else ++r;
        }
        out->window_start[t] = (uint32_t)(l + 1);
        out->window_len[t] = (uint32_t)(r - (l + 1));
        est += 3ull * (3ull * out->window_len[t] + 1);
    }
    free(tag);
    free(tgt);
    const uint64_t n_out = 3ull * T;
    out->term_ptr = (uint64_t *)malloc(sizeof(uint64_t) * (n_out + 1));
    out->term_feat = (uint32_t *)malloc(sizeof(uint32_t) * (est + 1));
    out->term_coef = (int32_t *)malloc(sizeof(int32_t) * (est + 1));
    if (!out->term_ptr || !out->term_feat || !out->term_coef) {
        oracle_synth_model_free(out);
        return -1;
    }
    const uint64_t kc = synth_key(seed, 13), kb = synth_key(seed, 14);
    uint64_t nt = 0;
    out->term_ptr[0] = 0;
    for (uint64_t o = 0; o < n_out; ++o) {
        const uint32_t t = (uint32_t)(o / 3);
        for (uint32_t q = 0; q < out->window_len[t]; ++q) {
            const uint32_t p = out->window_start[t] + q;
            for (uint32_t u = 0; u < 3; ++u) {
                const int32_t c = (int32_t)(synth_h(kc, o * 192 + q * 3 + u) % 16384u) - 8192;
                if (c == 0) continue;
                out->term_feat[nt] = 3 * p + u;
                out->term_coef[nt] = c;
                ++nt;
            }
        }
        out->term_feat[nt] = ORACLE_CONSTANT_FEATURE;
        out->term_coef[nt] = (int32_t)(synth_h(kb, o) % 16384u) - 8192;
        ++nt;
        out->term_ptr[o + 1] = nt;
    }
    out->n_out = n_out;
    out->n_terms = nt;
    return 0;
}
