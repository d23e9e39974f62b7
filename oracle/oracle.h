/*
 * oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's party-B scoring step
 * (`cloud_compute_score`, eval/idash.cpp:763-848) and of the two layouts the
 * GPU library adds beside it, used by tests/, by smoke() and by bench.py's
 * CPU-baseline leg as the checker.  Nothing in the product links, loads or
 * calls this library.
 *
 * Parity pin: oracle_trlwe_score is checked bit-for-bit against the
 * reference's own eval/idash.cpp compiled against oracle/tfhe_compat (the
 * committed fixtures under tests/golden/ were produced by that build).
 *
 * All Torus32 arithmetic is done on uint32_t (wrap-around mod 2^32).
 */
#ifndef IDASH_ORACLE_H
#define IDASH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_CONSTANT_FEATURE 0xFFFFFFFFu

/*
 * TRLWE-packed scoring, the reference's own loop (eval/idash.cpp:779-842):
 * for every output o (in CSR order):
 *   tmp[r] = 0 for every region r                                  (:795-797)
 *   for each term (feat, coef) in CSR order                        (:800-819)
 *     feat == CONSTANT: tmp[0].b[s] += coef*one_t32, s < num_samples
 *     else: tmp[feat % R] += coef * C[row_of_index[feat / R]]       (tLweAddMulTo)
 *   out = tmp[0]; out += X^(2N - r*RS) * tmp[r] for r >= 1          (:825-836)
 *   out.b[j] = 0 for j >= region_size                              (:839-841)
 * in_rows/out_rows are [rows][2][N] int32 (a then b).  Variance (optional)
 * follows TFHE's bookkeeping: region-0 accumulations add coef^2*var_in; the
 * folded regions contribute the rotation temporary's variance, which is 0.
 */
int oracle_trlwe_score(uint32_t N, uint32_t num_samples, uint32_t num_regions, uint32_t region_size,
                       int32_t one_t32, uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                       const int32_t *term_coef, const uint32_t *row_of_index, uint64_t n_index,
                       uint64_t n_rows, const int32_t *in_rows, const double *in_var,
                       int32_t *out_rows, double *out_var, int n_threads);

/*
 * Per-individual LWE scoring (one LWE sample of dimension n per individual and
 * input feature).  in: row f holds n_indiv samples of (n+1) int32 words
 * (a[0..n-1], b), rows in_row_stride words apart.  For outputs
 * [out_begin, out_end): out[o - out_begin] = sum coef * in[feat] and
 * b += bias * one_t32 for the constant feature.  This is SampleExtract of the
 * TRLWE form, slot by slot.
 */
int oracle_lwe_score(uint32_t n, uint32_t n_indiv, int32_t one_t32, uint64_t n_out,
                     const uint64_t *term_ptr, const uint32_t *term_feat, const int32_t *term_coef,
                     uint64_t n_feat_rows, const int32_t *in, uint64_t in_row_stride,
                     uint64_t out_begin, uint64_t out_end, int32_t *out, uint64_t out_row_stride,
                     int n_threads);

/*
 * Integer-polynomial x TRLWE scoring: out_o = sum_f W_{o,f}(X) * C_f(X) in
 * Z/2^32[X]/(X^N+1) on both polynomials, b[s] += bias_o*one_t32 for
 * s < num_samples, b[j] = 0 for j >= region_size.  Exact schoolbook product.
 * term_poly is [nnz][N] int16; term_feat indexes input rows directly.
 * Outputs [out_begin, out_end) only.
 */
int oracle_intpoly_score(uint32_t N, uint32_t num_samples, uint32_t region_size, int32_t one_t32,
                         uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                         const int16_t *term_poly, const int32_t *bias, uint64_t n_rows,
                         const int32_t *in_rows, uint64_t out_begin, uint64_t out_end,
                         int32_t *out_rows, int n_threads);

/* SampleExtract at slot s of a TRLWE (k=1): LWE a'[j] = a[s-j] (j<=s),
 * -a[N+s-j] (j>s); b' = b[s].  out has N+1 words. */
void oracle_sample_extract(uint32_t N, const int32_t *trlwe, uint32_t slot, int32_t *out);

/* Party A's decryption of TRLWE rows (decrypt_predictions,
 * eval/idash.cpp:682-761): phase = b - a*s (tLwePhase, eval/idash.cpp:714,
 * exact negacyclic product mod X^N+1 over Z/2^32 with the integer key s),
 * then out[r*num_samples + j] = (float)t32tod(phase[j]) (:718) for
 * j < num_samples.  rows: [n_rows][stride_words] int32, a at word 0, b at N. */
void oracle_trlwe_decrypt(uint32_t N, const int32_t *key, uint64_t n_rows, uint64_t stride_words,
                          const int32_t *rows, uint32_t num_samples, float *out, int n_threads);

/* Counter-based generator shared with the product's synthetic-workload
 * generator: splitmix64 finaliser over (seed, stream, index). */
uint64_t oracle_mix64(uint64_t z);
uint32_t oracle_hash32(uint64_t seed, uint64_t stream, uint64_t index);

/* Regenerate one synthetic LWE input row slice [w0, w0+count) of feature f
 * (see the product's synthetic generator for the definition). */
void oracle_synth_lwe_words(uint64_t seed, uint32_t n, uint32_t n_indiv, uint64_t feature,
                            uint64_t w0, uint64_t count, int32_t *out);

/* Seeded synthetic imputation model with the reference's shapes, the same
 * workload the product's idash_synth_model generates (restated here so that
 * the CPU reference arm builds its workload from the oracle alone):
 *   tag p at position 100 + 16p + h(seed, 10, p) % 16;
 *   targets at sorted positions lo + mix64(key(seed, 11) ^ t) % span;
 *   target t's neighbours: its k nearest tags, ties to the left
 *   (train/to_vw.py:33-34), k fixed or choices[h(seed, 12, t) % n_choices];
 *   outputs 3t..3t+2 (eval/idash.cpp:337-339), features 3p+u of tag p
 *   (:388-390), coefficient h(key(seed,13), o*192 + q*3 + u) % 16384 - 8192,
 *   zeros dropped (train/test_vw_hr.py:44), then the constant with
 *   h(key(seed,14), o) % 16384 - 8192.
 * Arrays are malloc'd; release with oracle_synth_model_free.  Returns 0, or
 * -1 on bad arguments / allocation failure. */
typedef struct {
    uint64_t n_out, n_terms;
    uint64_t *term_ptr;
    uint32_t *term_feat;
    int32_t *term_coef;
    uint32_t *window_start, *window_len;
} oracle_synth_model_t;
int oracle_synth_model(uint64_t seed, uint32_t n_tags, uint32_t n_targets, uint32_t neighbours, uint32_t n_choices,
                       const uint32_t *choices, oracle_synth_model_t *out);
void oracle_synth_model_free(oracle_synth_model_t *m);

#ifdef __cplusplus
}
#endif

#endif
