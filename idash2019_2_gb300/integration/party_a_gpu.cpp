// Drop-in GPU definitions of party A's two heavy functions, written against
// the reference's own eval/idash.h and TFHE types:
//   void decrypt_predictions(DecryptedPredictions &, const EncryptedPredictions &,
//                            const IdashKey &)                 (eval/idash.cpp:682-761)
//   void encrypt_data_ph1(EncryptedData &, const PlaintextData &,
//                         const IdashKey &)                     (eval/idash.cpp:615-641)
//
// To use them in the reference's build: compile eval/idash.cpp with
//   -Ddecrypt_predictions=decrypt_predictions_cpu
//   -Dencrypt_data_ph1=encrypt_data_ph1_cpu
// (or delete those definitions), add this file, and link libidash_gpu.so.
// encrypt_data_ph2 (the messages, a cheap host loop) stays the reference's.
// Behaviour kept: decrypt_predictions fills predictions.score[pos][snp] with
// NUM_SAMPLES floats t32tod(phase) per output position; encrypt_data_ph1
// hands out a pool of ceil(NUM_INPUT_FEATURES / NUM_REGIONS) fresh
// encryptions of zero (variance alpha^2) in the reference's first-visit order.
// Failures print and abort like REQUIRE_DRAMATICALLY (eval/idash.h:12).
#include <cstring>
#include <random>
#include <vector>

#include "idash.h"
#include "idash_gpu.h"

namespace {

void require_ok(idash_status s, idash_ctx *ctx, const char *what) {
    if (s != IDASH_OK) {
        std::cout << "ERROR: " << what << ": " << idash_status_string(s) << ": " << idash_last_error(ctx)
                  << std::endl;
        abort();
    }
}

idash_ctx *context() {
    static idash_ctx *ctx = nullptr;
    if (!ctx) require_ok(idash_open(&ctx, 0), nullptr, "idash_open");
    return ctx;
}

}  // namespace

void decrypt_predictions(DecryptedPredictions &predictions, const EncryptedPredictions &enc_preds,
                         const IdashKey &key) {
    const IdashParams &params = *key.idashParams;
    const uint32_t N = params.N, NS = params.NUM_SAMPLES;
    const uint64_t kStride = 16 + 8 * uint64_t(N);  // one record: index, tag, a|b, variance
    REQUIRE_DRAMATICALLY(key.tlweKey->params->k == 1 && key.tlweKey->params->N == (int32_t)N,
                         "only k = 1, N = IdashParams::N");
    idash_ctx *ctx = context();
    // the outputs the CSV names, in one dense record array
    std::vector<FeatBigIndex> outs;
    for (const auto &it : params.out_features_index)
        for (int snp = 0; snp < 3; ++snp) outs.push_back(it.second[snp]);
    const uint64_t n = outs.size();
    void *h_rec = nullptr, *d_rec = nullptr, *d_scores = nullptr;
    require_ok(idash_host_alloc(ctx, 16 + n * kStride, &h_rec), ctx, "idash_host_alloc");
    uint8_t *rec = static_cast<uint8_t *>(h_rec) + 8;  // payloads 16-byte aligned
    for (uint64_t i = 0; i < n; ++i) {
        const TLweSample *s = enc_preds.score.at(outs[i]);
        std::memcpy(rec + i * kStride + 8, s->a[0].coefsT, sizeof(Torus32) * N);
        std::memcpy(rec + i * kStride + 8 + 4 * N, s->b->coefsT, sizeof(Torus32) * N);
    }
    std::vector<float> scores(n * NS);
    require_ok(idash_device_alloc(ctx, 16 + n * kStride, &d_rec), ctx, "idash_device_alloc");
    require_ok(idash_device_alloc(ctx, scores.size() * sizeof(float) + 16, &d_scores), ctx, "idash_device_alloc");
    uint8_t *drec = static_cast<uint8_t *>(d_rec) + 8;
    require_ok(idash_copy_h2d(ctx, drec, rec, n * kStride), ctx, "copy in");
    const idash_row_layout lay{kStride, 8, -1, -1};
    require_ok(idash_decrypt_trlwe_device(ctx, key.tlweKey->key[0].coefs, N, drec, &lay, n, NS,
                                          static_cast<float *>(d_scores), nullptr),
               ctx, "idash_decrypt_trlwe_device");
    require_ok(idash_copy_d2h(ctx, scores.data(), d_scores, scores.size() * sizeof(float)), ctx, "copy out");
    require_ok(idash_sync(ctx), ctx, "idash_sync");
    uint64_t i = 0;
    for (const auto &it : params.out_features_index)
        for (int snp = 0; snp < 3; ++snp, ++i) {
            std::vector<float> &res = predictions.score[it.first][snp];
            res.assign(scores.begin() + i * NS, scores.begin() + (i + 1) * NS);
        }
    idash_device_free(ctx, d_rec);
    idash_device_free(ctx, d_scores);
    idash_host_free(ctx, h_rec);
}

void encrypt_data_ph1(EncryptedData &enc_data, const PlaintextData &plain_data, const IdashKey &key) {
    const IdashParams &params = *key.idashParams;
    const uint32_t N = params.N;
    const uint64_t kStride = 16 + 8 * uint64_t(N);  // one record: index, tag, a|b, variance
    REQUIRE_DRAMATICALLY(plain_data.data.size() == params.NUM_INPUT_POSITIONS, "Incomplete plaintext");
    REQUIRE_DRAMATICALLY(key.tlweKey->params->k == 1 && key.tlweKey->params->N == (int32_t)N,
                         "only k = 1, N = IdashParams::N");
    idash_ctx *ctx = context();
    const uint64_t pool_n = (params.NUM_INPUT_FEATURES + params.NUM_REGIONS - 1) / params.NUM_REGIONS;
    TLweSample *pool = new_TLweSample_array(pool_n, params.tlweParams);
    if (pool_n) {
        void *h_rec = nullptr, *d_rec = nullptr;
        require_ok(idash_host_alloc(ctx, 16 + pool_n * kStride, &h_rec), ctx, "idash_host_alloc");
        require_ok(idash_device_alloc(ctx, 16 + pool_n * kStride, &d_rec), ctx, "idash_device_alloc");
        uint8_t *drec = static_cast<uint8_t *>(d_rec) + 8, *rec = static_cast<uint8_t *>(h_rec) + 8;
        // encryptions of zero: no message slots (num_samples = 0)
        idash_encrypt_params p{};
        p.N = N;
        p.k = 1;
        p.num_samples = 0;
        p.num_regions = params.NUM_REGIONS;
        p.region_size = params.REGION_SIZE;
        p.record_tag = 0;
        p.alpha = params.alpha;
        std::random_device rd;
        const uint64_t seed = ((uint64_t(rd()) << 32) ^ rd()) | 1u;
        const idash_row_layout lay{kStride, 8, int64_t(8 + 8 * N), 0};
        require_ok(idash_encrypt_trlwe_device(ctx, &p, key.tlweKey->key[0].coefs, seed, pool_n, nullptr, nullptr, 0,
                                              nullptr, nullptr, drec, &lay, nullptr, nullptr),
                   ctx, "idash_encrypt_trlwe_device");
        require_ok(idash_copy_d2h(ctx, rec, drec, pool_n * kStride), ctx, "copy out");
        require_ok(idash_sync(ctx), ctx, "idash_sync");
        for (uint64_t i = 0; i < pool_n; ++i) {
            std::memcpy(pool[i].a[0].coefsT, rec + i * kStride + 8, sizeof(Torus32) * N);
            std::memcpy(pool[i].b->coefsT, rec + i * kStride + 8 + 4 * N, sizeof(Torus32) * N);
            std::memcpy(&pool[i].current_variance, rec + i * kStride + 8 + 8 * N, sizeof(double));
        }
        idash_device_free(ctx, d_rec);
        idash_host_free(ctx, h_rec);
    }
    // hand the pool out in the reference's first-visit order (:631-638)
    TLweSample *nextSample = pool;
    for (const auto &it : plain_data.data) {
        const uint64_t &pos = it.first;
        enc_data.ensure_exists(params.inBigIdx(pos, 0), nextSample, params);
        enc_data.ensure_exists(params.inBigIdx(pos, 1), nextSample, params);
        enc_data.ensure_exists(params.inBigIdx(pos, 2), nextSample, params);
    }
    REQUIRE_DRAMATICALLY(nextSample <= pool + pool_n, "memory error");
    REQUIRE_DRAMATICALLY(nextSample >= pool + pool_n - 10, "memory pb");
}
