// Drop-in GPU definition of the reference's
//   void cloud_compute_score(EncryptedPredictions &, const EncryptedData &,
//                            const Model &, const IdashParams &)
// (declared at eval/idash.h:251-252, defined at eval/idash.cpp:763-848),
// written against the reference's own eval/idash.h and TFHE types.
//
// To use it in the reference's build: compile eval/idash.cpp with
//   -Dcloud_compute_score=cloud_compute_score_cpu
// (or delete its definition), add this file, and link libidash_gpu.so.
// Behaviour kept: enc_preds gets one new TLweSample per model output
// (createAndGet, eval/idash.h:174-183), created in the model map's iteration
// order before any scoring, as eval/idash.cpp:772-777 creates them.  The
// order of insertion decides the iteration order of enc_preds.score, and so
// the record order write_encrypted_predictions writes (eval/idash.cpp:605-608):
// the prediction file comes out byte-identical to the reference's.
// Coefficients and current_variance are the reference's; failures print and
// abort like REQUIRE_DRAMATICALLY (eval/idash.h:12).
#include <algorithm>
#include <cstring>
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

void cloud_compute_score(EncryptedPredictions &enc_preds, const EncryptedData &enc_data, const Model &model,
                         const IdashParams &params) {
    const TLweParams *tp = params.tlweParams;
    REQUIRE_DRAMATICALLY(tp->k == 1 && tp->N == (int32_t)params.N, "only k = 1, N = IdashParams::N");
    const uint32_t N = params.N;
    const uint64_t kStride = 16 + 8 * uint64_t(N);  // one record: index, tag, a|b, variance
    idash_ctx *ctx = context();

    // The output samples first, in the model map's iteration order
    // (eval/idash.cpp:772-777): this fixes the record order of the file.
    std::vector<FeatBigIndex> outs;
    for (const auto &it : model.model) {
        enc_preds.createAndGet(it.first, tp);
        outs.push_back(it.first);
    }
    // Scored in FeatBigIndex order (neighbouring targets share input
    // windows), terms in each inner map's iteration order (the order of the
    // double variance sum, eval/idash.cpp:800-819).
    std::sort(outs.begin(), outs.end());
    std::vector<uint64_t> term_ptr(outs.size() + 1, 0);
    std::vector<uint32_t> term_feat;
    std::vector<int32_t> term_coef;
    for (size_t o = 0; o < outs.size(); ++o) {
        for (const auto &t : model.model.at(outs[o])) {
            term_feat.push_back(t.first);
            term_coef.push_back(t.second);
        }
        term_ptr[o + 1] = term_feat.size();
    }

    // Inputs: one page-locked record per FeatIndex (dense rows, index = row).
    uint64_t n_rows = 0;
    for (const auto &it : enc_data.enc_data) n_rows = std::max<uint64_t>(n_rows, uint64_t(it.first) + 1);
    void *h_in = nullptr, *h_out = nullptr;
    require_ok(idash_host_alloc(ctx, 16 + n_rows * kStride, &h_in), ctx, "idash_host_alloc");
    require_ok(idash_host_alloc(ctx, 16 + outs.size() * kStride, &h_out), ctx, "idash_host_alloc");
    uint8_t *in = static_cast<uint8_t *>(h_in) + 8;  // payloads 16-byte aligned
    uint8_t *out = static_cast<uint8_t *>(h_out) + 8;
    std::memset(in, 0, n_rows * kStride);
    for (const auto &it : enc_data.enc_data) {
        uint8_t *rec = in + uint64_t(it.first) * kStride;
        std::memcpy(rec + 8, it.second->a[0].coefsT, sizeof(Torus32) * N);
        std::memcpy(rec + 8 + 4 * N, it.second->b->coefsT, sizeof(Torus32) * N);
        std::memcpy(rec + 8 + 8 * N, &it.second->current_variance, sizeof(double));
    }

    // FeatIndex -> row; a term naming a TRLWE that enc_data lacks is an
    // IDASH_ERR_INDEX, where the reference aborts (eval/idash.h:164).
    std::vector<uint32_t> row_of_index(n_rows, 0xFFFFFFFFu);
    for (const auto &it : enc_data.enc_data) row_of_index[it.first] = it.first;

    idash_trlwe_params p{N, 1, params.NUM_SAMPLES, params.NUM_REGIONS, params.REGION_SIZE, params.ONE_IN_T32, 0};
    idash_model *m = nullptr;
    require_ok(idash_model_trlwe(ctx, &m, &p, outs.size(), outs.data(), nullptr, term_ptr.data(), term_feat.data(),
                                 term_coef.data(), n_rows, row_of_index.data(), n_rows),
               ctx, "idash_model_trlwe");
    const idash_row_layout in_l{kStride, 8, int64_t(8 + 8 * N), -1};
    const idash_row_layout out_l{kStride, 8, int64_t(8 + 8 * N), 0};
    require_ok(idash_score_trlwe_host(m, in, &in_l, n_rows, out, &out_l), ctx, "idash_score_trlwe_host");
    idash_model_free(m);

    for (size_t o = 0; o < outs.size(); ++o) {
        TLweSample *s = enc_preds.get(outs[o], tp);
        const uint8_t *rec = out + o * kStride;
        std::memcpy(s->a[0].coefsT, rec + 8, sizeof(Torus32) * N);
        std::memcpy(s->b->coefsT, rec + 8 + 4 * N, sizeof(Torus32) * N);
        std::memcpy(&s->current_variance, rec + 8 + 8 * N, sizeof(double));
    }
    idash_host_free(ctx, h_in);
    idash_host_free(ctx, h_out);
}
