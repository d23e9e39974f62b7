// Host side of the cloud step, mirroring the reference's interface for it
// (eval/idash.h): the same data roles, file formats and call sequence as
// eval/cloud.cpp, with ciphertexts kept as contiguous record images so that
// one copy moves them to or from the GPU.  Errors are returned, never
// aborted on.
#pragma once

#include <array>
#include <cstdint>
#include <iosfwd>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../../include/idash_gpu.h"

namespace idash_host {

typedef uint32_t FeatBigIndex;  // eval/idash.h:40
typedef uint32_t FeatIndex;     // eval/idash.h:41

// Size of one ciphertext record in encrypted_data.bin and
// encrypted_prediction.bin: uint32 index, int32 tag, 2N int32, double.
constexpr uint64_t kRecordBytes = 8 + 2 * 1024 * 4 + 8;  // 8208
constexpr int32_t kTlweSampleTag = 42;  // record tag of the ciphertext stream format

// eval/idash.h:45-111 (the fields the cloud step reads).
struct IdashParams {
    static constexpr uint32_t N = 1024;
    static constexpr uint32_t k = 1;
    static constexpr int32_t ONE_IN_T32 = 1 << 18;  // dtot32(2^-14), eval/idash.cpp:39
    uint32_t NUM_SAMPLES = 0, NUM_INPUT_POSITIONS = 0, NUM_OUTPUT_POSITIONS = 0;
    uint32_t NUM_INPUT_FEATURES = 0, NUM_OUTPUT_FEATURES = 0, NUM_REGIONS = 0, REGION_SIZE = 0;
    std::unordered_map<uint64_t, std::array<FeatBigIndex, 3>> in_features_index;
    std::unordered_map<uint64_t, std::array<FeatBigIndex, 3>> out_features_index;
    std::vector<std::pair<uint64_t, std::string>> out_position_names;

    FeatIndex feature_indexOf(FeatBigIndex b) const { return b / NUM_REGIONS; }
    uint32_t feature_regionOf(FeatBigIndex b) const { return b % NUM_REGIONS; }
    static FeatBigIndex constant_bigIndex() { return 0xFFFFFFFFu; }
};

// eval/idash.h:129-134: per output, input feature -> integer coefficient.
struct Model {
    std::unordered_map<FeatBigIndex, std::unordered_map<FeatBigIndex, int32_t>> model;
};

// A ciphertext file held as one image: 8-byte count, then `count` records.
struct RecordImage {
    uint8_t *data = nullptr;  // 16-byte aligned (pinned when a GPU is present)
    uint64_t bytes = 0, count = 0;
    bool pinned = false;
    RecordImage() = default;
    RecordImage(const RecordImage &) = delete;
    RecordImage &operator=(const RecordImage &) = delete;
    ~RecordImage();
    idash_status allocate(uint64_t count);
    uint8_t *record(uint64_t i) const { return data + 8 + i * kRecordBytes; }
    static idash_row_layout layout() { return idash_row_layout{kRecordBytes, 8, 8 + 2 * 1024 * 4, 0}; }
};

// eval/idash.h:136-167: FeatIndex -> the record that holds that TRLWE.
struct EncryptedData {
    RecordImage image;
    std::unordered_map<FeatIndex, uint64_t> record_of;
};

// eval/idash.h:169-188: FeatBigIndex -> output record.
struct EncryptedPredictions {
    RecordImage image;
    std::unordered_map<FeatBigIndex, uint64_t> record_of;
};

struct Status {
    idash_status code = IDASH_OK;
    std::string message;
    bool ok() const { return code == IDASH_OK; }
    static Status Ok() { return Status(); }
    static Status Err(idash_status c, std::string m) { return Status{c, std::move(m)}; }
};

// params.bin (eval/idash.cpp:128-186, 200-261).
Status read_params(IdashParams &params, const std::string &filename);
Status read_params_stream(IdashParams &params, std::istream &in);  // read_params_istream
Status write_params(const IdashParams &params, const std::string &filename);
// <dir>/<pos>_<snp>.hr for every output position (eval/idash.cpp:66-114,
// eval/parse_vw.cpp:8-30).
Status read_model(Model &model, const IdashParams &params, const std::string &path);
// encrypted_data.bin / encrypted_prediction.bin (eval/idash.cpp:513-613):
// the whole image moves as one range of the file.
Status read_encrypted_data(EncryptedData &data, const IdashParams &params, const std::string &filename);
Status write_encrypted_predictions(const EncryptedPredictions &preds, const std::string &filename);
// Writes a whole record image to `filename` (created or truncated).
Status write_image_file(const uint8_t *data, uint64_t bytes, const std::string &filename);
Status read_encrypted_predictions(EncryptedPredictions &preds, const std::string &filename);

struct CloudTiming {
    double plan_s = 0, score_s = 0;  // model planning; copies + kernels
    idash_model_info plan{};         // the plan the scoring ran (kernel kind, slice width)
};

// The tuned plan beside a model cache (`<cache>.plan`), keyed by the same
// fingerprint: apply_cached_plan pins its kernel kind and slice width on the
// context before the model is planned, so the autotuner only chooses among
// what is left (ring depth, CTAs per SM); save_plan records it after a run.
// Both are best effort: a missing or stale file changes nothing.
bool apply_cached_plan(idash_ctx *ctx, const std::string &cache_path, const std::string &params_file,
                       const std::string &model_dir);
void save_plan(const std::string &cache_path, const std::string &params_file, const std::string &model_dir,
               const idash_model_info &plan);

// The model as the GPU consumes it: outputs in FeatBigIndex order (so that
// neighbouring targets share input windows), each output's terms in the
// order the reference's map iterates them (the order of its variance sum,
// eval/idash.cpp:800-819), and the record each output takes in
// encrypted_prediction.bin (the order the reference writes, :607).
struct FlatModel {
    std::vector<FeatBigIndex> out_bidx;
    std::vector<uint32_t> out_row;
    std::vector<uint64_t> term_ptr;
    std::vector<uint32_t> term_feat;
    std::vector<int32_t> term_coef;
};
FlatModel flatten_model(const Model &model);

// Model-ingest cache: the flattened model in one file, tagged with a
// fingerprint of params.bin and the model directory's path.  Reading it
// replaces parsing one .hr file per output (eval/idash.cpp:66-114).  The
// cache does not watch the .hr files: remove it when they change.
uint64_t fingerprint(const std::string &params_file, const std::string &model_dir);
Status write_model_cache(const FlatModel &flat, uint64_t fp, const std::string &path);
Status read_model_cache(FlatModel *flat, uint64_t fp, const std::string &path);

// eval/idash.h:251-252 / eval/idash.cpp:763-848 on the GPU behind the C ABI.
// `preds` must be empty on entry.  Records come out in the order the
// reference's EncryptedPredictions map iterates, so the written file matches
// the reference's byte for byte.
Status cloud_compute_score(EncryptedPredictions &preds, const EncryptedData &data, const Model &model,
                           const IdashParams &params, idash_ctx *ctx, CloudTiming *timing = nullptr);
Status cloud_compute_score(EncryptedPredictions &preds, const EncryptedData &data, const FlatModel &flat,
                           const IdashParams &params, idash_ctx *ctx, CloudTiming *timing = nullptr);

// params.bin, model (from the cache at cache_path when it is valid, else
// parsed and, when cache_path is non-empty, cached there).
Status load_model(Model *parsed, FlatModel *flat, const IdashParams &params, const std::string &params_file,
                  const std::string &model_dir, const std::string &cache_path, bool *from_cache);

// ------------------------------------------------------------ decryption
// keys.bin (write_key / read_key, eval/idash.cpp:476-502): the params.bin
// content, then the TRLWE key record (int32 tag, int32 N, int32 k,
// double alpha_min, double alpha_max, k * N int32 coefficients).
struct IdashKey {
    IdashParams params;
    uint32_t N = 0, k = 0;
    double alpha_min = 0, alpha_max = 0;
    std::vector<int32_t> key;  // k * N coefficients
};
constexpr int32_t kTlweKeyTag = 52;  // record tag of the key stream format
Status read_key(IdashKey &key, const std::string &filename);

// ------------------------------------------------------------ encryption
// eval/idash.h:123-127: per tag position, NUM_SAMPLES genotypes (0/1/2, -1
// when missing).  Same container as the reference, filled in the same order,
// so it iterates in the same order.
struct PlaintextData {
    std::unordered_map<uint64_t, std::vector<int8_t>> data;
};
// read_plaintext_data (eval/idash.cpp:280-309).
Status read_plaintext_data(PlaintextData &plain, const IdashParams &params, const std::string &filename);
// Every plaintext position is an input position of params, and the features
// fill the reference's ciphertext pool (eval/idash.cpp:621-641).
Status check_plaintext(const PlaintextData &plain, const IdashParams &params);
// dtot32 (a double on the torus -> Torus32, fractional part truncated).
int32_t dtot32(double d);
// encrypt_data_ph1 + ph2 (eval/idash.cpp:615-679) on the GPU: one record
// per FeatIndex, in the order the reference's EncryptedData map iterates.
// seed: the mask / noise generator's key.
Status encrypt_data(EncryptedData &enc, const PlaintextData &plain, const IdashKey &key, idash_ctx *ctx,
                    uint64_t seed);
// write_encrypted_data (eval/idash.cpp:536-556): one bulk write.
Status write_encrypted_data(const EncryptedData &enc, const std::string &filename);

// eval/idash.h:190-211, held as one matrix: the scores of the prediction
// file's record r at [r * num_samples, (r + 1) * num_samples).
struct DecryptedPredictions {
    uint32_t num_samples = 0;
    std::vector<float> scores;
    std::unordered_map<FeatBigIndex, uint64_t> row_of;  // FeatBigIndex -> record
};
// Every output the params name has a record in the predictions.
Status check_predictions(const EncryptedPredictions &preds, const IdashParams &params);
// decrypt_predictions (eval/idash.cpp:682-761): every record's phase on the
// GPU, t32tod of coefficients [0, NUM_SAMPLES) as float.
Status decrypt_predictions(DecryptedPredictions &dec, const EncryptedPredictions &preds, const IdashKey &key,
                           idash_ctx *ctx);
// write_decrypted_predictions (eval/idash.cpp:436-469), byte for byte;
// formatted on all host threads.
Status write_decrypted_predictions(const DecryptedPredictions &dec, const IdashParams &params,
                                   const std::string &filename, bool print_pos_name, uint64_t *n_lines = nullptr);

}  // namespace idash_host
