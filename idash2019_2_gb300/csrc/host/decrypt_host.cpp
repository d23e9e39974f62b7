// Party A's decryption step on the GPU, mirroring eval/decrypt.cpp and the
// functions it calls: read_key (eval/idash.cpp:488-502),
// decrypt_predictions (:682-761) and write_decrypted_predictions (:436-469).
// The phase products run in one kernel launch over every prediction record;
// the CSV is formatted on all host threads, each float exactly as an iostream
// prints it (printf "%.6g" of the value, which std::to_chars with general
// format and precision 6 reproduces).
#include <cuda_runtime.h>

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <charconv>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <thread>
#include <vector>

#include "idash_host.hpp"

namespace idash_host {

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Appends v as `std::ostream << v` does for a float at the default precision.
inline char *put_float(char *p, char *end, float v) {
    return std::to_chars(p, end, v, std::chars_format::general, 6).ptr;
}

inline char *put_u64(char *p, char *end, uint64_t v) { return std::to_chars(p, end, v).ptr; }

}  // namespace

Status read_key(IdashKey &key, const std::string &filename) {
    std::ifstream in(filename, std::ios::binary);
    if (!in) return Status::Err(IDASH_ERR_IO, "cannot open key file '" + filename + "'");
    key = IdashKey();
    Status st = read_params_stream(key.params, in);
    if (!st.ok()) return Status::Err(st.code, filename + ": " + st.message);
    int32_t hdr[3] = {0, 0, 0};
    in.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
    in.read(reinterpret_cast<char *>(&key.alpha_min), sizeof(double));
    in.read(reinterpret_cast<char *>(&key.alpha_max), sizeof(double));
    if (!in || hdr[0] != kTlweKeyTag)
        return Status::Err(IDASH_ERR_FORMAT, filename + ": missing or malformed TRLWE key record");
    if (hdr[1] != int32_t(IdashParams::N) || hdr[2] != int32_t(IdashParams::k))
        return Status::Err(IDASH_ERR_UNSUPPORTED, filename + ": key is not N = 1024, k = 1");
    key.N = uint32_t(hdr[1]);
    key.k = uint32_t(hdr[2]);
    key.key.resize(size_t(key.N) * key.k);
    in.read(reinterpret_cast<char *>(key.key.data()), std::streamsize(key.key.size() * 4));
    if (size_t(in.gcount()) != key.key.size() * 4)
        return Status::Err(IDASH_ERR_FORMAT, filename + ": truncated key coefficients");
    return Status::Ok();
}

Status check_predictions(const EncryptedPredictions &preds, const IdashParams &params) {
    // every output the CSV names must have a record (the reference's
    // enc_preds.score.at(outBIdx) aborts otherwise, eval/idash.cpp:711)
    for (const auto &it : params.out_features_index)
        for (FeatBigIndex b : it.second)
            if (!preds.record_of.count(b))
                return Status::Err(IDASH_ERR_INDEX, "encrypted predictions hold no record for output " +
                                                        std::to_string(b));
    return Status::Ok();
}

Status decrypt_predictions(DecryptedPredictions &dec, const EncryptedPredictions &preds, const IdashKey &key,
                           idash_ctx *ctx) {
    const IdashParams &params = key.params;
    dec = DecryptedPredictions();
    dec.num_samples = params.NUM_SAMPLES;
    dec.row_of = preds.record_of;
    Status chk = check_predictions(preds, params);
    if (!chk.ok()) return chk;
    const uint64_t n = preds.image.count;
    if (n == 0 || dec.num_samples == 0) return Status::Ok();
    dec.scores.resize(n * dec.num_samples);
    void *d_img = nullptr;
    float *d_out = nullptr;
    auto cuda = [&](cudaError_t e, const char *what) {
        return e == cudaSuccess ? Status::Ok()
                                : Status::Err(e == cudaErrorMemoryAllocation ? IDASH_ERR_OUT_OF_MEMORY : IDASH_ERR_CUDA,
                                              std::string(what) + ": " + cudaGetErrorString(e));
    };
    Status st = cuda(cudaMalloc(&d_img, preds.image.bytes), "cudaMalloc(predictions)");
    if (st.ok()) st = cuda(cudaMalloc(&d_out, dec.scores.size() * sizeof(float)), "cudaMalloc(scores)");
    cudaStream_t s = static_cast<cudaStream_t>(idash_stream(ctx));
    if (st.ok())
        st = cuda(cudaMemcpyAsync(d_img, preds.image.data, preds.image.bytes, cudaMemcpyHostToDevice, s), "copy in");
    if (st.ok()) {
        const idash_row_layout lay = RecordImage::layout();
        idash_status code = idash_decrypt_trlwe_device(ctx, key.key.data(), key.N, static_cast<uint8_t *>(d_img) + 8,
                                                       &lay, n, dec.num_samples, d_out, nullptr);
        if (code != IDASH_OK) st = Status::Err(code, idash_last_error(ctx));
    }
    if (st.ok())
        st = cuda(cudaMemcpyAsync(dec.scores.data(), d_out, dec.scores.size() * sizeof(float), cudaMemcpyDeviceToHost,
                                  s),
                  "copy out");
    if (st.ok()) {
        idash_status code = idash_sync(ctx);
        if (code != IDASH_OK) st = Status::Err(code, idash_last_error(ctx));
    }
    cudaFree(d_img);
    cudaFree(d_out);
    return st;
}

Status write_decrypted_predictions(const DecryptedPredictions &dec, const IdashParams &params,
                                   const std::string &filename, bool print_pos_name, uint64_t *n_lines) {
    // per output position (CSV order), the score rows of its 3 genotypes
    const size_t P = params.out_position_names.size();
    std::vector<std::array<const float *, 3>> rows(P);
    for (size_t p = 0; p < P; ++p) {
        const auto it = params.out_features_index.find(params.out_position_names[p].first);
        if (it == params.out_features_index.end())
            return Status::Err(IDASH_ERR_FORMAT, "params: output position without feature indices");
        for (int g = 0; g < 3; ++g) {
            const auto r = dec.row_of.find(it->second[g]);
            if (r == dec.row_of.end())
                return Status::Err(IDASH_ERR_INDEX, "no decrypted scores for output " + std::to_string(it->second[g]));
            rows[p][g] = dec.scores.data() + r->second * dec.num_samples;
        }
    }
    const uint64_t S = params.NUM_SAMPLES;
    if (S > dec.num_samples) return Status::Err(IDASH_ERR_FORMAT, "fewer decrypted samples than NUM_SAMPLES");
    const int fd = ::open(filename.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return Status::Err(IDASH_ERR_IO, "cannot open '" + filename + "' for write");
    static const char kHeader[] = "Subject ID,target SNP,0,1,2\n";
    uint64_t offset = sizeof(kHeader) - 1;
    bool ok = ::pwrite(fd, kHeader, offset, 0) == ssize_t(offset);

    // Lines in the reference's order (sample-major, positions in CSV order).
    // Each round, every thread formats a chunk of samples into its own buffer
    // (allocated once, not cleared); the chunks are then written in order.
    // Writing them from one thread measured as fast as writing them in
    // parallel at their offsets: the write of a 3.2 GB file is bound by the
    // disk, not by the copy into the page cache.
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const uint64_t per_chunk = std::max<uint64_t>(1, (uint64_t(1) << 20) / std::max<uint64_t>(P, 1));  // ~1 M lines
    size_t name_max = 20;
    for (const auto &pn : params.out_position_names) name_max = std::max(name_max, pn.second.size());
    const size_t line_max = 20 + 1 + name_max + 1 + 3 * 16 + 4;
    const size_t buf_bytes = size_t(per_chunk) * P * line_max;
    std::vector<std::unique_ptr<char[]>> bufs(hw);
    std::vector<size_t> used(hw, 0);
    for (uint64_t s0 = 0; s0 < S && ok; s0 += per_chunk * hw) {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < hw; ++t) {
            const uint64_t a = s0 + t * per_chunk, b = std::min(S, a + per_chunk);
            used[t] = 0;
            if (a >= b) continue;
            pool.emplace_back([&, t, a, b]() {
                if (!bufs[t]) bufs[t].reset(new char[buf_bytes]);
                char *const begin = bufs[t].get();
                char *p = begin, *end = begin + buf_bytes;
                for (uint64_t smp = a; smp < b; ++smp)
                    for (size_t q = 0; q < P; ++q) {
                        p = put_u64(p, end, smp);
                        *p++ = ',';
                        if (print_pos_name) {
                            const std::string &nm = params.out_position_names[q].second;
                            std::memcpy(p, nm.data(), nm.size());
                            p += nm.size();
                        } else {
                            p = put_u64(p, end, params.out_position_names[q].first);
                        }
                        for (int g = 0; g < 3; ++g) {
                            *p++ = ',';
                            p = put_float(p, end, rows[q][g][smp]);
                        }
                        *p++ = '\n';
                    }
                used[t] = size_t(p - begin);
            });
        }
        for (auto &th : pool) th.join();
        for (unsigned t = 0; t < hw && ok; ++t) {
            size_t done = 0;
            while (done < used[t]) {
                const ssize_t r = ::pwrite(fd, bufs[t].get() + done, used[t] - done, off_t(offset + done));
                if (r < 0 && errno == EINTR) continue;
                if (r <= 0) {
                    ok = false;
                    break;
                }
                done += size_t(r);
            }
            offset += done;
        }
    }
    ok = (::close(fd) == 0) && ok;
    if (!ok) return Status::Err(IDASH_ERR_IO, "short write to '" + filename + "'");
    if (n_lines) *n_lines = S * P;
    return Status::Ok();
}

}  // namespace idash_host

using namespace idash_host;

extern "C" idash_status idash_decrypt_files(int device, const char *keys_file, const char *pred_file,
                                            const char *csv_file, int by_position, idash_decrypt_report *report,
                                            char *errbuf, size_t errbuf_len) {
    auto fail = [&](const Status &st) {
        if (errbuf && errbuf_len) std::snprintf(errbuf, errbuf_len, "%s", st.message.c_str());
        return st.code;
    };
    if (!keys_file || !pred_file || !csv_file) return fail(Status::Err(IDASH_ERR_INVALID_ARGUMENT, "null file name"));
    const double t0 = now_s();
    IdashKey key;
    EncryptedPredictions preds;
    Status st = read_key(key, keys_file);
    if (st.ok()) st = read_encrypted_predictions(preds, pred_file);
    if (st.ok()) st = check_predictions(preds, key.params);
    if (!st.ok()) return fail(st);  // inputs are validated before the device is touched
    const double t1 = now_s();
    idash_ctx *ctx = nullptr;
    idash_status s = idash_open(&ctx, device);
    if (s != IDASH_OK) return fail(Status::Err(s, idash_last_error(nullptr)));
    DecryptedPredictions dec;
    st = decrypt_predictions(dec, preds, key, ctx);
    idash_close(ctx);
    const double t2 = now_s();
    uint64_t lines = 0;
    if (st.ok()) st = write_decrypted_predictions(dec, key.params, csv_file, by_position == 0, &lines);
    const double t3 = now_s();
    if (!st.ok()) return fail(st);
    if (report) {
        report->read_s = t1 - t0;
        report->decrypt_s = t2 - t1;
        report->write_s = t3 - t2;
        report->n_records = preds.image.count;
        report->n_lines = lines;
    }
    if (errbuf && errbuf_len) errbuf[0] = '\0';
    return IDASH_OK;
}
