// Party A's encryption step on the GPU, mirroring eval/encrypt.cpp and the
// functions it calls: read_plaintext_data (eval/idash.cpp:280-309),
// encrypt_data_ph1 / ph2 (:615-679) and write_encrypted_data (:536-556).
//
// The host reproduces the reference's bookkeeping: positions are read into
// the same container in the same order, features are assigned to TRLWE rows
// in the order ph1 visits them, and the records are written in the order the
// reference's FeatIndex map iterates.  The device does the arithmetic: fresh
// encryptions of zero plus the one-hot messages, in one kernel launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <thread>
#include <vector>

#include "idash_host.hpp"

namespace idash_host {

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

constexpr double kAlpha = 2.9802322387695312e-08;  // IdashParams::alpha = 2^-25 (eval/idash.cpp:20)
constexpr double kInScaling = 1.0 / 16384;        // IN_SCALING_FACTOR (eval/idash.cpp:29)

}  // namespace

int32_t dtot32(double d) { return int32_t(uint32_t(uint64_t(int64_t((d - std::trunc(d)) * 4294967296.0)))); }

Status read_plaintext_data(PlaintextData &plain, const IdashParams &params, const std::string &filename) {
    std::ifstream challenge(filename);
    if (!challenge) return Status::Err(IDASH_ERR_IO, "cannot open challenge file '" + filename + "'");
    plain = PlaintextData();
    // The lines the reference reads (at most NUM_INPUT_POSITIONS), each parsed
    // as the reference parses it, token by token with an istringstream, on
    // host threads; then inserted into the map in file order, so that its
    // iteration order is the reference's.
    std::vector<std::string> lines;
    std::string line;
    for (std::getline(challenge, line); challenge && lines.size() < params.NUM_INPUT_POSITIONS;
         std::getline(challenge, line))
        lines.push_back(std::move(line));
    struct Parsed {
        uint64_t position = 0;
        std::vector<int8_t> values;
        Status st = Status::Ok();
    };
    std::vector<Parsed> parsed(lines.size());
    auto parse = [&](size_t i) {
        Parsed &out = parsed[i];
        std::istringstream iss(lines[i]);
        int chrom = 0;  // must be 22
        uint64_t position2 = 0;
        std::string name;
        iss >> chrom;
        if (chrom != 22) {
            out.st = Status::Err(IDASH_ERR_FORMAT, filename + ": line " + std::to_string(i + 1) +
                                                       " does not start with 22");
            return;
        }
        iss >> out.position >> position2 >> name;
        if (!iss) {
            out.st = Status::Err(IDASH_ERR_FORMAT, filename + ": line " + std::to_string(i + 1) + " is short");
            return;
        }
        out.values.resize(params.NUM_SAMPLES);
        std::string snp;
        for (uint32_t s = 0; s < params.NUM_SAMPLES; ++s) {
            iss >> snp;  // keeps the previous token when the line runs out, as the reference's loop does
            out.values[s] = (snp == "0" || snp == "1" || snp == "2") ? int8_t(snp[0] - '0') : int8_t(-1);
        }
    };
    const size_t n_threads =
        std::max<size_t>(1, std::min<size_t>({16, std::thread::hardware_concurrency(), lines.size() / 64 + 1}));
    std::vector<std::thread> threads;
    for (size_t t = 1; t < n_threads; ++t)
        threads.emplace_back([&, t] {
            for (size_t i = lines.size() * t / n_threads; i < lines.size() * (t + 1) / n_threads; ++i) parse(i);
        });
    for (size_t i = 0; i < lines.size() / n_threads; ++i) parse(i);
    for (auto &th : threads) th.join();
    for (Parsed &p : parsed) {
        if (!p.st.ok()) return p.st;  // the first failure in file order
        plain.data[p.position] = std::move(p.values);
    }
    if (parsed.size() != params.NUM_INPUT_POSITIONS)
        return Status::Err(IDASH_ERR_FORMAT, filename + ": missing positions in plaintext file");
    return Status::Ok();
}

Status check_plaintext(const PlaintextData &plain, const IdashParams &params) {
    std::unordered_map<FeatIndex, uint64_t> seen;
    for (const auto &it : plain.data) {
        const auto f = params.in_features_index.find(it.first);
        if (f == params.in_features_index.end())
            return Status::Err(IDASH_ERR_FORMAT, "plaintext position " + std::to_string(it.first) +
                                                     " is not an input position of params");
        for (int v = 0; v < 3; ++v) seen.emplace(params.feature_indexOf(f->second[v]), 0);
    }
    const uint64_t pool = (uint64_t(params.NUM_INPUT_FEATURES) + params.NUM_REGIONS - 1) / params.NUM_REGIONS;
    if (seen.size() > pool || seen.size() + 10 < pool)
        return Status::Err(IDASH_ERR_FORMAT, "plaintext features do not fill the ciphertext pool (eval/idash.cpp:640)");
    return Status::Ok();
}

Status encrypt_data(EncryptedData &enc, const PlaintextData &plain, const IdashKey &key, idash_ctx *ctx,
                    uint64_t seed) {
    const IdashParams &params = key.params;
    Status chk = check_plaintext(plain, params);
    if (!chk.ok()) return chk;
    const uint32_t R = params.NUM_REGIONS, NS = params.NUM_SAMPLES;
    // ph1: TRLWE rows handed out as the reference hands out its pool of
    // zero-encryptions, one per FeatIndex in first-visit order (:631-638)
    std::unordered_map<FeatIndex, uint64_t> enc_map;
    std::vector<FeatIndex> index_of_row;
    std::vector<std::array<uint32_t, 3>> slots_of_pos;  // per position: its 3 FeatBigIndex
    std::vector<const std::vector<int8_t> *> geno_rows;
    for (const auto &it : plain.data) {
        const auto f = params.in_features_index.find(it.first);
        if (f == params.in_features_index.end())
            return Status::Err(IDASH_ERR_FORMAT, "plaintext position " + std::to_string(it.first) +
                                                     " is not an input position of params");
        for (int v = 0; v < 3; ++v) {
            const FeatIndex fi = params.feature_indexOf(f->second[v]);
            if (enc_map.emplace(fi, index_of_row.size()).second) index_of_row.push_back(fi);
        }
        slots_of_pos.push_back(f->second);
        geno_rows.push_back(&it.second);
    }
    const uint64_t pool = (uint64_t(params.NUM_INPUT_FEATURES) + R - 1) / R;
    if (index_of_row.size() > pool || index_of_row.size() + 10 < pool)
        return Status::Err(IDASH_ERR_FORMAT, "plaintext features do not fill the ciphertext pool (eval/idash.cpp:640)");
    const uint64_t n_rows = index_of_row.size();
    // records in the map's iteration order (write_encrypted_data, :550-553)
    std::vector<uint32_t> row_out(n_rows);
    {
        uint32_t rec = 0;
        for (const auto &it : enc_map) row_out[it.second] = rec++;
    }
    // ph2's setScore targets: slot (row, region) -> plaintext feature 3p + v
    std::vector<uint32_t> slot_src(n_rows * R, 0xFFFFFFFFu);
    for (size_t p = 0; p < slots_of_pos.size(); ++p)
        for (uint32_t v = 0; v < 3; ++v) {
            const FeatBigIndex b = slots_of_pos[p][v];
            slot_src[enc_map.at(params.feature_indexOf(b)) * R + params.feature_regionOf(b)] = uint32_t(3 * p + v);
        }
    std::vector<int8_t> geno(geno_rows.size() * size_t(std::max<uint32_t>(NS, 1)));
    for (size_t p = 0; p < geno_rows.size(); ++p)
        std::memcpy(geno.data() + p * NS, geno_rows[p]->data(), NS);

    idash_status a = enc.image.allocate(n_rows);
    if (a != IDASH_OK) return Status::Err(a, "cannot allocate the record image");
    std::memcpy(enc.image.data, &n_rows, 8);
    enc.record_of.clear();
    for (uint64_t r = 0; r < n_rows; ++r) enc.record_of.emplace(index_of_row[r], row_out[r]);

    auto cuda = [&](cudaError_t e, const char *what) {
        return e == cudaSuccess ? Status::Ok()
                                : Status::Err(e == cudaErrorMemoryAllocation ? IDASH_ERR_OUT_OF_MEMORY : IDASH_ERR_CUDA,
                                              std::string(what) + ": " + cudaGetErrorString(e));
    };
    cudaStream_t s = static_cast<cudaStream_t>(idash_stream(ctx));
    uint32_t *d_src = nullptr, *d_index = nullptr, *d_out_row = nullptr;
    int8_t *d_geno = nullptr;
    uint8_t *d_img = nullptr;
    Status st = cuda(cudaMalloc(&d_src, slot_src.size() * 4), "cudaMalloc");
    if (st.ok()) st = cuda(cudaMalloc(&d_index, n_rows * 4), "cudaMalloc");
    if (st.ok()) st = cuda(cudaMalloc(&d_out_row, n_rows * 4), "cudaMalloc");
    if (st.ok()) st = cuda(cudaMalloc(&d_geno, std::max<size_t>(geno.size(), 1)), "cudaMalloc");
    if (st.ok()) st = cuda(cudaMalloc(&d_img, enc.image.bytes), "cudaMalloc");
    if (st.ok()) st = cuda(cudaMemcpyAsync(d_src, slot_src.data(), slot_src.size() * 4, cudaMemcpyHostToDevice, s), "copy");
    if (st.ok()) st = cuda(cudaMemcpyAsync(d_index, index_of_row.data(), n_rows * 4, cudaMemcpyHostToDevice, s), "copy");
    if (st.ok()) st = cuda(cudaMemcpyAsync(d_out_row, row_out.data(), n_rows * 4, cudaMemcpyHostToDevice, s), "copy");
    if (st.ok() && !geno.empty())
        st = cuda(cudaMemcpyAsync(d_geno, geno.data(), geno.size(), cudaMemcpyHostToDevice, s), "copy");
    if (st.ok()) {
        idash_encrypt_params p{};
        p.N = IdashParams::N;
        p.k = IdashParams::k;
        p.num_samples = NS;
        p.num_regions = R;
        p.region_size = params.REGION_SIZE;
        p.one_t32 = dtot32(kInScaling);
        p.nan_t32[0] = dtot32(3. / 6. * kInScaling);
        p.nan_t32[1] = dtot32(2. / 6. * kInScaling);
        p.nan_t32[2] = dtot32(1. / 6. * kInScaling);
        p.record_tag = kTlweSampleTag;
        p.alpha = kAlpha;
        const idash_row_layout lay = RecordImage::layout();
        idash_status code = idash_encrypt_trlwe_device(ctx, &p, key.key.data(), seed, n_rows, d_src, d_geno,
                                                       std::max<uint32_t>(NS, 1), d_index, d_out_row, d_img + 8, &lay,
                                                       nullptr, nullptr);
        if (code != IDASH_OK) st = Status::Err(code, idash_last_error(ctx));
    }
    if (st.ok())
        st = cuda(cudaMemcpyAsync(enc.image.data + 8, d_img + 8, enc.image.bytes - 8, cudaMemcpyDeviceToHost, s),
                  "copy out");
    if (st.ok()) {
        idash_status code = idash_sync(ctx);
        if (code != IDASH_OK) st = Status::Err(code, idash_last_error(ctx));
    }
    cudaFree(d_src);
    cudaFree(d_index);
    cudaFree(d_out_row);
    cudaFree(d_geno);
    cudaFree(d_img);
    return st;
}

Status write_encrypted_data(const EncryptedData &enc, const std::string &filename) {
    return write_image_file(enc.image.data, enc.image.bytes, filename);
}

}  // namespace idash_host

using namespace idash_host;

extern "C" idash_status idash_encrypt_files(int device, const char *keys_file, const char *challenge_file,
                                            const char *data_file, uint64_t seed, idash_encrypt_report *report,
                                            char *errbuf, size_t errbuf_len) {
    auto fail = [&](const Status &st) {
        if (errbuf && errbuf_len) std::snprintf(errbuf, errbuf_len, "%s", st.message.c_str());
        return st.code;
    };
    if (!keys_file || !challenge_file || !data_file)
        return fail(Status::Err(IDASH_ERR_INVALID_ARGUMENT, "null file name"));
    const double t0 = now_s();
    IdashKey key;
    PlaintextData plain;
    Status st = read_key(key, keys_file);
    if (st.ok()) st = read_plaintext_data(plain, key.params, challenge_file);
    if (st.ok()) st = check_plaintext(plain, key.params);
    if (!st.ok()) return fail(st);  // inputs are validated before the device is touched
    const double t1 = now_s();
    if (seed == 0) {
        std::random_device rd;
        seed = (uint64_t(rd()) << 32) ^ rd();
        if (seed == 0) seed = 1;
    }
    idash_ctx *ctx = nullptr;
    idash_status s = idash_open(&ctx, device);
    if (s != IDASH_OK) return fail(Status::Err(s, idash_last_error(nullptr)));
    EncryptedData enc;
    st = encrypt_data(enc, plain, key, ctx, seed);
    idash_close(ctx);
    const double t2 = now_s();
    if (st.ok()) st = write_encrypted_data(enc, data_file);
    const double t3 = now_s();
    if (!st.ok()) return fail(st);
    if (report) {
        report->read_s = t1 - t0;
        report->encrypt_s = t2 - t1;
        report->write_s = t3 - t2;
        report->n_positions = plain.data.size();
        report->n_records = enc.image.count;
    }
    if (errbuf && errbuf_len) errbuf[0] = '\0';
    return IDASH_OK;
}
