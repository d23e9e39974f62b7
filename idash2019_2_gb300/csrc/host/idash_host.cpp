// Host side of the cloud step (see idash_host.hpp).
#include "idash_host.hpp"

#include <cuda_runtime.h>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <thread>
#include <vector>

namespace idash_host {

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

bool read_exact(std::istream &in, void *dst, size_t n) {
    in.read(static_cast<char *>(dst), std::streamsize(n));
    return size_t(in.gcount()) == n;
}

// "<pos>_<snp>" -> (pos, snp), as split() at eval/idash.cpp:50-57.
bool split_feature(const std::string &s, uint64_t *pos, uint32_t *snp) {
    const size_t k = s.find('_');
    if (k == std::string::npos || k == 0 || k + 1 >= s.size()) return false;
    char *end = nullptr;
    const unsigned long long p = std::strtoull(s.c_str(), &end, 10);
    if (end != s.c_str() + k) return false;
    const unsigned long v = std::strtoul(s.c_str() + k + 1, &end, 10);
    if (*end != '\0') return false;
    *pos = p;
    *snp = uint32_t(v);
    return true;
}

// One .hr file into a name -> coefficient map, line by line as
// eval/parse_vw.cpp:8-30 fills its map (later lines overwrite earlier ones).
Status read_hr(const std::string &file, std::unordered_map<std::string, int32_t> *coefs) {
    FILE *f = std::fopen(file.c_str(), "r");
    if (!f) return Status::Err(IDASH_ERR_IO, "cannot open model file '" + file + "'");
    char buf[256];
    while (std::fgets(buf, sizeof(buf), f)) {
        char name[256];
        int value = 0;
        if (std::sscanf(buf, "%255s %d", name, &value) != 2) continue;
        (*coefs)[name] = int32_t(value);
    }
    std::fclose(f);
    return Status::Ok();
}

}  // namespace

RecordImage::~RecordImage() {
    if (!data) return;
    if (pinned) cudaFreeHost(data);
    else std::free(data);
}

idash_status RecordImage::allocate(uint64_t n) {
    const uint64_t need = 8 + n * kRecordBytes;
    if (data && bytes >= need) {
        count = n;
        bytes = need;
        return IDASH_OK;
    }
    if (data) {
        if (pinned) cudaFreeHost(data);
        else std::free(data);
        data = nullptr;
    }
    void *p = nullptr;
    if (cudaMallocHost(&p, need) == cudaSuccess) {
        pinned = true;
    } else {
        cudaGetLastError();
        pinned = false;
        p = std::aligned_alloc(64, (need + 63) / 64 * 64);
        if (!p) return IDASH_ERR_OUT_OF_MEMORY;
    }
    data = static_cast<uint8_t *>(p);
    bytes = need;
    count = n;
    std::memcpy(data, &count, 8);
    return IDASH_OK;
}

Status read_params(IdashParams &params, const std::string &filename) {
    std::ifstream in(filename, std::ios::binary);
    if (!in) return Status::Err(IDASH_ERR_IO, "cannot open parameters file '" + filename + "'");
    return read_params_stream(params, in);
}

Status read_params_stream(IdashParams &params, std::istream &in) {
    uint32_t hdr[7];
    if (!read_exact(in, hdr, sizeof(hdr))) return Status::Err(IDASH_ERR_FORMAT, "params.bin: truncated header");
    params = IdashParams();
    params.NUM_SAMPLES = hdr[0];
    params.NUM_INPUT_POSITIONS = hdr[1];
    params.NUM_OUTPUT_POSITIONS = hdr[2];
    params.NUM_INPUT_FEATURES = hdr[3];
    params.NUM_OUTPUT_FEATURES = hdr[4];
    params.NUM_REGIONS = hdr[5];
    params.REGION_SIZE = hdr[6];
    for (uint32_t i = 0; i < params.NUM_INPUT_POSITIONS; ++i) {
        uint64_t pos;
        std::array<FeatBigIndex, 3> b;
        if (!read_exact(in, &pos, 8) || !read_exact(in, b.data(), sizeof(b)))
            return Status::Err(IDASH_ERR_FORMAT, "params.bin: truncated input table");
        params.in_features_index.emplace(pos, std::array<FeatBigIndex, 3>());
        params.in_features_index.at(pos) = b;
    }
    if (params.in_features_index.size() != params.NUM_INPUT_POSITIONS)
        return Status::Err(IDASH_ERR_FORMAT, "params.bin: NUM_INPUT_POSITIONS != in_features_index.size()");
    for (uint32_t i = 0; i < params.NUM_OUTPUT_POSITIONS; ++i) {
        uint64_t pos;
        if (!read_exact(in, &pos, 8)) return Status::Err(IDASH_ERR_FORMAT, "params.bin: truncated output table");
        std::string name;
        for (int c = in.get(); c > 0; c = in.get()) name.push_back(char(c));
        std::array<FeatBigIndex, 3> b;
        if (!read_exact(in, b.data(), sizeof(b)))
            return Status::Err(IDASH_ERR_FORMAT, "params.bin: truncated output table");
        params.out_position_names.push_back({pos, name});
        params.out_features_index.emplace(pos, std::array<FeatBigIndex, 3>());
        params.out_features_index.at(pos) = b;
    }
    if (params.out_features_index.size() != params.NUM_OUTPUT_POSITIONS ||
        params.out_position_names.size() != params.NUM_OUTPUT_POSITIONS)
        return Status::Err(IDASH_ERR_FORMAT, "params.bin: NUM_OUTPUT_POSITIONS != out_features_index.size()");
    if (params.NUM_REGIONS == 0 || params.REGION_SIZE == 0 ||
        uint64_t(params.NUM_REGIONS) * params.REGION_SIZE > IdashParams::N || params.NUM_SAMPLES > params.REGION_SIZE)
        return Status::Err(IDASH_ERR_FORMAT, "params.bin: inconsistent NUM_REGIONS / REGION_SIZE / NUM_SAMPLES");
    return Status::Ok();
}

Status write_params(const IdashParams &params, const std::string &filename) {
    std::ofstream out(filename, std::ios::binary);
    if (!out) return Status::Err(IDASH_ERR_IO, "cannot open parameters file '" + filename + "' for write");
    const uint32_t hdr[7] = {params.NUM_SAMPLES,         params.NUM_INPUT_POSITIONS, params.NUM_OUTPUT_POSITIONS,
                             params.NUM_INPUT_FEATURES,  params.NUM_OUTPUT_FEATURES, params.NUM_REGIONS,
                             params.REGION_SIZE};
    out.write(reinterpret_cast<const char *>(hdr), sizeof(hdr));
    if (params.in_features_index.size() != params.NUM_INPUT_POSITIONS ||
        params.out_features_index.size() != params.NUM_OUTPUT_POSITIONS ||
        params.out_position_names.size() != params.NUM_OUTPUT_POSITIONS)
        return Status::Err(IDASH_ERR_FORMAT, "params: position counts disagree with the index tables");
    for (const auto &e : params.in_features_index) {
        out.write(reinterpret_cast<const char *>(&e.first), 8);
        out.write(reinterpret_cast<const char *>(e.second.data()), sizeof(e.second));
    }
    for (const auto &e : params.out_position_names) {
        out.write(reinterpret_cast<const char *>(&e.first), 8);
        out.write(e.second.c_str(), std::streamsize(e.second.size() + 1));
        const auto &b = params.out_features_index.at(e.first);
        out.write(reinterpret_cast<const char *>(b.data()), sizeof(b));
    }
    if (!out) return Status::Err(IDASH_ERR_IO, "write failed: '" + filename + "'");
    return Status::Ok();
}

Status read_model(Model &model, const IdashParams &params, const std::string &path) {
    // The files are read and parsed on host threads, each into its terms in
    // the iteration order of its name -> coefficient map (what the reference
    // iterates); the model's maps are then filled on this thread in the
    // reference's order, so every unordered_map sees the same insertions.
    struct File {
        FeatBigIndex out;
        std::string name;
        std::vector<std::pair<FeatBigIndex, int32_t>> terms;
        Status st = Status::Ok();
    };
    std::vector<File> files;
    files.reserve(params.out_features_index.size() * 3);
    for (const auto &elem : params.out_features_index)
        for (uint32_t snp = 0; snp < 3; ++snp)
            files.push_back(File{elem.second[snp],
                                 path + "/" + std::to_string(elem.first) + "_" + std::to_string(snp) + ".hr", {}});
    auto parse = [&](File &f) {
        std::unordered_map<std::string, int32_t> coefs;
        f.st = read_hr(f.name, &coefs);
        if (!f.st.ok()) return;
        f.terms.reserve(coefs.size());
        for (const auto &c : coefs) {
            if (c.first == "Constant") {
                f.terms.emplace_back(IdashParams::constant_bigIndex(), c.second);
                continue;
            }
            uint64_t in_pos;
            uint32_t in_snp;
            if (!split_feature(c.first, &in_pos, &in_snp)) {
                f.st = Status::Err(IDASH_ERR_FORMAT, "model: bad feature name '" + c.first + "'");
                return;
            }
            const auto it = params.in_features_index.find(in_pos);
            if (it == params.in_features_index.end() || in_snp >= 3) {
                f.st = Status::Err(IDASH_ERR_INDEX, "model: feature '" + c.first + "' is not a tag SNP of params");
                return;
            }
            f.terms.emplace_back(it->second[in_snp], c.second);
        }
    };
    const size_t n_threads =
        std::max<size_t>(1, std::min<size_t>({16, std::thread::hardware_concurrency(), files.size() / 256 + 1}));
    std::vector<std::thread> threads;
    for (size_t t = 1; t < n_threads; ++t)
        threads.emplace_back([&, t] {
            for (size_t i = files.size() * t / n_threads; i < files.size() * (t + 1) / n_threads; ++i) parse(files[i]);
        });
    for (size_t i = 0; i < files.size() / n_threads; ++i) parse(files[i]);
    for (auto &th : threads) th.join();
    for (File &f : files) {
        if (!f.st.ok()) return f.st;  // the first failure in the reference's reading order
        auto &mc = model.model[f.out] = std::unordered_map<FeatBigIndex, int32_t>();
        for (const auto &t : f.terms) mc[t.first] = t.second;
        std::vector<std::pair<FeatBigIndex, int32_t>>().swap(f.terms);
    }
    return Status::Ok();
}

// Reads (or writes) bytes [off, off + bytes) of fd into (from) buf: a
// record image is one contiguous range, so up to 8 threads each move a
// slice of it with pread/pwrite (one thread below 64 MiB a slice).
static bool parallel_io(int fd, uint8_t *buf, size_t bytes, uint64_t off, bool write) {
    constexpr size_t kSlice = size_t(64) << 20;
    const size_t n_threads = std::max<size_t>(1, std::min<size_t>(8, bytes / kSlice));
    std::atomic<bool> ok{true};
    auto run = [&](size_t t) {
        const size_t lo = bytes * t / n_threads, hi = bytes * (t + 1) / n_threads;
        for (size_t done = lo; done < hi && ok.load();) {
            const ssize_t r = write ? ::pwrite(fd, buf + done, hi - done, off_t(off + done))
                                    : ::pread(fd, buf + done, hi - done, off_t(off + done));
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) {
                ok = false;
                break;
            }
            done += size_t(r);
        }
    };
    std::vector<std::thread> threads;
    for (size_t t = 1; t < n_threads; ++t) threads.emplace_back(run, t);
    run(0);
    for (auto &th : threads) th.join();
    return ok.load();
}

static Status read_image(RecordImage &img, const std::string &filename) {
    const int fd = ::open(filename.c_str(), O_RDONLY);
    if (fd < 0) return Status::Err(IDASH_ERR_IO, "cannot open '" + filename + "'");
    struct stat sb {};
    uint64_t count = 0;
    if (::fstat(fd, &sb) != 0 || sb.st_size < 8 || ::pread(fd, &count, 8, 0) != 8) {
        ::close(fd);
        return Status::Err(IDASH_ERR_FORMAT, "'" + filename + "': missing record count");
    }
    const uint64_t size = uint64_t(sb.st_size);
    if (count > (size - 8) / kRecordBytes || size != 8 + count * kRecordBytes) {
        ::close(fd);
        return Status::Err(IDASH_ERR_FORMAT, "'" + filename + "': size is not 8 + count * 8208");
    }
    idash_status s = img.allocate(count);
    if (s != IDASH_OK) {
        ::close(fd);
        return Status::Err(s, "cannot allocate the record image");
    }
    const bool ok = parallel_io(fd, img.data, size_t(size), 0, false);
    ::close(fd);
    if (!ok) return Status::Err(IDASH_ERR_IO, "'" + filename + "': short read");
    return Status::Ok();
}

Status read_encrypted_data(EncryptedData &data, const IdashParams &params, const std::string &filename) {
    (void)params;
    Status st = read_image(data.image, filename);
    if (!st.ok()) return st;
    data.record_of.clear();
    data.record_of.reserve(data.image.count);
    for (uint64_t i = 0; i < data.image.count; ++i) {
        FeatIndex idx;
        std::memcpy(&idx, data.image.record(i), 4);
        data.record_of.emplace(idx, i);  // first record of an index wins, as eval/idash.cpp:531
    }
    return Status::Ok();
}

Status read_encrypted_predictions(EncryptedPredictions &preds, const std::string &filename) {
    Status st = read_image(preds.image, filename);
    if (!st.ok()) return st;
    preds.record_of.clear();
    for (uint64_t i = 0; i < preds.image.count; ++i) {
        FeatBigIndex idx;
        std::memcpy(&idx, preds.image.record(i), 4);
        preds.record_of.emplace(idx, i);
    }
    return Status::Ok();
}

Status write_image_file(const uint8_t *data, uint64_t bytes, const std::string &filename) {
    const int fd = ::open(filename.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return Status::Err(IDASH_ERR_IO, "cannot open '" + filename + "' for write");
    bool ok = data && parallel_io(fd, const_cast<uint8_t *>(data), size_t(bytes), 0, true);
    ok = ::close(fd) == 0 && ok;
    if (!ok) return Status::Err(IDASH_ERR_IO, "short write to '" + filename + "'");
    return Status::Ok();
}

Status write_encrypted_predictions(const EncryptedPredictions &preds, const std::string &filename) {
    return write_image_file(preds.image.data, preds.image.bytes, filename);
}

FlatModel flatten_model(const Model &model) {
    FlatModel f;
    // Record order of the output file: the reference creates one sample per
    // model entry in model-iteration order (eval/idash.cpp:772-777) in an
    // unordered_map and writes that map in its iteration order (:607).
    std::unordered_map<FeatBigIndex, uint64_t> score;
    for (const auto &it : model.model) score.emplace(it.first, 0);
    uint64_t rec = 0;
    for (auto &it : score) it.second = rec++;
    const uint64_t n_out = score.size();
    // Outputs numbered by FeatBigIndex (neighbouring targets adjacent); each
    // output's terms in the model map's iteration order (the variance sum
    // order of eval/idash.cpp:800-819).
    f.out_bidx.reserve(n_out);
    for (const auto &it : model.model) f.out_bidx.push_back(it.first);
    std::sort(f.out_bidx.begin(), f.out_bidx.end());
    f.term_ptr.assign(n_out + 1, 0);
    f.out_row.resize(n_out);
    for (uint64_t o = 0; o < n_out; ++o) {
        for (const auto &t : model.model.at(f.out_bidx[o])) {
            f.term_feat.push_back(t.first);
            f.term_coef.push_back(t.second);
        }
        f.term_ptr[o + 1] = f.term_feat.size();
        f.out_row[o] = uint32_t(score.at(f.out_bidx[o]));
    }
    return f;
}

namespace {
constexpr char kCacheMagic[8] = {'I', 'D', 'A', 'S', 'H', 'F', 'M', '1'};

uint64_t fnv1a(uint64_t h, const void *data, size_t n) {
    const uint8_t *p = static_cast<const uint8_t *>(data);
    for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 0x100000001B3ull;
    return h;
}
}  // namespace

uint64_t fingerprint(const std::string &params_file, const std::string &model_dir) {
    uint64_t h = 0xCBF29CE484222325ull;
    FILE *f = std::fopen(params_file.c_str(), "rb");
    if (f) {
        char buf[1 << 16];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) h = fnv1a(h, buf, n);
        std::fclose(f);
    }
    return fnv1a(h, model_dir.data(), model_dir.size());
}

Status write_model_cache(const FlatModel &flat, uint64_t fp, const std::string &path) {
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return Status::Err(IDASH_ERR_IO, "cannot write model cache '" + tmp + "'");
    const uint64_t hdr[3] = {fp, flat.out_bidx.size(), flat.term_feat.size()};
    bool ok = std::fwrite(kCacheMagic, 1, 8, f) == 8 && std::fwrite(hdr, 8, 3, f) == 3;
    auto put = [&](const void *d, size_t bytes) { ok = ok && (bytes == 0 || std::fwrite(d, 1, bytes, f) == bytes); };
    put(flat.out_bidx.data(), flat.out_bidx.size() * 4);
    put(flat.out_row.data(), flat.out_row.size() * 4);
    put(flat.term_ptr.data(), flat.term_ptr.size() * 8);
    put(flat.term_feat.data(), flat.term_feat.size() * 4);
    put(flat.term_coef.data(), flat.term_coef.size() * 4);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        return Status::Err(IDASH_ERR_IO, "cannot write model cache '" + path + "'");
    }
    return Status::Ok();
}

Status read_model_cache(FlatModel *flat, uint64_t fp, const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return Status::Err(IDASH_ERR_IO, "no model cache at '" + path + "'");
    char magic[8];
    uint64_t hdr[3];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCacheMagic, 8) == 0 &&
              std::fread(hdr, 8, 3, f) == 3;
    if (ok && hdr[0] != fp) {
        std::fclose(f);
        return Status::Err(IDASH_ERR_FORMAT, "model cache is for other params/model");
    }
    if (ok && (hdr[1] > (1ull << 32) || hdr[2] > (1ull << 40))) ok = false;
    if (ok) {
        flat->out_bidx.resize(hdr[1]);
        flat->out_row.resize(hdr[1]);
        flat->term_ptr.resize(hdr[1] + 1);
        flat->term_feat.resize(hdr[2]);
        flat->term_coef.resize(hdr[2]);
    }
    auto get = [&](void *d, size_t bytes) { ok = ok && (bytes == 0 || std::fread(d, 1, bytes, f) == bytes); };
    get(flat->out_bidx.data(), hdr[1] * 4);
    get(flat->out_row.data(), hdr[1] * 4);
    get(flat->term_ptr.data(), (hdr[1] + 1) * 8);
    get(flat->term_feat.data(), hdr[2] * 4);
    get(flat->term_coef.data(), hdr[2] * 4);
    std::fclose(f);
    if (!ok || flat->term_ptr.back() != hdr[2]) return Status::Err(IDASH_ERR_FORMAT, "model cache is damaged");
    return Status::Ok();
}

namespace {
constexpr char kPlanMagic[8] = {'I', 'D', 'G', 'P', 'L', 'A', 'N', '1'};
// idash_model_info::kernel (0 window, 1 direct, 2 pipe, 3 warp-specialised,
// 4 tensor cores) as the "kernel" option's value (2, 1, 3, 4, 5)
constexpr int64_t kKernelOption[5] = {2, 1, 3, 4, 5};
constexpr uint64_t kMaxKernel = 4;
}  // namespace

bool apply_cached_plan(idash_ctx *ctx, const std::string &cache_path, const std::string &params_file,
                       const std::string &model_dir) {
    if (cache_path.empty()) return false;
    FILE *f = std::fopen((cache_path + ".plan").c_str(), "rb");
    if (!f) return false;
    char magic[8];
    uint64_t rec[3];
    const bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kPlanMagic, 8) == 0 &&
                    std::fread(rec, 8, 3, f) == 3;
    std::fclose(f);
    if (!ok || rec[0] != fingerprint(params_file, model_dir) || rec[1] > kMaxKernel) return false;
    return idash_set_option(ctx, "kernel", kKernelOption[rec[1]]) == IDASH_OK &&
           idash_set_option(ctx, "slice_words", int64_t(rec[2])) == IDASH_OK;
}

void save_plan(const std::string &cache_path, const std::string &params_file, const std::string &model_dir,
               const idash_model_info &plan) {
    if (cache_path.empty() || plan.kernel > kMaxKernel || plan.slice_words == 0) return;
    const std::string path = cache_path + ".plan", tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    const uint64_t rec[3] = {fingerprint(params_file, model_dir), plan.kernel, plan.slice_words};
    bool ok = std::fwrite(kPlanMagic, 1, 8, f) == 8 && std::fwrite(rec, 8, 3, f) == 3;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

Status load_model(Model *parsed, FlatModel *flat, const IdashParams &params, const std::string &params_file,
                  const std::string &model_dir, const std::string &cache_path, bool *from_cache) {
    *from_cache = false;
    uint64_t fp = 0;
    if (!cache_path.empty()) {
        fp = fingerprint(params_file, model_dir);
        if (read_model_cache(flat, fp, cache_path).ok()) {
            *from_cache = true;
            return Status::Ok();
        }
    }
    Status st = read_model(*parsed, params, model_dir);
    if (!st.ok()) return st;
    *flat = flatten_model(*parsed);
    if (!cache_path.empty()) write_model_cache(*flat, fp, cache_path);  // best effort
    return Status::Ok();
}

Status cloud_compute_score(EncryptedPredictions &preds, const EncryptedData &data, const Model &model,
                           const IdashParams &params, idash_ctx *ctx, CloudTiming *timing) {
    const double t0 = now_s();
    const FlatModel flat = flatten_model(model);
    const double t_flat = now_s() - t0;
    Status st = cloud_compute_score(preds, data, flat, params, ctx, timing);
    if (st.ok() && timing) timing->plan_s += t_flat;
    return st;
}

Status cloud_compute_score(EncryptedPredictions &preds, const EncryptedData &data, const FlatModel &flat,
                           const IdashParams &params, idash_ctx *ctx, CloudTiming *timing) {
    if (!preds.record_of.empty()) return Status::Err(IDASH_ERR_STATE, "predictions must be empty on entry");
    const double t0 = now_s();
    const uint64_t n_out = flat.out_bidx.size();
    uint64_t n_index = 0;
    for (const auto &it : data.record_of) n_index = std::max<uint64_t>(n_index, uint64_t(it.first) + 1);
    std::vector<uint32_t> row_of_index(n_index, 0xFFFFFFFFu);
    for (const auto &it : data.record_of) row_of_index[it.first] = uint32_t(it.second);

    idash_trlwe_params tp{IdashParams::N, IdashParams::k, params.NUM_SAMPLES, params.NUM_REGIONS,
                          params.REGION_SIZE, IdashParams::ONE_IN_T32, kTlweSampleTag};
    idash_model *m = nullptr;
    idash_status s = idash_model_trlwe(ctx, &m, &tp, n_out, flat.out_bidx.data(), flat.out_row.data(),
                                       flat.term_ptr.data(), flat.term_feat.data(), flat.term_coef.data(), n_index,
                                       row_of_index.data(), data.image.count);
    if (s != IDASH_OK) return Status::Err(s, idash_last_error(ctx));
    const double t1 = now_s();

    s = preds.image.allocate(n_out);
    void *d_in = nullptr, *d_out = nullptr;
    if (s == IDASH_OK) s = idash_device_alloc(ctx, data.image.bytes, &d_in);
    if (s == IDASH_OK) s = idash_device_alloc(ctx, preds.image.bytes, &d_out);
    if (s == IDASH_OK) s = idash_copy_h2d(ctx, d_in, data.image.data, data.image.bytes);
    idash_row_layout in_l = RecordImage::layout();
    in_l.header_offset = -1;
    const idash_row_layout out_l = RecordImage::layout();
    if (s == IDASH_OK)
        s = idash_score_trlwe_device(m, static_cast<uint8_t *>(d_in) + 8, &in_l, static_cast<uint8_t *>(d_out) + 8,
                                     &out_l, nullptr);
    if (s == IDASH_OK) s = idash_sync(ctx);
    if (s == IDASH_OK) s = idash_copy_d2h(ctx, preds.image.data + 8, static_cast<uint8_t *>(d_out) + 8,
                                          preds.image.bytes - 8);
    Status st = s == IDASH_OK ? Status::Ok() : Status::Err(s, idash_last_error(ctx));
    if (d_in) idash_device_free(ctx, d_in);
    if (d_out) idash_device_free(ctx, d_out);
    if (st.ok() && timing) idash_model_get_info(m, &timing->plan);
    idash_model_free(m);
    if (!st.ok()) return st;
    std::memcpy(preds.image.data, &preds.image.count, 8);
    preds.record_of.clear();
    for (uint64_t o = 0; o < n_out; ++o) preds.record_of.emplace(flat.out_bidx[o], flat.out_row[o]);
    if (timing) {
        timing->plan_s = t1 - t0;
        timing->score_s = now_s() - t1;
    }
    return Status::Ok();
}

}  // namespace idash_host

using namespace idash_host;

extern "C" idash_status idash_cloud_files(int device, const char *params_file, const char *model_dir,
                                          const char *data_file, const char *pred_file, idash_cloud_report *report,
                                          char *errbuf, size_t errbuf_len) {
    auto fail = [&](const Status &st) {
        if (errbuf && errbuf_len) std::snprintf(errbuf, errbuf_len, "%s", st.message.c_str());
        return st.code;
    };
    if (!params_file || !model_dir || !data_file || !pred_file)
        return fail(Status::Err(IDASH_ERR_INVALID_ARGUMENT, "null file name"));
    const double t0 = now_s();
    IdashParams params;
    Model model;
    FlatModel flat;
    EncryptedData data;
    EncryptedPredictions preds;
    CloudTiming tm;
    const char *cache_env = std::getenv("IDASH_MODEL_CACHE");
    bool cached = false;
    Status st = read_params(params, params_file);
    if (st.ok()) st = load_model(&model, &flat, params, params_file, model_dir, cache_env ? cache_env : "", &cached);
    if (st.ok()) st = read_encrypted_data(data, params, data_file);
    if (!st.ok()) return fail(st);  // every input is validated before the device is touched
    const double t1 = now_s();
    idash_ctx *ctx = nullptr;
    idash_status s = idash_open(&ctx, device);
    if (s != IDASH_OK) return fail(Status::Err(s, idash_last_error(nullptr)));
    const std::string cache_path = cache_env ? cache_env : "";
    const bool plan_cached = apply_cached_plan(ctx, cache_path, params_file, model_dir);
    if (st.ok()) st = cloud_compute_score(preds, data, flat, params, ctx, &tm);
    if (st.ok() && !plan_cached) save_plan(cache_path, params_file, model_dir, tm.plan);
    const double t2 = now_s();
    if (st.ok()) st = write_encrypted_predictions(preds, pred_file);
    const double t3 = now_s();
    idash_close(ctx);
    if (!st.ok()) return fail(st);
    if (report) {
        report->read_s = t1 - t0;
        report->plan_s = tm.plan_s;
        report->score_s = tm.score_s;
        report->write_s = t3 - t2;
        report->n_in_records = data.image.count;
        report->n_out_records = preds.image.count;
        report->model_from_cache = cached ? 1 : 0;
    }
    if (errbuf && errbuf_len) errbuf[0] = '\0';
    return IDASH_OK;
}
