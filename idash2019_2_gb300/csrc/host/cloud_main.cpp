// idash_cloud: the party-B cloud binary on the GPU.  Same argv, file names and
// BENCHMARK block as the reference's eval/cloud.cpp:3-28, so make rules and
// log scrapers (eval/parse_log.py) keep working:
//   idash_cloud [model_dir]   in a directory holding params.bin and
//                             encrypted_data.bin; writes encrypted_prediction.bin.
// Optional: IDASH_DEVICE (CUDA device ordinal, default 0); IDASH_MODEL_CACHE
// (file holding the flattened model, read when it matches params.bin and the
// model directory, written otherwise).
#include <sys/resource.h>

#include <chrono>
#include <cstdlib>
#include <iostream>

#include "idash_host.hpp"

using namespace idash_host;

static double wall() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char **argv) {
    const double t0 = wall();
    std::string model_dir = "../../ml/model/final";  // eval/idash.h:17
    if (argc >= 2) model_dir = argv[1];
    std::cout << "using model dir: " << model_dir << std::endl;
    const char *dev_env = std::getenv("IDASH_DEVICE");
    const int device = dev_env ? std::atoi(dev_env) : 0;

    idash_ctx *ctx = nullptr;
    idash_status s = idash_open(&ctx, device);
    if (s != IDASH_OK) {
        std::cout << "ERROR: " << idash_status_string(s) << ": " << idash_last_error(nullptr) << std::endl;
        return 1;
    }
    IdashParams params;
    Model model;
    FlatModel flat;
    EncryptedData data;
    EncryptedPredictions preds;
    const char *cache_env = std::getenv("IDASH_MODEL_CACHE");
    bool cached = false;
    Status st = read_params(params, "params.bin");
    if (st.ok()) st = load_model(&model, &flat, params, "params.bin", model_dir, cache_env ? cache_env : "", &cached);
    if (st.ok()) st = read_encrypted_data(data, params, "encrypted_data.bin");
    if (cached) std::cout << "model from cache: " << cache_env << std::endl;
    const double t_start = wall();
    CloudTiming tm;
    const std::string cache_path = cache_env ? cache_env : "";
    const bool plan_cached = st.ok() && apply_cached_plan(ctx, cache_path, "params.bin", model_dir);
    if (st.ok()) st = cloud_compute_score(preds, data, flat, params, ctx, &tm);
    if (st.ok() && !plan_cached) save_plan(cache_path, "params.bin", model_dir, tm.plan);
    const double t_end = wall();
    if (st.ok()) st = write_encrypted_predictions(preds, "encrypted_prediction.bin");
    const double t_write = wall();
    idash_close(ctx);
    if (!st.ok()) {
        std::cout << "ERROR: " << idash_status_string(st.code) << ": " << st.message << std::endl;
        return 1;
    }
    struct rusage ru;
    getrusage(RUSAGE_SELF, &ru);
    std::cout << "----------------- BENCHMARK ----------------- " << std::endl;
    std::cout << "fhe wall time (seconds)..........: " << t_end - t_start << std::endl;
    std::cout << "  of which planning (seconds)....: " << tm.plan_s << std::endl;
    std::cout << "  of which gpu + copies (seconds): " << tm.score_s << std::endl;
    std::cout << "serialization wall time (seconds): " << (t_write - t_end) + (t_start - t0) << std::endl;
    std::cout << "total wall time (seconds)........: " << t_write - t0 << std::endl;
    std::cout << "RAM usage (MB)...................: " << double(ru.ru_maxrss) * 1000 / 1e6 << std::endl;
    return 0;
}
