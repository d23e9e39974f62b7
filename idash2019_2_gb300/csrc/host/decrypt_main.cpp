// idash_decrypt: party A's decryption binary on the GPU.  Same file names,
// argv and BENCHMARK block as the reference's eval/decrypt.cpp:13-48:
//   idash_decrypt           reads keys.bin and encrypted_prediction.bin,
//                           writes result.csv (target SNPs by name);
//   idash_decrypt <any>     writes result_bypos.csv (target SNPs by position).
// Optional: IDASH_DEVICE (CUDA device ordinal, default 0).
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
    (void)argv;
    const double t0 = wall();
    const char *dev_env = std::getenv("IDASH_DEVICE");
    const int device = dev_env ? std::atoi(dev_env) : 0;
    IdashKey key;
    EncryptedPredictions preds;
    Status st = read_key(key, "keys.bin");
    if (st.ok()) st = read_encrypted_predictions(preds, "encrypted_prediction.bin");
    if (!st.ok()) {
        std::cout << "ERROR: " << idash_status_string(st.code) << ": " << st.message << std::endl;
        return 1;
    }
    idash_ctx *ctx = nullptr;
    idash_status s = idash_open(&ctx, device);
    if (s != IDASH_OK) {
        std::cout << "ERROR: " << idash_status_string(s) << ": " << idash_last_error(nullptr) << std::endl;
        return 1;
    }
    const double t_start = wall();
    DecryptedPredictions dec;
    st = decrypt_predictions(dec, preds, key, ctx);
    const double t_end = wall();
    idash_close(ctx);
    if (st.ok()) st = write_decrypted_predictions(dec, key.params, argc == 1 ? "result.csv" : "result_bypos.csv",
                                                  argc == 1);
    const double t_write = wall();
    if (!st.ok()) {
        std::cout << "ERROR: " << idash_status_string(st.code) << ": " << st.message << std::endl;
        return 1;
    }
    struct rusage ru;
    getrusage(RUSAGE_SELF, &ru);
    std::cout << "----------------- BENCHMARK ----------------- " << std::endl;
    std::cout << "decrypt wall time (seconds)......: " << t_end - t_start << std::endl;
    std::cout << "serialization wall time (seconds): " << (t_write - t_end) + (t_start - t0) << std::endl;
    std::cout << "total wall time (seconds)........: " << t_write - t0 << std::endl;
    std::cout << "RAM usage (MB)...................: " << double(ru.ru_maxrss) * 1000 / 1e6 << std::endl;
    return 0;
}
