// idash_encrypt: party A's encryption binary on the GPU.  Same file names,
// argv and BENCHMARK block as the reference's eval/encrypt.cpp:14-38:
//   idash_encrypt [challenge_file]   reads keys.bin and the tag genotypes
//                                    (default ../../data/tag_testing.txt,
//                                    eval/idash.h:16), writes encrypted_data.bin.
// Optional: IDASH_DEVICE (CUDA device ordinal, default 0); IDASH_SEED (the
// mask / noise generator's key; default: drawn from the operating system).
#include <sys/resource.h>

#include <chrono>
#include <cstdlib>
#include <iostream>
#include <random>

#include "idash_host.hpp"

using namespace idash_host;

static double wall() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char **argv) {
    const double t0 = wall();
    std::string challenge = "../../data/tag_testing.txt";
    if (argc >= 2) challenge = argv[1];
    std::cout << "using tag file (challenge): " << challenge << std::endl;
    const char *dev_env = std::getenv("IDASH_DEVICE");
    const int device = dev_env ? std::atoi(dev_env) : 0;
    const char *seed_env = std::getenv("IDASH_SEED");
    uint64_t seed = seed_env ? std::strtoull(seed_env, nullptr, 10) : 0;
    if (seed == 0) {
        std::random_device rd;
        seed = ((uint64_t(rd()) << 32) ^ rd()) | 1u;
    }
    IdashKey key;
    PlaintextData plain;
    Status st = read_key(key, "keys.bin");
    if (st.ok()) st = read_plaintext_data(plain, key.params, challenge);
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
    EncryptedData enc;
    st = encrypt_data(enc, plain, key, ctx, seed);
    const double t_end = wall();
    idash_close(ctx);
    if (st.ok()) st = write_encrypted_data(enc, "encrypted_data.bin");
    const double t_write = wall();
    if (!st.ok()) {
        std::cout << "ERROR: " << idash_status_string(st.code) << ": " << st.message << std::endl;
        return 1;
    }
    struct rusage ru;
    getrusage(RUSAGE_SELF, &ru);
    std::cout << "----------------- BENCHMARK ----------------- " << std::endl;
    std::cout << "encrypt wall time (seconds)......: " << t_end - t_start << std::endl;
    std::cout << "serialization wall time (seconds): " << (t_write - t_end) + (t_start - t0) << std::endl;
    std::cout << "total wall time (seconds)........: " << t_write - t0 << std::endl;
    std::cout << "RAM usage (MB)...................: " << double(ru.ru_maxrss) * 1000 / 1e6 << std::endl;
    return 0;
}
