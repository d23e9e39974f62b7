/*
 * tfhe_compat — TEST INFRASTRUCTURE (oracle only).  Implementation of the TFHE
 * subset declared in tfhe.h, written from the mathematics:
 *   Torus32 is Z/2^32 (stored as int32, computed as uint32);
 *   a TorusPolynomial is an element of T[X]/(X^N+1);
 *   a TRLWE sample (a_0..a_{k-1}, b) encrypts mu with phase b - sum_i a_i*s_i.
 */
#include "tfhe.h"

#include <atomic>
#include <cstring>

namespace {

inline uint32_t u(int32_t x) { return (uint32_t)x; }
inline int32_t s(uint32_t x) { return (int32_t)x; }

/* splitmix64: a 64-bit counter-based mixer (Steele, Lea, Flood 2014). */
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

std::atomic<uint64_t> g_stream_counter{0};

struct Rng {
    uint64_t state;
    Rng() {
        const char *env = std::getenv("TFHE_COMPAT_SEED");
        uint64_t seed = env ? std::strtoull(env, nullptr, 0) : 0x1DA52019ull;
        uint64_t stream = g_stream_counter.fetch_add(1);
        state = mix64(seed ^ mix64(stream + 0x5157u));
    }
    uint64_t next() { state += 0x9E3779B97F4A7C15ull; return mix64(state); }
    uint32_t next32() { return (uint32_t)(next() >> 32); }
    double uniform01() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    /* Box-Muller transform: one standard normal deviate. */
    double normal() {
        const double u1 = uniform01(), u2 = uniform01();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

thread_local Rng g_rng;

/* result += sign * (key_poly * torus_poly) mod X^N+1, exact schoolbook product
 * of a {0,1} integer polynomial with a torus polynomial. */
void add_binary_product(uint32_t *acc, const int32_t *key, const int32_t *poly, int32_t N, bool subtract) {
    for (int32_t i = 0; i < N; ++i) {
        if (key[i] == 0) continue;
        const uint32_t ki = u(key[i]);
        for (int32_t j = 0; j < N; ++j) {
            const int32_t t = i + j;
            uint32_t term = ki * u(poly[j]);
            if (t >= N) term = 0u - term;   // X^N = -1
            const int32_t pos = t >= N ? t - N : t;
            acc[pos] = subtract ? acc[pos] - term : acc[pos] + term;
        }
    }
}

}  // namespace

Torus32 dtot32(double d) {
    /* fractional part of d, scaled by 2^32, truncated toward zero, mod 2^32 */
    const double frac = d - std::trunc(d);
    const int64_t v = (int64_t)(frac * 4294967296.0);
    return s((uint32_t)(uint64_t)v);
}

double t32tod(Torus32 x) { return (double)x / 4294967296.0; }

TLweParams *new_TLweParams(int32_t N, int32_t k, double alpha_min, double alpha_max) {
    TLweParams *p = new TLweParams;
    p->N = N;
    p->k = k;
    p->alpha_min = alpha_min;
    p->alpha_max = alpha_max;
    return p;
}

void delete_TLweParams(TLweParams *p) { delete p; }

TorusPolynomial *new_TorusPolynomial(int32_t N) {
    TorusPolynomial *p = new TorusPolynomial;
    p->N = N;
    p->coefsT = new Torus32[N]();
    return p;
}

void delete_TorusPolynomial(TorusPolynomial *p) {
    delete[] p->coefsT;
    delete p;
}

static void init_sample(TLweSample *s, const TLweParams *params) {
    s->k = params->k;
    s->a = new TorusPolynomial[params->k + 1];
    for (int32_t i = 0; i <= params->k; ++i) {
        s->a[i].N = params->N;
        s->a[i].coefsT = new Torus32[params->N]();
    }
    s->b = s->a + params->k;
    s->current_variance = 0.0;
}

static void free_sample(TLweSample *s) {
    for (int32_t i = 0; i <= s->k; ++i) delete[] s->a[i].coefsT;
    delete[] s->a;
}

TLweSample *new_TLweSample(const TLweParams *params) {
    TLweSample *s = new TLweSample;
    init_sample(s, params);
    return s;
}

TLweSample *new_TLweSample_array(int32_t nbelts, const TLweParams *params) {
    TLweSample *arr = new TLweSample[nbelts];
    for (int32_t i = 0; i < nbelts; ++i) init_sample(arr + i, params);
    return arr;
}

void delete_TLweSample(TLweSample *s) {
    free_sample(s);
    delete s;
}

void delete_TLweSample_array(int32_t nbelts, TLweSample *s) {
    for (int32_t i = 0; i < nbelts; ++i) free_sample(s + i);
    delete[] s;
}

TLweKey *new_TLweKey(const TLweParams *params) {
    TLweKey *key = new TLweKey;
    key->params = params;
    key->key = new IntPolynomial[params->k];
    for (int32_t i = 0; i < params->k; ++i) {
        key->key[i].N = params->N;
        key->key[i].coefs = new int32_t[params->N]();
    }
    return key;
}

void delete_TLweKey(TLweKey *key) {
    for (int32_t i = 0; i < key->params->k; ++i) delete[] key->key[i].coefs;
    delete[] key->key;
    delete key;
}

void tLweClear(TLweSample *result, const TLweParams *params) {
    for (int32_t i = 0; i <= params->k; ++i)
        std::memset(result->a[i].coefsT, 0, sizeof(Torus32) * params->N);
    result->current_variance = 0.0;
}

void tLweCopy(TLweSample *result, const TLweSample *sample, const TLweParams *params) {
    for (int32_t i = 0; i <= params->k; ++i)
        std::memcpy(result->a[i].coefsT, sample->a[i].coefsT, sizeof(Torus32) * params->N);
    result->current_variance = sample->current_variance;
}

void tLweAddTo(TLweSample *result, const TLweSample *sample, const TLweParams *params) {
    for (int32_t i = 0; i <= params->k; ++i)
        for (int32_t j = 0; j < params->N; ++j)
            result->a[i].coefsT[j] = s(u(result->a[i].coefsT[j]) + u(sample->a[i].coefsT[j]));
    result->current_variance += sample->current_variance;
}

void tLweAddMulTo(TLweSample *result, int32_t p, const TLweSample *sample, const TLweParams *params) {
    const uint32_t up = u(p);
    for (int32_t i = 0; i <= params->k; ++i)
        for (int32_t j = 0; j < params->N; ++j)
            result->a[i].coefsT[j] = s(u(result->a[i].coefsT[j]) + up * u(sample->a[i].coefsT[j]));
    result->current_variance += (double)p * (double)p * sample->current_variance;
}

void torusPolynomialMulByXai(TorusPolynomial *result, int32_t a, const TorusPolynomial *source) {
    /* result = X^a * source in T[X]/(X^N+1), a in [0, 2N) */
    const int32_t N = source->N;
    if (a < 0 || a >= 2 * N) {
        std::cerr << "torusPolynomialMulByXai: exponent out of [0,2N)" << std::endl;
        std::abort();
    }
    for (int32_t j = 0; j < N; ++j) {
        int32_t t = j + a;
        bool neg = false;
        if (t >= 2 * N) t -= 2 * N;
        if (t >= N) { t -= N; neg = true; }
        const uint32_t v = u(source->coefsT[j]);
        result->coefsT[t] = s(neg ? 0u - v : v);
    }
}

void tLweKeyGen(TLweKey *result) {
    const int32_t N = result->params->N;
    for (int32_t i = 0; i < result->params->k; ++i)
        for (int32_t j = 0; j < N; ++j) result->key[i].coefs[j] = (int32_t)(g_rng.next32() & 1u);
}

void tLweSymEncryptZero(TLweSample *result, double alpha, const TLweKey *key) {
    const int32_t N = key->params->N;
    const int32_t k = key->params->k;
    uint32_t *b = (uint32_t *)result->b->coefsT;
    for (int32_t j = 0; j < N; ++j) b[j] = u(dtot32(alpha * g_rng.normal()));
    for (int32_t i = 0; i < k; ++i) {
        for (int32_t j = 0; j < N; ++j) result->a[i].coefsT[j] = s(g_rng.next32());
        add_binary_product(b, key->key[i].coefs, result->a[i].coefsT, N, false);
    }
    result->current_variance = alpha * alpha;
}

void tLwePhase(TorusPolynomial *phase, const TLweSample *sample, const TLweKey *key) {
    const int32_t N = key->params->N;
    std::memcpy(phase->coefsT, sample->b->coefsT, sizeof(Torus32) * N);
    for (int32_t i = 0; i < key->params->k; ++i)
        add_binary_product((uint32_t *)phase->coefsT, key->key[i].coefs, sample->a[i].coefsT, N, true);
}

void export_tlweSample_toStream(std::ostream &F, const TLweSample *sample, const TLweParams *params) {
    F.write((const char *)&TFHE_COMPAT_TLWE_SAMPLE_TAG, sizeof(int32_t));
    for (int32_t i = 0; i <= params->k; ++i)
        F.write((const char *)sample->a[i].coefsT, sizeof(Torus32) * params->N);
    F.write((const char *)&sample->current_variance, sizeof(double));
}

void import_tlweSample_fromStream(std::istream &F, TLweSample *sample, const TLweParams *params) {
    int32_t tag = 0;
    F.read((char *)&tag, sizeof(int32_t));
    if (!F || tag != TFHE_COMPAT_TLWE_SAMPLE_TAG) {
        std::cerr << "import_tlweSample_fromStream: bad record tag" << std::endl;
        std::abort();
    }
    for (int32_t i = 0; i <= params->k; ++i)
        F.read((char *)sample->a[i].coefsT, sizeof(Torus32) * params->N);
    F.read((char *)&sample->current_variance, sizeof(double));
    if (!F) {
        std::cerr << "import_tlweSample_fromStream: truncated record" << std::endl;
        std::abort();
    }
}

void export_tlweKey_toStream(std::ostream &F, const TLweKey *key) {
    const int32_t hdr[3] = {TFHE_COMPAT_TLWE_KEY_TAG, key->params->N, key->params->k};
    F.write((const char *)hdr, sizeof(hdr));
    F.write((const char *)&key->params->alpha_min, sizeof(double));
    F.write((const char *)&key->params->alpha_max, sizeof(double));
    for (int32_t i = 0; i < key->params->k; ++i)
        F.write((const char *)key->key[i].coefs, sizeof(int32_t) * key->params->N);
}

TLweKey *new_tlweKey_fromStream(std::istream &F) {
    int32_t hdr[3] = {0, 0, 0};
    double amin = 0, amax = 0;
    F.read((char *)hdr, sizeof(hdr));
    F.read((char *)&amin, sizeof(double));
    F.read((char *)&amax, sizeof(double));
    if (!F || hdr[0] != TFHE_COMPAT_TLWE_KEY_TAG) {
        std::cerr << "new_tlweKey_fromStream: bad key record" << std::endl;
        std::abort();
    }
    TLweParams *params = new_TLweParams(hdr[1], hdr[2], amin, amax);
    TLweKey *key = new_TLweKey(params);
    for (int32_t i = 0; i < params->k; ++i)
        F.read((char *)key->key[i].coefs, sizeof(int32_t) * params->N);
    return key;
}
