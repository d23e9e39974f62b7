/*
 * tfhe_compat — TEST INFRASTRUCTURE (oracle only; never linked into the product).
 *
 * A small, project-written stand-in for the subset of the TFHE library
 * (https://github.com/tfhe/tfhe, git submodule `tfhe` of the reference,
 * `.gitmodules:1-3`; the pinned commit is not recoverable offline) that the
 * reference's party-B pipeline calls.  It exists so that the reference's own
 * `eval/idash.cpp`, `eval/parse_vw.cpp` and `eval/{keygen,encrypt,cloud,decrypt}.cpp`
 * compile unmodified against it and act as the oracle for the GPU path.
 *
 * Every function is written from the published mathematical definition of the
 * TFHE primitive it stands in for (Torus32 = Z/2^32, negacyclic polynomials
 * mod X^N+1); the names and argument order follow TFHE's public API because the
 * reference calls them by those names:
 *   - hot path (eval/idash.cpp:796,817,825,832,835): tLweClear, tLweAddMulTo,
 *     tLweCopy, torusPolynomialMulByXai, tLweAddTo;
 *   - encryption / decryption (eval/idash.cpp:151,625,714): tLweSymEncryptZero,
 *     tLwePhase, tLweKeyGen (exact integer polynomial products, not FFT);
 *   - conversions (eval/idash.cpp:39-45,718): dtot32, t32tod;
 *   - streams (eval/idash.cpp:483,498,529,552,586,609).
 * Integer arithmetic is carried out on uint32_t so that wrap-around mod 2^32 is
 * defined behaviour.  Randomness comes from a seedable, thread-local counter
 * generator (TFHE_COMPAT_SEED env var), not from TFHE's std::default_random_engine,
 * so encryptions are reproducible but not bit-identical to upstream TFHE's.
 */
#ifndef IDASH_TFHE_COMPAT_TFHE_H
#define IDASH_TFHE_COMPAT_TFHE_H

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <iostream>

typedef int32_t Torus32;

struct IntPolynomial {
    int32_t N;
    int32_t *coefs;
};

struct TorusPolynomial {
    int32_t N;
    Torus32 *coefsT;
};

struct TLweParams {
    int32_t N;
    int32_t k;
    double alpha_min;
    double alpha_max;
};

struct TLweKey {
    const TLweParams *params;
    IntPolynomial *key;  // k binary polynomials
};

/* a[0..k-1] is the mask, b aliases a[k]; current_variance tracks the noise. */
struct TLweSample {
    TorusPolynomial *a;
    TorusPolynomial *b;
    double current_variance;
    int32_t k;
};

/* ---- conversions ---- */
Torus32 dtot32(double d);
double t32tod(Torus32 x);

/* ---- allocation ---- */
TLweParams *new_TLweParams(int32_t N, int32_t k, double alpha_min, double alpha_max);
void delete_TLweParams(TLweParams *p);
TorusPolynomial *new_TorusPolynomial(int32_t N);
void delete_TorusPolynomial(TorusPolynomial *p);
TLweSample *new_TLweSample(const TLweParams *params);
TLweSample *new_TLweSample_array(int32_t nbelts, const TLweParams *params);
void delete_TLweSample(TLweSample *s);
void delete_TLweSample_array(int32_t nbelts, TLweSample *s);
TLweKey *new_TLweKey(const TLweParams *params);
void delete_TLweKey(TLweKey *key);

/* ---- arithmetic on TRLWE samples (all coefficients mod 2^32) ---- */
void tLweClear(TLweSample *result, const TLweParams *params);
void tLweCopy(TLweSample *result, const TLweSample *sample, const TLweParams *params);
void tLweAddTo(TLweSample *result, const TLweSample *sample, const TLweParams *params);
void tLweAddMulTo(TLweSample *result, int32_t p, const TLweSample *sample, const TLweParams *params);
void torusPolynomialMulByXai(TorusPolynomial *result, int32_t a, const TorusPolynomial *source);

/* ---- keys, encryption, phase ---- */
void tLweKeyGen(TLweKey *result);
void tLweSymEncryptZero(TLweSample *result, double alpha, const TLweKey *key);
void tLwePhase(TorusPolynomial *phase, const TLweSample *sample, const TLweKey *key);

/* ---- streams ---- */
void export_tlweSample_toStream(std::ostream &F, const TLweSample *sample, const TLweParams *params);
void import_tlweSample_fromStream(std::istream &F, TLweSample *sample, const TLweParams *params);
void export_tlweKey_toStream(std::ostream &F, const TLweKey *key);
TLweKey *new_tlweKey_fromStream(std::istream &F);

/* Record tag written before each TLweSample payload: the stream layout is
 * int32 tag | (k+1)*N int32 coefficients | double current_variance. */
static const int32_t TFHE_COMPAT_TLWE_SAMPLE_TAG = 42;
static const int32_t TFHE_COMPAT_TLWE_KEY_TAG = 52;

#endif
