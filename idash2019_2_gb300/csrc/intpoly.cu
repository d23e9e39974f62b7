// Exact integer-polynomial x TRLWE scoring:
//   out_o = sum_f W_{o,f}(X) * C_f(X)  in Z/2^32[X]/(X^N + 1), on a and b,
// then b[s] += bias_o * one for s < num_samples and b[j] = 0 for
// j >= region_size, as the TRLWE form does (eval/idash.cpp:805-810, 839-841).
// The reference's own terms are the special case W = coef * X^(-r*REGION_SIZE)
// (eval/idash.cpp:817, 830-833); the only dense polynomial products in the
// reference are TFHE's double FFT inside encryption and decryption
// (eval/idash.cpp:625, 714), which cannot be exact here: a term is bounded by
// N * 2^13 * 2^31 = 2^54 and a 60-term sum by ~2^60, beyond 53 bits.
//
// Exactness: every coefficient's true integer value S (ciphertext words taken
// as signed 32-bit) satisfies |S| <= terms * max|W| * N * 2^31 < p1*p2 / 2,
// checked when the model is built.  S is computed modulo two NTT primes
// p1, p2 < 2^31 (p = 1 mod 2N) and recovered by CRT, then reduced mod 2^32.
//
// Kernels: k_ntt_model (model polynomials -> NTT, once per model), k_ntt_rows
// (input TRLWE rows -> NTT, once per call), both stored as centred residues,
// and k_intpoly_score (one CTA per group of outputs: pointwise
// multiply-accumulate over the terms as exact 64-bit sums, inverse NTT, CRT,
// epilogue).  Negacyclic NTTs are the
// Cooley-Tukey / Gentleman-Sande pair with bit-reversed powers of a primitive
// 2N-th root psi (Longa & Naehrig, CANS 2016).
#include <algorithm>
#include <cstring>
#include <vector>

#include "capi_internal.hpp"
#include "common.cuh"

namespace idash {

namespace {

constexpr uint32_t kPrimes[2] = {2147473409u, 2147389441u};  // both = 1 mod 2048
constexpr uint32_t kPsi2048[2] = {383167813u, 211808905u};   // primitive 2048-th roots of unity
constexpr int kNttThreads = 256;
constexpr uint32_t kIpN = 1024;  // polynomial size of the row and scoring kernels: 256 threads x 4 points

// 2^32 mod p is small for both primes (20478 and 188414), so folding the high
// word of a 64-bit sum onto the low one with it shrinks the sum below 2^49.
static_assert((uint64_t(1) << 32) % kPrimes[0] < (1u << 18) && (uint64_t(1) << 32) % kPrimes[1] < (1u << 18),
              "fold bound");

struct NttConsts {
    uint32_t p[2];
    uint32_t pinv[2];       // -p^-1 mod 2^32
    int32_t r1[2];          // R mod p, R = 2^32
    uint32_t nscale[2];     // N^-1 * R^2 mod p: Montgomery factor of the last inverse stage
    uint32_t nscale_tw[2];  // nscale * (that stage's twiddle) mod p
    uint32_t p1inv_m;       // p1^-1 * R mod p2
    uint64_t M, M_half;     // p1 * p2 and floor(M / 2)
};

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t p) { return uint64_t((unsigned __int128)a * b % p); }
uint64_t powmod(uint64_t a, uint64_t e, uint64_t p) {
    uint64_t r = 1;
    for (a %= p; e; e >>= 1, a = mulmod(a, a, p))
        if (e & 1) r = mulmod(r, a, p);
    return r;
}

__device__ __forceinline__ uint32_t mod_add(uint32_t a, uint32_t b, uint32_t p) {
    const uint32_t s = a + b;
    return s >= p ? s - p : s;
}
__device__ __forceinline__ uint32_t mod_sub(uint32_t a, uint32_t b, uint32_t p) { return a >= b ? a - b : a + p - b; }

// Montgomery product a*b*2^-32 mod p for a, b < p < 2^31.
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    const uint64_t t = uint64_t(a) * b;
    const uint32_t m = uint32_t(t) * pinv;
    const uint32_t r = uint32_t((t + uint64_t(m) * p) >> 32);
    return r >= p ? r - p : r;
}

// A signed 32-bit word (or int16) as a residue mod p, for 2^30 < p < 2^31:
// v + 2p is positive and below 4p, so at most two corrections either way.
__device__ __forceinline__ uint32_t residue(int32_t v, uint32_t p) {
    int64_t x = v;
    x += x < 0 ? int64_t(p) : 0;
    x += x < 0 ? int64_t(p) : 0;
    x -= x >= int64_t(p) ? int64_t(p) : 0;
    return uint32_t(x);
}
static_assert(kPrimes[0] > (1u << 30) && kPrimes[1] > (1u << 30), "residue() needs p > 2^30");

// Cooley-Tukey butterfly of the forward transform: (u, v) -> (u + v*S, u - v*S).
__device__ __forceinline__ void ct_butterfly(uint32_t &u, uint32_t &v, uint32_t S, uint32_t p, uint32_t pinv) {
    const uint32_t w = mont_mul(v, S, p, pinv);
    v = mod_sub(u, w, p);
    u = mod_add(u, w, p);
}

// A residue x in [0, p) as the congruent value in (-p/2, p/2]: transforms are
// stored this way so that a product of two has magnitude below 2^60.
__device__ __forceinline__ int32_t centred(uint32_t x, uint32_t p) { return x > p / 2 ? int32_t(x - p) : int32_t(x); }

// In-place negacyclic NTTs (Cooley-Tukey) of `narr` arrays of length N = 2^logn
// in shared memory; array i uses prime prime_of(i) and its twiddles tw[prime][N].
template <typename PrimeOf>
__device__ void ntt_forward(uint32_t *arr, int narr, uint32_t logn, const uint32_t *tw, const NttConsts &k,
                            PrimeOf prime_of) {
    const uint32_t N = 1u << logn, half = N / 2;
    for (uint32_t m = 1, lt = logn - 1; m < N; m <<= 1, --lt) {  // butterfly span t = 2^lt
        const uint32_t t = 1u << lt;
        for (uint32_t x = threadIdx.x; x < half * narr; x += blockDim.x) {
            const uint32_t a = x >> (logn - 1), b = x & (half - 1);
            const uint32_t q = prime_of(a);
            const uint32_t i = b >> lt, j = (i << (lt + 1)) + (b & (t - 1));
            uint32_t *v = arr + a * N;
            const uint32_t S = tw[q * N + m + i];
            const uint32_t U = v[j], V = mont_mul(v[j + t], S, k.p[q], k.pinv[q]);
            v[j] = mod_add(U, V, k.p[q]);
            v[j + t] = mod_sub(U, V, k.p[q]);
        }
        __syncthreads();
    }
}

// Gentleman-Sande butterfly of the inverse transform: (u, v) -> (u + v, (u - v) * S).
__device__ __forceinline__ void gs_butterfly(uint32_t &u, uint32_t &v, uint32_t S, uint32_t p, uint32_t pinv) {
    const uint32_t d = mod_sub(u, v, p);
    u = mod_add(u, v, p);
    v = mont_mul(d, S, p, pinv);
}

// Model polynomials (int16, [term][N]) -> NTT, centred residues, [term][prime][N].
// Coefficients beyond max_abs break the exactness bound: reported, not used.
__global__ void __launch_bounds__(kNttThreads) k_ntt_model(const int16_t *w, uint64_t n_terms, uint32_t N,
                                                           const uint32_t *tw, NttConsts k, int32_t max_abs,
                                                           uint32_t *w_hat, uint32_t *err) {
    extern __shared__ uint32_t sh[];
    uint32_t *tws = sh;           // 2 * N forward twiddles
    uint32_t *arr = sh + 2 * N;   // 2 arrays (one per prime)
    for (uint32_t x = threadIdx.x; x < 2 * N; x += blockDim.x) tws[x] = tw[x];
    __syncthreads();
    for (uint64_t t = blockIdx.x; t < n_terms; t += gridDim.x) {
        const int16_t *src = w + t * N;
        for (uint32_t x = threadIdx.x; x < N; x += blockDim.x) {
            const int32_t v = src[x];
            if (v > max_abs || v < -max_abs) report_error(err, kDevBadIndex);
            arr[x] = residue(v, k.p[0]);
            arr[N + x] = residue(v, k.p[1]);
        }
        __syncthreads();
        ntt_forward(arr, 2, uint32_t(__ffs(N) - 1), tws, k, [](uint32_t a) { return a; });
        uint32_t *dst = w_hat + t * 2 * N;
        for (uint32_t x = threadIdx.x; x < 2 * N; x += blockDim.x) {
            dst[x] = uint32_t(centred(arr[x], k.p[x / N]));
        }
        __syncthreads();
    }
}

// Input TRLWE rows (a | b, signed words) -> NTT, centred residues,
// [row][poly][prime][N], N = kIpN, kNttThreads threads.  The stage of span t
// pairs points j and j + t with twiddle tw[N / (2t) + j / (2t)].  Per row:
// (1) thread r loads points r + 256e of both polynomials and does the stages
// 512 and 256 in registers, for both primes; (2) stages (128, 64), (32, 16),
// (8, 4) as radix-4 passes in shared memory; (3) stages 2 and 1 in registers
// on 4 consecutive points, stored straight to global memory.  Two shared
// buffers alternate between rows.
__global__ void __launch_bounds__(kNttThreads) k_ntt_rows(const uint8_t *in, uint64_t stride, uint64_t n_rows,
                                                          const uint32_t *tw, NttConsts k, uint32_t *c_hat) {
    constexpr uint32_t N = kIpN, Q = N / 4;
    extern __shared__ uint32_t sh[];
    uint32_t *tws = sh;  // 2 * N
    for (uint32_t x = threadIdx.x; x < 2 * N; x += blockDim.x) tws[x] = tw[x];
    __syncthreads();
    const uint32_t tid = threadIdx.x;
    uint32_t buf = 0;
    for (uint64_t row = blockIdx.x; row < n_rows; row += gridDim.x, buf ^= 1u) {
        uint32_t *arr = sh + 2 * N + buf * 4 * N;  // 4 arrays: (a,p1) (a,p2) (b,p1) (b,p2)
        const int32_t *src = reinterpret_cast<const int32_t *>(in + row * stride);
        // (1)
#pragma unroll
        for (uint32_t poly = 0; poly < 2; ++poly) {
            int32_t v[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) v[e] = src[poly * N + tid + e * Q];
#pragma unroll
            for (uint32_t q = 0; q < 2; ++q) {
                const uint32_t p = k.p[q], pinv = k.pinv[q];
                uint32_t x0 = residue(v[0], p), x1 = residue(v[1], p), x2 = residue(v[2], p), x3 = residue(v[3], p);
                const uint32_t *t = tws + q * N;
                ct_butterfly(x0, x2, t[1], p, pinv);
                ct_butterfly(x1, x3, t[1], p, pinv);
                ct_butterfly(x0, x1, t[2], p, pinv);
                ct_butterfly(x2, x3, t[3], p, pinv);
                uint32_t *a = arr + (2 * poly + q) * N + tid;
                a[0] = x0;
                a[Q] = x1;
                a[2 * Q] = x2;
                a[3 * Q] = x3;
            }
        }
        __syncthreads();
        // (2) item w: points base + r + {0, T/2, T, 3T/2}, base = 2T * (w / (T/2))
#pragma unroll 1
        for (uint32_t lt = 7; lt >= 3; lt -= 2) {  // T = 2^lt
            const uint32_t T = 1u << lt, h = T / 2, m = N >> (lt + 1);
            for (uint32_t x = tid; x < 4 * Q; x += blockDim.x) {
                const uint32_t ar = x / Q, w = x % Q;
                const uint32_t kb = w >> (lt - 1), r = w & (h - 1);
                const uint32_t q = ar & 1u;
                const uint32_t p = k.p[q], pinv = k.pinv[q];
                const uint32_t *t = tws + q * N;
                uint32_t *va = arr + ar * N + 2 * T * kb + r;
                uint32_t x0 = va[0], x1 = va[h], x2 = va[T], x3 = va[T + h];
                const uint32_t s = t[m + kb];
                ct_butterfly(x0, x2, s, p, pinv);
                ct_butterfly(x1, x3, s, p, pinv);
                ct_butterfly(x0, x1, t[2 * m + 2 * kb], p, pinv);
                ct_butterfly(x2, x3, t[2 * m + 2 * kb + 1], p, pinv);
                va[0] = x0;
                va[h] = x1;
                va[T] = x2;
                va[T + h] = x3;
            }
            __syncthreads();
        }
        // (3) points 4w..4w+3: stage 2 (twiddle N/4 + w), stage 1 (N/2 + 2w, N/2 + 2w + 1)
        uint4 *dst = reinterpret_cast<uint4 *>(c_hat + row * 4 * N);
        for (uint32_t x = tid; x < 4 * Q; x += blockDim.x) {
            const uint32_t ar = x / Q, w = x % Q;
            const uint32_t q = ar & 1u;
            const uint32_t p = k.p[q], pinv = k.pinv[q];
            const uint32_t *t = tws + q * N;
            const uint4 v = reinterpret_cast<const uint4 *>(arr)[x];
            uint32_t x0 = v.x, x1 = v.y, x2 = v.z, x3 = v.w;
            const uint32_t s = t[N / 4 + w];
            ct_butterfly(x0, x2, s, p, pinv);
            ct_butterfly(x1, x3, s, p, pinv);
            ct_butterfly(x0, x1, t[N / 2 + 2 * w], p, pinv);
            ct_butterfly(x2, x3, t[N / 2 + 2 * w + 1], p, pinv);
            dst[x] = make_uint4(uint32_t(centred(x0, p)), uint32_t(centred(x1, p)), uint32_t(centred(x2, p)),
                                uint32_t(centred(x3, p)));
        }
        // the other buffer is free: its last reader finished before the
        // barriers of this row
    }
}

struct IntpolyArgs {
    const uint64_t *term_ptr;
    const uint32_t *term_row;
    const uint64_t *group_first;  // group g: outputs [group_first[g], group_first[g + 1])
    uint64_t group_begin, group_end;  // groups scored by this launch
    const uint32_t *w_hat;
    const uint32_t *c_hat;
    const int32_t *bias;
    const uint32_t *itw;
    NttConsts k;
    uint32_t N, num_samples, region_size, n_rows;
    int32_t one;
    uint64_t out_begin, out_end;  // outputs written (output o -> row o - out_begin)
    uint8_t *out;  // payload of output row 0
    uint64_t out_stride;
    uint32_t *err;
};

constexpr uint32_t kGroupMax = 3;     // outputs sharing one term-row list (a target's genotypes)
constexpr int kScoreThreads = 256 * kGroupMax;  // k_intpoly_score consumers: 256 threads per group member
constexpr int kScoreBlock = kScoreThreads + 32;  // and one producer warp
constexpr uint32_t kScoreStages = 4;             // row steps in flight per CTA
// Products of centred residues have magnitude below 2^60; a folded sum is
// below 2^49, so kFoldSteps products more stay below 2^63.
constexpr uint32_t kFoldSteps = 7;

// c + a * b with a 64-bit result: one widening multiply-add.
__device__ __forceinline__ int64_t mad_wide(int32_t a, int32_t b, int64_t c) {
    int64_t d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// hi * 2^32 + lo  ->  hi * (2^32 mod p) + lo: same residue, magnitude < 2^49
// for |T| < 2^63.
__device__ __forceinline__ int64_t fold(int64_t T, int32_t r1) {
    int64_t d;
    asm("{\n\t.reg .b32 lo, hi;\n\t.reg .b64 z;\n\t"
        "mov.b64 {lo, hi}, %1;\n\t"
        "mov.b64 z, {lo, 0};\n\t"
        "mad.wide.s32 %0, hi, %2, z;\n\t}"
        : "=l"(d)
        : "l"(T), "r"(r1));
    return d;
}

// Stage layout: the input row's transform (2 polynomials x 2 primes x N
// words), then the weight transforms (2 primes x N words) of up to kGroupMax
// outputs at the same term position.
__host__ __device__ constexpr uint32_t ip_stage_words(uint32_t N) { return (4 + 2 * kGroupMax) * N; }
__host__ __device__ constexpr size_t ip_score_smem(uint32_t N) {
    return 128 + (size_t(kScoreStages) * ip_stage_words(N) + 4 * size_t(kGroupMax) * N + 2 * size_t(N)) * 4;
}

// Consumer-only synchronisation (named barrier 1): the producer warp takes
// no part in the pointwise phase or the inverse NTT.
__device__ __forceinline__ void consumers_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(kScoreThreads) : "memory");
}
__device__ __forceinline__ bool consumers_and(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(v ? 1u : 0u), "n"(kScoreThreads)
        : "memory");
    return r != 0;
}

// One CTA per output group (grid-stride): the outputs of a group read the
// same input rows in the same order (normally the three genotype outputs of a
// target), so each row step brings one input transform (16 KiB) and one
// weight transform (8 KiB) per output.  A producer warp (one lane) keeps
// kScoreStages row steps in flight with cp.async.bulk into a ring: stage s
// completes on full[s], and is refilled once every consumer warp has arrived
// on empty[s], across group boundaries.  Consumer thread x takes group member
// x / 256 and NTT points 4q..4q+3 of its four arrays (q = x % 256); warps run
// through the row steps without a CTA-wide barrier.  A product is one signed
// widening multiply-add into a 64-bit sum; every kFoldSteps terms the sums
// are folded with 2^32 mod p, which keeps them exact without a Montgomery
// reduction per product.  The consumers agree once per group that every copy
// landed, then run the inverse NTTs, CRT and the a1 epilogue.  Every wait is
// bounded; after a failed wait the consumers stop together at the group's
// agreement, and the producer drains its copies in flight before it returns.
__global__ void __launch_bounds__(kScoreBlock, 1) k_intpoly_score(const IntpolyArgs a) {
    extern __shared__ __align__(128) uint8_t ip_smem[];
    constexpr uint32_t N = kIpN;  // a.N, checked on the host
    uint64_t *full = reinterpret_cast<uint64_t *>(ip_smem);             // [kScoreStages]
    uint64_t *empty = full + kScoreStages;                              // [kScoreStages]
    uint32_t *stage0 = reinterpret_cast<uint32_t *>(ip_smem + 128);     // kScoreStages x stage
    uint32_t *arr = stage0 + kScoreStages * ip_stage_words(N);          // [output][poly][prime][N]
    uint32_t *itws = arr + 4 * kGroupMax * N;                           // 2N inverse twiddles
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        for (uint32_t s = 0; s < kScoreStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kScoreThreads / 32);
        }
        fence_mbar_init();
    }
    for (uint32_t x = tid; x < 2 * N; x += blockDim.x) itws[x] = a.itw[x];
    __syncthreads();

    if (tid >= kScoreThreads) {
        // ------------------------------------------------------------ producer
        if (tid != kScoreThreads) return;
        // Fetch cursor: the next (group, row step) of this CTA, with the row
        // of that step loaded one issue ahead.
        uint64_t f_g = a.group_begin + blockIdx.x, f_i = 0, f_n = 0;
        uint64_t f_w[kGroupMax] = {0, 0, 0};  // weight index of the group's first term, per member
        uint32_t f_m = 0;                     // members of the group
        uint32_t pre_r = 0;
        auto open_group = [&]() {
            const uint64_t o0 = a.group_first[f_g];
            f_m = uint32_t(a.group_first[f_g + 1] - o0);
#pragma unroll
            for (uint32_t m = 0; m < kGroupMax; ++m) f_w[m] = m < f_m ? a.term_ptr[o0 + m] : 0;
            f_i = 0;
            f_n = a.term_ptr[o0 + 1] - f_w[0];
        };
        auto advance = [&]() {
            while (f_g < a.group_end && f_i >= f_n) {  // skip finished and empty groups
                f_g += gridDim.x;
                if (f_g < a.group_end) open_group();
            }
            if (f_g < a.group_end) pre_r = a.term_row[f_w[0] + f_i];
        };
        if (f_g >= a.group_end) return;
        open_group();
        advance();
        uint64_t issued = 0;
        bool ok = true;
        while (f_g < a.group_end) {
            const uint32_t s = uint32_t(issued % kScoreStages);
            if (issued >= kScoreStages &&
                !mbar_wait_bounded(&empty[s], uint32_t((issued / kScoreStages - 1) & 1u), a.err)) {
                ok = false;
                break;
            }
            uint32_t r = pre_r;
            if (r >= a.n_rows) {
                report_error(a.err, kDevBadIndex);
                r = 0;  // read a valid row; the output is reported invalid
            }
            uint32_t *st = stage0 + s * ip_stage_words(N);
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&full[s], (4 + 2 * f_m) * N * 4);
            bulk_g2s(st, a.c_hat + uint64_t(r) * 4 * N, 4 * N * 4, &full[s]);
#pragma unroll
            for (uint32_t m = 0; m < kGroupMax; ++m)
                if (m < f_m) bulk_g2s(st + (4 + 2 * m) * N, a.w_hat + (f_w[m] + f_i) * 2 * N, 2 * N * 4, &full[s]);
            ++issued;
            ++f_i;
            advance();
        }
        if (!ok) {
            // the consumers stopped: let the copies still in flight land
            for (uint64_t k = issued > kScoreStages ? issued - kScoreStages : 0; k < issued; ++k)
                mbar_wait_bounded(&full[k % kScoreStages], uint32_t((k / kScoreStages) & 1u), nullptr);
        }
        return;
    }

    // --------------------------------------------------------------- consumers
    const uint32_t p0 = a.k.p[0], p1 = a.k.p[1], i0 = a.k.pinv[0], i1 = a.k.pinv[1];
    const int32_t f0 = a.k.r1[0], f1 = a.k.r1[1];
    const uint32_t me = tid >> 8, q4 = tid & 255u;  // group member, point quad
    uint64_t consumed = 0;
    for (uint64_t g = a.group_begin + blockIdx.x; g < a.group_end; g += gridDim.x) {
        const uint64_t o0 = a.group_first[g];
        const uint32_t gm = uint32_t(a.group_first[g + 1] - o0);
        const uint64_t nt = a.term_ptr[o0 + 1] - a.term_ptr[o0];
        const bool active = me < gm;
        // exact sums of products of centred residues (one widening multiply-add
        // each), folded every kFoldSteps terms and reduced mod p after the last
        int64_t acc[16];  // [poly * 2 + prime][4]
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[e] = 0;
        uint32_t since_fold = 0;
        bool got = true;  // every copy of this group's steps landed
        for (uint64_t i = 0; i < nt && got; ++i) {
            const uint32_t s = uint32_t(consumed % kScoreStages);
            got = mbar_wait_bounded(&full[s], uint32_t((consumed / kScoreStages) & 1u), a.err);
            if (!got) break;  // the stage is not released: its copy may still land
            if (active) {
                const uint32_t *st = stage0 + s * ip_stage_words(N);
                const uint4 *cv = reinterpret_cast<const uint4 *>(st);
                const uint4 *wv = reinterpret_cast<const uint4 *>(st + (4 + 2 * me) * N);
                const uint4 w0 = wv[q4], w1 = wv[N / 4 + q4];
                const int32_t W[2][4] = {{int32_t(w0.x), int32_t(w0.y), int32_t(w0.z), int32_t(w0.w)},
                                         {int32_t(w1.x), int32_t(w1.y), int32_t(w1.z), int32_t(w1.w)}};
#pragma unroll
                for (int ap = 0; ap < 4; ++ap) {  // (poly, prime)
                    const uint4 c = cv[ap * (N / 4) + q4];
                    const int32_t Cv[4] = {int32_t(c.x), int32_t(c.y), int32_t(c.z), int32_t(c.w)};
                    const int q = ap & 1;
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[ap * 4 + e] = mad_wide(W[q][e], Cv[e], acc[ap * 4 + e]);
                }
                if (++since_fold == kFoldSteps) {
                    since_fold = 0;
#pragma unroll
                    for (int e = 0; e < 16; ++e) acc[e] = fold(acc[e], (e >> 2) & 1 ? f1 : f0);
                }
            }
            ++consumed;
            // this warp is done with the stage
            __syncwarp();
            if ((tid & 31u) == 0) mbar_arrive(&empty[s]);
        }
        if (!consumers_and(got)) return;  // a copy never landed: all consumers stop here
        // Inverse NTT (Gentleman-Sande; the stage of span t pairs points j and
        // j + t with twiddle itw[N / (2t) + j / (2t)]), in three parts.
        // (1) Each sum to its residue times 2^-32 (REDC), then the stages t = 1
        // and 2, which stay inside this thread's points 4q..4q+3.
        if (active) {
#pragma unroll
            for (int ap = 0; ap < 4; ++ap) {
                const int q = ap & 1;
                const uint32_t p = q ? p1 : p0, pinv = q ? i1 : i0;
                uint32_t v[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    // fold below 2^49 and lift by p * 2^19 to a positive T < p * 2^32
                    const uint64_t T = uint64_t(fold(acc[ap * 4 + e], q ? f1 : f0) + (int64_t(p) << 19));
                    const uint32_t m = uint32_t(T) * pinv;
                    const uint32_t u = uint32_t((T + uint64_t(m) * p) >> 32);
                    v[e] = u >= p ? u - p : u;
                }
                const uint32_t *tw = itws + q * N;
                gs_butterfly(v[0], v[1], tw[N / 2 + 2 * q4], p, pinv);
                gs_butterfly(v[2], v[3], tw[N / 2 + 2 * q4 + 1], p, pinv);
                const uint32_t s2 = tw[N / 4 + q4];
                gs_butterfly(v[0], v[2], s2, p, pinv);
                gs_butterfly(v[1], v[3], s2, p, pinv);
                reinterpret_cast<uint4 *>(arr + (4 * me + ap) * N)[q4] = make_uint4(v[0], v[1], v[2], v[3]);
            }
        }
        consumers_sync();
        // (2) Stages (4, 8), (16, 32), (64, 128) as radix-4 passes: item w of
        // an array takes points base + r + {0, t, 2t, 3t}, base = 4t * (w / t).
#pragma unroll 1
        for (uint32_t lt = 2; lt <= 6; lt += 2) {
            const uint32_t t = 1u << lt, h = N >> (lt + 1);
            for (uint32_t x = tid; x < 4 * gm * (N / 4); x += kScoreThreads) {
                const uint32_t ar = x / (N / 4), w = x % (N / 4);
                const uint32_t kb = w >> lt, r = w & (t - 1);
                const uint32_t q = ar & 1u;
                const uint32_t p = q ? p1 : p0, pinv = q ? i1 : i0;
                uint32_t *va = arr + ar * N + 4 * t * kb + r;
                const uint32_t *tw = itws + q * N;
                uint32_t x0 = va[0], x1 = va[t], x2 = va[2 * t], x3 = va[3 * t];
                gs_butterfly(x0, x1, tw[h + 2 * kb], p, pinv);
                gs_butterfly(x2, x3, tw[h + 2 * kb + 1], p, pinv);
                const uint32_t s = tw[h / 2 + kb];
                gs_butterfly(x0, x2, s, p, pinv);
                gs_butterfly(x1, x3, s, p, pinv);
                va[0] = x0;
                va[t] = x1;
                va[2 * t] = x2;
                va[3 * t] = x3;
            }
            consumers_sync();
        }
        // (3) Stages 256 and 512 in registers, scaled by N^-1 * 2^32 (which
        // also undoes the REDC factor), then CRT and the epilogue: item
        // (member, poly, r) finishes points r + 256e of both primes.
        for (uint32_t x = tid; x < gm * 2 * (N / 4); x += kScoreThreads) {
            const uint32_t m = x / (N / 2), pl = (x / (N / 4)) & 1u, r = x % (N / 4);
            const uint64_t o = o0 + m;
            if (o < a.out_begin || o >= a.out_end) continue;
            uint32_t y[2][4];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const uint32_t p = q ? p1 : p0, pinv = q ? i1 : i0;
                const uint32_t *va = arr + (4 * m + 2 * pl + q) * N + r;
                const uint32_t *tw = itws + q * N;
                uint32_t x0 = va[0], x1 = va[N / 4], x2 = va[N / 2], x3 = va[3 * N / 4];
                gs_butterfly(x0, x1, tw[2], p, pinv);
                gs_butterfly(x2, x3, tw[3], p, pinv);
                y[q][0] = mont_mul(mod_add(x0, x2, p), a.k.nscale[q], p, pinv);
                y[q][1] = mont_mul(mod_add(x1, x3, p), a.k.nscale[q], p, pinv);
                y[q][2] = mont_mul(mod_sub(x0, x2, p), a.k.nscale_tw[q], p, pinv);
                y[q][3] = mont_mul(mod_sub(x1, x3, p), a.k.nscale_tw[q], p, pinv);
            }
            uint32_t *dst = reinterpret_cast<uint32_t *>(a.out + (o - a.out_begin) * a.out_stride) + pl * N;
            const uint32_t add = pl == 1 && a.bias ? uint32_t(a.bias[o]) * uint32_t(a.one) : 0u;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                // CRT: x = x1 + p1 * ((x2 - x1) / p1 mod p2), signed, then mod 2^32
                const uint32_t j = r + e * (N / 4);
                const uint32_t x1 = y[0][e], x2 = y[1][e];
                const uint32_t x1m = x1 >= p1 ? x1 - p1 : x1;
                const uint32_t t = mont_mul(mod_sub(x2, x1m, p1), a.k.p1inv_m, p1, i1);
                const uint64_t v = uint64_t(x1) + uint64_t(p0) * t;
                uint32_t w = uint32_t(v);
                if (v > a.k.M_half) w -= uint32_t(a.k.M);
                if (pl == 1) {
                    if (j < a.num_samples) w += add;
                    if (j >= a.region_size) w = 0;
                }
                dst[j] = w;
            }
        }
        consumers_sync();  // arr is read before the next group overwrites it
    }
}

__global__ void k_synth_int16(uint64_t seed, uint64_t n, int32_t max_abs, int16_t *out) {
    const uint64_t key = mix64(seed + mix64(15));
    const uint32_t span = uint32_t(2 * max_abs);
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
        out[i] = int16_t(int32_t(uint32_t(mix64(key ^ i) >> 32) % span) - max_abs);
}

NttConsts make_consts(uint32_t N) {
    NttConsts k{};
    for (int q = 0; q < 2; ++q) {
        const uint64_t p = kPrimes[q];
        k.p[q] = uint32_t(p);
        uint32_t inv = 1;  // Newton iteration for p^-1 mod 2^32
        for (int it = 0; it < 5; ++it) inv *= 2u - uint32_t(p) * inv;
        k.pinv[q] = 0u - inv;
        const uint64_t R = (uint64_t(1) << 32) % p;
        k.r1[q] = int32_t(R);
        const uint64_t nscale = mulmod(powmod(N, p - 2, p), mulmod(R, R, p), p);
        k.nscale[q] = uint32_t(nscale);
        // the last inverse stage's twiddle: psi^-(N/2) (bit-reversed index 1)
        const uint64_t psi = powmod(kPsi2048[q], 2048 / (2 * N), p);
        k.nscale_tw[q] = uint32_t(mulmod(powmod(powmod(psi, p - 2, p), N / 2, p), nscale, p));
    }
    const uint64_t p0 = kPrimes[0], p1 = kPrimes[1];
    k.p1inv_m = uint32_t(mulmod(powmod(p0 % p1, p1 - 2, p1), (uint64_t(1) << 32) % p1, p1));
    k.M = p0 * p1;
    k.M_half = k.M / 2;
    return k;
}

// Bit-reversed powers of psi (forward) and psi^-1 (inverse), Montgomery form,
// [prime][N] each.  psi is a primitive 2N-th root: psi_2048^(2048 / 2N).
void make_twiddles(uint32_t N, std::vector<uint32_t> *fwd, std::vector<uint32_t> *inv) {
    uint32_t logn = 0;
    while ((1u << logn) < N) ++logn;
    fwd->assign(2 * N, 0);
    inv->assign(2 * N, 0);
    for (int q = 0; q < 2; ++q) {
        const uint64_t p = kPrimes[q];
        const uint64_t psi = powmod(kPsi2048[q], 2048 / (2 * N), p);
        const uint64_t psi_inv = powmod(psi, p - 2, p);
        const uint64_t R = (uint64_t(1) << 32) % p;
        for (uint32_t i = 0; i < N; ++i) {
            uint32_t rev = 0;
            for (uint32_t b = 0; b < logn; ++b)
                if (i & (1u << b)) rev |= 1u << (logn - 1 - b);
            (*fwd)[q * N + i] = uint32_t(mulmod(powmod(psi, rev, p), R, p));
            (*inv)[q * N + i] = uint32_t(mulmod(powmod(psi_inv, rev, p), R, p));
        }
    }
}

}  // namespace

struct IntpolyModel {
    uint32_t N = 0, num_samples = 0, region_size = 0;
    int32_t one = 0, max_abs = 0;
    uint64_t n_out = 0, n_terms = 0, n_rows = 0;
    NttConsts k{};
    uint64_t *d_term_ptr = nullptr;
    uint32_t *d_term_row = nullptr;
    // Output groups: consecutive outputs (at most kGroupMax) with identical
    // term-row lists; group g is outputs [group_first[g], group_first[g + 1]).
    std::vector<uint64_t> group_first;
    uint64_t *d_group_first = nullptr;
    int32_t *d_bias = nullptr;
    uint32_t *d_w_hat = nullptr;
    uint32_t *d_tw = nullptr;   // forward twiddles [2][N]
    uint32_t *d_itw = nullptr;  // inverse twiddles [2][N]
    uint32_t *d_c_hat = nullptr;
    uint64_t c_hat_rows = 0;
    ~IntpolyModel() {
        cudaFree(d_term_ptr);
        cudaFree(d_term_row);
        cudaFree(d_group_first);
        cudaFree(d_bias);
        cudaFree(d_w_hat);
        cudaFree(d_tw);
        cudaFree(d_itw);
        cudaFree(d_c_hat);
    }
};

}  // namespace idash

using namespace idash;

void idash_model::free_intpoly() {
    delete intpoly;
    intpoly = nullptr;
}

extern "C" idash_status idash_model_intpoly(idash_ctx *ctx, idash_model **model, const idash_intpoly_params *p,
                                            uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                                            const int32_t *bias, uint64_t n_in_rows, const int16_t *term_poly,
                                            int term_poly_on_device) {
    if (!ctx || !model || !p || (n_out && !term_ptr)) return IDASH_ERR_INVALID_ARGUMENT;
    *model = nullptr;
    if (p->N != kIpN)
        return ctx->fail(IDASH_ERR_UNSUPPORTED, "the integer-polynomial kernels are built for N = 1024");
    if (p->num_samples > p->region_size || p->region_size > p->N)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "need num_samples <= region_size <= N");
    if (p->max_abs_coef <= 0 || p->max_abs_coef > 32767)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "max_abs_coef must be in [1, 32767]");
    const uint64_t nnz = n_out ? term_ptr[n_out] : 0;
    if (nnz && (!term_feat || !term_poly)) return IDASH_ERR_INVALID_ARGUMENT;
    const NttConsts k = make_consts(p->N);
    // exactness: terms * max|W| * N * 2^31 < M / 2 for every output
    const double cap = double(k.M_half) / (double(p->max_abs_coef) * p->N * 2147483648.0);
    for (uint64_t o = 0; o < n_out; ++o) {
        if (term_ptr[o + 1] < term_ptr[o]) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "term_ptr not monotone");
        if (double(term_ptr[o + 1] - term_ptr[o]) >= cap)
            return ctx->fail(IDASH_ERR_UNSUPPORTED, "output " + std::to_string(o) + " has too many terms for an "
                                                    "exact two-prime product at this max_abs_coef");
    }
    for (uint64_t t = 0; t < nnz; ++t)
        if (term_feat[t] >= n_in_rows) return ctx->fail(IDASH_ERR_INDEX, "a term names a row outside the input");

    idash_model *m = new idash_model();
    m->ctx = ctx;
    m->form = Form::kIntPoly;
    m->n_out = n_out;
    m->n_in_rows = n_in_rows;
    m->intpoly = new IntpolyModel();
    IntpolyModel &ip = *m->intpoly;
    ip.N = p->N;
    ip.num_samples = p->num_samples;
    ip.region_size = p->region_size;
    ip.one = p->one_t32;
    ip.max_abs = p->max_abs_coef;
    ip.n_out = n_out;
    ip.n_terms = nnz;
    ip.n_rows = n_in_rows;
    ip.k = k;
    std::vector<uint32_t> fwd, inv;
    make_twiddles(p->N, &fwd, &inv);
    std::vector<int32_t> bias_v(n_out, 0);
    if (bias) std::memcpy(bias_v.data(), bias, n_out * 4);
    auto fail = [&](idash_status s) {
        idash_model_free(m);
        return s;
    };
    idash_status s = IDASH_OK;
    auto up = [&](void **dst, const void *src, size_t bytes, const char *what) {
        if (s != IDASH_OK) return;
        s = ctx->check_cuda(cudaMalloc(dst, std::max<size_t>(bytes, 16)), what);
        if (s == IDASH_OK && bytes) s = ctx->check_cuda(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), what);
    };
    // groups of outputs that read the same rows in the same order
    ip.group_first.clear();
    for (uint64_t o = 0; o < n_out;) {
        uint64_t e = o + 1;
        const uint64_t len = term_ptr[o + 1] - term_ptr[o];
        while (e < n_out && e - o < kGroupMax && term_ptr[e + 1] - term_ptr[e] == len &&
               std::equal(term_feat + term_ptr[o], term_feat + term_ptr[o + 1], term_feat + term_ptr[e]))
            ++e;
        ip.group_first.push_back(o);
        o = e;
    }
    ip.group_first.push_back(n_out);
    up(reinterpret_cast<void **>(&ip.d_group_first), ip.group_first.data(), ip.group_first.size() * 8,
       "intpoly groups");
    up(reinterpret_cast<void **>(&ip.d_term_ptr), term_ptr, (n_out + 1) * 8, "intpoly term_ptr");
    up(reinterpret_cast<void **>(&ip.d_term_row), term_feat, nnz * 4, "intpoly term rows");
    up(reinterpret_cast<void **>(&ip.d_bias), bias_v.data(), n_out * 4, "intpoly bias");
    up(reinterpret_cast<void **>(&ip.d_tw), fwd.data(), fwd.size() * 4, "intpoly twiddles");
    up(reinterpret_cast<void **>(&ip.d_itw), inv.data(), inv.size() * 4, "intpoly twiddles");
    if (s == IDASH_OK)
        s = ctx->check_cuda(cudaMalloc(&ip.d_w_hat, std::max<size_t>(nnz * 2 * p->N * 4, 16)), "cudaMalloc(W^)");
    if (s != IDASH_OK) return fail(s);
    // Model polynomials -> NTT, through a bounded device staging buffer when on the host.
    const size_t smem = size_t(4) * p->N * 4;
    const uint64_t chunk = term_poly_on_device ? nnz : std::min<uint64_t>(nnz, (uint64_t(1) << 28) / p->N);
    int16_t *stage = nullptr;
    if (!term_poly_on_device && nnz &&
        (s = ctx->check_cuda(cudaMalloc(&stage, chunk * p->N * 2), "cudaMalloc(model staging)")) != IDASH_OK)
        return fail(s);
    for (uint64_t t0 = 0; t0 < nnz && s == IDASH_OK; t0 += chunk) {
        const uint64_t n = std::min(chunk, nnz - t0);
        const int16_t *src = term_poly + t0 * p->N;
        if (!term_poly_on_device) {
            s = ctx->check_cuda(cudaMemcpy(stage, src, n * p->N * 2, cudaMemcpyHostToDevice), "model upload");
            src = stage;
        }
        if (s != IDASH_OK) break;
        const uint32_t grid = uint32_t(std::min<uint64_t>(n, uint64_t(ctx->sm_count) * 8));
        k_ntt_model<<<grid, kNttThreads, smem, ctx->stream>>>(src, n, p->N, ip.d_tw, k, p->max_abs_coef,
                                                             ip.d_w_hat + t0 * 2 * p->N, ctx->d_err);
        s = ctx->check_cuda(cudaGetLastError(), "k_ntt_model launch");
        if (s == IDASH_OK) s = idash_sync(ctx);
    }
    cudaFree(stage);
    if (s != IDASH_OK) {
        if (s == IDASH_ERR_INDEX) ctx->last_error = "a model coefficient exceeds max_abs_coef";
        return fail(s);
    }
    ctx->models.insert(m);
    *model = m;
    return IDASH_OK;
}

extern "C" idash_status idash_model_intpoly_set_weights(idash_model *m, const int16_t *d_term_poly, void *stream) {
    if (!m) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kIntPoly || !m->intpoly) return ctx->fail(IDASH_ERR_STATE, "not an integer-polynomial model");
    IntpolyModel &ip = *m->intpoly;
    if (ip.n_terms == 0) return IDASH_OK;
    if (!d_term_poly) return IDASH_ERR_INVALID_ARGUMENT;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const uint32_t grid = uint32_t(std::min<uint64_t>(ip.n_terms, uint64_t(ctx->sm_count) * 8));
    k_ntt_model<<<grid, kNttThreads, size_t(4) * ip.N * 4, st>>>(d_term_poly, ip.n_terms, ip.N, ip.d_tw, ip.k,
                                                                ip.max_abs, ip.d_w_hat, ctx->d_err);
    return ctx->check_cuda(cudaGetLastError(), "k_ntt_model launch");
}

extern "C" idash_status idash_score_intpoly_device(idash_model *m, const void *d_in, const idash_row_layout *il,
                                                   uint64_t out_begin, uint64_t out_end, void *d_out,
                                                   const idash_row_layout *ol, void *stream) {
    if (!m || !d_in || !d_out || !il || !ol) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kIntPoly || !m->intpoly) return ctx->fail(IDASH_ERR_STATE, "not an integer-polynomial model");
    IntpolyModel &ip = *m->intpoly;
    if (out_begin > out_end || out_end > ip.n_out) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "bad output range");
    const uint64_t payload = uint64_t(2) * ip.N * 4;
    if (il->row_stride % 16 || ol->row_stride % 16 || il->payload_offset + payload > il->row_stride ||
        ol->payload_offset + payload > ol->row_stride ||
        ((reinterpret_cast<uintptr_t>(d_in) + il->payload_offset) & 15u) ||
        ((reinterpret_cast<uintptr_t>(d_out) + ol->payload_offset) & 15u))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "row layout: stride or alignment");
    if (out_begin == out_end) return IDASH_OK;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    idash_status s = IDASH_OK;
    if (ip.c_hat_rows < ip.n_rows) {
        if ((s = ctx->check_cuda(cudaStreamSynchronize(st), "sync before growing C^")) != IDASH_OK) return s;
        cudaFree(ip.d_c_hat);
        ip.d_c_hat = nullptr;
        ip.c_hat_rows = 0;
        if ((s = ctx->check_cuda(cudaMalloc(&ip.d_c_hat, std::max<uint64_t>(ip.n_rows, 1) * 4 * ip.N * 4),
                                 "cudaMalloc(C^)")) != IDASH_OK)
            return s;
        ip.c_hat_rows = ip.n_rows;
    }
    const size_t smem_rows = size_t(10) * kIpN * 4;  // twiddles and two row buffers
    int rows_per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rows_per_sm, k_ntt_rows, kNttThreads, smem_rows) != cudaSuccess ||
        rows_per_sm < 1)
        rows_per_sm = 1;
    const uint32_t grid_rows = uint32_t(std::min<uint64_t>(ip.n_rows, uint64_t(ctx->sm_count) * rows_per_sm));
    if (grid_rows) {
        k_ntt_rows<<<grid_rows, kNttThreads, smem_rows, st>>>(static_cast<const uint8_t *>(d_in) + il->payload_offset,
                                                             il->row_stride, ip.n_rows, ip.d_tw, ip.k, ip.d_c_hat);
        if ((s = ctx->check_cuda(cudaGetLastError(), "k_ntt_rows launch")) != IDASH_OK) return s;
    }
    IntpolyArgs a{};
    a.term_ptr = ip.d_term_ptr;
    a.term_row = ip.d_term_row;
    a.group_first = ip.d_group_first;
    {
        // groups holding outputs of [out_begin, out_end)
        const auto &G = ip.group_first;
        a.group_begin = uint64_t(std::upper_bound(G.begin(), G.end() - 1, out_begin) - G.begin()) - 1;
        a.group_end = uint64_t(std::lower_bound(G.begin(), G.end() - 1, out_end) - G.begin());
    }
    a.w_hat = ip.d_w_hat;
    a.c_hat = ip.d_c_hat;
    a.bias = ip.d_bias;
    a.itw = ip.d_itw;
    a.k = ip.k;
    a.N = ip.N;
    a.num_samples = ip.num_samples;
    a.region_size = ip.region_size;
    a.n_rows = uint32_t(ip.n_rows);
    a.one = ip.one;
    a.out_begin = out_begin;
    a.out_end = out_end;
    a.out = static_cast<uint8_t *>(d_out) + ol->payload_offset;
    a.out_stride = ol->row_stride;
    a.err = ctx->d_err;
    const size_t smem = ip_score_smem(ip.N);
    // the ring needs more than the default 48 KiB of dynamic shared memory
    if ((s = ctx->check_cuda(cudaFuncSetAttribute(k_intpoly_score, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  int(smem)),
                             "k_intpoly_score shared memory")) != IDASH_OK)
        return s;
    // one wave of resident CTAs, each striding over the groups
    int resident = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_intpoly_score, kScoreBlock, smem) != cudaSuccess ||
        resident < 1)
        resident = 1;
    const uint32_t grid = uint32_t(
        std::min<uint64_t>(a.group_end - a.group_begin, uint64_t(ctx->sm_count) * uint64_t(resident)));
    k_intpoly_score<<<grid, kScoreBlock, smem, st>>>(a);
    s = ctx->check_cuda(cudaGetLastError(), "k_intpoly_score launch");
    if (s == IDASH_OK) ctx->stats.kernel_launches += 2;
    return s;
}

extern "C" idash_status idash_synth_int16_device(idash_ctx *ctx, uint64_t seed, uint64_t n, int32_t max_abs,
                                                 int16_t *d_out, void *stream) {
    if (!ctx || !d_out || max_abs <= 0 || max_abs > 16383) return IDASH_ERR_INVALID_ARGUMENT;
    if (n == 0) return IDASH_OK;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const uint32_t grid = uint32_t(std::min<uint64_t>((n + 255) / 256, uint64_t(ctx->sm_count) * 16));
    k_synth_int16<<<grid, 256, 0, st>>>(seed, n, max_abs, d_out);
    return ctx->check_cuda(cudaGetLastError(), "k_synth_int16 launch");
}
