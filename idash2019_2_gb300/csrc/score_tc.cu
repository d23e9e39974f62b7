// Scoring on the tensor cores: out_o = bias_o + sum_k coef[o][k] * row_k, per
// column, in Z/2^32 - the accumulate of cloud_compute_score
// (tLweAddMulTo per term, eval/idash.cpp:800-819) as a dense product
//   D[outputs x columns] = A[outputs x rows] * B[rows x columns]
// per block of up to 128 consecutive outputs, on tcgen05.mma.
//
// Exactness.  The operands are small integers held exactly in fp16 and
// summed exactly in fp32: an error-free splitting of an integer product into
// digit products, as in the published tensor-core methods that emulate exact
// or high-precision matrix products by splitting (Mukunoki, Ozaki, Ogita and
// Imamura, "DGEMM using Tensor Cores, and Its Accurate and Reproducible
// Versions", ISC 2020).  A ciphertext word x is written as four balanced
// base-256 digits x = sum_i b_i 256^i (mod 2^32), b_i = byte_i(x + 0x80808080)
// - 128 in [-128, 127]; a coefficient c as c0 + 256 c1, c0 in [-128, 127].
// Digit products land in four accumulators by shift: D_s = sum over i + j = s
// of A_j * B_i, s = 0..3 (seven MMAs per K-step), and
//   out = sum_s 256^s D_s  (mod 2^32).
// The planner bounds K so that every partial sum stays below 2^22 in
// magnitude (plan.hpp), where fp32 holds integers exactly; the epilogue turns
// D_s into an integer by adding 1.5 * 2^23 and reading the bits.
//
// Structure (one CTA of 10 warps per SM, persistent over work units of
// (block, run of 64-column slices)):
//   warp 4     producer: the block's coefficient digits (one bulk copy, kept
//              in shared memory for the unit) and, per chunk of 32 rows, the
//              rows' 64-column slices: one 2D tensor copy
//              (cp.async.bulk.tensor) when the chunk's rows are consecutive,
//              else one cp.async.bulk per row; completed on mbarriers;
//   warps 6-9  converters: raw words -> four fp16 digit planes in the MMA's
//              no-swizzle K-major layout;
//   warp 5     allocates the 512 TMEM columns; lane 0 issues tcgen05.mma
//              (M = 128, N = 64, K = 16) into a double-buffered set of four
//              fp32 accumulators and commits to mbarriers;
//   warps 0-3  epilogue: tcgen05.ld of the accumulators (warp w reads TMEM
//              lanes 32w..32w+31, one output each), the digit recombination,
//              bias and zeroed columns; each warp stages its 32 rows in
//              shared memory and stores them row by row with coalesced
//              16-byte streaming stores (no barrier across warps).
// Every wait is bounded; a wait that expires records IDASH_ERR_DEVICE_TIMEOUT,
// raises a CTA-wide abort flag that ends the other roles' waits, and each
// role then waits (bounded) for its own copies and MMAs in flight before the
// TMEM columns are freed.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "common.cuh"
#include "score_kernels.cuh"

namespace idash {

namespace {

constexpr uint32_t kN = kTcSliceWords;  // 64 columns per tile
constexpr uint32_t kM = kTcRows;        // 128 outputs per block
constexpr uint32_t kChunk = 32;         // rows per pipeline chunk (two MMA K-steps)
constexpr uint32_t kRawStages = 4, kDigStages = 2, kAccStages = 2;
constexpr uint32_t kRawRow = kN + 4;                    // words per row slice in a raw stage (bank padding)
constexpr uint32_t kRawStageBytes = kChunk * kRawRow * 4;
constexpr uint32_t kPlaneBytes = kChunk * kN * 2;       // one fp16 digit plane of a chunk
constexpr uint32_t kDigStageBytes = 4 * kPlaneBytes;
constexpr uint32_t kOutRow = kN + 4;                    // words per output row in the staging buffer
constexpr uint32_t kOutBytes = kM * kOutRow * 4;
constexpr uint32_t kHeader = 1024;
constexpr uint32_t kThreads = 320;
constexpr uint32_t kProducerWarp = 4, kMmaWarp = 5, kConvWarp0 = 6;
constexpr uint32_t kTmemCols = 512;                     // 2 stages x 4 accumulators x 64 columns
constexpr uint32_t kMagic = 0x4B400000u;                // bits of 1.5 * 2^23
constexpr uint32_t kMagicSum = kMagic + (kMagic << 8) + (kMagic << 16) + (kMagic << 24);
// one CTA per SM, so the CTA owns all of TMEM
constexpr size_t kMinSmem = 120 * 1024;

struct TcBars {
    uint64_t a_full, a_empty, drain;
    uint64_t raw_full[kRawStages], raw_empty[kRawStages];
    uint64_t dig_full[kDigStages], dig_empty[kDigStages];
    uint64_t acc_full[kAccStages], acc_empty[kAccStages];
    uint32_t tmem_base;
    uint32_t abort;
};
static_assert(sizeof(TcBars) <= kHeader, "barrier area");

__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool aborted(const TcBars &sh) {
    return *reinterpret_cast<const volatile uint32_t *>(&sh.abort) != 0;
}

// Bounded wait that also ends when another role raised the abort flag.
__device__ __forceinline__ bool tc_wait(TcBars &sh, uint64_t *bar, uint32_t parity, uint32_t *err) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait_sleep(bar, parity, 20000u)) {
        if (aborted(sh)) return false;
        if (clock64() - t0 > kWaitLimitCycles) {
            report_error(err, kDevTimeout);
            *reinterpret_cast<volatile uint32_t *>(&sh.abort) = 1u;
            return false;
        }
    }
    return true;
}

// Lane 0 waits, the warp follows its verdict.
__device__ __forceinline__ bool warp_wait(TcBars &sh, uint64_t *bar, uint32_t parity, uint32_t *err, uint32_t lane) {
    uint32_t ok = 1;
    if (lane == 0) ok = tc_wait(sh, bar, parity, err) ? 1u : 0u;
    return __shfl_sync(0xFFFFFFFFu, ok, 0) != 0;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: start address, LBO = bytes
// between core matrices along K, SBO = bytes between 8-row groups.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// D (fp32, TMEM) (+)= A (fp16, K-major) * B (fp16, K-major), M = 128, N = 64.
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    constexpr uint32_t idesc = (1u << 4) | ((kN >> 3) << 17) | ((kM >> 4) << 24);
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr)
        : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 2D tensor copy of the box at (x = column, y = row) into shared memory,
// completed on `bar` as transaction bytes.  x * 4 is a multiple of 16.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int32_t x, int32_t y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ uint4 lds_v4p(const uint32_t *p) {
    uint4 v;
    asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(smem_addr(p)));
    return v;
}

__device__ __forceinline__ void sts_v4(uint32_t *p, uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
    asm volatile("st.shared.v4.u32 [%0], {%1,%2,%3,%4};" ::"r"(smem_addr(p)), "r"(x), "r"(y), "r"(z), "r"(w)
                 : "memory");
}

// fp16x2 bits {lo: v_lo - 128, hi: v_hi - 128} from r = [v_lo, 0x64, v_hi, 0x64]
// (fp16 1024 + v, exact) minus 1152.
__device__ __forceinline__ uint32_t digits_minus_128(uint32_t r) {
    const __half2 h = __hsub2(*reinterpret_cast<const __half2 *>(&r), __half2(__half(1152.f), __half(1152.f)));
    return *reinterpret_cast<const uint32_t *>(&h);
}

struct Unit {
    PlanBlock blk;
    uint32_t s0, s1, k_pad, n_chunks;
};

__device__ __forceinline__ Unit unit_of(const ScoreArgs &a, uint32_t u) {
    Unit x;
    x.blk = a.blocks[a.block_lo + u / a.units_per_block];
    x.s0 = (u % a.units_per_block) * a.unit_slices;
    x.s1 = min(x.s0 + a.unit_slices, a.n_slices);
    x.k_pad = x.blk.n_groups;
    x.n_chunks = (x.k_pad + kChunk - 1) / kChunk;
    return x;
}

__global__ void __launch_bounds__(kThreads, 1) k_score_tc(const ScoreArgs a, const __grid_constant__ CUtensorMap rows_map) {
    extern __shared__ __align__(1024) uint8_t smem[];
    TcBars &sh = *reinterpret_cast<TcBars *>(smem);
    uint8_t *smA = smem + kHeader;
    uint8_t *raw = smA + a.tc_a_max_bytes;
    uint8_t *dig = raw + kRawStages * kRawStageBytes;
    uint8_t *stage_out = dig + kDigStages * kDigStageBytes;
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        mbar_init(&sh.a_full, 1);
        mbar_init(&sh.a_empty, 1);
        mbar_init(&sh.drain, 1);
        for (uint32_t s = 0; s < kRawStages; ++s) {
            mbar_init(&sh.raw_full[s], 1);
            mbar_init(&sh.raw_empty[s], 4);
        }
        for (uint32_t s = 0; s < kDigStages; ++s) {
            mbar_init(&sh.dig_full[s], 4);
            mbar_init(&sh.dig_empty[s], 1);
        }
        for (uint32_t s = 0; s < kAccStages; ++s) {
            mbar_init(&sh.acc_full[s], 1);
            mbar_init(&sh.acc_empty[s], 4);
        }
        sh.abort = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&sh.tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem_base;

    if (warp == kProducerWarp) {
        // ------------------------------------------------------------ producer
        uint32_t rc = 0, a_loads = 0;
        bool ok = true;
        for (uint32_t u = blockIdx.x, uc = 0; ok && u < a.n_units; u += gridDim.x, ++uc) {
            const Unit x = unit_of(a, u);
            if (uc > 0 && !(ok = warp_wait(sh, &sh.a_empty, (uc - 1) & 1u, a.err, lane))) break;
            if (lane == 0) {
                const uint32_t bytes = 4u * kM * x.k_pad;  // tc_a_bytes(k_pad): two fp16 digit planes
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&sh.a_full, bytes);
                bulk_g2s(smA, a.tc_a + uint64_t(x.blk.group_begin) * 16, bytes, &sh.a_full);
            }
            ++a_loads;
            for (uint32_t sl = x.s0; ok && sl < x.s1; ++sl) {
                const uint32_t c0 = sl * kN;
                const uint32_t valid = min(kN, a.row_words - c0);
                const uint32_t copy_bytes = ((valid + 3u) & ~3u) * 4u;
                for (uint32_t c = 0; c < x.n_chunks; ++c) {
                    const uint32_t st = rc % kRawStages;
                    if (rc >= kRawStages &&
                        !(ok = warp_wait(sh, &sh.raw_empty[st], ((rc / kRawStages) - 1) & 1u, a.err, lane)))
                        break;
                    if (lane == 0) fence_proxy_async_smem();
                    __syncwarp();
                    const uint32_t k_lo = c * kChunk, k_hi = min(k_lo + kChunk, uint32_t(x.blk.n_slots));
                    uint8_t *dst = raw + st * kRawStageBytes;
                    if (a.tc_use_map && k_hi > k_lo && ((x.blk.term_begin >> c) & 1u)) {
                        // consecutive rows: the whole chunk (32 rows x 68 words) in one tensor copy
                        if (lane == 0) {
                            const uint32_t r0 = a.slots[x.blk.slot_begin + k_lo].row - a.row_base;
                            if (r0 >= a.n_rows || r0 + (k_hi - k_lo) > a.n_rows) {
                                report_error(a.err, kDevBadIndex);
                            } else {
                                expect_tx(&sh.raw_full[st], kRawStageBytes);
                                tma_load_2d(dst, &rows_map, int32_t(c0), int32_t(r0), &sh.raw_full[st]);
                            }
                        }
                    } else {
                        for (uint32_t k = k_lo + lane; k < k_hi; k += 32) {
                            const uint32_t r = a.slots[x.blk.slot_begin + k].row - a.row_base;
                            if (r >= a.n_rows) {
                                report_error(a.err, kDevBadIndex);
                                continue;
                            }
                            expect_tx(&sh.raw_full[st], copy_bytes);
                            bulk_g2s(dst + (k - k_lo) * kRawRow * 4,
                                     a.in + uint64_t(r) * a.in_stride + uint64_t(c0) * 4, copy_bytes,
                                     &sh.raw_full[st]);
                        }
                    }
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&sh.raw_full[st]);
                    ++rc;
                }
            }
        }
        // let every copy this CTA issued land: the last fill of each raw
        // stage and the last digit load (immediate when nothing aborted)
        if (lane == 0) {
            for (uint32_t k = 1; k <= kRawStages && k <= rc; ++k) {
                const uint32_t j = rc - k;
                mbar_wait_bounded(&sh.raw_full[j % kRawStages], (j / kRawStages) & 1u, nullptr);
            }
            if (a_loads) mbar_wait_bounded(&sh.a_full, (a_loads - 1) & 1u, nullptr);
        }
    } else if (warp >= kConvWarp0) {
        // ---------------------------------------------------------- converters
        // thread -> row pair kp (rows 2kp, 2kp+1 of the chunk) and columns
        // nl + 8i: raw reads and digit stores both hit 32 distinct banks
        const uint32_t cw = warp - kConvWarp0;
        const uint32_t kp = 4 * cw + lane / 8, nl = lane % 8;
        uint32_t rc = 0;
        bool ok = true;
        for (uint32_t u = blockIdx.x; ok && u < a.n_units; u += gridDim.x) {
            const Unit x = unit_of(a, u);
            for (uint32_t sl = x.s0; ok && sl < x.s1; ++sl) {
                for (uint32_t c = 0; c < x.n_chunks; ++c, ++rc) {
                    const uint32_t st = rc % kRawStages, dg = rc % kDigStages;
                    if (!(ok = warp_wait(sh, &sh.raw_full[st], (rc / kRawStages) & 1u, a.err, lane))) break;
                    if (rc >= kDigStages &&
                        !(ok = warp_wait(sh, &sh.dig_empty[dg], ((rc / kDigStages) - 1) & 1u, a.err, lane)))
                        break;
                    const uint32_t rows = min(kChunk, x.k_pad - c * kChunk);
                    if (2 * kp < rows) {
                        const uint32_t *rw =
                            reinterpret_cast<const uint32_t *>(raw + st * kRawStageBytes) + 2 * kp * kRawRow + nl;
                        uint32_t *dp = reinterpret_cast<uint32_t *>(dig + dg * kDigStageBytes) + (kp / 4) * 256 +
                                       nl * 4 + (kp % 4);
#pragma unroll
                        for (uint32_t i = 0; i < kN / 8; ++i) {
                            const uint32_t ya = rw[8 * i] + 0x80808080u, yb = rw[kRawRow + 8 * i] + 0x80808080u;
                            const uint32_t lo = __byte_perm(ya, yb, 0x5140), hi = __byte_perm(ya, yb, 0x7362);
                            constexpr uint32_t k64 = 0x64646464u;
                            uint32_t *q = dp + 32 * i;
                            q[0] = digits_minus_128(__byte_perm(lo, k64, 0x4140));
                            q[kPlaneBytes / 4] = digits_minus_128(__byte_perm(lo, k64, 0x4342));
                            q[2 * kPlaneBytes / 4] = digits_minus_128(__byte_perm(hi, k64, 0x4140));
                            q[3 * kPlaneBytes / 4] = digits_minus_128(__byte_perm(hi, k64, 0x4342));
                        }
                    }
                    fence_proxy_async_smem();  // the digits are read by the tensor cores (async proxy)
                    __syncwarp();
                    if (lane == 0) {
                        mbar_arrive(&sh.raw_empty[st]);
                        mbar_arrive(&sh.dig_full[dg]);
                    }
                }
            }
        }
    } else if (warp == kMmaWarp) {
        // ----------------------------------------------------------------- MMA
        if (lane == 0) {
            uint32_t rc = 0, tcount = 0;
            bool ok = true;
            const uint32_t a_base = smem_addr(smA), d_base = smem_addr(dig);
            for (uint32_t u = blockIdx.x, uc = 0; ok && u < a.n_units; u += gridDim.x, ++uc) {
                const Unit x = unit_of(a, u);
                if (!(ok = tc_wait(sh, &sh.a_full, uc & 1u, a.err))) break;
                const uint32_t a_plane = x.k_pad * 256;  // bytes per coefficient digit plane
                for (uint32_t sl = x.s0; ok && sl < x.s1; ++sl, ++tcount) {
                    const uint32_t acc = tcount % kAccStages;
                    if (tcount >= kAccStages &&
                        !(ok = tc_wait(sh, &sh.acc_empty[acc], ((tcount / kAccStages) - 1) & 1u, a.err)))
                        break;
                    tc_fence_after();
                    const uint32_t d0 = tmem + acc * 256;
                    for (uint32_t c = 0; c < x.n_chunks; ++c, ++rc) {
                        const uint32_t dg = rc % kDigStages;
                        if (!(ok = tc_wait(sh, &sh.dig_full[dg], (rc / kDigStages) & 1u, a.err))) break;
                        tc_fence_after();
                        const uint32_t steps = min(kChunk, x.k_pad - c * kChunk) / 16;
                        const uint32_t b_base = d_base + dg * kDigStageBytes;
                        for (uint32_t j = 0; j < steps; ++j) {
                            const uint32_t s = c * 2 + j, on = s > 0 ? 1u : 0u;
                            const uint64_t a0 = umma_desc(a_base + s * 4096, 2048, 128);
                            const uint64_t a1 = umma_desc(a_base + a_plane + s * 4096, 2048, 128);
                            const uint64_t b0 = umma_desc(b_base + j * 2048, 1024, 128);
                            const uint64_t b1 = umma_desc(b_base + kPlaneBytes + j * 2048, 1024, 128);
                            const uint64_t b2 = umma_desc(b_base + 2 * kPlaneBytes + j * 2048, 1024, 128);
                            const uint64_t b3 = umma_desc(b_base + 3 * kPlaneBytes + j * 2048, 1024, 128);
                            umma_f16(d0, a0, b0, on);
                            umma_f16(d0 + 64, a0, b1, on);
                            umma_f16(d0 + 64, a1, b0, 1u);
                            umma_f16(d0 + 128, a0, b2, on);
                            umma_f16(d0 + 128, a1, b1, 1u);
                            umma_f16(d0 + 192, a0, b3, on);
                            umma_f16(d0 + 192, a1, b2, 1u);
                        }
                        umma_commit(&sh.dig_empty[dg]);
                    }
                    if (ok) umma_commit(&sh.acc_full[acc]);
                }
                if (ok) umma_commit(&sh.a_empty);
            }
            // every MMA issued has completed before TMEM is released
            umma_commit(&sh.drain);
            mbar_wait_bounded(&sh.drain, 0, nullptr);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const uint32_t row = warp * 32 + lane;
        const uint32_t t_lane = (warp * 32) << 16;
        uint32_t *stage_rows = reinterpret_cast<uint32_t *>(stage_out);
        uint32_t *srow = stage_rows + row * kOutRow;
        uint32_t tcount = 0;
        bool ok = true;
        for (uint32_t u = blockIdx.x; ok && u < a.n_units; u += gridDim.x) {
            const Unit x = unit_of(a, u);
            const uint32_t o = x.blk.out_lo + row;
            const bool has = o < x.blk.out_hi && o >= a.out_lo && o < a.out_hi;
            const uint32_t bias = has ? a.tc_bias[o] : 0u;
            uint8_t *orow = has ? a.out + (a.out_row_map ? uint64_t(a.out_row_map[o]) : uint64_t(o) - a.out_row_base) *
                                              a.out_stride
                                : nullptr;
            for (uint32_t sl = x.s0; ok && sl < x.s1; ++sl, ++tcount) {
                const uint32_t acc = tcount % kAccStages;
                if (!(ok = warp_wait(sh, &sh.acc_full[acc], (tcount / kAccStages) & 1u, a.err, lane))) break;
                tc_fence_after();
                const uint32_t c0 = sl * kN;
                const uint32_t valid = min(kN, a.row_words - c0);
                const bool full = valid == kN;
                // columns (relative to c0) that take the bias, and that are zeroed
                uint32_t b_lo = 0, b_hi = 0, z_lo = 0, z_hi = 0;
                if (a.form == kFormTrlwe) {
                    auto rel = [&](uint32_t c) { return c <= c0 ? 0u : min(c - c0, kN); };
                    b_lo = rel(a.N);
                    b_hi = rel(a.N + a.num_samples);
                    z_lo = rel(a.N + a.region_size);
                    z_hi = rel(2 * a.N);
                } else {
                    const uint32_t first = (a.lwe_n1 - 1u) - c0 % a.lwe_n1;  // next column c with c % n1 == n
                    b_lo = min(first, kN);
                    b_hi = min(first + 1u, kN);
                }
                // warp-uniform fast path: the bias on every column or none, nothing zeroed
                const bool uniform = z_lo >= z_hi && (b_lo >= b_hi || (b_lo == 0 && b_hi == kN));
                const uint32_t add_all = (b_lo == 0 && b_hi == kN ? bias : 0u) - kMagicSum;
                const uint32_t base = tmem + t_lane + acc * 256;
#pragma unroll
                for (uint32_t cc = 0; cc < kN / 16; ++cc) {
                    uint32_t d0[16], d1[16], d2[16], d3[16];
                    tmem_ld16(base + cc * 16, d0);
                    tmem_ld16(base + 64 + cc * 16, d1);
                    tmem_ld16(base + 128 + cc * 16, d2);
                    tmem_ld16(base + 192 + cc * 16, d3);
                    tmem_wait_ld();
                    uint32_t v[16];
#pragma unroll
                    for (uint32_t j = 0; j < 16; ++j) {
                        const uint32_t u0 = __float_as_uint(__fadd_rn(__uint_as_float(d0[j]), 12582912.0f));
                        const uint32_t u1 = __float_as_uint(__fadd_rn(__uint_as_float(d1[j]), 12582912.0f));
                        const uint32_t u2 = __float_as_uint(__fadd_rn(__uint_as_float(d2[j]), 12582912.0f));
                        const uint32_t u3 = __float_as_uint(__fadd_rn(__uint_as_float(d3[j]), 12582912.0f));
                        v[j] = ((u3 * 256u + u2) * 256u + u1) * 256u + u0;
                    }
                    if (uniform) {
#pragma unroll
                        for (uint32_t j = 0; j < 16; ++j) v[j] += add_all;
                    } else {
#pragma unroll
                        for (uint32_t j = 0; j < 16; ++j) {
                            const uint32_t col = cc * 16 + j;
                            v[j] += (col >= b_lo && col < b_hi ? bias : 0u) - kMagicSum;
                            if (col >= z_lo && col < z_hi) v[j] = 0u;
                        }
                    }
                    if (full) {
#pragma unroll
                        for (uint32_t j = 0; j < 16; j += 4) sts_v4(srow + cc * 16 + j, v[j], v[j + 1], v[j + 2], v[j + 3]);
                    } else if (has) {
                        uint32_t *g = reinterpret_cast<uint32_t *>(orow) + c0 + cc * 16;
#pragma unroll
                        for (uint32_t j = 0; j < 16; ++j)
                            if (cc * 16 + j < valid) g[j] = v[j];
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&sh.acc_empty[acc]);
                if (full) {
                    // the warp's 32 staged rows, row by row: lanes 0-15 and
                    // 16-31 each store one row's 256 bytes as coalesced
                    // 16-byte stores; row r's address comes from lane r
                    __syncwarp();
                    const uint32_t half = lane / 16, q = lane % 16;
                    const uint64_t mine = reinterpret_cast<uint64_t>(orow);
#pragma unroll 4
                    for (uint32_t i = 0; i < 16; ++i) {
                        const uint32_t r = 2 * i + half;
                        const uint64_t dst = __shfl_sync(0xFFFFFFFFu, mine, r);
                        const uint4 w = lds_v4p(stage_rows + (warp * 32 + r) * kOutRow + 4 * q);
                        if (dst)
                            stg_cs_v4(reinterpret_cast<uint8_t *>(dst) + uint64_t(c0) * 4 + 16 * q,
                                      make_int4(int(w.x), int(w.y), int(w.z), int(w.w)));
                    }
                    __syncwarp();  // the warp has read its staged rows before the next tile writes them
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kMmaWarp)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// The input rows as a 2D tensor (row_words columns x n_rows rows, uint32,
// row stride in_stride bytes) read in boxes of 68 columns x 32 rows: one
// chunk of a raw stage.  False when the layout cannot be encoded (the kernel
// then copies row by row).
bool encode_rows_map(const ScoreArgs &a, CUtensorMap *map) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || a.n_rows == 0 || a.in_stride % 16 || (reinterpret_cast<uintptr_t>(a.in) & 15u)) return false;
    const cuuint64_t dims[2] = {a.row_words, a.n_rows};
    const cuuint64_t strides[1] = {a.in_stride};
    const cuuint32_t box[2] = {kRawRow, kChunk};
    const cuuint32_t elem[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<uint8_t *>(a.in), dims, strides, box, elem,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t tc_smem_bytes(uint32_t max_k_pad) {
    const size_t need = kHeader + size_t(tc_a_bytes(max_k_pad)) + size_t(kRawStages) * kRawStageBytes +
                        size_t(kDigStages) * kDigStageBytes + kOutBytes;
    return need < kMinSmem ? kMinSmem : need;
}

cudaError_t configure_tc_kernel(size_t max_smem) {
    return cudaFuncSetAttribute(k_score_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(max_smem));
}

cudaError_t launch_score_tc(const ScoreArgs &a_in, uint32_t ctas, cudaStream_t stream) {
    if (a_in.n_units == 0) return cudaSuccess;
    if (a_in.accumulate || a_in.digest || a_in.units_per_block == 0 || a_in.unit_slices == 0)
        return cudaErrorInvalidValue;
    ScoreArgs a = a_in;
    CUtensorMap map;
    std::memset(&map, 0, sizeof(map));
    a.tc_use_map = encode_rows_map(a, &map) ? 1u : 0u;
    const size_t smem = tc_smem_bytes(a.tc_a_max_bytes / uint32_t(tc_a_bytes(1)));
    const uint32_t grid = ctas < a.n_units ? ctas : a.n_units;
    k_score_tc<<<grid, kThreads, smem, stream>>>(a, map);
    return cudaGetLastError();
}

}  // namespace idash
