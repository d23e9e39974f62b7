// Scoring kernels: out_o = sum_terms coef * X^(-m) * row + bias, per column
// slice of the ciphertext rows, all in Z/2^32.  This is the arithmetic of
// cloud_compute_score (eval/idash.cpp:800-841) reorganised for the GPU:
//   - tLweAddMulTo per term (eval/idash.cpp:817) becomes one IMAD per word;
//   - the fold of region r (torusPolynomialMulByXai by 2N - r*REGION_SIZE then
//     tLweAddTo, :826-836) is applied per term as a rotated read, which is the
//     same value because the rotation is linear over Z/2^32;
//   - the bias on b[0..NUM_SAMPLES) (:805-810) and the zeroing of
//     b[REGION_SIZE..N) (:839-841) are the epilogue.
//
// k_score_window  (batched): persistent CTAs pull (block, slice) tiles from an
//   atomic counter; each tile's input window is staged into shared memory with
//   cp.async.bulk (completed on an mbarrier, waits bounded), then every thread
//   accumulates Q quads of columns x G outputs from 16-byte shared loads.
// k_score_direct  (plain): one CTA per tile, each output read straight from
//   global memory term by term - the reference's per-output loop on the GPU.
//
// A thread owns Q quads (4 consecutive columns each); quad k of the thread at
// lane l of its team sits at column 4*l + 4*k*TEAM of the slice, so a warp's
// 16-byte loads and stores of one quad are contiguous.
#include "common.cuh"
#include "score_kernels.cuh"

namespace idash {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Epilogue masks over the thread's 4Q columns (bit 4k+e: quad k, element e):
// which columns receive the bias, which are zeroed.  Worked out per quad: a
// quad's four columns are consecutive and start at a multiple of 4, and N is
// a multiple of 256, so a TRLWE quad lies wholly in the mask part (columns
// < N) or wholly in the body part.
template <int Q, int TEAM>
__device__ __forceinline__ void column_masks(const ScoreArgs &a, uint32_t c0, uint32_t lane, uint32_t &bias_mask,
                                             uint32_t &zero_mask) {
    bias_mask = 0;
    zero_mask = 0;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const uint32_t c = c0 + 4 * lane + 4 * k * TEAM;  // the quad's first column
        uint32_t b = 0, z = 0;
        if (a.form == kFormTrlwe) {
            if (c >= a.N) {
                const uint32_t j = c - a.N;  // body coefficients j .. j+3
                // coefficients below NUM_SAMPLES take the bias
                if (j < a.num_samples) b = 0xFu >> (4u - min(a.num_samples - j, 4u));
                // coefficients from REGION_SIZE on are zeroed
                if (j + 4u > a.region_size) z = (0xFu << (a.region_size > j ? a.region_size - j : 0u)) & 0xFu;
            }
        } else {
            // LWE: column c+e is a sample's body word when (c+e) % (n+1) == n
            uint32_t r = c % a.lwe_n1;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (r == a.lwe_n1 - 1) b |= 1u << e;
                r = r + 1 == a.lwe_n1 ? 0u : r + 1;
            }
        }
        bias_mask |= b << (4 * k);
        zero_mask |= z << (4 * k);
    }
}

__device__ __forceinline__ void store_quad(uint8_t *row, uint32_t q, uint32_t valid, uint4 v) {
    if (q + 4 <= valid) {
        stg_cs_v4(row + size_t(q) * 4, make_int4(int(v.x), int(v.y), int(v.z), int(v.w)));
    } else {
        uint32_t *p = reinterpret_cast<uint32_t *>(row) + q;
        if (q + 0 < valid) p[0] = v.x;
        if (q + 1 < valid) p[1] = v.y;
        if (q + 2 < valid) p[2] = v.z;
        if (q + 3 < valid) p[3] = v.w;
    }
}

// Accumulators start at the bias on the columns that take it (the bias of
// eval/idash.cpp:805-810 folded in before the terms; addition commutes).
template <int G, int Q>
__device__ __forceinline__ void init_acc(uint32_t (&acc)[G][4 * Q], const PlanGroup &gr, uint32_t bias_mask) {
#pragma unroll
    for (int m = 0; m < G; ++m)
#pragma unroll
        for (int e = 0; e < 4 * Q; ++e) acc[m][e] = 0;
    if (bias_mask) {
#pragma unroll
        for (int m = 0; m < G; ++m)
#pragma unroll
            for (int e = 0; e < 4 * Q; ++e)
                if (bias_mask & (1u << e)) acc[m][e] = uint32_t(gr.bias[m]);
    }
}

template <int Q>
__device__ __forceinline__ constexpr uint32_t all_columns() {
    return (1u << (4 * Q)) - 1u;
}

template <int G, int Q, int TEAM>
__device__ __forceinline__ void write_outputs(const ScoreArgs &a, const PlanGroup &gr, uint32_t (&acc)[G][4 * Q],
                                              uint32_t c0, uint32_t lane, uint32_t valid, uint32_t zero_mask) {
    constexpr uint32_t W = 4 * Q * TEAM;
    // Output ordinals, output rows and the row stride are below 2^32 (the
    // launch checks the stride): 32-bit compares and one wide multiply-add
    // per row address.
    const uint32_t lo = uint32_t(min(a.out_lo, uint64_t(kNoOutput)));
    const uint32_t hi = uint32_t(min(a.out_hi, uint64_t(kNoOutput)));
    uint8_t *const out_c0 = a.out + uint64_t(c0) * 4;
#pragma unroll
    for (int m = 0; m < G; ++m) {
        const uint32_t o = gr.out[m];
        if (o - lo >= hi - lo) continue;  // outside [out_lo, out_hi), kNoOutput included
        if (zero_mask) {
#pragma unroll
            for (int e = 0; e < 4 * Q; ++e)
                if (zero_mask & (1u << e)) acc[m][e] = 0;
        }
        const uint32_t r = a.out_row_map ? a.out_row_map[o] : o - uint32_t(a.out_row_base);
        uint8_t *row = out_c0 + uint64_t(r) * uint32_t(a.out_stride);
        if (a.accumulate) {
            // a later part of a split group: add what the earlier launches
            // wrote (zeroed columns stay zero: both terms are zero there)
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                const uint32_t q = 4 * lane + 4 * k * TEAM;
                if (q + 4 <= valid) {
                    const int4 v = ldg_nc_v4(row + size_t(q) * 4);
                    acc[m][4 * k + 0] += uint32_t(v.x);
                    acc[m][4 * k + 1] += uint32_t(v.y);
                    acc[m][4 * k + 2] += uint32_t(v.z);
                    acc[m][4 * k + 3] += uint32_t(v.w);
                } else {
                    const uint32_t *p = reinterpret_cast<const uint32_t *>(row) + q;
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (q + e < valid) acc[m][4 * k + e] += p[e];
                }
            }
        }
        if (valid >= W) {  // a full slice: every quad is inside the row
#pragma unroll
            for (int k = 0; k < Q; ++k)
                stg_cs_v4(row + size_t(4 * lane + 4 * k * TEAM) * 4,
                          make_int4(int(acc[m][4 * k]), int(acc[m][4 * k + 1]), int(acc[m][4 * k + 2]),
                                    int(acc[m][4 * k + 3])));
            continue;
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const uint32_t q = 4 * lane + 4 * k * TEAM;
            if (q < valid)
                store_quad(row, q, valid,
                           make_uint4(acc[m][4 * k], acc[m][4 * k + 1], acc[m][4 * k + 2], acc[m][4 * k + 3]));
        }
    }
}

// The fused digest: adds the quad hashes (common.cuh) of the words
// write_outputs stored (acc holds the stored values) to `dig`.  A thread's
// quad k starts at word c0 + 4*lane + 4*k*TEAM of its row, a multiple of 4 of
// the output layout (digest_base, the row stride and c0 are), so each quad is
// hashed whole from registers.  When the low word of the slice's first quad
// index leaves room for the slice, every key is that index's key plus a
// constant.
template <int W, int G, int Q, int TEAM>
__device__ __forceinline__ void digest_outputs(const ScoreArgs &a, const PlanGroup &gr,
                                               const uint32_t (&acc)[G][4 * Q], uint32_t c0, uint32_t lane,
                                               uint32_t valid, uint64_t &dig) {
    const uint64_t row_words = a.out_stride / 4;
    const uint32_t lo = uint32_t(min(a.out_lo, uint64_t(kNoOutput)));
    const uint32_t hi = uint32_t(min(a.out_hi, uint64_t(kNoOutput)));
#pragma unroll
    for (int m = 0; m < G; ++m) {
        const uint32_t o = gr.out[m];
        if (o - lo >= hi - lo) continue;  // outside [out_lo, out_hi), kNoOutput included
        const uint32_t r = a.out_row_map ? a.out_row_map[o] : o - uint32_t(a.out_row_base);
        const uint64_t quad0 = (a.digest_base + uint64_t(r) * row_words + c0) / 4;  // the slice's first quad
        if (valid >= W && uint32_t(quad0) <= 0xFFFFFFFFu - uint32_t(W / 4)) {
            const uint32_t key0 = hash_index_key(quad0) + lane * kHashLo;
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                uint32_t h = key0 + uint32_t(k * TEAM) * kHashLo;
#pragma unroll
                for (int e = 0; e < 4; ++e) h = hash_step(h, acc[m][4 * k + e]);
                dig += hash_finish(h);
            }
        } else {
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                const uint32_t q = 4 * lane + 4 * k * TEAM;
                if (q >= valid) continue;
                uint32_t h = hash_index_key(quad0 + q / 4);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (q + e < valid) h = hash_step(h, acc[m][4 * k + e]);
                dig += hash_finish(h);
            }
        }
    }
}

template <int G, int Q>
__device__ __forceinline__ void mac(uint32_t (&acc)[G][4 * Q], const PlanTerm &tm, const uint4 (&x)[Q]) {
    const uint32_t c[3] = {uint32_t(tm.c0), uint32_t(tm.c1), uint32_t(tm.c2)};
#pragma unroll
    for (int m = 0; m < G; ++m)
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            acc[m][4 * k + 0] += c[m] * x[k].x;
            acc[m][4 * k + 1] += c[m] * x[k].y;
            acc[m][4 * k + 2] += c[m] * x[k].z;
            acc[m][4 * k + 3] += c[m] * x[k].w;
        }
}

// One group's accumulation over its terms from the shared-memory window
// (wlane: the thread's first column in slot 0).  The first term initialises
// the accumulators (IMAD with the bias as addend where the thread's columns
// all take it), so no separate zeroing pass; a slice that crosses the edge of
// the biased columns adds the bias per column afterwards (addition commutes
// in Z/2^32).  Columns that the epilogue zeroes skip the arithmetic.
template <int W, int G, int Q, int TEAM>
__device__ __forceinline__ void accumulate_group(uint32_t (&acc)[G][4 * Q], const PlanGroup &gr,
                                                 const PlanTerm *tp, const uint32_t *wlane, uint32_t bias_mask,
                                                 uint32_t zero_mask) {
    constexpr uint32_t kAll = all_columns<Q>();
    const bool all_bias = bias_mask == kAll;
    uint32_t b[G];
#pragma unroll
    for (int m = 0; m < G; ++m) b[m] = all_bias ? uint32_t(gr.bias[m]) : 0u;
    if (gr.n_terms == 0 || zero_mask == kAll) {
#pragma unroll
        for (int m = 0; m < G; ++m)
#pragma unroll
            for (int e = 0; e < 4 * Q; ++e) acc[m][e] = b[m];
    } else {
        // 32-bit shared addresses throughout: a term is {c0, c1, c2, slot},
        // the slot's column slice starts slot * W words into the window.
        const uint32_t wbase = smem_addr(wlane);
        uint32_t taddr = smem_addr(tp);
        {
            const uint4 tv = lds_v4(taddr);
            const uint32_t w = wbase + tv.w * (W * 4);
            uint4 x[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) x[k] = lds_v4(w + 16 * k * TEAM);
            const uint32_t c[3] = {tv.x, tv.y, tv.z};
#pragma unroll
            for (int m = 0; m < G; ++m)
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    acc[m][4 * k + 0] = b[m] + c[m] * x[k].x;
                    acc[m][4 * k + 1] = b[m] + c[m] * x[k].y;
                    acc[m][4 * k + 2] = b[m] + c[m] * x[k].z;
                    acc[m][4 * k + 3] = b[m] + c[m] * x[k].w;
                }
        }
        const uint32_t tend = taddr + 16 * gr.n_terms;
        // terms in flight per thread: two at four quads (measured best there).
        // One quad carries little arithmetic per pair of dependent loads (term,
        // then window), so more terms go in flight: on the uneven LWE form
        // (128-word slices) unroll 2 / 4 / 8 / 16 ran 1.74 / 1.58 / 1.55 / 1.53 s
        constexpr int kUnroll = Q == 1 ? 16 : 2;
#pragma unroll kUnroll
        for (taddr += 16; taddr != tend; taddr += 16) {
            const uint4 tv = lds_v4(taddr);
            const uint32_t w = wbase + tv.w * (W * 4);
            uint4 x[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) x[k] = lds_v4(w + 16 * k * TEAM);
            const uint32_t c[3] = {tv.x, tv.y, tv.z};
#pragma unroll
            for (int m = 0; m < G; ++m)
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    acc[m][4 * k + 0] += c[m] * x[k].x;
                    acc[m][4 * k + 1] += c[m] * x[k].y;
                    acc[m][4 * k + 2] += c[m] * x[k].z;
                    acc[m][4 * k + 3] += c[m] * x[k].w;
                }
        }
    }
    if (bias_mask != 0 && !all_bias) {
#pragma unroll
        for (int m = 0; m < G; ++m)
#pragma unroll
            for (int e = 0; e < 4 * Q; ++e)
                if (bias_mask & (1u << e)) acc[m][e] += uint32_t(gr.bias[m]);
    }
}

// Value of column c (of the 2N-word TRLWE row) of X^(-m) * row:
// (X^(-m) P)[j] = P[j+m] if j+m < N else -P[j+m-N], per polynomial.
__device__ __forceinline__ uint32_t rotated_word(const uint32_t *src, uint32_t c, uint32_t m, uint32_t N) {
    const uint32_t p = c >= N ? 1u : 0u;
    const uint32_t j = c - p * N;
    const uint32_t t = j + m;
    return t < N ? src[p * N + t] : 0u - src[p * N + t - N];
}

template <int W, int G, int Q>
__global__ void __launch_bounds__(kThreads) k_score_window(const ScoreArgs a) {
    constexpr int TEAM = W / (4 * Q);
    constexpr int NTEAMS = kThreads / TEAM;
    static_assert(TEAM >= 32 && kThreads % TEAM == 0, "a team is one or more whole warps");
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *tile_s = reinterpret_cast<uint32_t *>(smem + 8);
    uint32_t *win = reinterpret_cast<uint32_t *>(smem + 128);
    PlanTerm *terms_s = reinterpret_cast<PlanTerm *>(smem + 128 + size_t(a.max_slots) * W * 4);
    PlanGroup *groups_s = reinterpret_cast<PlanGroup *>(terms_s + a.max_terms);

    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    const uint32_t team = tid / TEAM, lane = tid % TEAM;
    uint32_t phase = 0;

    for (;;) {
        if (tid == 0) *tile_s = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const uint32_t tile = *tile_s;
        if (tile >= a.n_tiles) break;
        const uint32_t b = a.block_lo + tile % a.n_blocks;
        const uint32_t slice = tile / a.n_blocks;
        const PlanBlock blk = a.blocks[b];
        const uint32_t c0 = slice * W;
        const uint32_t valid = min(uint32_t(W), a.row_words - c0);
        const uint32_t copy_bytes = ((valid + 3u) & ~3u) * 4u;

        // Producer warp: bulk-copy the block's terms, groups and the
        // unrotated slots' column slices; lane 0 arrives once all lanes
        // registered their transaction bytes.
        if (tid < 32) {
            if (tid == 0) fence_proxy_async_smem();
            __syncwarp();
            const uint32_t n_unrot = uint32_t(blk.n_slots) - blk.n_rot;
            for (uint32_t s = tid; s < n_unrot; s += 32) {
                const PlanSlot sl = a.slots[blk.slot_begin + s];
                if (sl.row - a.row_base >= a.n_rows) {
                    report_error(a.err, kDevBadIndex);
                    continue;
                }
                mbar_expect_tx(bar, copy_bytes);
                bulk_g2s(win + size_t(s) * W, a.in + uint64_t(sl.row - a.row_base) * a.in_stride + uint64_t(c0) * 4, copy_bytes,
                         bar);
            }
            if (tid == 0) {
                if (blk.n_terms) {
                    mbar_expect_tx(bar, blk.n_terms * uint32_t(sizeof(PlanTerm)));
                    bulk_g2s(terms_s, a.terms + blk.term_begin, blk.n_terms * uint32_t(sizeof(PlanTerm)), bar);
                }
                mbar_expect_tx(bar, blk.n_groups * uint32_t(sizeof(PlanGroup)));
                bulk_g2s(groups_s, a.groups + blk.group_begin, blk.n_groups * uint32_t(sizeof(PlanGroup)), bar);
            }
            __syncwarp();
            if (tid == 0) mbar_arrive(bar);
        }
        // Rotated slots (TRLWE with NUM_REGIONS > 1): gathered by all threads.
        if (blk.n_rot) {
            for (uint32_t s = uint32_t(blk.n_slots) - blk.n_rot; s < blk.n_slots; ++s) {
                const PlanSlot sl = a.slots[blk.slot_begin + s];
                if (sl.row - a.row_base >= a.n_rows) continue;
                const uint32_t *src = reinterpret_cast<const uint32_t *>(a.in + uint64_t(sl.row - a.row_base) * a.in_stride);
                for (uint32_t x = tid; x < valid; x += kThreads)
                    win[size_t(s) * W + x] = rotated_word(src, c0 + x, sl.rot, a.N);
            }
        }
        __syncthreads();
        const bool ok = mbar_wait_bounded(bar, phase, a.err);
        if (__syncthreads_or(!ok)) {
            // A copy never completed: wait (bounded) once more so no copy is
            // still writing shared memory when the CTA exits.
            mbar_wait_bounded(bar, phase, nullptr);
            return;
        }
        phase ^= 1u;

        uint32_t bias_mask, zero_mask;
        column_masks<Q, TEAM>(a, c0, lane, bias_mask, zero_mask);
        const uint32_t *wlane = win + 4 * lane;
        for (uint32_t g = team; g < blk.n_groups; g += NTEAMS) {
            const PlanGroup gr = groups_s[g];
            uint32_t acc[G][4 * Q];
            accumulate_group<W, G, Q, TEAM>(acc, gr, terms_s + gr.term_begin, wlane, bias_mask, zero_mask);
            write_outputs<G, Q, TEAM>(a, gr, acc, c0, lane, valid, zero_mask);
        }
        __syncthreads();
    }
}

// Issues the bulk copies of one tile (terms, groups, unrotated slot slices)
// into one buffer; called by warp 0, lane 0 arrives on the buffer's barrier.
template <int W>
__device__ __forceinline__ void issue_tile_loads(const ScoreArgs &a, const PlanBlock &blk, uint32_t c0,
                                                 uint32_t copy_bytes, uint32_t *win, PlanTerm *terms_s,
                                                 PlanGroup *groups_s, uint64_t *bar, uint32_t lane) {
    if (lane == 0) fence_proxy_async_smem();
    __syncwarp();
    const uint32_t n_unrot = uint32_t(blk.n_slots) - blk.n_rot;
    for (uint32_t s = lane; s < n_unrot; s += 32) {
        const PlanSlot sl = a.slots[blk.slot_begin + s];
        if (sl.row - a.row_base >= a.n_rows) {
            report_error(a.err, kDevBadIndex);
            continue;
        }
        mbar_expect_tx(bar, copy_bytes);
        bulk_g2s(win + size_t(s) * W, a.in + uint64_t(sl.row - a.row_base) * a.in_stride + uint64_t(c0) * 4, copy_bytes, bar);
    }
    if (lane == 0) {
        if (blk.n_terms) {
            mbar_expect_tx(bar, blk.n_terms * uint32_t(sizeof(PlanTerm)));
            bulk_g2s(terms_s, a.terms + blk.term_begin, blk.n_terms * uint32_t(sizeof(PlanTerm)), bar);
        }
        mbar_expect_tx(bar, blk.n_groups * uint32_t(sizeof(PlanGroup)));
        bulk_g2s(groups_s, a.groups + blk.group_begin, blk.n_groups * uint32_t(sizeof(PlanGroup)), bar);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(bar);
}

constexpr int kPipeThreads = 512;

// k_score_pipe (batched, double-buffered): one 512-thread CTA per SM; while
// all warps accumulate tile i from one shared-memory buffer, warp 0 has
// already issued the bulk copies of tile i+1 into the other, so the input
// window's load latency hides behind the previous tile's arithmetic.
template <int W, int G, int Q>
__global__ void __launch_bounds__(kPipeThreads, 1) k_score_pipe(const ScoreArgs a) {
    constexpr int TEAM = W / (4 * Q);
    constexpr int NTEAMS = kPipeThreads / TEAM;
    static_assert(TEAM >= 32 && kPipeThreads % TEAM == 0, "a team is one or more whole warps");
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);  // bar[0], bar[1]
    uint32_t *tile_s = reinterpret_cast<uint32_t *>(smem + 16);
    const uint32_t buf_bytes = a.max_slots * W * 4 + a.max_terms * uint32_t(sizeof(PlanTerm)) +
                               a.max_groups * uint32_t(sizeof(PlanGroup));
    const uint32_t terms_off = a.max_slots * W * 4;
    const uint32_t groups_off = terms_off + a.max_terms * uint32_t(sizeof(PlanTerm));
    // buffer i: window at smem+128+i*buf_bytes, then terms, then groups
    auto win_of = [&](uint32_t i) { return reinterpret_cast<uint32_t *>(smem + 128 + i * buf_bytes); };
    auto terms_of = [&](uint32_t i) { return reinterpret_cast<PlanTerm *>(smem + 128 + i * buf_bytes + terms_off); };
    auto groups_of = [&](uint32_t i) {
        return reinterpret_cast<PlanGroup *>(smem + 128 + i * buf_bytes + groups_off);
    };
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        *tile_s = atomicAdd(a.tile_counter, 1u);
    }
    __syncthreads();
    uint32_t cur = *tile_s;
    const uint32_t team = tid / TEAM, lane = tid % TEAM;
    uint32_t phase = 0;  // bit i: parity of the next completion of bar[i]
    auto tile_geom = [&](uint32_t tile, PlanBlock &blk, uint32_t &c0, uint32_t &valid) {
        blk = a.blocks[a.block_lo + tile % a.n_blocks];
        c0 = (tile / a.n_blocks) * W;
        valid = min(uint32_t(W), a.row_words - c0);
    };
    if (cur < a.n_tiles && tid < 32) {
        PlanBlock blk;
        uint32_t c0, valid;
        tile_geom(cur, blk, c0, valid);
        issue_tile_loads<W>(a, blk, c0, ((valid + 3u) & ~3u) * 4u, win_of(0), terms_of(0), groups_of(0), &bar[0], tid);
    }
    for (uint32_t i = 0; cur < a.n_tiles; ++i) {
        const uint32_t b = i & 1u;
        __syncthreads();  // every thread is done with buffer b^1 (tile i-1) and has read *tile_s
        if (tid == 0) *tile_s = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const uint32_t nxt = *tile_s;
        if (nxt < a.n_tiles && tid < 32) {
            PlanBlock nb;
            uint32_t n0, nvalid;
            tile_geom(nxt, nb, n0, nvalid);
            issue_tile_loads<W>(a, nb, n0, ((nvalid + 3u) & ~3u) * 4u, win_of(b ^ 1u), terms_of(b ^ 1u),
                                groups_of(b ^ 1u), &bar[b ^ 1u], tid);
        }
        PlanBlock blk;
        uint32_t c0, valid;
        tile_geom(cur, blk, c0, valid);
        uint32_t *win = win_of(b);
        if (blk.n_rot) {
            for (uint32_t s = uint32_t(blk.n_slots) - blk.n_rot; s < blk.n_slots; ++s) {
                const PlanSlot sl = a.slots[blk.slot_begin + s];
                if (sl.row - a.row_base >= a.n_rows) continue;
                const uint32_t *src = reinterpret_cast<const uint32_t *>(a.in + uint64_t(sl.row - a.row_base) * a.in_stride);
                for (uint32_t x = tid; x < valid; x += kPipeThreads)
                    win[size_t(s) * W + x] = rotated_word(src, c0 + x, sl.rot, a.N);
            }
            __syncthreads();
        }
        const bool ok = mbar_wait_bounded(&bar[b], (phase >> b) & 1u, a.err);
        if (__syncthreads_or(!ok)) {
            // drain: every copy this CTA issued must land before it exits
            mbar_wait_bounded(&bar[b], (phase >> b) & 1u, nullptr);
            if (nxt < a.n_tiles) mbar_wait_bounded(&bar[b ^ 1u], (phase >> (b ^ 1u)) & 1u, nullptr);
            return;
        }
        phase ^= 1u << b;

        uint32_t bias_mask, zero_mask;
        column_masks<Q, TEAM>(a, c0, lane, bias_mask, zero_mask);
        const uint32_t *wlane = win + 4 * lane;
        const PlanTerm *terms_s = terms_of(b);
        const PlanGroup *groups_s = groups_of(b);
        for (uint32_t g = team; g < blk.n_groups; g += NTEAMS) {
            const PlanGroup gr = groups_s[g];
            uint32_t acc[G][4 * Q];
            accumulate_group<W, G, Q, TEAM>(acc, gr, terms_s + gr.term_begin, wlane, bias_mask, zero_mask);
            write_outputs<G, Q, TEAM>(a, gr, acc, c0, lane, valid, zero_mask);
        }
        cur = nxt;
    }
}

constexpr int kWsConsumers = 15;                     // consumer warps per CTA (512 threads: 128 registers each)
constexpr int kWsThreads = (kWsConsumers + 1) * 32;  // + one producer warp
constexpr uint32_t kWsMaxStages = 4;

// Per-stage header written by the producer before it signals the stage full.
struct WsStageHeader {
    PlanBlock blk;       // the tile's block
    uint32_t tile;       // tile index, >= n_tiles marks the end of work
    uint32_t next_unit;  // work counter: consumers take (group, part) units from it
    uint32_t job;        // multi-job launches: the tile's job
    uint32_t pad[5];
};

// Multi-job launches: the job of launch tile `tile` (the last job whose
// tiles begin at or before it).
__device__ __forceinline__ uint32_t job_of(const ScoreArgs &a, uint32_t tile) {
    uint32_t lo = 0, hi = a.n_jobs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (a.jobs[mid].tile_begin <= tile) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The launch arguments as one job sees them; `tile` becomes the job's own
// tile index.
__device__ __forceinline__ void with_job(ScoreArgs &a, const ScoreJob &j, uint32_t &tile) {
    tile -= j.tile_begin;
    a.in = j.in;
    a.out = j.out;
    a.digest = j.digest;
    a.out_lo = j.out_lo;
    a.out_hi = j.out_hi;
    a.out_row_base = j.out_row_base;
    a.digest_base = j.digest_base;
    a.in_stride = j.stride;
    a.out_stride = j.stride;
    a.block_lo = j.block_lo;
    a.n_blocks = j.n_blocks;
    a.row_base = j.row_base;
    a.n_rows = j.n_rows;
    a.row_words = j.row_words;
    a.num_samples = j.num_samples;
}
static_assert(sizeof(WsStageHeader) == 64, "stage header layout");
static_assert(2 * kWsMaxStages * 8 + kWsMaxStages * sizeof(WsStageHeader) <= kWsHeaderBytes,
              "barriers and stage headers fit the header area");

// k_score_ws (batched, warp-specialised): one CTA of 1 producer + 15 consumer
// warps per SM.  The producer fills a ring of shared-memory stages (window +
// terms + groups, with the tile's block header) by bulk copies and signals
// `full[s]`.  Consumer warps take work units - one group's columns handled by
// one warp (a TEAM / 32 part of the group's slice) - from the stage's shared
// counter, so uneven groups balance across warps; a warp that runs out of
// units arrives on `empty[s]` and moves on to the next stage.  No CTA-wide
// barrier: the next stages' copies overlap this stage's arithmetic.
//
// DIG: the instance that also takes the serving digest of what it writes
// (ScoreArgs::digest); one atomic add per consumer warp at the end.
template <int W, int G, int Q, bool DIG>
__global__ void __launch_bounds__(kWsThreads, 1) k_score_ws(const ScoreArgs a) {
    constexpr int TEAM = W / (4 * Q);
    constexpr int PARTS = TEAM / 32;  // warps per group-slice
    static_assert(TEAM >= 32 && TEAM % 32 == 0, "a team is one or more whole warps");
    extern __shared__ __align__(128) uint8_t smem[];
    const uint32_t n_stages = a.n_stages;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem);   // [kWsMaxStages]
    uint64_t *empty = full + kWsMaxStages;                  // [kWsMaxStages]
    WsStageHeader *hdr = reinterpret_cast<WsStageHeader *>(smem + 2 * kWsMaxStages * 8);
    const uint32_t buf_bytes = a.max_slots * W * 4 + a.max_terms * uint32_t(sizeof(PlanTerm)) +
                               a.max_groups * uint32_t(sizeof(PlanGroup));
    const uint32_t terms_off = a.max_slots * W * 4;
    const uint32_t groups_off = terms_off + a.max_terms * uint32_t(sizeof(PlanTerm));
    auto win_of = [&](uint32_t s) { return reinterpret_cast<uint32_t *>(smem + kWsHeaderBytes + s * buf_bytes); };
    auto terms_of = [&](uint32_t s) {
        return reinterpret_cast<PlanTerm *>(smem + kWsHeaderBytes + s * buf_bytes + terms_off);
    };
    auto groups_of = [&](uint32_t s) {
        return reinterpret_cast<PlanGroup *>(smem + kWsHeaderBytes + s * buf_bytes + groups_off);
    };
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < n_stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kWsConsumers);
        }
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == kWsConsumers) {
        // ------------------------------------------------------------ producer
        uint32_t pending = 0;  // stages with copies not yet consumed
        uint32_t it = 0;
        uint32_t tile = 0;
        uint32_t job = 0;  // multi-job launches: the job of the last tile
        if (lane == 0) tile = atomicAdd(a.tile_counter, 1u);
        tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
        for (;; ++it) {
            const uint32_t s = it % n_stages, round = it / n_stages;
            if (round > 0) {
                bool ok = true;
                if (lane == 0) ok = mbar_wait_bounded(&empty[s], (round - 1) & 1u, a.err);
                ok = __shfl_sync(0xFFFFFFFFu, ok ? 1 : 0, 0) != 0;
                if (!ok) break;
                pending &= ~(1u << s);
            }
            if (tile >= a.n_tiles) {
                if (lane == 0) {
                    hdr[s].tile = tile;
                    mbar_arrive(&full[s]);  // end-of-work marker
                }
                return;
            }
            ScoreArgs aj = a;
            uint32_t lt = tile;
            if (DIG && a.n_jobs) {
                // a CTA's tiles come from one counter in increasing order, so
                // its job index only moves forward
                if (a.jobs[job].tile_begin > tile) job = job_of(a, tile);
                while (job + 1 < a.n_jobs && a.jobs[job + 1].tile_begin <= tile) ++job;
                with_job(aj, a.jobs[job], lt);
            }
            const PlanBlock blk = aj.blocks[aj.block_lo + lt % aj.n_blocks];
            const uint32_t c0 = (lt / aj.n_blocks) * W;
            const uint32_t valid = min(uint32_t(W), aj.row_words - c0);
            if (lane == 0) {
                hdr[s].blk = blk;
                hdr[s].tile = tile;
                hdr[s].next_unit = 0;
                hdr[s].job = job;
            }
            uint32_t *win = win_of(s);
            // rotated slots (NUM_REGIONS > 1): gathered by the producer lanes
            for (uint32_t sl_i = uint32_t(blk.n_slots) - blk.n_rot; sl_i < blk.n_slots; ++sl_i) {
                const PlanSlot sl = aj.slots[blk.slot_begin + sl_i];
                if (sl.row - aj.row_base >= aj.n_rows) continue;
                const uint32_t *src =
                    reinterpret_cast<const uint32_t *>(aj.in + uint64_t(sl.row - aj.row_base) * aj.in_stride);
                for (uint32_t x = lane; x < valid; x += 32)
                    win[size_t(sl_i) * W + x] = rotated_word(src, c0 + x, sl.rot, aj.N);
            }
            issue_tile_loads<W>(aj, blk, c0, ((valid + 3u) & ~3u) * 4u, win, terms_of(s), groups_of(s), &full[s],
                                lane);
            pending |= 1u << s;
            // the next tile's index, fetched while this stage's copies fly
            if (lane == 0) tile = atomicAdd(a.tile_counter, 1u);
            tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
        }
        // A wait expired: let every copy this CTA issued land before exiting.
        // The last n_stages iterations issued each stage's newest copies.
        for (uint32_t k = 1; k <= n_stages && k <= it; ++k) {
            const uint32_t j = it - k, sj = j % n_stages;
            if (((pending >> sj) & 1u) && lane == 0) mbar_wait_bounded(&full[sj], (j / n_stages) & 1u, nullptr);
        }
        return;
    }

    // --------------------------------------------------------------- consumers
    uint64_t dig = 0;                                 // DIG only
    unsigned long long *dig_to = a.n_jobs ? nullptr : a.digest;  // where dig goes
    auto flush_digest = [&]() {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) dig += __shfl_xor_sync(0xFFFFFFFFu, dig, off);
        if (lane == 0 && dig && dig_to) atomicAdd(dig_to, (unsigned long long)dig);
        dig = 0;
    };
    for (uint32_t it = 0;; ++it) {
        const uint32_t s = it % n_stages, round = it / n_stages;
        if (!mbar_wait_bounded(&full[s], round & 1u, a.err)) return;
        const uint32_t tile = hdr[s].tile;
        if (tile >= a.n_tiles) {
            if (DIG) flush_digest();
            return;
        }
        ScoreArgs aj = a;
        uint32_t lt = tile;
        if (DIG && a.n_jobs) {
            with_job(aj, a.jobs[hdr[s].job], lt);
            if (DIG && aj.digest != dig_to) {  // a new job: the last one's digest is complete here
                flush_digest();
                dig_to = aj.digest;
            }
        }
        const PlanBlock blk = hdr[s].blk;
        const uint32_t c0 = (lt / aj.n_blocks) * W;
        const uint32_t valid = min(uint32_t(W), aj.row_words - c0);
        uint32_t bmask[PARTS], zmask[PARTS];
#pragma unroll
        for (int p = 0; p < PARTS; ++p) column_masks<Q, TEAM>(aj, c0, 32 * p + lane, bmask[p], zmask[p]);
        const PlanTerm *terms_s = terms_of(s);
        const PlanGroup *groups_s = groups_of(s);
        const uint32_t n_units = blk.n_groups * PARTS;
        uint32_t *next_unit = &hdr[s].next_unit;
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(next_unit, 1u);
        u = __shfl_sync(0xFFFFFFFFu, u, 0);
        while (u < n_units) {
            uint32_t u_next = 0;  // taken now, its latency hides behind this unit
            if (lane == 0) u_next = atomicAdd(next_unit, 1u);
            const uint32_t g = u / PARTS, part = u % PARTS;
            const uint32_t tlane = 32 * part + lane;
            uint32_t bias_mask = bmask[0], zero_mask = zmask[0];
#pragma unroll
            for (int p = 1; p < PARTS; ++p)
                if (part == uint32_t(p)) {
                    bias_mask = bmask[p];
                    zero_mask = zmask[p];
                }
            const PlanGroup gr = groups_s[g];
            uint32_t acc[G][4 * Q];
            accumulate_group<W, G, Q, TEAM>(acc, gr, terms_s + gr.term_begin, win_of(s) + 4 * tlane, bias_mask,
                                            zero_mask);
            write_outputs<G, Q, TEAM>(aj, gr, acc, c0, tlane, valid, zero_mask);
            if (DIG && dig_to) digest_outputs<W, G, Q, TEAM>(aj, gr, acc, c0, tlane, valid, dig);
            u = __shfl_sync(0xFFFFFFFFu, u_next, 0);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

template <int W, int G, int Q>
__global__ void __launch_bounds__(kThreads) k_score_direct(const ScoreArgs a) {
    constexpr int TEAM = W / (4 * Q);
    constexpr int NTEAMS = kThreads / TEAM;
    const uint32_t tid = threadIdx.x;
    const uint32_t team = tid / TEAM, lane = tid % TEAM;
    const uint32_t tile = blockIdx.x;
    if (tile >= a.n_tiles) return;
    const uint32_t b = a.block_lo + tile % a.n_blocks;
    const uint32_t slice = tile / a.n_blocks;
    const PlanBlock blk = a.blocks[b];
    const uint32_t c0 = slice * W;
    const uint32_t valid = min(uint32_t(W), a.row_words - c0);
    const uint32_t vpad = (valid + 3u) & ~3u;

    uint32_t bias_mask, zero_mask;
    column_masks<Q, TEAM>(a, c0, lane, bias_mask, zero_mask);
    for (uint32_t g = team; g < blk.n_groups; g += NTEAMS) {
        const PlanGroup gr = a.groups[blk.group_begin + g];
        uint32_t acc[G][4 * Q];
        init_acc<G, Q>(acc, gr, bias_mask);
        const PlanTerm *tp = a.terms + blk.term_begin + gr.term_begin;
        for (uint32_t t = 0; t < gr.n_terms; ++t) {
            const PlanTerm tm = tp[t];
            const PlanSlot sl = a.slots[blk.slot_begin + tm.slot];
            if (sl.row - a.row_base >= a.n_rows) {
                report_error(a.err, kDevBadIndex);
                continue;
            }
            const uint8_t *src = a.in + uint64_t(sl.row - a.row_base) * a.in_stride;
            uint4 x[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                const uint32_t q = 4 * lane + 4 * k * TEAM;
                x[k] = make_uint4(0, 0, 0, 0);
                if (sl.rot == 0) {
                    if (q < vpad) {
                        const int4 v = ldg_nc_v4(src + (uint64_t(c0) + q) * 4);
                        x[k] = make_uint4(uint32_t(v.x), uint32_t(v.y), uint32_t(v.z), uint32_t(v.w));
                    }
                } else {
                    const uint32_t *s32 = reinterpret_cast<const uint32_t *>(src);
                    x[k].x = q + 0 < valid ? rotated_word(s32, c0 + q + 0, sl.rot, a.N) : 0u;
                    x[k].y = q + 1 < valid ? rotated_word(s32, c0 + q + 1, sl.rot, a.N) : 0u;
                    x[k].z = q + 2 < valid ? rotated_word(s32, c0 + q + 2, sl.rot, a.N) : 0u;
                    x[k].w = q + 3 < valid ? rotated_word(s32, c0 + q + 3, sl.rot, a.N) : 0u;
                }
            }
            mac<G, Q>(acc, tm, x);
        }
        write_outputs<G, Q, TEAM>(a, gr, acc, c0, lane, valid, zero_mask);
    }
}

__global__ void k_finalize(const FinalizeArgs a) {
    const uint64_t o = a.o_begin + uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (o >= a.o_end) return;
    uint8_t *row = a.out_rows + (a.out_row_map ? uint64_t(a.out_row_map[o]) : o - a.out_row_base) * a.out_stride;
    if (a.out_hdr_off >= 0) {
        *reinterpret_cast<uint32_t *>(row + a.out_hdr_off) = a.out_index ? a.out_index[o] : uint32_t(o);
        *reinterpret_cast<int32_t *>(row + a.out_hdr_off + 4) = a.tag;
    }
    if (a.out_var_off >= 0) {
        // TFHE bookkeeping of tLweAddMulTo: variance += coef^2 * var_in, in
        // CSR order, without contraction (matches the host's rounding).
        double v = 0.0;
        if (a.in_var_off >= 0) {
            for (uint64_t t = a.var_ptr[o]; t < a.var_ptr[o + 1]; ++t) {
                const int64_t c = a.var_coef[t];
                const double vin =
                    *reinterpret_cast<const double *>(a.in_rows + uint64_t(a.var_row[t] - a.in_row_base) * a.in_stride +
                                                      a.in_var_off);
                v = __dadd_rn(v, __dmul_rn(double(c * c), vin));
            }
        }
        *reinterpret_cast<double *>(row + a.out_var_off) = v;
    }
}

using KernelFn = void (*)(const ScoreArgs);

// Columns per thread: 16 (4 quads) from 512-word slices up, 8 at 256 and 4 at
// 128 (a team is always whole warps); the direct kernel keeps 8 (4 at 128)
// so that each output has a full CTA of loads in flight.
template <int G>
KernelFn pick(KernelKind kind, uint32_t w) {
    switch (kind) {
        case KernelKind::kWindow:
            switch (w) {
                case 128: return k_score_window<128, G, 1>;
                case 256: return k_score_window<256, G, 2>;
                case 512: return k_score_window<512, G, 4>;
                case 1024: return k_score_window<1024, G, 4>;
                case 2048: return k_score_window<2048, G, 4>;
            }
            break;
        case KernelKind::kPipe:
            switch (w) {
                case 128: return k_score_pipe<128, G, 1>;
                case 256: return k_score_pipe<256, G, 2>;
                case 512: return k_score_pipe<512, G, 4>;
                case 1024: return k_score_pipe<1024, G, 4>;
                case 2048: return k_score_pipe<2048, G, 4>;
            }
            break;
        case KernelKind::kWs:
            switch (w) {
                case 128: return k_score_ws<128, G, 1, false>;
                case 256: return k_score_ws<256, G, 2, false>;
                case 512: return k_score_ws<512, G, 4, false>;
                case 1024: return k_score_ws<1024, G, 4, false>;
                case 2048: return k_score_ws<2048, G, 4, false>;
            }
            break;
        case KernelKind::kDirect:
            switch (w) {
                case 128: return k_score_direct<128, G, 1>;
                case 256: return k_score_direct<256, G, 2>;
                case 512: return k_score_direct<512, G, 2>;
                case 1024: return k_score_direct<1024, G, 2>;
                case 2048: return k_score_direct<2048, G, 2>;
            }
            break;
    }
    return nullptr;
}

KernelFn pick_kernel(KernelKind kind, uint32_t w, uint32_t g) {
    return g == 1 ? pick<1>(kind, w) : g == 3 ? pick<3>(kind, w) : nullptr;
}

// The fused-digest instances: the warp-specialised kernel, groups of 3.
KernelFn pick_digest(KernelKind kind, uint32_t w, uint32_t g) {
    if (kind != KernelKind::kWs || g != 3) return nullptr;
    switch (w) {
        case 128: return k_score_ws<128, 3, 1, true>;
        case 256: return k_score_ws<256, 3, 2, true>;
        case 512: return k_score_ws<512, 3, 4, true>;
        case 1024: return k_score_ws<1024, 3, 4, true>;
        case 2048: return k_score_ws<2048, 3, 4, true>;
    }
    return nullptr;
}

uint32_t threads_of(KernelKind kind) {
    return kind == KernelKind::kPipe ? kPipeThreads : kind == KernelKind::kWs ? kWsThreads : kThreads;
}

}  // namespace

bool digest_fusable(KernelKind kind, uint32_t w, uint32_t g) { return pick_digest(kind, w, g) != nullptr; }

bool slice_supported(uint32_t w) { return w == 128 || w == 256 || w == 512 || w == 1024 || w == 2048; }

size_t buffer_bytes(uint32_t slice_words, uint32_t max_slots, uint32_t max_terms, uint32_t max_groups) {
    return size_t(max_slots) * slice_words * 4 + size_t(max_terms) * sizeof(PlanTerm) +
           size_t(max_groups) * sizeof(PlanGroup);
}

size_t kernel_smem_bytes(KernelKind kind, uint32_t slice_words, uint32_t max_slots, uint32_t max_terms,
                         uint32_t max_groups, uint32_t n_stages) {
    const size_t buf = buffer_bytes(slice_words, max_slots, max_terms, max_groups);
    switch (kind) {
        case KernelKind::kWindow: return 128 + buf;
        case KernelKind::kPipe: return 128 + 2 * buf;
        case KernelKind::kWs: return kWsHeaderBytes + size_t(n_stages) * buf;
        default: return 0;
    }
}

cudaError_t configure_window_kernels(size_t max_smem) {
    for (KernelKind kind : {KernelKind::kWindow, KernelKind::kPipe, KernelKind::kWs})
        for (uint32_t w : {128u, 256u, 512u, 1024u, 2048u})
            for (uint32_t g : {1u, 3u}) {
                for (KernelFn fn : {pick_kernel(kind, w, g), pick_digest(kind, w, g)}) {
                    if (!fn) continue;
                    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(max_smem));
                    if (e != cudaSuccess) return e;
                }
            }
    return cudaSuccess;
}

int resident_ctas_per_sm(KernelKind kind, uint32_t slice_words, uint32_t group_size, size_t smem_bytes) {
    KernelFn fn = pick_kernel(kind, slice_words, group_size);
    if (!fn || kind == KernelKind::kDirect) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, int(threads_of(kind)), smem_bytes) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_score(KernelKind kind, uint32_t slice_words, uint32_t group_size, const ScoreArgs &a,
                         uint32_t ctas, cudaStream_t stream) {
    // job tables run on the fused-digest instances (a job without a digest
    // pointer takes none)
    const bool dig = a.digest || a.n_jobs;
    KernelFn fn = dig ? pick_digest(kind, slice_words, group_size) : pick_kernel(kind, slice_words, group_size);
    if (!fn || (dig && a.accumulate) || (a.n_jobs && kind != KernelKind::kWs)) return cudaErrorInvalidValue;
    if (a.out_stride > 0xFFFFFFFFull) return cudaErrorInvalidValue;  // write_outputs' 32-bit row addressing
    if (a.n_tiles == 0) return cudaSuccess;
    if (kind == KernelKind::kDirect) {
        fn<<<a.n_tiles, kThreads, 0, stream>>>(a);
    } else {
        if (kind == KernelKind::kWs && (a.n_stages < 2 || a.n_stages > kWsMaxStages)) return cudaErrorInvalidValue;
        const size_t smem = kernel_smem_bytes(kind, slice_words, a.max_slots, a.max_terms, a.max_groups, a.n_stages);
        cudaError_t e = cudaMemsetAsync(a.tile_counter, 0, sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
        fn<<<ctas < a.n_tiles ? ctas : a.n_tiles, threads_of(kind), smem, stream>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_finalize(const FinalizeArgs &a, cudaStream_t stream) {
    if (a.o_end <= a.o_begin || (a.out_var_off < 0 && a.out_hdr_off < 0)) return cudaSuccess;
    const uint32_t threads = 256;
    const uint64_t blocks = (a.o_end - a.o_begin + threads - 1) / threads;
    k_finalize<<<uint32_t(blocks), threads, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace idash
