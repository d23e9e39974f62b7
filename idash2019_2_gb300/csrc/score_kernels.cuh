// Launch-side view of the scoring kernels (score_kernels.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_status.hpp"
#include "plan.hpp"

namespace idash {

enum : uint32_t { kFormTrlwe = 0, kFormLwe = 1 };

// One job of a multi-job launch (the warp-specialised kernel): a range of
// plan blocks scored from its own input buffer into its own output buffer,
// e.g. one block of individuals of one serving request.  Its tiles are
// [tile_begin, tile_begin + n_blocks * n_slices) of the launch, block-major
// within a slice as in a single-job launch.
struct ScoreJob {
    const uint8_t *in;           // coefficient 0 of the input row holding plan row row_base
    uint8_t *out;                // coefficient 0 of output row 0 (output out_row_base)
    unsigned long long *digest;  // the job's digest (null: none)
    uint64_t out_lo, out_hi;     // outputs written: [out_lo, out_hi)
    uint64_t out_row_base;
    uint64_t digest_base;
    uint64_t stride;             // bytes between rows, inputs and outputs
    uint32_t block_lo, n_blocks;
    uint32_t row_base, n_rows;
    uint32_t row_words, num_samples;
    uint32_t tile_begin, n_slices;
};

struct ScoreArgs {
    const PlanBlock *blocks;
    const PlanSlot *slots;
    const PlanGroup *groups;
    const PlanTerm *terms;
    uint32_t block_lo, n_blocks;  // blocks [block_lo, block_lo + n_blocks)
    uint32_t n_slices;            // column slices per row
    uint32_t row_words;           // valid int32 words per row
    uint32_t n_tiles;             // n_blocks * n_slices
    uint32_t n_rows;              // input rows held at `in` (bounds guard)
    uint32_t row_base;            // plan row r is held at row (r - row_base) of `in`
    const uint8_t *in;            // coefficient 0 of input row 0
    uint64_t in_stride;           // bytes
    uint8_t *out;                 // coefficient 0 of output row 0
    uint64_t out_stride;          // bytes
    uint64_t out_lo, out_hi;      // outputs written: [out_lo, out_hi)
    uint64_t out_row_base;        // output o goes to row (o - out_row_base) ...
    const uint32_t *out_row_map;  // ... or to row out_row_map[o] when non-null
    uint32_t form;                // kFormTrlwe / kFormLwe
    uint32_t N, num_samples, region_size;  // TRLWE epilogue
    uint32_t lwe_n1;                       // LWE: n + 1 words per sample
    uint32_t max_slots, max_terms, max_groups;  // shared-memory carve-up (one buffer)
    uint32_t n_stages;                          // warp-specialised kernel: buffers in the ring
    uint32_t accumulate;          // 1: add to the outputs (later parts of split groups)
    uint32_t *tile_counter;       // persistent kernel: next tile (zeroed before launch)
    uint32_t *err;                // device error word
    // k_score_ws with the fused digest only (null otherwise): the digest of
    // the words written (the quad hashes of common.cuh), word (r, c) at
    // global index digest_base + r * out_stride / 4 + c, is added to *digest.
    unsigned long long *digest;
    uint64_t digest_base;         // a multiple of 4
    // KernelKind::kTc only.  tc_a: per block, the coefficient digits in the
    // MMA's shared-memory layout (PlanBlock::group_begin is the block's
    // offset in 16-byte units, PlanBlock::n_groups its padded K); tc_bias:
    // every output's bias.  Work unit u covers column slices
    // [(u % units_per_block) * unit_slices, + unit_slices) of block
    // block_lo + u / units_per_block.
    const uint8_t *tc_a;
    const uint32_t *tc_bias;
    uint32_t unit_slices, units_per_block, n_units;
    uint32_t tc_a_max_bytes;      // shared-memory room for one block's digits
    uint32_t tc_use_map;          // set by the launch: consecutive-row chunks come by 2D tensor copy
    // Multi-job launches (KernelKind::kWs only): n_jobs > 0 replaces the
    // per-launch input, output, row window, columns, bias rows and digest by
    // the job of each tile; jobs sorted by tile_begin, n_tiles their total.
    // They run on the fused-digest instance (a job whose digest pointer is
    // null takes none), so the plain instance carries no per-job state.
    const ScoreJob *jobs;
    uint32_t n_jobs;
};

// kWindow: persistent, 256 threads, one shared-memory buffer, 1-2 CTAs/SM.
// kDirect: one CTA per tile, inputs read from global memory (plain form).
// kPipe:   persistent, 512 threads, two buffers (next tile loads while the
//          current one computes), one CTA per SM.
// kWs:     persistent, warp-specialised: one CTA of 1 producer + 15 consumer
//          warps per SM over a ring of n_stages buffers handed over with
//          mbarriers; consumers take (group, part) units from a shared counter.
// kTc:     persistent, tensor cores (tcgen05.mma, fp16 digits, fp32
//          accumulators in TMEM): one CTA per SM; blocks of up to 128
//          outputs x 64-column slices (score_tc.cu).
enum class KernelKind : int { kWindow = 0, kDirect = 1, kPipe = 2, kWs = 3, kTc = 4 };
constexpr uint32_t kTcSliceWords = 64;  // columns per tensor-core tile (the MMA's N)
constexpr uint32_t kMaxStages = 4;
constexpr uint32_t kWsHeaderBytes = 512;  // kWs: barriers + per-stage headers before the ring

// Slice widths the kernels are instantiated for.
bool slice_supported(uint32_t slice_words);

// One shared-memory buffer (window + terms + groups) for the given limits.
size_t buffer_bytes(uint32_t slice_words, uint32_t max_slots, uint32_t max_terms, uint32_t max_groups);
// Dynamic shared memory of one CTA of `kind` (0 for the direct kernel);
// n_stages counts the kWs ring's buffers.
size_t kernel_smem_bytes(KernelKind kind, uint32_t slice_words, uint32_t max_slots, uint32_t max_terms,
                         uint32_t max_groups, uint32_t n_stages = 1);
inline size_t window_smem_bytes(uint32_t slice_words, uint32_t max_slots, uint32_t max_terms, uint32_t max_groups) {
    return kernel_smem_bytes(KernelKind::kWindow, slice_words, max_slots, max_terms, max_groups);
}

// Whether the kernel kind can take the fused digest (ScoreArgs::digest).
bool digest_fusable(KernelKind kind, uint32_t slice_words, uint32_t group_size);

// Launches one scoring kernel.  `ctas` is the persistent grid size (window
// and pipe kernels) and is ignored by the direct kernel (one CTA per tile).
cudaError_t launch_score(KernelKind kind, uint32_t slice_words, uint32_t group_size, const ScoreArgs &a,
                         uint32_t ctas, cudaStream_t stream);

// Allows every persistent kernel instance up to `max_smem` bytes of dynamic
// shared memory (once per device, before any launch or capture).
cudaError_t configure_window_kernels(size_t max_smem);

// Largest resident CTA count per SM for a persistent kernel at this smem size.
int resident_ctas_per_sm(KernelKind kind, uint32_t slice_words, uint32_t group_size, size_t smem_bytes);
inline int window_ctas_per_sm(uint32_t slice_words, uint32_t group_size, size_t smem_bytes) {
    return resident_ctas_per_sm(KernelKind::kWindow, slice_words, group_size, smem_bytes);
}

struct FinalizeArgs {
    const uint64_t *var_ptr;
    const uint32_t *var_row;
    const int32_t *var_coef;
    const uint32_t *out_index;  // may be null: index = o
    const uint32_t *out_row_map;  // may be null: row = o
    uint64_t o_begin, o_end;    // outputs finalised: [o_begin, o_end)
    const uint8_t *in_rows;     // input row 0 start (record start, not payload)
    uint32_t in_row_base;       // plan row r is at row (r - in_row_base) of in_rows
    uint64_t in_stride;
    int64_t in_var_off;         // -1: inputs carry no variance (outputs get 0)
    uint8_t *out_rows;          // output row 0 start
    uint64_t out_row_base;      // without a map, output o is row (o - out_row_base)
    uint64_t out_stride;
    int64_t out_var_off, out_hdr_off;
    int32_t tag;
};
cudaError_t launch_finalize(const FinalizeArgs &a, cudaStream_t stream);

// Tensor-core kernel (score_tc.cu): dynamic shared memory for a plan whose
// largest padded K is max_k_pad, its launch (grid = ctas, one per SM at
// most), and the one-off shared-memory attribute.
size_t tc_smem_bytes(uint32_t max_k_pad);
cudaError_t launch_score_tc(const ScoreArgs &a, uint32_t ctas, cudaStream_t stream);
cudaError_t configure_tc_kernel(size_t max_smem);

}  // namespace idash
