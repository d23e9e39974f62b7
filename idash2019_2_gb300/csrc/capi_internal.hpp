// Internal state behind the C ABI (include/idash_gpu.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <set>
#include <string>
#include <vector>

#include "../../include/idash_gpu.h"
#include "plan.hpp"
#include "score_kernels.cuh"

namespace idash {
struct IntpolyModel;  // integer-polynomial form (intpoly.cu)
// Synthetic TRLWE rows [row_begin, row_end) of the generator behind
// idash_synth_trlwe_device, written to d_out (row row_begin at d_out).
cudaError_t synth_trlwe_rows(uint64_t seed, const idash_trlwe_params &p, uint64_t n_features, uint64_t row_begin,
                             uint64_t row_end, uint8_t *d_out, const idash_row_layout &layout, cudaStream_t s);
// Uniformly random rows [row_begin, row_begin + n_rows) of row_words words
// (as idash_synth_uniform_device), row row_begin at d_out.
cudaError_t fill_uniform_rows(uint64_t seed, uint64_t row_begin, uint64_t n_rows, uint32_t row_words, uint8_t *d_out,
                              uint64_t row_stride, int sm_count, cudaStream_t s);
// Adds to *d_digest the order-independent digest of n_words output words at
// global word indices index_base + i (the quad hashes of common.cuh).
cudaError_t digest_words(const uint32_t *words, uint64_t n_words, uint64_t index_base, uint64_t *d_digest,
                         int sm_count, cudaStream_t s);
uint64_t digest_host(const uint32_t *words, uint64_t n_words, uint64_t index_base);
// idash_score_trlwe_range that can also take the digest of the outputs it
// writes, added to *digest (the one of digest_words over the output image,
// with index_base = digest_base).  *fused tells whether it did; when not,
// the caller digests the outputs itself.
idash_status score_trlwe_range(idash_model *m, uint64_t out_begin, uint64_t out_end, uint32_t num_samples,
                               const void *d_in, const idash_row_layout *il, uint64_t in_row_base, uint64_t n_in_rows,
                               void *d_out, const idash_row_layout *ol, void *stream, uint64_t *digest,
                               uint64_t digest_base, bool *fused);

// The nonzero coefficients of an integer key polynomial (positions, values),
// staged on the device for launches on `s` and released stream-ordered after
// them, so concurrent calls with different keys never share a buffer.
struct StagedKey {
    uint32_t *idx = nullptr;
    int32_t *val = nullptr;
    uint32_t n_nz = 0;
    bool binary = true;  // every nonzero coefficient is 1
    void *buf = nullptr;
};
cudaError_t stage_key(const int32_t *key, uint32_t N, cudaStream_t s, StagedKey *out);
void release_key(StagedKey *k, cudaStream_t s);
}  // namespace idash

// Message returned by idash_last_error(NULL) on this thread (entry points
// that have no context: idash_open failures, idash_score_trlwe_noalloc).
void idash_set_thread_error(const std::string &msg);

struct idash_ctx {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;  // max dynamic shared memory per CTA
    cudaStream_t stream = nullptr, h2d = nullptr, d2h = nullptr;
    cudaEvent_t join_in = nullptr, join_out = nullptr;
    uint32_t *d_err = nullptr;
    uint32_t *d_counters = nullptr;  // per-launch tile counters
    static constexpr uint32_t kCounters = 256;
    uint32_t next_counter = 0;

    // options
    int64_t opt_kernel = 0;        // 0 autotuned, 1 direct (plain), 2 window, 3 pipe, 4 ws, 5 tensor cores
    int64_t opt_slice_words = 0;   // 0 = autotune
    int64_t opt_ctas_per_sm = 0;   // 0 = autotune / occupancy
    int64_t opt_graph = 1;
    int64_t opt_max_window_slots = 0;
    int64_t opt_max_group_terms = 0;
    int64_t opt_split = 1;  // batched plans split neighbourhoods larger than a window

    idash_stats stats{};
    std::string last_error;
    std::set<idash_model *> models;  // live models; idash_close frees what is left

    // buffers for the host-memory path (grow only)
    uint8_t *d_in_buf = nullptr, *d_out_buf = nullptr;
    size_t d_in_cap = 0, d_out_cap = 0;
    std::vector<cudaEvent_t> events;

    idash_status fail(idash_status s, const std::string &msg) {
        last_error = msg;
        return s;
    }
    idash_status check_cuda(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return IDASH_OK;
        last_error = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? IDASH_ERR_OUT_OF_MEMORY : IDASH_ERR_CUDA;
    }
    uint32_t *counter() { return d_counters + (next_counter++ % kCounters); }
    cudaEvent_t event(size_t i);
};

struct idash_model {
    idash_ctx *ctx = nullptr;
    idash::Form form = idash::Form::kTrlwe;
    idash_trlwe_params tp{};
    idash_lwe_params lp{};
    uint64_t n_out = 0, n_in_rows = 0;
    std::vector<uint64_t> term_ptr;
    std::vector<uint32_t> term_feat;
    std::vector<int32_t> term_coef;
    std::vector<uint32_t> out_index;
    std::vector<uint32_t> out_row;
    std::vector<uint32_t> row_of_index;

    idash::Plan plan;
    idash::KernelKind kind = idash::KernelKind::kWindow;
    uint32_t slice_words = 1024, group_size = 3;
    uint32_t n_stages = 1;  // warp-specialised kernel's ring depth
    uint32_t max_slots = 0, max_terms = 0, max_groups = 0;
    uint32_t ctas = 0;
    bool tuned = false;

    idash::PlanBlock *d_blocks = nullptr;
    idash::PlanSlot *d_slots = nullptr;
    idash::PlanGroup *d_groups = nullptr;
    idash::PlanTerm *d_terms = nullptr;
    uint64_t *d_var_ptr = nullptr;
    uint32_t *d_var_row = nullptr;
    int32_t *d_var_coef = nullptr;
    uint32_t *d_out_index = nullptr;
    uint32_t *d_out_row = nullptr;
    uint8_t *d_tc_a = nullptr;      // tensor-core plans: coefficient digits per block
    uint32_t *d_tc_bias = nullptr;  // tensor-core plans: bias per output

    // cached CUDA graph of the last device-path call
    cudaGraphExec_t graph = nullptr;
    const void *g_in = nullptr;
    void *g_out = nullptr;
    idash_row_layout g_in_layout{}, g_out_layout{};

    idash::IntpolyModel *intpoly = nullptr;  // set for Form::kIntPoly

    void free_device();
    void drop_graph();
    void free_intpoly();
};
