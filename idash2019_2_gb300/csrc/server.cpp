// Continuous-batching serving loop for a resident TRLWE model
// (idash_serve_trlwe).  No counterpart in the reference, whose cloud binary
// scores one batch per process (eval/cloud.cpp:3-28); this serves a stream of
// imputation requests against one resident model.
//
// A request is a batch of individuals and a contiguous range of target SNPs.
// Its individuals are packed up to REGION_SIZE per TRLWE block (the model is
// planned with NUM_REGIONS = 1), so a request of I individuals is
// ceil(I / REGION_SIZE) blocks.  Each block needs the input rows its targets
// read (idash_model_input_rows) and 3 output rows per target.
//
// The loop admits requests in arrival order whenever a stream slot is free
// and the request's device memory fits the HBM budget (first fit in one arena
// allocated at start).  Admitted requests run concurrently, one stream each:
// ciphertext synthesis (standing in for the request's payload), range
// scoring, and an order-independent digest of the outputs (taken by the
// scoring kernel as it stores them when the model's kernel can, else by a
// pass over the outputs).  Memory returns to
// the arena when a request completes.  Completion times come from CUDA events.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <vector>

#include "capi_internal.hpp"

using namespace idash;

namespace {

constexpr uint64_t kAlign = 256;

// First-fit allocator over one device arena.
class Arena {
   public:
    explicit Arena(uint64_t size) { free_[0] = size; }
    bool alloc(uint64_t bytes, uint64_t *off) {
        bytes = (bytes + kAlign - 1) / kAlign * kAlign;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const uint64_t rest = it->second - bytes, at = it->first + bytes;
            free_.erase(it);
            if (rest) free_[at] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes) {
        bytes = (bytes + kAlign - 1) / kAlign * kAlign;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }

   private:
    std::map<uint64_t, uint64_t> free_;
};

struct Shape {
    uint64_t out_begin, out_end, row_begin, row_end;
    uint32_t blocks;
    uint64_t in_bytes_per_block, out_bytes_per_block;
    uint64_t bytes() const { return blocks * (in_bytes_per_block + out_bytes_per_block); }
};

// Seed of the ciphertexts of individual block b of a request.
uint64_t request_block_seed(uint64_t seed, uint32_t b) { return seed * 0x9E3779B97F4A7C15ull + b; }

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    int64_t req = -1;
    uint64_t off = 0, bytes = 0;
};

}  // namespace

extern "C" idash_status idash_serve_trlwe(idash_model *m, const idash_serve_config *cfg, const idash_request *reqs,
                                          uint64_t n, idash_request_result *results, void *const *host_out) {
    if (!m || !cfg || (n && (!reqs || !results))) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kTrlwe) return ctx->fail(IDASH_ERR_STATE, "serving needs a TRLWE model");
    if (m->tp.num_regions != 1) return ctx->fail(IDASH_ERR_UNSUPPORTED, "serving needs a model with NUM_REGIONS = 1");
    if (cfg->max_inflight == 0 || cfg->max_inflight > 64 || cfg->hbm_budget == 0)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "max_inflight in [1, 64] and a non-zero budget");
    const uint32_t N = m->tp.N, RS = m->tp.region_size;
    const uint64_t row_bytes = uint64_t(2) * N * 4;
    const idash_row_layout dense{row_bytes, 0, -1, -1};

    for (uint64_t i = 0; i < n; ++i) {
        const idash_request &r = reqs[i];
        if (r.n_indiv == 0 || r.target_end <= r.target_begin || 3 * r.target_end > m->n_out)
            return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "request " + std::to_string(i) + ": empty or out of range");
    }

    uint8_t *arena_base = nullptr;
    uint64_t *d_digest = nullptr;
    idash_status st = ctx->check_cuda(cudaMalloc(&arena_base, cfg->hbm_budget), "cudaMalloc(serving arena)");
    if (st != IDASH_OK) return st;
    st = ctx->check_cuda(cudaMalloc(&d_digest, std::max<uint64_t>(n, 1) * 8), "cudaMalloc(digests)");
    if (st == IDASH_OK) st = ctx->check_cuda(cudaMemset(d_digest, 0, std::max<uint64_t>(n, 1) * 8), "memset");
    std::vector<Slot> slots(cfg->max_inflight);
    for (Slot &s : slots) {
        if (st != IDASH_OK) break;
        st = ctx->check_cuda(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate");
        if (st == IDASH_OK) st = ctx->check_cuda(cudaEventCreate(&s.done), "cudaEventCreate");
    }
    cudaEvent_t t0_evt = nullptr;
    if (st == IDASH_OK) st = ctx->check_cuda(cudaEventCreate(&t0_evt), "cudaEventCreate");

    // Autotune the model once, outside the served window, on arena memory.
    if (st == IDASH_OK && !m->tuned && m->ctx->opt_kernel != 1) {
        const uint64_t in_b = m->n_in_rows * row_bytes, out_b = m->n_out * row_bytes;
        if (in_b + out_b <= cfg->hbm_budget) {
            st = idash_score_trlwe_device(m, arena_base, &dense, arena_base + in_b, &dense, nullptr);
            if (st == IDASH_OK) st = idash_sync(ctx);
        }
    }

    // Shapes under the final plan (blocks decide which input rows a range
    // reads) and admission limits: a request that can never fit fails with
    // IDASH_ERR_ADMISSION before any request runs.
    std::vector<Shape> shape(n);
    for (uint64_t i = 0; i < n && st == IDASH_OK; ++i) {
        const idash_request &r = reqs[i];
        Shape &s = shape[i];
        s.out_begin = 3 * r.target_begin;
        s.out_end = 3 * r.target_end;
        idash_model_input_rows(m, s.out_begin, s.out_end, &s.row_begin, &s.row_end);
        s.blocks = (r.n_indiv + RS - 1) / RS;
        s.in_bytes_per_block = std::max<uint64_t>(s.row_end - s.row_begin, 1) * row_bytes;
        s.out_bytes_per_block = (s.out_end - s.out_begin) * row_bytes;
        if (s.bytes() > cfg->hbm_budget)
            st = ctx->fail(IDASH_ERR_ADMISSION, "request " + std::to_string(i) + " needs more than the HBM budget");
    }

    Arena arena(cfg->hbm_budget);
    std::deque<uint64_t> queue;
    uint64_t next_arrival = 0, completed = 0;
    using clock = std::chrono::steady_clock;
    const clock::time_point t0 = clock::now();
    auto now_s = [&]() { return std::chrono::duration<double>(clock::now() - t0).count(); };
    if (st == IDASH_OK) st = ctx->check_cuda(cudaEventRecord(t0_evt, slots[0].stream), "event");
    if (st == IDASH_OK) st = ctx->check_cuda(cudaEventSynchronize(t0_evt), "event");

    while (st == IDASH_OK && completed < n) {
        bool progress = false;
        for (Slot &s : slots) {
            if (s.req < 0) continue;
            const cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaErrorNotReady) continue;
            if ((st = ctx->check_cuda(q, "request completion")) != IDASH_OK) break;
            float ms = 0;
            if ((st = ctx->check_cuda(cudaEventElapsedTime(&ms, t0_evt, s.done), "completion time")) != IDASH_OK)
                break;
            idash_request_result &res = results[s.req];
            res.done_s = ms * 1e-3;
            res.device_bytes = s.bytes;
            if (host_out && host_out[s.req]) {
                const Shape &sh = shape[s.req];
                const uint64_t ob = sh.out_bytes_per_block;
                for (uint32_t b = 0; b < sh.blocks && st == IDASH_OK; ++b)
                    st = ctx->check_cuda(cudaMemcpy(static_cast<uint8_t *>(host_out[s.req]) + b * ob,
                                                    arena_base + s.off + sh.blocks * sh.in_bytes_per_block + b * ob,
                                                    ob, cudaMemcpyDeviceToHost),
                                         "copy outputs");
            }
            arena.release(s.off, s.bytes);
            s.req = -1;
            ++completed;
            progress = true;
        }
        if (st != IDASH_OK) break;
        const double now = now_s();
        while (next_arrival < n && reqs[next_arrival].arrival_s <= now) queue.push_back(next_arrival++);
        while (!queue.empty()) {
            Slot *free_slot = nullptr;
            for (Slot &s : slots)
                if (s.req < 0) {
                    free_slot = &s;
                    break;
                }
            if (!free_slot) break;
            const uint64_t i = queue.front();
            const Shape &sh = shape[i];
            uint64_t off;
            if (!arena.alloc(sh.bytes(), &off)) break;  // wait for memory to come back
            queue.pop_front();
            Slot &s = *free_slot;
            s.req = int64_t(i);
            s.off = off;
            s.bytes = sh.bytes();
            results[i].admit_s = now_s();
            const idash_request &r = reqs[i];
            uint8_t *in0 = arena_base + off;
            uint8_t *out0 = in0 + sh.blocks * sh.in_bytes_per_block;
            for (uint32_t b = 0; b < sh.blocks && st == IDASH_OK; ++b) {
                const uint32_t ns = std::min<uint32_t>(RS, r.n_indiv - b * RS);
                uint8_t *in_b = in0 + b * sh.in_bytes_per_block;
                uint8_t *out_b = out0 + b * sh.out_bytes_per_block;
                st = ctx->check_cuda(fill_uniform_rows(request_block_seed(r.seed, b), sh.row_begin,
                                                       sh.row_end - sh.row_begin, 2 * N, in_b, row_bytes,
                                                       ctx->sm_count, s.stream),
                                     "request ciphertexts");
                const uint64_t index_base = uint64_t(b) * (sh.out_bytes_per_block / 4);
                bool fused = false;
                if (st == IDASH_OK)
                    st = score_trlwe_range(m, sh.out_begin, sh.out_end, ns, in_b, &dense, sh.row_begin,
                                           sh.row_end - sh.row_begin, out_b, &dense, s.stream, d_digest + i,
                                           index_base, &fused);
                if (st == IDASH_OK && !fused)
                    st = ctx->check_cuda(digest_words(reinterpret_cast<const uint32_t *>(out_b),
                                                      sh.out_bytes_per_block / 4, index_base, d_digest + i,
                                                      ctx->sm_count, s.stream),
                                         "digest");
            }
            if (st == IDASH_OK) st = ctx->check_cuda(cudaEventRecord(s.done, s.stream), "event");
            progress = true;
        }
        if (!progress) {
            // idle: sleep briefly, never past the next arrival
            double wait = 20e-6;
            if (queue.empty() && next_arrival < n) wait = std::min(wait, std::max(0.0, reqs[next_arrival].arrival_s - now_s()));
            std::this_thread::sleep_for(std::chrono::duration<double>(wait));
        }
    }
    for (Slot &s : slots)
        if (s.stream) cudaStreamSynchronize(s.stream);
    if (st == IDASH_OK) st = idash_sync(ctx);
    if (st == IDASH_OK && n) {
        std::vector<uint64_t> dig(n);
        st = ctx->check_cuda(cudaMemcpy(dig.data(), d_digest, n * 8, cudaMemcpyDeviceToHost), "digests");
        for (uint64_t i = 0; i < n && st == IDASH_OK; ++i) results[i].digest = dig[i];
    }
    for (Slot &s : slots) {
        if (s.done) cudaEventDestroy(s.done);
        if (s.stream) cudaStreamDestroy(s.stream);
    }
    if (t0_evt) cudaEventDestroy(t0_evt);
    cudaFree(d_digest);
    cudaFree(arena_base);
    return st;
}

extern "C" uint64_t idash_digest_host(const uint32_t *words, uint64_t n_words, uint64_t index_base) {
    return digest_host(words, n_words, index_base);
}
