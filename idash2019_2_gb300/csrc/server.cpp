// Serving engine (idash_server_*, include/idash_gpu.h).  No counterpart in the
// reference, whose cloud binary scores one batch per process
// (eval/cloud.cpp:3-28); this serves a stream of imputation requests against
// one resident model while they arrive.
//
// Requests are submitted from any thread into a FIFO.  One scheduler thread
// owns every CUDA call of the server:
//   admission   in submission order, while fewer than max_inflight requests
//               are admitted and one device arena (the HBM budget, allocated
//               at open) holds the request's first segment: a range of its
//               outputs and the input rows those outputs read;
//   staging     segments of admitted requests as the arena frees up (at most
//               two per request at a time); a staged segment's input rows are
//               copied in from host memory (or generated from the request's
//               seed) on the input stream;
//   launches    every staged segment of every admitted request goes into one
//               job table - one job per (segment, block of individuals) - and
//               one launch of the warp-specialised kernel scores them all
//               (ScoreJob, score_kernels.cuh), after the jobs' inputs have
//               landed; at most two launches are outstanding, so segments
//               staged while one runs form the next.  A launch issued onto
//               an idle device takes about half of what is staged (whole
//               segments), and the rest follows at once behind it: the
//               device then always has a launch queued while the requests
//               of the one before complete and new ones are staged;
//   completion  a launched segment's outputs go back to host memory on the
//               output stream (when the request has a host buffer), its
//               segment memory returns to the arena; when every segment of a
//               request is back, its digest is read and it completes.
// The digest of a request is taken by the scoring kernel as it stores the
// outputs, per job, into the request's own digest slot: it depends only on the
// request's own outputs, not on what shared the launch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "capi_internal.hpp"

using namespace idash;

namespace {

constexpr uint64_t kAlign = 256;
constexpr uint32_t kLaunchRing = 2;        // launches outstanding at once
constexpr uint32_t kSegmentsPerRequest = 2;  // output segments of one request staged at once
constexpr uint32_t kCounters = 8;

// First-fit allocator over one device arena.
class Arena {
   public:
    void reset(uint64_t size) {
        free_.clear();
        free_[0] = size;
    }
    bool alloc(uint64_t bytes, uint64_t *off) {
        bytes = round(bytes);
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
        bytes = round(bytes);
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
    static uint64_t round(uint64_t b) { return (std::max<uint64_t>(b, 1) + kAlign - 1) / kAlign * kAlign; }

   private:
    std::map<uint64_t, uint64_t> free_;
};

// Seed of the generated inputs of block b of a request.
uint64_t request_block_seed(uint64_t seed, uint32_t b) { return seed * 0x9E3779B97F4A7C15ull + b; }

enum class SegState { kWaiting, kStaged, kLaunched, kCopying, kDone };

struct Segment {
    uint64_t o_lo = 0, o_hi = 0;  // outputs
    uint64_t r_lo = 0, r_hi = 0;  // the input rows they read
    uint64_t in_off = 0, in_bytes = 0;  // arena memory of its input rows (all blocks)
    uint64_t off = 0, bytes = 0;  // arena memory of its outputs (all blocks)
    cudaEvent_t in_ready = nullptr;
    SegState state = SegState::kWaiting;
    uint32_t launch = 0;          // launch ring slot
    uint64_t launch_seq = 0;
    cudaEvent_t copied = nullptr;
};

enum class ReqState { kQueued, kAdmitted, kFinishing, kDone, kFailed };

struct Req {
    idash_serve_request r{};
    uint64_t out_begin = 0, out_end = 0, row_begin = 0, row_end = 0;
    uint32_t blocks = 1;
    uint32_t row_words = 0;     // valid words per row
    uint64_t row_bytes = 0;     // row stride in bytes (inputs and outputs)
    std::vector<Segment> segs;
    size_t next_seg = 0, segs_done = 0;
    uint32_t digest_slot = 0;
    cudaEvent_t finished = nullptr;
    ReqState state = ReqState::kQueued;
    idash_status status = IDASH_PENDING;
    idash_request_result res{};
    uint64_t seg_bytes(const Segment &s) const { return blocks * (s.o_hi - s.o_lo) * row_bytes; }
    uint64_t seg_in_bytes(const Segment &s) const { return blocks * std::max<uint64_t>(s.r_hi - s.r_lo, 1) * row_bytes; }
};

}  // namespace

struct idash_server {
    idash_model *m = nullptr;
    idash_ctx *ctx = nullptr;
    idash_serve_config cfg{};
    bool lwe = false;
    uint8_t *arena_base = nullptr;
    Arena arena;
    unsigned long long *d_digest = nullptr;  // one slot per admissible request
    uint64_t *h_digest = nullptr;            // page-locked mirror
    std::vector<uint32_t> free_slots;
    uint32_t *d_counters = nullptr;
    uint32_t next_counter = 0;
    cudaStream_t compute = nullptr, h2d = nullptr, d2h = nullptr;
    cudaEvent_t t0 = nullptr;
    ScoreJob *d_jobs[kLaunchRing] = {};
    ScoreJob *h_jobs[kLaunchRing] = {};
    size_t jobs_cap = 0;
    cudaEvent_t launch_start[kLaunchRing] = {}, launch_done[kLaunchRing] = {};
    uint64_t launch_seq = 0;     // launches issued
    uint64_t launch_retired = 0; // launches known complete
    std::atomic<uint64_t> launches{0};
    idash_server_stats stats{};  // under mu
    std::vector<cudaEvent_t> event_pool;

    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req *> queued;
    std::map<uint64_t, Req *> all;
    uint64_t next_id = 1;
    bool closing = false;
    std::string error;         // why the scheduler failed ("" while it has not)
    std::string submit_error;  // why the last refused submit was refused
    std::vector<Req *> admitted;  // scheduler thread only
    std::thread worker;
    std::chrono::steady_clock::time_point t0_host;

    double now_s() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_host).count();
    }
    cudaEvent_t take_event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void give_event(cudaEvent_t &e) {
        if (e) event_pool.push_back(e);
        e = nullptr;
    }
    bool fail(const std::string &msg) {
        std::lock_guard<std::mutex> lock(mu);
        if (error.empty()) error = msg;
        return false;
    }
    bool check(cudaError_t e, const char *what) {
        return e == cudaSuccess ? true : fail(std::string(what) + ": " + cudaGetErrorString(e));
    }
    bool admit(Req *q);
    bool stage(Req *q, Segment &g);
    bool stage_segments();
    bool launch();
    bool complete();
    void run();
};

namespace {

// Shape of a request under the model's plan; "" or why it cannot be served.
std::string shape_request(const idash_server *s, const idash_serve_request &r, Req *q) {
    idash_model *m = s->m;
    if (r.n_indiv == 0 || r.target_end <= r.target_begin || 3 * r.target_end > m->n_out)
        return "request is empty or its targets are out of range";
    q->r = r;
    q->out_begin = 3 * r.target_begin;
    q->out_end = 3 * r.target_end;
    idash_model_input_rows(m, q->out_begin, q->out_end, &q->row_begin, &q->row_end);
    if (s->lwe) {
        if (r.n_indiv > m->lp.n_indiv) return "request has more individuals than the model";
        q->blocks = 1;
        q->row_words = r.n_indiv * (m->lp.n + 1);
        q->row_bytes = uint64_t((q->row_words + 3) / 4 * 4) * 4;
    } else {
        q->blocks = (r.n_indiv + m->tp.region_size - 1) / m->tp.region_size;
        q->row_words = 2 * m->tp.N;
        q->row_bytes = uint64_t(q->row_words) * 4;
    }
    const uint64_t seg = s->cfg.segment_outputs ? s->cfg.segment_outputs : (s->lwe ? 2048 : q->out_end - q->out_begin);
    uint64_t need = 0;
    for (uint64_t lo = q->out_begin; lo < q->out_end; lo += seg) {
        Segment g;
        g.o_lo = lo;
        g.o_hi = std::min(q->out_end, lo + seg);
        idash_model_input_rows(m, g.o_lo, g.o_hi, &g.r_lo, &g.r_hi);
        g.bytes = q->seg_bytes(g);
        g.in_bytes = q->seg_in_bytes(g);
        need = std::max(need, Arena::round(g.in_bytes) + Arena::round(g.bytes));
        q->segs.push_back(g);
    }
    if (need > s->cfg.hbm_budget) return "request needs more than the HBM budget";
    return "";
}

}  // namespace

// Takes arena memory for segment g and starts its input rows on their way.
bool idash_server::stage(Req *q, Segment &g) {
    if (!arena.alloc(g.in_bytes, &g.in_off)) return false;
    if (!arena.alloc(g.bytes, &g.off)) {
        arena.release(g.in_off, g.in_bytes);
        return false;
    }
    g.state = SegState::kStaged;
    uint8_t *in0 = arena_base + g.in_off;
    const uint64_t n_rows = g.r_hi - g.r_lo, block_bytes = std::max<uint64_t>(n_rows, 1) * q->row_bytes;
    bool ok = true;
    for (uint32_t b = 0; b < q->blocks && ok && n_rows; ++b) {
        uint8_t *dst = in0 + b * block_bytes;
        if (q->r.h_in) {
            const uint8_t *src = static_cast<const uint8_t *>(q->r.h_in) +
                                 (uint64_t(b) * (q->row_end - q->row_begin) + (g.r_lo - q->row_begin)) * q->row_bytes;
            ok = check(cudaMemcpyAsync(dst, src, n_rows * q->row_bytes, cudaMemcpyHostToDevice, h2d), "request inputs");
            std::lock_guard<std::mutex> lock(mu);
            stats.h2d_bytes += n_rows * q->row_bytes;
        } else {
            ok = check(fill_uniform_rows(request_block_seed(q->r.seed, b), g.r_lo, n_rows, q->row_words, dst,
                                         q->row_bytes, ctx->sm_count, h2d),
                       "request inputs");
        }
    }
    g.in_ready = take_event();
    return ok && check(cudaEventRecord(g.in_ready, h2d), "event");
}

bool idash_server::admit(Req *q) {
    if (!stage(q, q->segs[0])) {
        if (q->segs[0].state == SegState::kStaged) return fail("staging a request's inputs");
        return false;  // no memory yet
    }
    q->next_seg = 1;
    q->digest_slot = free_slots.back();
    free_slots.pop_back();
    q->res.admit_s = now_s();
    q->res.device_bytes = Arena::round(q->segs[0].in_bytes) + Arena::round(q->segs[0].bytes);
    q->state = ReqState::kAdmitted;
    // the digest slot is cleared before any launch reads the segment's inputs
    bool ok = check(cudaMemsetAsync(d_digest + q->digest_slot, 0, 8, h2d), "digest reset");
    ok = ok && check(cudaEventRecord(q->segs[0].in_ready, h2d), "event");
    admitted.push_back(q);
    return ok;
}

bool idash_server::stage_segments() {
    for (Req *q : admitted) {
        size_t open = 0;
        for (size_t i = 0; i < q->next_seg; ++i) open += q->segs[i].state != SegState::kDone;
        while (q->next_seg < q->segs.size() && open < kSegmentsPerRequest) {
            Segment &g = q->segs[q->next_seg];
            if (!stage(q, g)) return g.state != SegState::kStaged;  // no memory: wait, keeping submission order
            ++q->next_seg;
            ++open;
        }
    }
    return true;
}

bool idash_server::launch() {
    if (launch_seq - launch_retired >= kLaunchRing) return true;
    const uint32_t W = m->slice_words;
    // the staged segments in admission order, with their plan blocks and tiles
    struct Pick {
        Req *q;
        Segment *g;
        uint32_t b_lo, b_hi, n_slices;
        uint64_t tiles;
    };
    std::vector<Pick> picks;
    uint64_t staged_tiles = 0;
    for (Req *q : admitted)
        for (Segment &g : q->segs) {
            if (g.state != SegState::kStaged) continue;
            const auto &B = m->plan.blocks;
            const auto first = std::partition_point(B.begin(), B.end(), [&](const PlanBlock &b) { return b.out_hi <= g.o_lo; });
            const auto last = std::partition_point(first, B.end(), [&](const PlanBlock &b) { return b.out_lo < g.o_hi; });
            Pick p{q, &g, uint32_t(first - B.begin()), uint32_t(last - B.begin()), (q->row_words + W - 1) / W, 0};
            p.tiles = uint64_t(q->blocks) * (p.b_hi - p.b_lo) * p.n_slices;
            staged_tiles += p.tiles;
            picks.push_back(p);
        }
    if (picks.empty()) return true;
    // onto an idle device: about half now, the rest queued right behind it
    if (launch_seq == launch_retired && picks.size() > 1) {
        uint64_t taken = 0;
        size_t n = 0;
        while (n < picks.size() && 2 * taken < staged_tiles) taken += picks[n++].tiles;
        picks.resize(n);
    }
    std::vector<ScoreJob> jobs;
    std::vector<Segment *> segs;
    uint64_t tiles = 0;
    for (const Pick &p : picks) {
        {
            Req *q = p.q;
            Segment &g = *p.g;
            const uint32_t b_lo = p.b_lo, b_hi = p.b_hi, n_slices = p.n_slices;
            const uint64_t in_block_bytes = std::max<uint64_t>(g.r_hi - g.r_lo, 1) * q->row_bytes;
            if (!check(cudaStreamWaitEvent(compute, g.in_ready, 0), "wait for inputs")) return false;
            for (uint32_t b = 0; b < q->blocks && b_hi > b_lo; ++b) {
                ScoreJob j{};
                j.in = arena_base + g.in_off + b * in_block_bytes;
                j.out = arena_base + g.off + uint64_t(b) * (g.o_hi - g.o_lo) * q->row_bytes;
                j.digest = d_digest + q->digest_slot;
                j.out_lo = g.o_lo;
                j.out_hi = g.o_hi;
                j.out_row_base = g.o_lo;
                const uint64_t req_row = lwe ? (g.o_lo - q->out_begin)
                                             : uint64_t(b) * (q->out_end - q->out_begin) + (g.o_lo - q->out_begin);
                j.digest_base = req_row * (q->row_bytes / 4);
                j.stride = q->row_bytes;
                j.block_lo = b_lo;
                j.n_blocks = b_hi - b_lo;
                j.row_base = uint32_t(g.r_lo);
                j.n_rows = uint32_t(g.r_hi - g.r_lo);
                j.row_words = q->row_words;
                j.num_samples = lwe ? 0u : std::min<uint32_t>(m->tp.region_size, q->r.n_indiv - b * m->tp.region_size);
                j.tile_begin = uint32_t(tiles);
                j.n_slices = n_slices;
                tiles += uint64_t(j.n_blocks) * n_slices;
                jobs.push_back(j);
            }
            segs.push_back(&g);
        }
    }
    if (tiles >= 0xFFFFFFFFull) return fail("one launch would exceed 2^32 tiles; lower segment_outputs");
    const uint32_t k = uint32_t(launch_seq % kLaunchRing);
    // the job table of the launch that last used this slot has been consumed
    if (launch_seq >= kLaunchRing && !check(cudaEventSynchronize(launch_done[k]), "launch slot")) return false;
    if (jobs.size() > jobs_cap) {
        const size_t cap = std::max<size_t>(jobs.size() * 2, 256);
        for (uint32_t i = 0; i < kLaunchRing; ++i) {
            if (i != k && launch_seq >= kLaunchRing && !check(cudaEventSynchronize(launch_done[i]), "launch slot"))
                return false;
            cudaFree(d_jobs[i]);
            cudaFreeHost(h_jobs[i]);
            d_jobs[i] = nullptr;
            h_jobs[i] = nullptr;
            if (!check(cudaMalloc(&d_jobs[i], cap * sizeof(ScoreJob)), "job table") ||
                !check(cudaMallocHost(&h_jobs[i], cap * sizeof(ScoreJob)), "job table"))
                return false;
        }
        jobs_cap = cap;
    }
    std::memcpy(h_jobs[k], jobs.data(), jobs.size() * sizeof(ScoreJob));
    if (!check(cudaMemcpyAsync(d_jobs[k], h_jobs[k], jobs.size() * sizeof(ScoreJob), cudaMemcpyHostToDevice, compute),
               "job table"))
        return false;
    ScoreArgs a{};
    a.blocks = m->d_blocks;
    a.slots = m->d_slots;
    a.groups = m->d_groups;
    a.terms = m->d_terms;
    a.n_tiles = uint32_t(tiles);
    a.form = lwe ? kFormLwe : kFormTrlwe;
    a.N = m->tp.N;
    a.region_size = m->tp.region_size;
    a.lwe_n1 = m->lp.n + 1;
    a.max_slots = m->max_slots;
    a.max_terms = m->max_terms;
    a.max_groups = m->max_groups;
    a.n_stages = m->n_stages;
    a.tile_counter = d_counters + (next_counter++ % kCounters);
    a.err = ctx->d_err;
    a.jobs = d_jobs[k];
    a.n_jobs = uint32_t(jobs.size());
    if (!check(cudaEventRecord(launch_start[k], compute), "event")) return false;
    if (!check(launch_score(KernelKind::kWs, W, m->group_size, a, m->ctas, compute), "scoring launch")) return false;
    if (!check(cudaEventRecord(launch_done[k], compute), "event")) return false;
    for (Segment *g : segs) {
        g->state = SegState::kLaunched;
        g->launch = k;
        g->launch_seq = launch_seq;
    }
    ++launch_seq;
    launches.fetch_add(1);
    {
        std::lock_guard<std::mutex> lock(mu);
        ++stats.launches;
    }
    return true;
}

bool idash_server::complete() {
    // retire finished launches in order
    while (launch_retired < launch_seq) {
        const uint32_t k = uint32_t(launch_retired % kLaunchRing);
        const cudaError_t e = cudaEventQuery(launch_done[k]);
        if (e == cudaErrorNotReady) break;
        if (!check(e, "launch")) return false;
        float ms = 0;
        if (!check(cudaEventElapsedTime(&ms, launch_start[k], launch_done[k]), "launch time")) return false;
        {
            std::lock_guard<std::mutex> lock(mu);
            stats.busy_s += ms * 1e-3;
        }
        ++launch_retired;
    }
    for (size_t i = 0; i < admitted.size();) {
        Req *q = admitted[i];
        for (Segment &g : q->segs) {
            if (g.state == SegState::kLaunched && g.launch_seq < launch_retired) {
                if (q->r.h_out) {
                    const uint64_t n_req = q->out_end - q->out_begin, n_seg = g.o_hi - g.o_lo;
                    for (uint32_t b = 0; b < q->blocks; ++b) {
                        uint8_t *dst = static_cast<uint8_t *>(q->r.h_out) +
                                       (uint64_t(b) * n_req + (g.o_lo - q->out_begin)) * q->row_bytes;
                        if (!check(cudaMemcpyAsync(dst, arena_base + g.off + uint64_t(b) * n_seg * q->row_bytes,
                                                   n_seg * q->row_bytes, cudaMemcpyDeviceToHost, d2h),
                                   "request outputs"))
                            return false;
                    }
                    {
                        std::lock_guard<std::mutex> lock(mu);
                        stats.d2h_bytes += q->blocks * n_seg * q->row_bytes;
                    }
                    g.copied = take_event();
                    if (!check(cudaEventRecord(g.copied, d2h), "event")) return false;
                    g.state = SegState::kCopying;
                } else {
                    g.state = SegState::kDone;
                    arena.release(g.off, g.bytes);
                    arena.release(g.in_off, g.in_bytes);
                    give_event(g.in_ready);
                    ++q->segs_done;
                }
            }
            if (g.state == SegState::kCopying) {
                const cudaError_t e = cudaEventQuery(g.copied);
                if (e == cudaErrorNotReady) continue;
                if (!check(e, "output copy")) return false;
                give_event(g.copied);
                g.state = SegState::kDone;
                arena.release(g.off, g.bytes);
                arena.release(g.in_off, g.in_bytes);
                give_event(g.in_ready);
                ++q->segs_done;
            }
        }
        if (q->state == ReqState::kAdmitted && q->segs_done == q->segs.size()) {
            // every launch of this request is complete: read its digest
            if (!check(cudaMemcpyAsync(h_digest + q->digest_slot, d_digest + q->digest_slot, 8,
                                       cudaMemcpyDeviceToHost, d2h),
                       "digest"))
                return false;
            q->finished = take_event();
            if (!check(cudaEventRecord(q->finished, d2h), "event")) return false;
            q->state = ReqState::kFinishing;
        }
        if (q->state == ReqState::kFinishing) {
            const cudaError_t e = cudaEventQuery(q->finished);
            if (e != cudaErrorNotReady) {
                if (!check(e, "request completion")) return false;
                float ms = 0;
                if (!check(cudaEventElapsedTime(&ms, t0, q->finished), "completion time")) return false;
                give_event(q->finished);
                {
                    std::lock_guard<std::mutex> lock(mu);
                    q->res.done_s = ms * 1e-3;
                    q->res.digest = h_digest[q->digest_slot];
                    q->status = IDASH_OK;
                    q->state = ReqState::kDone;
                    ++stats.requests_done;
                }
                free_slots.push_back(q->digest_slot);
                cv.notify_all();
                admitted.erase(admitted.begin() + long(i));
                continue;
            }
        }
        ++i;
    }
    return true;
}

void idash_server::run() {
    cudaSetDevice(ctx->device);
    bool ok = true;
    while (ok) {
        bool idle = true;
        {
            std::unique_lock<std::mutex> lock(mu);
            if (closing && queued.empty() && admitted.empty()) break;
        }
        // admission in submission order
        while (ok) {
            Req *q = nullptr;
            {
                std::lock_guard<std::mutex> lock(mu);
                if (queued.empty() || admitted.size() >= cfg.max_inflight) break;
                q = queued.front();
            }
            if (!admit(q)) {
                std::lock_guard<std::mutex> lock(mu);
                if (error.empty()) break;  // no memory yet
                ok = false;
                break;
            }
            std::lock_guard<std::mutex> lock(mu);
            queued.pop_front();
            idle = false;
        }
        const uint64_t before = launch_seq + launch_retired;
        ok = ok && stage_segments() && launch() && complete();
        if (launch_seq + launch_retired != before) idle = false;
        if (idle) {
            std::unique_lock<std::mutex> lock(mu);
            cv.wait_for(lock, std::chrono::microseconds(admitted.empty() ? 2000 : 20));
        }
    }
    if (!ok) {
        // fail everything not complete
        cudaStreamSynchronize(compute);
        cudaStreamSynchronize(h2d);
        cudaStreamSynchronize(d2h);
        std::lock_guard<std::mutex> lock(mu);
        for (auto &kv : all)
            if (kv.second->state != ReqState::kDone) {
                kv.second->state = ReqState::kFailed;
                kv.second->status = IDASH_ERR_CUDA;
            }
        queued.clear();
        admitted.clear();
        cv.notify_all();
    }
}

extern "C" {

idash_status idash_server_open(idash_model *m, const idash_serve_config *cfg, idash_server **out) {
    if (!m || !cfg || !out) return IDASH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    idash_ctx *ctx = m->ctx;
    if (m->form == Form::kIntPoly) return ctx->fail(IDASH_ERR_UNSUPPORTED, "serving covers the TRLWE and LWE forms");
    if (m->form == Form::kTrlwe && m->tp.num_regions != 1)
        return ctx->fail(IDASH_ERR_UNSUPPORTED, "serving needs a TRLWE model with NUM_REGIONS = 1");
    if (cfg->max_inflight == 0 || cfg->max_inflight > 4096 || cfg->hbm_budget == 0)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "max_inflight in [1, 4096] and a non-zero budget");
    idash_status st = IDASH_OK;
    if (m->kind != KernelKind::kWs) {
        // plan for the warp-specialised kernel (the one that takes job tables)
        const int64_t saved = ctx->opt_kernel;
        ctx->opt_kernel = 4;
        st = idash_model_replan(m);
        ctx->opt_kernel = saved;
        if (st != IDASH_OK) return st;
        if (m->kind != KernelKind::kWs)
            return ctx->fail(IDASH_ERR_UNSUPPORTED, "no warp-specialised plan holds this model's neighbourhoods");
    }
    if (m->plan.phase_begin.size() > 2)
        return ctx->fail(IDASH_ERR_UNSUPPORTED, "serving needs a plan without split neighbourhoods");
    idash_server *s = new idash_server();
    s->m = m;
    s->ctx = ctx;
    s->cfg = *cfg;
    s->lwe = m->form == Form::kLwe;
    auto bad = [&](idash_status code) {
        s->closing = true;
        idash_server_close(s);
        return code;
    };
    if ((st = ctx->check_cuda(cudaMalloc(&s->arena_base, cfg->hbm_budget), "cudaMalloc(serving arena)")) != IDASH_OK)
        return bad(st);
    s->arena.reset(cfg->hbm_budget);
    const size_t slots = cfg->max_inflight;
    if ((st = ctx->check_cuda(cudaMalloc(&s->d_digest, slots * 8), "cudaMalloc(digests)")) != IDASH_OK) return bad(st);
    if ((st = ctx->check_cuda(cudaMallocHost(&s->h_digest, slots * 8), "cudaMallocHost(digests)")) != IDASH_OK)
        return bad(st);
    for (uint32_t i = 0; i < slots; ++i) s->free_slots.push_back(uint32_t(slots - 1 - i));
    if ((st = ctx->check_cuda(cudaMalloc(&s->d_counters, kCounters * 4), "cudaMalloc(counters)")) != IDASH_OK)
        return bad(st);
    for (cudaStream_t *x : {&s->compute, &s->h2d, &s->d2h})
        if ((st = ctx->check_cuda(cudaStreamCreateWithFlags(x, cudaStreamNonBlocking), "cudaStreamCreate")) != IDASH_OK)
            return bad(st);
    for (uint32_t i = 0; i < kLaunchRing; ++i)
        for (cudaEvent_t *e : {&s->launch_start[i], &s->launch_done[i]})
            if ((st = ctx->check_cuda(cudaEventCreate(e), "event")) != IDASH_OK) return bad(st);
    if ((st = ctx->check_cuda(cudaEventCreate(&s->t0), "event")) != IDASH_OK) return bad(st);
    // tune the model once, on arena memory, before the clock starts
    if (!m->tuned && !s->lwe) {
        const uint64_t in_b = m->n_in_rows * 8 * uint64_t(m->tp.N), out_b = m->n_out * 8 * uint64_t(m->tp.N);
        if (in_b + out_b <= cfg->hbm_budget) {
            const idash_row_layout dense{8 * uint64_t(m->tp.N), 0, -1, -1};
            const int64_t saved = ctx->opt_kernel;
            ctx->opt_kernel = 4;
            st = idash_score_trlwe_device(m, s->arena_base, &dense, s->arena_base + in_b, &dense, nullptr);
            ctx->opt_kernel = saved;
            if (st == IDASH_OK) st = idash_sync(ctx);
            if (st != IDASH_OK) return bad(st);
        }
    }
    s->t0_host = std::chrono::steady_clock::now();
    if ((st = ctx->check_cuda(cudaEventRecord(s->t0, s->compute), "event")) != IDASH_OK) return bad(st);
    if ((st = ctx->check_cuda(cudaEventSynchronize(s->t0), "event")) != IDASH_OK) return bad(st);
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return IDASH_OK;
}

idash_status idash_server_submit(idash_server *s, const idash_serve_request *r, uint64_t *ticket) {
    if (!s || !r || !ticket) return IDASH_ERR_INVALID_ARGUMENT;
    Req *q = new Req();
    const std::string why = shape_request(s, *r, q);
    if (!why.empty()) {
        delete q;
        std::lock_guard<std::mutex> lock(s->mu);
        s->submit_error = why;
        return why.find("budget") != std::string::npos ? IDASH_ERR_ADMISSION : IDASH_ERR_INVALID_ARGUMENT;
    }
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->closing) {
            delete q;
            return IDASH_ERR_STATE;
        }
        *ticket = s->next_id++;
        s->all[*ticket] = q;
        s->queued.push_back(q);
    }
    s->cv.notify_all();
    return IDASH_OK;
}

idash_status idash_server_poll(idash_server *s, uint64_t ticket, idash_request_result *res) {
    if (!s) return IDASH_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return IDASH_ERR_INVALID_ARGUMENT;
    if (it->second->status == IDASH_OK && res) *res = it->second->res;
    return it->second->status;
}

idash_status idash_server_wait(idash_server *s, uint64_t ticket, idash_request_result *res) {
    if (!s) return IDASH_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return IDASH_ERR_INVALID_ARGUMENT;
    Req *q = it->second;
    s->cv.wait(lock, [&] { return q->status != IDASH_PENDING; });
    if (q->status == IDASH_OK && res) *res = q->res;
    return q->status;
}

uint64_t idash_server_launches(const idash_server *s) { return s ? s->launches.load() : 0; }

idash_status idash_server_get_stats(idash_server *s, idash_server_stats *out) {
    if (!s || !out) return IDASH_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->stats;
    return IDASH_OK;
}

const char *idash_server_last_error(const idash_server *s) {
    if (!s) return "";
    return s->error.empty() ? s->submit_error.c_str() : s->error.c_str();
}

idash_status idash_server_close(idash_server *s) {
    if (!s) return IDASH_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->closing = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    idash_status st = IDASH_OK;
    if (!s->error.empty()) st = s->ctx->fail(IDASH_ERR_CUDA, s->error);
    for (cudaStream_t x : {s->compute, s->h2d, s->d2h})
        if (x) cudaStreamSynchronize(x);
    if (st == IDASH_OK) st = idash_sync(s->ctx);
    for (auto &kv : s->all) {
        for (Segment &g : kv.second->segs) {
            if (g.copied) cudaEventDestroy(g.copied);
            if (g.in_ready) cudaEventDestroy(g.in_ready);
        }
        if (kv.second->finished) cudaEventDestroy(kv.second->finished);
        delete kv.second;
    }
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    for (uint32_t i = 0; i < kLaunchRing; ++i) {
        if (s->launch_start[i]) cudaEventDestroy(s->launch_start[i]);
        if (s->launch_done[i]) cudaEventDestroy(s->launch_done[i]);
        cudaFree(s->d_jobs[i]);
        cudaFreeHost(s->h_jobs[i]);
    }
    if (s->t0) cudaEventDestroy(s->t0);
    for (cudaStream_t x : {s->compute, s->h2d, s->d2h})
        if (x) cudaStreamDestroy(x);
    cudaFree(s->d_counters);
    cudaFree(s->d_digest);
    cudaFreeHost(s->h_digest);
    cudaFree(s->arena_base);
    delete s;
    return st;
}

idash_status idash_serve_trlwe(idash_model *m, const idash_serve_config *cfg, const idash_request *reqs, uint64_t n,
                               idash_request_result *results, void *const *host_out) {
    if (!m || !cfg || (n && (!reqs || !results))) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kTrlwe) return ctx->fail(IDASH_ERR_STATE, "idash_serve_trlwe needs a TRLWE model");
    idash_server *s = nullptr;
    idash_status st = idash_server_open(m, cfg, &s);
    if (st != IDASH_OK) return st;
    // every request must fit before anything runs
    for (uint64_t i = 0; i < n; ++i) {
        Req probe;
        idash_serve_request r{};
        r.n_indiv = reqs[i].n_indiv;
        r.target_begin = reqs[i].target_begin;
        r.target_end = reqs[i].target_end;
        const std::string why = shape_request(s, r, &probe);
        if (!why.empty()) {
            idash_server_close(s);
            return ctx->fail(why.find("budget") != std::string::npos ? IDASH_ERR_ADMISSION : IDASH_ERR_INVALID_ARGUMENT,
                             "request " + std::to_string(i) + ": " + why);
        }
    }
    std::vector<uint64_t> tickets(n);
    for (uint64_t i = 0; i < n && st == IDASH_OK; ++i) {
        const double wait = reqs[i].arrival_s - s->now_s();
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(wait));
        idash_serve_request r{};
        r.n_indiv = reqs[i].n_indiv;
        r.target_begin = reqs[i].target_begin;
        r.target_end = reqs[i].target_end;
        r.h_out = host_out ? host_out[i] : nullptr;
        r.seed = reqs[i].seed;
        st = idash_server_submit(s, &r, &tickets[i]);
    }
    for (uint64_t i = 0; i < n && st == IDASH_OK; ++i) st = idash_server_wait(s, tickets[i], &results[i]);
    const idash_status cs = idash_server_close(s);
    return st != IDASH_OK ? st : cs;
}

uint64_t idash_digest_host(const uint32_t *words, uint64_t n_words, uint64_t index_base) {
    return digest_host(words, n_words, index_base);
}

}  // extern "C"
