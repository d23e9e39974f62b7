// C ABI (include/idash_gpu.h): contexts, resident models, the autotuner,
// CUDA-graph replay and the pipelined host-memory path.
#include <algorithm>
#include <cstring>
#include <string>
#include <thread>

#include "capi_internal.hpp"

using namespace idash;

namespace {

constexpr size_t kSmemReserve = 1024;  // per-CTA shared memory the runtime keeps
thread_local std::string g_open_error;   // why the last idash_open on this thread failed

bool aligned16(const void *p, uint64_t off) { return ((reinterpret_cast<uintptr_t>(p) + off) & 15u) == 0; }

idash_status check_layout(idash_ctx *ctx, const void *base, const idash_row_layout *l, uint64_t payload_bytes,
                          bool output) {
    if (!l) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "row layout is null");
    if (l->row_stride % 16 != 0) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "row_stride must be a multiple of 16");
    if (!aligned16(base, l->payload_offset))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "row payload (base + payload_offset) must be 16-byte aligned");
    if (l->payload_offset + payload_bytes > l->row_stride)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "payload does not fit in row_stride");
    auto overlaps = [&](int64_t off, uint64_t len) {
        return off >= 0 && (uint64_t(off) + len > l->row_stride ||
                            (uint64_t(off) < l->payload_offset + payload_bytes && uint64_t(off) + len > l->payload_offset));
    };
    if (overlaps(l->variance_offset, 8) ||
        (l->variance_offset >= 0 && ((reinterpret_cast<uintptr_t>(base) + l->variance_offset) % 8) != 0))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "variance field overlaps the payload or is misaligned");
    if (output && overlaps(l->header_offset, 8))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "header field overlaps the payload");
    return IDASH_OK;
}

template <typename T>
idash_status upload(idash_ctx *ctx, T **dst, const std::vector<T> &src) {
    *dst = nullptr;
    const size_t bytes = std::max<size_t>(src.size(), 1) * sizeof(T);
    idash_status s = ctx->check_cuda(cudaMalloc(dst, bytes), "cudaMalloc(plan)");
    if (s != IDASH_OK) return s;
    if (!src.empty()) s = ctx->check_cuda(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice),
                                          "cudaMemcpy(plan)");
    return s;
}

struct Candidate {
    KernelKind kind;
    uint32_t w, g, slots, terms, groups, cps;
    uint32_t stages = 1;  // kWs: buffers in the ring
    bool split = false;   // plan neighbourhoods larger than a window as parts
};

// Shared-memory carve-up of one buffer: a window-kernel CTA for `cps` CTAs
// per SM, or one of the two buffers of a pipe-kernel CTA (one per SM).
bool window_limits(const idash_ctx *ctx, KernelKind kind, uint32_t w, uint32_t cps, Candidate *c,
                   uint32_t stages = 1) {
    const size_t per_sm = 233472;  // 228 KB of shared memory per SM
    size_t budget = std::min(per_sm / cps - kSmemReserve, ctx->smem_optin);
    if (kind == KernelKind::kPipe) budget = (budget - 128) / 2;
    if (kind == KernelKind::kWs) budget = (budget - kWsHeaderBytes) / stages;
    const uint32_t groups = 64;
    const size_t fixed = 128 + size_t(groups) * sizeof(PlanGroup);
    if (budget <= fixed) return false;
    // a quarter of what is left for the block's terms, the rest for the window
    uint32_t terms = uint32_t((budget - fixed) / 4 / sizeof(PlanTerm));
    if (ctx->opt_max_group_terms > 0) terms = uint32_t(std::min<int64_t>(terms, ctx->opt_max_group_terms));
    const size_t left = budget - fixed - size_t(terms) * sizeof(PlanTerm);
    uint32_t slots = uint32_t(left / (size_t(w) * 4));
    if (ctx->opt_max_window_slots > 0) slots = uint32_t(std::min<int64_t>(slots, ctx->opt_max_window_slots));
    if (slots == 0) return false;
    *c = Candidate{kind, w, 3, slots, terms, groups, kind == KernelKind::kPipe ? 1u : cps, stages};
    return true;
}

uint32_t row_words_of(const idash_model *m, uint32_t n_indiv) {
    return m->form == Form::kTrlwe ? 2 * m->tp.N : n_indiv * (m->lp.n + 1);
}

// A candidate's plan, built on the host only (safe to run on several threads
// at once: it reads the model's arrays and writes nothing shared).
struct BuiltPlan {
    Plan plan;
    std::string err;
    bool index_error = false;
};

BuiltPlan make_plan(const idash_model *m, const Candidate &c) {
    PlanInput in;
    in.form = m->form;
    in.n_out = m->n_out;
    in.term_ptr = m->term_ptr.data();
    in.term_feat = m->term_feat.data();
    in.term_coef = m->term_coef.data();
    in.n_rows = m->n_in_rows;
    if (m->form == Form::kTrlwe) {
        in.one_t32 = m->tp.one_t32;
        in.N = m->tp.N;
        in.num_regions = m->tp.num_regions;
        in.region_size = m->tp.region_size;
        in.row_of_index = m->row_of_index.empty() ? nullptr : m->row_of_index.data();
        in.n_index = m->row_of_index.size();
    } else {
        in.one_t32 = m->lp.one_t32;
    }
    BuiltPlan b;
    if (c.kind == KernelKind::kTc) {
        TcLimits tl;
        tl.max_k = c.slots;
        b.err = build_tc_plan(in, tl, &b.plan, &b.index_error);
        return b;
    }
    PlanLimits lim;
    lim.group_size = c.g;
    lim.max_slots = c.slots;
    lim.max_terms = c.terms;
    lim.max_groups = c.groups;
    // batched kinds split neighbourhoods larger than one window into parts
    // (later launches accumulate); the direct kernel reads global memory
    lim.split = c.split && c.kind != KernelKind::kDirect;
    b.err = build_plan(in, lim, &b.plan, &b.index_error);
    if (b.err.empty() && (b.plan.blocks.size() >= 0xFFFFFFFFull || b.plan.terms.size() >= 0xFFFFFFFFull))
        b.err = "model too large for 32-bit plan indices";
    return b;
}

// Makes a built plan the model's: device arrays, kernel shape, CTAs.
idash_status upload_plan(idash_model *m, const Candidate &c, BuiltPlan &&b) {
    idash_ctx *ctx = m->ctx;
    if (!b.err.empty()) return ctx->fail(b.index_error ? IDASH_ERR_INDEX : IDASH_ERR_UNSUPPORTED, b.err);
    Plan plan = std::move(b.plan);
    m->drop_graph();
    m->free_device();
    idash_status s;
    if ((s = upload(ctx, &m->d_blocks, plan.blocks)) != IDASH_OK) return s;
    if ((s = upload(ctx, &m->d_slots, plan.slots)) != IDASH_OK) return s;
    if ((s = upload(ctx, &m->d_groups, plan.groups)) != IDASH_OK) return s;
    if ((s = upload(ctx, &m->d_terms, plan.terms)) != IDASH_OK) return s;
    if (c.kind == KernelKind::kTc) {
        if ((s = upload(ctx, &m->d_tc_a, plan.tc_a)) != IDASH_OK) return s;
        if ((s = upload(ctx, &m->d_tc_bias, plan.tc_bias)) != IDASH_OK) return s;
    }
    if (m->form == Form::kTrlwe) {
        if ((s = upload(ctx, &m->d_var_ptr, plan.var_ptr)) != IDASH_OK) return s;
        if ((s = upload(ctx, &m->d_var_row, plan.var_row)) != IDASH_OK) return s;
        if ((s = upload(ctx, &m->d_var_coef, plan.var_coef)) != IDASH_OK) return s;
        if (!m->out_index.empty() && (s = upload(ctx, &m->d_out_index, m->out_index)) != IDASH_OK) return s;
        if (!m->out_row.empty() && (s = upload(ctx, &m->d_out_row, m->out_row)) != IDASH_OK) return s;
    }
    m->plan = std::move(plan);
    m->kind = c.kind;
    m->slice_words = c.w;
    m->group_size = c.g;
    m->n_stages = c.stages;
    m->max_slots = m->plan.max_block_slots;
    m->max_terms = m->plan.max_block_terms;
    m->max_groups = m->plan.max_block_groups;
    uint32_t cps = c.cps;
    if (c.kind == KernelKind::kTc) {
        if (tc_smem_bytes(m->max_terms) > ctx->smem_optin)
            return ctx->fail(IDASH_ERR_UNSUPPORTED, "tensor-core plan needs more shared memory than a CTA has");
        cps = 1;  // one CTA per SM: it owns the SM's tensor memory
    } else if (c.kind != KernelKind::kDirect) {
        const size_t smem = kernel_smem_bytes(c.kind, c.w, m->max_slots, m->max_terms, m->max_groups, c.stages);
        const int occ = resident_ctas_per_sm(c.kind, c.w, c.g, smem);
        if (occ <= 0) return ctx->fail(IDASH_ERR_CUDA, "scoring kernel cannot be resident with this shared memory");
        cps = std::min<uint32_t>(cps ? cps : uint32_t(occ), uint32_t(occ));
        if (ctx->opt_ctas_per_sm > 0 && c.kind == KernelKind::kWindow)
            cps = std::min<uint32_t>(uint32_t(ctx->opt_ctas_per_sm), uint32_t(occ));
    }
    m->ctas = uint32_t(ctx->sm_count) * std::max<uint32_t>(cps, 1);
    return IDASH_OK;
}

idash_status build_and_upload(idash_model *m, const Candidate &c) { return upload_plan(m, c, make_plan(m, c)); }


ScoreArgs make_args(idash_model *m, const uint8_t *in_payload, uint64_t in_stride, uint8_t *out_payload,
                    uint64_t out_stride, uint32_t row_words, uint32_t b_lo, uint32_t b_hi, uint64_t out_lo,
                    uint64_t out_hi, uint64_t out_row_base) {
    ScoreArgs a{};
    a.blocks = m->d_blocks;
    a.slots = m->d_slots;
    a.groups = m->d_groups;
    a.terms = m->d_terms;
    a.block_lo = b_lo;
    a.n_blocks = b_hi - b_lo;
    a.row_words = row_words;
    a.n_slices = (row_words + m->slice_words - 1) / m->slice_words;
    a.n_tiles = a.n_blocks * a.n_slices;
    a.n_rows = uint32_t(std::min<uint64_t>(m->n_in_rows, 0xFFFFFFFFull));
    a.in = in_payload;
    a.in_stride = in_stride;
    a.out = out_payload;
    a.out_stride = out_stride;
    a.out_lo = out_lo;
    a.out_hi = out_hi;
    a.out_row_base = out_row_base;
    a.out_row_map = m->d_out_row;
    a.form = m->form == Form::kTrlwe ? kFormTrlwe : kFormLwe;
    a.N = m->tp.N;
    a.num_samples = m->tp.num_samples;
    a.region_size = m->tp.region_size;
    a.lwe_n1 = m->lp.n + 1;
    a.max_slots = m->max_slots;
    a.max_terms = m->max_terms;
    a.max_groups = m->max_groups;
    a.n_stages = m->n_stages;
    a.tile_counter = m->ctx->counter();
    a.err = m->ctx->d_err;
    if (m->kind == KernelKind::kTc) {
        // work units of whole column-slice runs of one block, about 32 per
        // CTA so the persistent grid balances; the block's coefficient digits
        // are loaded once per unit
        a.tc_a = m->d_tc_a;
        a.tc_bias = m->d_tc_bias;
        a.tc_a_max_bytes = uint32_t(tc_a_bytes(m->max_terms));
        const uint64_t tiles = uint64_t(a.n_blocks) * a.n_slices;
        const uint64_t want = std::max<uint64_t>(1, uint64_t(m->ctas) * 32);
        a.unit_slices = uint32_t(std::min<uint64_t>(a.n_slices, std::max<uint64_t>(1, (tiles + want - 1) / want)));
        a.units_per_block = (a.n_slices + a.unit_slices - 1) / a.unit_slices;
        a.n_units = a.n_blocks * a.units_per_block;
    }
    return a;
}

idash_status launch(idash_model *m, const ScoreArgs &a, cudaStream_t s) {
    if (uint64_t(a.n_blocks) * a.n_slices >= 0xFFFFFFFFull)
        return m->ctx->fail(IDASH_ERR_UNSUPPORTED, "too many tiles in one launch; score a smaller output range");
    if (m->kind == KernelKind::kTc && uint64_t(a.n_blocks) * a.units_per_block >= 0xFFFFFFFFull)
        return m->ctx->fail(IDASH_ERR_UNSUPPORTED, "too many work units in one launch; score a smaller output range");
    const cudaError_t e = m->kind == KernelKind::kTc
                              ? launch_score_tc(a, m->ctas, s)
                              : launch_score(m->kind, m->slice_words, m->group_size, a, m->ctas, s);
    idash_status st = m->ctx->check_cuda(e, "scoring kernel launch");
    if (st == IDASH_OK && a.n_tiles) m->ctx->stats.kernel_launches++;
    return st;
}

uint32_t n_phases(const idash_model *m) {
    return m->plan.phase_begin.size() > 1 ? uint32_t(m->plan.phase_begin.size() - 1) : 1u;
}

// Blocks [lo, hi) of phase p whose outputs intersect [o_begin, o_end).
void block_range(const idash_model *m, uint32_t p, uint64_t o_begin, uint64_t o_end, uint32_t *lo, uint32_t *hi) {
    const auto &B = m->plan.blocks;
    const auto &P = m->plan.phase_begin;
    const auto b0 = B.begin() + (P.size() > 1 ? P[p] : 0);
    const auto b1 = B.begin() + (P.size() > 1 ? P[p + 1] : B.size());
    const auto first = std::partition_point(b0, b1, [&](const PlanBlock &b) { return b.out_hi <= o_begin; });
    const auto last = std::partition_point(first, b1, [&](const PlanBlock &b) { return b.out_lo < o_end; });
    *lo = uint32_t(first - B.begin());
    *hi = uint32_t(last - B.begin());
}

// Launches the scoring kernel over every phase's blocks that touch outputs
// [o_lo, o_hi), phase by phase on `s` (later phases add to what earlier ones
// wrote); args(b_lo, b_hi) builds one launch's arguments.
template <class F>
idash_status launch_phases(idash_model *m, uint64_t o_lo, uint64_t o_hi, cudaStream_t s, F args) {
    for (uint32_t p = 0; p < n_phases(m); ++p) {
        uint32_t lo, hi;
        block_range(m, p, o_lo, o_hi, &lo, &hi);
        if (lo == hi) continue;
        ScoreArgs a = args(lo, hi);
        a.accumulate = p > 0 ? 1u : 0u;
        idash_status st = launch(m, a, s);
        if (st != IDASH_OK) return st;
    }
    return IDASH_OK;
}

// Enqueues the whole device-path TRLWE scoring (kernel + record finalize).
idash_status enqueue_trlwe(idash_model *m, const void *d_in, const idash_row_layout *il, void *d_out,
                           const idash_row_layout *ol, cudaStream_t s) {
    const uint8_t *in = static_cast<const uint8_t *>(d_in);
    uint8_t *out = static_cast<uint8_t *>(d_out);
    idash_status st = launch_phases(m, 0, m->n_out, s, [&](uint32_t lo, uint32_t hi) {
        return make_args(m, in + il->payload_offset, il->row_stride, out + ol->payload_offset, ol->row_stride,
                         row_words_of(m, 0), lo, hi, 0, m->n_out, 0);
    });
    if (st != IDASH_OK) return st;
    FinalizeArgs f{};
    f.var_ptr = m->d_var_ptr;
    f.var_row = m->d_var_row;
    f.var_coef = m->d_var_coef;
    f.out_index = m->d_out_index;
    f.out_row_map = m->d_out_row;
    f.o_begin = 0;
    f.o_end = m->n_out;
    f.in_rows = in;
    f.in_stride = il->row_stride;
    f.in_var_off = il->variance_offset;
    f.out_rows = out;
    f.out_stride = ol->row_stride;
    f.out_var_off = ol->variance_offset;
    f.out_hdr_off = ol->header_offset;
    f.tag = m->tp.record_tag;
    return m->ctx->check_cuda(launch_finalize(f, s), "finalize launch");
}

bool same_layout(const idash_row_layout &x, const idash_row_layout &y) { return std::memcmp(&x, &y, sizeof(x)) == 0; }

// Orders `waiter` after the work enqueued so far on `done` (through the
// context's event number `ev`).
idash_status stream_after(idash_ctx *ctx, cudaStream_t waiter, cudaStream_t done, size_t ev) {
    cudaEvent_t e = ctx->event(ev);
    if (!e) return ctx->fail(IDASH_ERR_CUDA, "cudaEventCreate failed");
    idash_status s = ctx->check_cuda(cudaEventRecord(e, done), "cudaEventRecord");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaStreamWaitEvent(waiter, e, 0), "cudaStreamWaitEvent");
    return s;
}

// Milliseconds per run of `reps` runs of `run` on `s` between two events;
// -1 when a run, an event or the stream fails.
template <class F>
float time_runs(cudaEvent_t e0, cudaEvent_t e1, cudaStream_t s, int reps, F run) {
    if (!e0 || !e1 || run() != IDASH_OK) return -1.f;  // the first run warms up
    if (cudaEventRecord(e0, s) != cudaSuccess) return -1.f;
    for (int r = 0; r < reps; ++r)
        if (run() != IDASH_OK) return -1.f;
    if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return -1.f;
    return ms / reps;
}

// Times `reps` runs of the current plan on the caller's buffers.
float time_candidate(idash_model *m, const void *d_in, const idash_row_layout *il, void *d_out,
                     const idash_row_layout *ol, cudaStream_t s, int reps) {
    return time_runs(m->ctx->event(0), m->ctx->event(1), s, reps,
                     [&]() { return enqueue_trlwe(m, d_in, il, d_out, ol, s); });
}

float time_candidate_lwe(idash_model *m, uint32_t n_indiv, const int32_t *d_in, uint64_t in_stride, uint64_t o_lo,
                         uint64_t o_hi, int32_t *d_out, uint64_t out_stride, cudaStream_t s, int reps) {
    const uint32_t rw = row_words_of(m, n_indiv);
    auto run = [&]() {
        return launch_phases(m, o_lo, o_hi, s, [&](uint32_t lo, uint32_t hi) {
            return make_args(m, reinterpret_cast<const uint8_t *>(d_in), in_stride * 4,
                             reinterpret_cast<uint8_t *>(d_out), out_stride * 4, rw, lo, hi, o_lo, o_hi, o_lo);
        });
    };
    return time_runs(m->ctx->event(0), m->ctx->event(1), s, reps, run);
}

std::vector<Candidate> candidates(idash_model *m) {
    idash_ctx *ctx = m->ctx;
    std::vector<Candidate> out;
    if (ctx->opt_kernel == 1) {
        const uint32_t w = ctx->opt_slice_words ? uint32_t(ctx->opt_slice_words) : 1024;
        out.push_back(Candidate{KernelKind::kDirect, w, 1, 0xFFFFFFFFu, 0xFFFFFFFFu, 8, 0});
        return out;
    }
    std::vector<uint32_t> ws;
    if (ctx->opt_slice_words) ws.push_back(uint32_t(ctx->opt_slice_words));
    else if (m->form == Form::kTrlwe) ws = {2048, 1024, 512};
    else ws = {1024, 512, 256, 128};
    std::vector<uint32_t> cpss;
    if (ctx->opt_ctas_per_sm > 0) cpss.push_back(uint32_t(ctx->opt_ctas_per_sm));
    else cpss = {1, 2};
    // the tensor-core kernel first: exact digit products on tcgen05 (TRLWE
    // with NUM_REGIONS = 1, and the LWE form), 64-column slices, K up to 192
    if ((ctx->opt_kernel == 0 || ctx->opt_kernel == 5) && (ctx->opt_slice_words == 0 || ctx->opt_slice_words == 64) &&
        (m->form == Form::kLwe || (m->form == Form::kTrlwe && m->tp.num_regions == 1))) {
        Candidate c{KernelKind::kTc, kTcSliceWords, 1, 192, 0, 0, 1};
        out.push_back(c);
    }
    if (ctx->opt_kernel == 5) return out;
    const bool window = ctx->opt_kernel == 0 || ctx->opt_kernel == 2;
    const bool pipe = ctx->opt_kernel == 0 || ctx->opt_kernel == 3;
    const bool use_ws = ctx->opt_kernel == 0 || ctx->opt_kernel == 4;
    for (uint32_t w : ws) {
        Candidate c;
        if (window)
            for (uint32_t cps : cpss)
                if (window_limits(ctx, KernelKind::kWindow, w, cps, &c)) out.push_back(c);
        if (pipe && window_limits(ctx, KernelKind::kPipe, w, 1, &c)) out.push_back(c);
        if (use_ws)  // one 512-thread CTA per SM (register file)
            for (uint32_t stages : {2u, 3u})
                if (window_limits(ctx, KernelKind::kWs, w, 1, &c, stages)) out.push_back(c);
    }
    // then the same shapes with split plans: used only when no shape fits
    // the model whole (the autotuner skips them once one has)
    if (ctx->opt_split) {
        const size_t n = out.size();
        for (size_t i = 0; i < n; ++i) {
            Candidate c = out[i];
            if (c.kind == KernelKind::kTc) continue;
            c.split = true;
            out.push_back(c);
        }
    }
    return out;
}

// Plans with the first feasible candidate (the model's default until tuned).
idash_status plan_default(idash_model *m) {
    idash_status last = IDASH_ERR_UNSUPPORTED;
    for (const Candidate &c : candidates(m)) {
        last = build_and_upload(m, c);
        if (last == IDASH_OK || last == IDASH_ERR_INDEX) return last;
    }
    if (last == IDASH_ERR_UNSUPPORTED && m->ctx->opt_kernel != 1) {
        // Neighbourhoods too large for any window: fall back to the direct kernel.
        Candidate c{KernelKind::kDirect, 512, 1, 0xFFFFFFFFu, 0xFFFFFFFFu, 8, 0};
        last = build_and_upload(m, c);
    }
    return last;
}

bool autotune_wanted(idash_model *m) { return !m->tuned && m->ctx->opt_kernel != 1 && candidates(m).size() > 1; }

// Autotuning: the candidates' plans are built on host threads, one per
// host core up to kPlanThreads at a time, then each is uploaded and timed in order by
// time_fn (milliseconds per unit, <= 0 when it failed).  Split candidates
// are tried only when no whole one worked.  The fastest becomes the model's
// plan (or the first feasible one, when none could be timed).
constexpr size_t kPlanThreads = 16;

template <typename TimeFn>
idash_status autotune(idash_model *m, TimeFn time_fn) {
    const std::vector<Candidate> cands = candidates(m);
    float best = -1.f;
    Candidate best_c{};
    BuiltPlan best_plan;
    bool stop = false;
    const size_t width = std::max<size_t>(1, std::min<size_t>(kPlanThreads, std::thread::hardware_concurrency()));
    for (size_t i = 0; i < cands.size() && !stop; i += width) {
        const size_t n = std::min(width, cands.size() - i);
        std::vector<BuiltPlan> built(n);
        std::vector<std::thread> threads;
        for (size_t k = 0; k < n; ++k)
            threads.emplace_back([&, k] { built[k] = make_plan(m, cands[i + k]); });
        for (auto &t : threads) t.join();
        for (size_t k = 0; k < n; ++k) {
            const Candidate &c = cands[i + k];
            if (c.split && best >= 0) {
                stop = true;
                break;
            }
            if (upload_plan(m, c, std::move(built[k])) != IDASH_OK) continue;
            const float ms = time_fn();
            if (ms > 0 && (best < 0 || ms < best)) {
                best = ms;
                best_c = c;
                best_plan.plan = std::move(m->plan);  // the next upload replaces the model's plan anyway
            }
        }
    }
    idash_status s = best < 0 ? plan_default(m) : upload_plan(m, best_c, std::move(best_plan));
    if (s == IDASH_OK) m->tuned = true;
    return s;
}

}  // namespace

void idash_set_thread_error(const std::string &msg) { g_open_error = msg; }

namespace idash {

cudaError_t stage_key(const int32_t *key, uint32_t N, cudaStream_t s, StagedKey *out) {
    *out = StagedKey();
    std::vector<uint32_t> words;  // positions, then values
    for (uint32_t i = 0; i < N; ++i)
        if (key[i] != 0) {
            words.push_back(i);
            out->binary = out->binary && key[i] == 1;
        }
    out->n_nz = uint32_t(words.size());
    for (uint32_t q = 0; q < out->n_nz; ++q) words.push_back(uint32_t(key[words[q]]));
    if (words.empty()) return cudaSuccess;
    cudaError_t e = cudaMallocAsync(&out->buf, words.size() * 4, s);
    if (e != cudaSuccess) return e;
    // pageable source: the copy returns once the bytes are staged
    e = cudaMemcpyAsync(out->buf, words.data(), words.size() * 4, cudaMemcpyHostToDevice, s);
    out->idx = static_cast<uint32_t *>(out->buf);
    out->val = reinterpret_cast<int32_t *>(out->idx + out->n_nz);
    return e;
}

void release_key(StagedKey *k, cudaStream_t s) {
    if (k->buf) cudaFreeAsync(k->buf, s);
    *k = StagedKey();
}

}  // namespace idash

cudaEvent_t idash_ctx::event(size_t i) {
    while (events.size() <= i) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;  // the caller's timing fails
        events.push_back(e);
    }
    return events[i];
}

void idash_model::free_device() {
    cudaFree(d_blocks);
    cudaFree(d_slots);
    cudaFree(d_groups);
    cudaFree(d_terms);
    cudaFree(d_var_ptr);
    cudaFree(d_var_row);
    cudaFree(d_var_coef);
    cudaFree(d_out_index);
    cudaFree(d_out_row);
    cudaFree(d_tc_a);
    cudaFree(d_tc_bias);
    d_tc_a = nullptr;
    d_tc_bias = nullptr;
    d_out_row = nullptr;
    d_blocks = nullptr;
    d_slots = nullptr;
    d_groups = nullptr;
    d_terms = nullptr;
    d_var_ptr = nullptr;
    d_var_row = nullptr;
    d_var_coef = nullptr;
    d_out_index = nullptr;
}

void idash_model::drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    g_in = nullptr;
    g_out = nullptr;
}

extern "C" {

const char *idash_status_string(idash_status s) {
    switch (s) {
        case IDASH_OK: return "ok";
        case IDASH_ERR_INVALID_ARGUMENT: return "invalid argument";
        case IDASH_ERR_CUDA: return "CUDA error";
        case IDASH_ERR_OUT_OF_MEMORY: return "out of memory";
        case IDASH_ERR_INDEX: return "feature index without input ciphertext";
        case IDASH_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case IDASH_ERR_IO: return "I/O error";
        case IDASH_ERR_FORMAT: return "format error";
        case IDASH_ERR_UNSUPPORTED: return "unsupported parameters";
        case IDASH_ERR_ADMISSION: return "request exceeds the HBM budget";
        case IDASH_ERR_STATE: return "invalid call order";
        case IDASH_PENDING: return "request still in flight";
    }
    return "unknown status";
}

int idash_abi_version(void) { return IDASH_GPU_ABI_VERSION; }

idash_status idash_open(idash_ctx **out, int device) {
    if (!out) return IDASH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    idash_ctx *ctx = new idash_ctx();
    ctx->device = device;
    idash_status s = ctx->check_cuda(cudaSetDevice(device), "cudaSetDevice");
    cudaDeviceProp prop{};
    if (s == IDASH_OK) s = ctx->check_cuda(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (s == IDASH_OK && prop.major < 10) {
        ctx->last_error = "device is not a Blackwell (sm_100+) GPU";
        s = IDASH_ERR_UNSUPPORTED;
    }
    if (s == IDASH_OK) {
        ctx->sm_count = prop.multiProcessorCount;
        ctx->smem_optin = prop.sharedMemPerBlockOptin;
        s = ctx->check_cuda(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    if (s == IDASH_OK) s = ctx->check_cuda(configure_window_kernels(ctx->smem_optin), "configure kernels");
    if (s == IDASH_OK) s = ctx->check_cuda(configure_tc_kernel(ctx->smem_optin), "configure tensor-core kernel");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking), "cudaStreamCreate");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking), "cudaStreamCreate");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaEventCreateWithFlags(&ctx->join_in, cudaEventDisableTiming), "cudaEventCreate");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaEventCreateWithFlags(&ctx->join_out, cudaEventDisableTiming), "cudaEventCreate");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaMalloc(&ctx->d_err, sizeof(uint32_t)), "cudaMalloc(err)");
    if (s == IDASH_OK)
        s = ctx->check_cuda(cudaMalloc(&ctx->d_counters, sizeof(uint32_t) * idash_ctx::kCounters), "cudaMalloc(counters)");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaMemset(ctx->d_err, 0, sizeof(uint32_t)), "cudaMemset");
    if (s != IDASH_OK) {
        g_open_error = ctx->last_error;
        idash_close(ctx);
        return s;
    }
    *out = ctx;
    return IDASH_OK;
}

void idash_close(idash_ctx *ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    while (!ctx->models.empty()) idash_model_free(*ctx->models.begin());
    for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
    if (ctx->join_in) cudaEventDestroy(ctx->join_in);
    if (ctx->join_out) cudaEventDestroy(ctx->join_out);
    cudaFree(ctx->d_err);
    cudaFree(ctx->d_counters);
    cudaFree(ctx->d_in_buf);
    cudaFree(ctx->d_out_buf);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->h2d) cudaStreamDestroy(ctx->h2d);
    if (ctx->d2h) cudaStreamDestroy(ctx->d2h);
    delete ctx;
}

const char *idash_last_error(const idash_ctx *ctx) { return ctx ? ctx->last_error.c_str() : g_open_error.c_str(); }

void *idash_stream(idash_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

idash_status idash_sync(idash_ctx *ctx) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    idash_status s = ctx->check_cuda(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    if (s != IDASH_OK) return s;
    uint32_t err = 0;
    s = ctx->check_cuda(cudaMemcpy(&err, ctx->d_err, sizeof(err), cudaMemcpyDeviceToHost), "read error word");
    if (s != IDASH_OK) return s;
    if (err != kDevOk) {
        cudaMemset(ctx->d_err, 0, sizeof(uint32_t));
        if (err == kDevTimeout) return ctx->fail(IDASH_ERR_DEVICE_TIMEOUT, "a device-side wait expired");
        return ctx->fail(IDASH_ERR_INDEX, "a kernel met an input row outside its buffer");
    }
    return IDASH_OK;
}

idash_status idash_set_option(idash_ctx *ctx, const char *name, int64_t value) {
    if (!ctx || !name) return IDASH_ERR_INVALID_ARGUMENT;
    const std::string n(name);
    if (n == "kernel") {
        if (value < 0 || value > 5) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "kernel must be 0 .. 5");
        ctx->opt_kernel = value;
    } else if (n == "slice_words") {
        if (value != 0 && value != int64_t(kTcSliceWords) && !slice_supported(uint32_t(value)))
            return ctx->fail(IDASH_ERR_INVALID_ARGUMENT,
                             "slice_words must be 0, 64 (tensor-core kernel), 128, 256, 512, 1024 or 2048");
        ctx->opt_slice_words = value;
    } else if (n == "ctas_per_sm") {
        if (value < 0 || value > 8) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "ctas_per_sm must be in [0, 8]");
        ctx->opt_ctas_per_sm = value;
    } else if (n == "graph") {
        ctx->opt_graph = value ? 1 : 0;
    } else if (n == "max_window_slots") {
        if (value < 0) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "max_window_slots must be >= 0");
        ctx->opt_max_window_slots = value;
    } else if (n == "max_group_terms") {
        if (value < 0) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "max_group_terms must be >= 0");
        ctx->opt_max_group_terms = value;
    } else if (n == "split") {
        ctx->opt_split = value ? 1 : 0;
    } else {
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "unknown option " + n);
    }
    return IDASH_OK;
}

idash_status idash_get_option(const idash_ctx *ctx, const char *name, int64_t *value) {
    if (!ctx || !name || !value) return IDASH_ERR_INVALID_ARGUMENT;
    const std::string n(name);
    if (n == "kernel") *value = ctx->opt_kernel;
    else if (n == "slice_words") *value = ctx->opt_slice_words;
    else if (n == "ctas_per_sm") *value = ctx->opt_ctas_per_sm;
    else if (n == "graph") *value = ctx->opt_graph;
    else if (n == "max_window_slots") *value = ctx->opt_max_window_slots;
    else if (n == "max_group_terms") *value = ctx->opt_max_group_terms;
    else if (n == "split") *value = ctx->opt_split;
    else return IDASH_ERR_INVALID_ARGUMENT;
    return IDASH_OK;
}

idash_status idash_get_stats(const idash_ctx *ctx, idash_stats *out) {
    if (!ctx || !out) return IDASH_ERR_INVALID_ARGUMENT;
    *out = ctx->stats;
    return IDASH_OK;
}

idash_status idash_device_alloc(idash_ctx *ctx, size_t bytes, void **ptr) {
    if (!ctx || !ptr) return IDASH_ERR_INVALID_ARGUMENT;
    *ptr = nullptr;
    return ctx->check_cuda(cudaMalloc(ptr, std::max<size_t>(bytes, 1)), "cudaMalloc");
}
idash_status idash_device_free(idash_ctx *ctx, void *ptr) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(ctx->stream);
    return ctx->check_cuda(cudaFree(ptr), "cudaFree");
}
idash_status idash_host_alloc(idash_ctx *ctx, size_t bytes, void **ptr) {
    if (!ctx || !ptr) return IDASH_ERR_INVALID_ARGUMENT;
    *ptr = nullptr;
    return ctx->check_cuda(cudaMallocHost(ptr, std::max<size_t>(bytes, 1)), "cudaMallocHost");
}
idash_status idash_host_free(idash_ctx *ctx, void *ptr) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    return ctx->check_cuda(cudaFreeHost(ptr), "cudaFreeHost");
}
idash_status idash_copy_h2d(idash_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    idash_status s = ctx->check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaStreamSynchronize(ctx->stream), "h2d sync");
    return s;
}
idash_status idash_copy_d2h(idash_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    idash_status s = ctx->check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "d2h");
    if (s == IDASH_OK) s = ctx->check_cuda(cudaStreamSynchronize(ctx->stream), "d2h sync");
    return s;
}
idash_status idash_memset_device(idash_ctx *ctx, void *dst, int value, size_t bytes) {
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    return ctx->check_cuda(cudaMemsetAsync(dst, value, bytes, ctx->stream), "memset");
}

idash_status idash_model_trlwe(idash_ctx *ctx, idash_model **model, const idash_trlwe_params *p, uint64_t n_out,
                               const uint32_t *out_index, const uint32_t *out_row, const uint64_t *term_ptr,
                               const uint32_t *term_feat, const int32_t *term_coef, uint64_t n_in_index,
                               const uint32_t *in_row_of_index, uint64_t n_in_rows) {
    if (!ctx || !model || !p || (n_out && !term_ptr)) return IDASH_ERR_INVALID_ARGUMENT;
    *model = nullptr;
    if (p->k != 1) return ctx->fail(IDASH_ERR_UNSUPPORTED, "only k = 1 TRLWE is supported (eval/idash.cpp:768)");
    if (p->N == 0 || p->N % 256 != 0 || p->N > 4096)
        return ctx->fail(IDASH_ERR_UNSUPPORTED, "N must be a multiple of 256 up to 4096");
    if (p->num_regions == 0 || p->region_size == 0 || uint64_t(p->num_regions) * p->region_size > p->N ||
        p->num_samples > p->region_size)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT,
                         "need NUM_REGIONS*REGION_SIZE <= N and NUM_SAMPLES <= REGION_SIZE (eval/idash.cpp:409-412)");
    const uint64_t nnz = n_out ? term_ptr[n_out] : 0;
    if (nnz && (!term_feat || !term_coef)) return IDASH_ERR_INVALID_ARGUMENT;
    idash_model *m = new idash_model();
    m->ctx = ctx;
    m->form = Form::kTrlwe;
    m->tp = *p;
    m->n_out = n_out;
    m->n_in_rows = n_in_rows;
    m->term_ptr.assign(term_ptr, term_ptr + (n_out ? n_out + 1 : 0));
    if (m->term_ptr.empty()) m->term_ptr.push_back(0);
    m->term_feat.assign(term_feat, term_feat + nnz);
    m->term_coef.assign(term_coef, term_coef + nnz);
    if (out_index) m->out_index.assign(out_index, out_index + n_out);
    if (out_row) {
        std::vector<uint8_t> hit(n_out, 0);
        for (uint64_t o = 0; o < n_out; ++o) {
            if (out_row[o] >= n_out || hit[out_row[o]]) {
                idash_model_free(m);
                return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "out_row must be a permutation of [0, n_out)");
            }
            hit[out_row[o]] = 1;
        }
        m->out_row.assign(out_row, out_row + n_out);
    }
    if (in_row_of_index) m->row_of_index.assign(in_row_of_index, in_row_of_index + n_in_index);
    idash_status s = plan_default(m);
    if (s != IDASH_OK) {
        idash_model_free(m);
        return s;
    }
    ctx->models.insert(m);
    *model = m;
    return IDASH_OK;
}

idash_status idash_model_lwe(idash_ctx *ctx, idash_model **model, const idash_lwe_params *p, uint64_t n_out,
                             const uint64_t *term_ptr, const uint32_t *term_feat, const int32_t *term_coef,
                             uint64_t n_feat_rows) {
    if (!ctx || !model || !p || (n_out && !term_ptr)) return IDASH_ERR_INVALID_ARGUMENT;
    *model = nullptr;
    if (p->n == 0 || p->n_indiv == 0 || uint64_t(p->n_indiv) * (p->n + 1) >= (1ull << 31))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "LWE row (n_indiv * (n+1) words) must be non-empty and < 2^31");
    const uint64_t nnz = n_out ? term_ptr[n_out] : 0;
    if (nnz && (!term_feat || !term_coef)) return IDASH_ERR_INVALID_ARGUMENT;
    idash_model *m = new idash_model();
    m->ctx = ctx;
    m->form = Form::kLwe;
    m->lp = *p;
    m->n_out = n_out;
    m->n_in_rows = n_feat_rows;
    m->term_ptr.assign(term_ptr, term_ptr + (n_out ? n_out + 1 : 0));
    if (m->term_ptr.empty()) m->term_ptr.push_back(0);
    m->term_feat.assign(term_feat, term_feat + nnz);
    m->term_coef.assign(term_coef, term_coef + nnz);
    idash_status s = plan_default(m);
    if (s != IDASH_OK) {
        idash_model_free(m);
        return s;
    }
    ctx->models.insert(m);
    *model = m;
    return IDASH_OK;
}

idash_status idash_model_get_info(const idash_model *m, idash_model_info *info) {
    if (!m || !info) return IDASH_ERR_INVALID_ARGUMENT;
    info->n_out = m->n_out;
    info->n_terms = m->plan.n_terms_in;
    info->n_groups = m->plan.groups.size();
    info->n_blocks = m->plan.blocks.size();
    info->n_slots = m->plan.slots.size();
    info->slice_words = m->slice_words;
    info->max_window_slots = m->max_slots;
    info->kernel = uint32_t(m->kind);
    info->algorithmic_in_rows = m->plan.distinct_rows;
    info->dense_k = 0;
    if (m->kind == KernelKind::kTc)
        for (const PlanBlock &b : m->plan.blocks) info->dense_k += b.n_groups;
    return IDASH_OK;
}

idash_status idash_model_replan(idash_model *m) {
    if (!m) return IDASH_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(m->ctx->stream);
    m->tuned = false;
    return plan_default(m);
}

void idash_model_free(idash_model *m) {
    if (!m) return;
    if (m->ctx) {
        if (m->ctx->stream) cudaStreamSynchronize(m->ctx->stream);
        m->ctx->models.erase(m);
    }
    m->free_intpoly();
    m->drop_graph();
    m->free_device();
    delete m;
}

idash_status idash_score_trlwe_device(idash_model *m, const void *d_in, const idash_row_layout *il, void *d_out,
                                      const idash_row_layout *ol, void *stream) {
    if (!m || !d_in || !d_out || !il || !ol) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kTrlwe) return ctx->fail(IDASH_ERR_STATE, "model is not a TRLWE model");
    const uint64_t payload = uint64_t(2) * m->tp.N * 4;
    idash_status s = check_layout(ctx, d_in, il, payload, false);
    if (s == IDASH_OK) s = check_layout(ctx, d_out, ol, payload, true);
    if (s != IDASH_OK) return s;
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    cudaStream_t cs = ctx->stream;
    if (user && user != cs) {
        if ((s = ctx->check_cuda(cudaEventRecord(ctx->join_in, user), "join")) != IDASH_OK) return s;
        if ((s = ctx->check_cuda(cudaStreamWaitEvent(cs, ctx->join_in, 0), "join")) != IDASH_OK) return s;
    }
    if (autotune_wanted(m)) {
        // Autotune on the caller's buffers: plan every candidate, time it, keep the best.
        if ((s = autotune(m, [&]() { return time_candidate(m, d_in, il, d_out, ol, cs, 3); })) != IDASH_OK) return s;
    }
    if (ctx->opt_graph) {
        if (!(m->graph && m->g_in == d_in && m->g_out == d_out && same_layout(m->g_in_layout, *il) &&
              same_layout(m->g_out_layout, *ol))) {
            m->drop_graph();
            cudaGraph_t g = nullptr;
            if ((s = ctx->check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture")) != IDASH_OK)
                return s;
            idash_status es = enqueue_trlwe(m, d_in, il, d_out, ol, cs);
            cudaError_t ce = cudaStreamEndCapture(cs, &g);
            if (es != IDASH_OK) {
                if (g) cudaGraphDestroy(g);
                return es;
            }
            if ((s = ctx->check_cuda(ce, "end capture")) != IDASH_OK) return s;
            s = ctx->check_cuda(cudaGraphInstantiate(&m->graph, g, 0), "graph instantiate");
            cudaGraphDestroy(g);
            if (s != IDASH_OK) return s;
            m->g_in = d_in;
            m->g_out = d_out;
            m->g_in_layout = *il;
            m->g_out_layout = *ol;
        }
        if ((s = ctx->check_cuda(cudaGraphLaunch(m->graph, cs), "graph launch")) != IDASH_OK) return s;
        ctx->stats.graph_launches++;
        ctx->stats.kernel_launches++;
    } else {
        if ((s = enqueue_trlwe(m, d_in, il, d_out, ol, cs)) != IDASH_OK) return s;
    }
    if (user && user != cs) {
        if ((s = ctx->check_cuda(cudaEventRecord(ctx->join_out, cs), "join")) != IDASH_OK) return s;
        if ((s = ctx->check_cuda(cudaStreamWaitEvent(user, ctx->join_out, 0), "join")) != IDASH_OK) return s;
    }
    return IDASH_OK;
}

idash_status idash_score_trlwe_host(idash_model *m, const void *h_in, const idash_row_layout *il, uint64_t n_in_rows,
                                    void *h_out, const idash_row_layout *ol) {
    if (!m || !h_in || !h_out || !il || !ol) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kTrlwe) return ctx->fail(IDASH_ERR_STATE, "model is not a TRLWE model");
    if (n_in_rows < m->n_in_rows) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "fewer input rows than the model reads");
    if (!m->out_row.empty())
        return ctx->fail(IDASH_ERR_STATE, "the host-memory path writes output o to row o (model has out_row)");
    const uint64_t payload = uint64_t(2) * m->tp.N * 4;
    idash_status s = check_layout(ctx, h_in, il, payload, false);
    if (s == IDASH_OK) s = check_layout(ctx, h_out, ol, payload, true);
    if (s != IDASH_OK) return s;
    // Device copies keep the host buffers' alignment phase mod 16.
    const uint64_t in_shift = reinterpret_cast<uintptr_t>(h_in) & 15u;
    const uint64_t out_shift = reinterpret_cast<uintptr_t>(h_out) & 15u;
    const uint64_t in_bytes = n_in_rows * il->row_stride, out_bytes = m->n_out * ol->row_stride;
    if (ctx->d_in_cap < in_bytes + 16) {
        cudaFree(ctx->d_in_buf);
        ctx->d_in_buf = nullptr;
        ctx->d_in_cap = 0;
        if ((s = ctx->check_cuda(cudaMalloc(&ctx->d_in_buf, in_bytes + 16), "cudaMalloc(input)")) != IDASH_OK) return s;
        ctx->d_in_cap = in_bytes + 16;
    }
    if (ctx->d_out_cap < out_bytes + 16) {
        cudaFree(ctx->d_out_buf);
        ctx->d_out_buf = nullptr;
        ctx->d_out_cap = 0;
        if ((s = ctx->check_cuda(cudaMalloc(&ctx->d_out_buf, out_bytes + 16), "cudaMalloc(output)")) != IDASH_OK)
            return s;
        ctx->d_out_cap = out_bytes + 16;
    }
    uint8_t *d_in = ctx->d_in_buf + in_shift;
    uint8_t *d_out = ctx->d_out_buf + out_shift;
    const uint8_t *host_in = static_cast<const uint8_t *>(h_in);
    uint8_t *host_out = static_cast<uint8_t *>(h_out);
    if (autotune_wanted(m)) {
        // tune once on the device copies of this call's inputs
        if ((s = ctx->check_cuda(cudaMemcpyAsync(d_in, host_in, in_bytes, cudaMemcpyHostToDevice, ctx->stream), "h2d")) !=
            IDASH_OK)
            return s;
        if ((s = idash_score_trlwe_device(m, d_in, il, d_out, ol, nullptr)) != IDASH_OK) return s;
        if ((s = ctx->check_cuda(cudaStreamSynchronize(ctx->stream), "sync")) != IDASH_OK) return s;
    }

    // Chunks of whole phase-0 blocks (which cover every output once); each
    // chunk waits only for the input rows it reads, its later-phase parts
    // run after it, and its outputs stream back while later chunks compute.
    const uint32_t nb = m->plan.phase_begin.size() > 1 ? m->plan.phase_begin[1] : uint32_t(m->plan.blocks.size());
    const uint32_t n_chunks = std::max<uint32_t>(1, std::min<uint32_t>(nb, 12));
    std::vector<uint32_t> cb(n_chunks + 1);
    for (uint32_t c = 0; c <= n_chunks; ++c) cb[c] = uint32_t(uint64_t(nb) * c / n_chunks);
    // input rows needed by each chunk (prefix maximum of the blocks' rows)
    uint64_t rows_sent = 0;
    const uint32_t row_words = row_words_of(m, 0);
    size_t ev = 2;
    for (uint32_t c = 0; c < n_chunks; ++c) {
        uint32_t need = 0;
        for (uint32_t b = cb[c]; b < cb[c + 1]; ++b) need = std::max(need, m->plan.block_max_row[b] + 1);
        if (cb[c + 1] > cb[c])
            for (uint32_t p = 1; p < n_phases(m); ++p) {
                uint32_t lo, hi;
                block_range(m, p, m->plan.blocks[cb[c]].out_lo, m->plan.blocks[cb[c + 1] - 1].out_hi, &lo, &hi);
                for (uint32_t b = lo; b < hi; ++b) need = std::max(need, m->plan.block_max_row[b] + 1);
            }
        if (need > rows_sent) {
            // send the rows in [rows_sent, need) plus a lookahead of the next chunk's share
            uint64_t upto = std::min<uint64_t>(n_in_rows, std::max<uint64_t>(need, rows_sent + (n_in_rows + n_chunks - 1) / n_chunks));
            if (c == n_chunks - 1) upto = std::max<uint64_t>(upto, need);
            s = ctx->check_cuda(cudaMemcpyAsync(d_in + rows_sent * il->row_stride, host_in + rows_sent * il->row_stride,
                                                (upto - rows_sent) * il->row_stride, cudaMemcpyHostToDevice, ctx->h2d),
                                "h2d chunk");
            if (s != IDASH_OK) return s;
            ctx->stats.h2d_bytes += (upto - rows_sent) * il->row_stride;
            rows_sent = upto;
            if ((s = stream_after(ctx, ctx->stream, ctx->h2d, ev++)) != IDASH_OK) return s;
        }
        if (cb[c + 1] == cb[c]) continue;
        const uint64_t o_lo = m->plan.blocks[cb[c]].out_lo, o_hi = m->plan.blocks[cb[c + 1] - 1].out_hi;
        s = launch_phases(m, o_lo, o_hi, ctx->stream, [&](uint32_t lo, uint32_t hi) {
            ScoreArgs a = make_args(m, d_in + il->payload_offset, il->row_stride, d_out + ol->payload_offset,
                                    ol->row_stride, row_words, lo, hi, o_lo, o_hi, 0);
            a.out_row_map = nullptr;
            return a;
        });
        if (s != IDASH_OK) return s;
        FinalizeArgs f{};
        f.var_ptr = m->d_var_ptr;
        f.var_row = m->d_var_row;
        f.var_coef = m->d_var_coef;
        f.out_index = m->d_out_index;
        f.out_row_map = nullptr;
        f.o_begin = o_lo;
        f.o_end = o_hi;
        f.in_rows = d_in;
        f.in_stride = il->row_stride;
        f.in_var_off = il->variance_offset;
        f.out_rows = d_out;
        f.out_stride = ol->row_stride;
        f.out_var_off = ol->variance_offset;
        f.out_hdr_off = ol->header_offset;
        f.tag = m->tp.record_tag;
        if ((s = ctx->check_cuda(launch_finalize(f, ctx->stream), "finalize")) != IDASH_OK) return s;
        if ((s = stream_after(ctx, ctx->d2h, ctx->stream, ev++)) != IDASH_OK) return s;
        s = ctx->check_cuda(cudaMemcpyAsync(host_out + o_lo * ol->row_stride, d_out + o_lo * ol->row_stride,
                                            (o_hi - o_lo) * ol->row_stride, cudaMemcpyDeviceToHost, ctx->d2h),
                            "d2h chunk");
        if (s != IDASH_OK) return s;
        ctx->stats.d2h_bytes += (o_hi - o_lo) * ol->row_stride;
    }
    (void)row_words;
    if ((s = ctx->check_cuda(cudaStreamSynchronize(ctx->d2h), "d2h sync")) != IDASH_OK) return s;
    if ((s = ctx->check_cuda(cudaStreamSynchronize(ctx->h2d), "h2d sync")) != IDASH_OK) return s;
    return idash_sync(ctx);
}

idash_status idash_model_input_rows(const idash_model *m, uint64_t out_begin, uint64_t out_end, uint64_t *row_begin,
                                    uint64_t *row_end) {
    if (!m || !row_begin || !row_end || out_begin > out_end || out_end > m->n_out) return IDASH_ERR_INVALID_ARGUMENT;
    uint64_t lo = UINT64_MAX, hi = 0;
    for (uint32_t p = 0; p < n_phases(m); ++p) {
        uint32_t b_lo, b_hi;
        block_range(m, p, out_begin, out_end, &b_lo, &b_hi);
        for (uint32_t b = b_lo; b < b_hi; ++b) {
            if (m->plan.blocks[b].n_slots == 0) continue;
            lo = std::min<uint64_t>(lo, m->plan.block_min_row[b]);
            hi = std::max<uint64_t>(hi, uint64_t(m->plan.block_max_row[b]) + 1);
        }
    }
    if (lo == UINT64_MAX) lo = hi = 0;
    *row_begin = lo;
    *row_end = hi;
    return IDASH_OK;
}

}  // extern "C"

namespace idash {

idash_status score_trlwe_range(idash_model *m, uint64_t out_begin, uint64_t out_end, uint32_t num_samples,
                               const void *d_in, const idash_row_layout *il, uint64_t in_row_base, uint64_t n_in_rows,
                               void *d_out, const idash_row_layout *ol, void *stream, uint64_t *digest,
                               uint64_t digest_base, bool *fused) {
    if (fused) *fused = false;
    if (!m || !d_in || !d_out || !il || !ol) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kTrlwe) return ctx->fail(IDASH_ERR_STATE, "model is not a TRLWE model");
    if (out_begin > out_end || out_end > m->n_out) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "bad output range");
    if (num_samples > m->tp.region_size)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "num_samples must not exceed REGION_SIZE");
    if (in_row_base > 0xFFFFFFFFull || n_in_rows > 0xFFFFFFFFull)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "input rows beyond 32-bit indices");
    const uint64_t payload = uint64_t(2) * m->tp.N * 4;
    idash_status s = check_layout(ctx, d_in, il, payload, false);
    if (s == IDASH_OK) s = check_layout(ctx, d_out, ol, payload, true);
    if (s != IDASH_OK) return s;
    if (out_begin == out_end) return IDASH_OK;
    uint64_t r_lo, r_hi;
    idash_model_input_rows(m, out_begin, out_end, &r_lo, &r_hi);
    if (r_hi > r_lo && (r_lo < in_row_base || r_hi > in_row_base + n_in_rows))
        return ctx->fail(IDASH_ERR_INDEX, "the outputs read input rows outside [in_row_base, in_row_base + n_in_rows)");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const uint8_t *in = static_cast<const uint8_t *>(d_in);
    uint8_t *out = static_cast<uint8_t *>(d_out);
    // The digest rides in the scoring kernel when every output word is
    // written once, by one launch, into dense rows (word c of row r is word
    // r * 2N + c of the output image).
    const bool fuse = digest && n_phases(m) == 1 && ol->payload_offset == 0 && ol->row_stride == payload &&
                      ol->variance_offset < 0 && ol->header_offset < 0 && digest_base % 4 == 0 &&
                      digest_fusable(m->kind, m->slice_words, m->group_size);
    s = launch_phases(m, out_begin, out_end, st, [&](uint32_t lo, uint32_t hi) {
        ScoreArgs a = make_args(m, in + il->payload_offset, il->row_stride, out + ol->payload_offset, ol->row_stride,
                                row_words_of(m, 0), lo, hi, out_begin, out_end, out_begin);
        a.out_row_map = nullptr;
        a.row_base = uint32_t(in_row_base);
        a.n_rows = uint32_t(n_in_rows);
        if (num_samples) a.num_samples = num_samples;
        if (fuse) {
            a.digest = reinterpret_cast<unsigned long long *>(digest);
            a.digest_base = digest_base;
        }
        return a;
    });
    if (s != IDASH_OK) return s;
    if (fused) *fused = fuse;
    FinalizeArgs f{};
    f.var_ptr = m->d_var_ptr;
    f.var_row = m->d_var_row;
    f.var_coef = m->d_var_coef;
    f.out_index = m->d_out_index;
    f.out_row_map = nullptr;
    f.o_begin = out_begin;
    f.o_end = out_end;
    f.in_rows = in;
    f.in_row_base = uint32_t(in_row_base);
    f.in_stride = il->row_stride;
    f.in_var_off = il->variance_offset;
    f.out_rows = out;
    f.out_row_base = out_begin;
    f.out_stride = ol->row_stride;
    f.out_var_off = ol->variance_offset;
    f.out_hdr_off = ol->header_offset;
    f.tag = m->tp.record_tag;
    return ctx->check_cuda(launch_finalize(f, st), "finalize launch");
}

}  // namespace idash

extern "C" {

idash_status idash_score_trlwe_range(idash_model *m, uint64_t out_begin, uint64_t out_end, uint32_t num_samples,
                                     const void *d_in, const idash_row_layout *il, uint64_t in_row_base,
                                     uint64_t n_in_rows, void *d_out, const idash_row_layout *ol, void *stream) {
    return score_trlwe_range(m, out_begin, out_end, num_samples, d_in, il, in_row_base, n_in_rows, d_out, ol, stream,
                             nullptr, 0, nullptr);
}

idash_status idash_score_lwe_device(idash_model *m, uint32_t n_indiv, const int32_t *d_in, uint64_t in_row_stride,
                                    uint64_t out_begin, uint64_t out_end, int32_t *d_out, uint64_t out_row_stride,
                                    void *stream) {
    if (!m || !d_in || !d_out) return IDASH_ERR_INVALID_ARGUMENT;
    idash_ctx *ctx = m->ctx;
    if (m->form != Form::kLwe) return ctx->fail(IDASH_ERR_STATE, "model is not an LWE model");
    if (n_indiv == 0 || n_indiv > m->lp.n_indiv)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "n_indiv must be in [1, model n_indiv]");
    const uint64_t L = uint64_t(n_indiv) * (m->lp.n + 1);
    const uint64_t Lpad = (L + 3) & ~3ull;
    if (in_row_stride < Lpad || in_row_stride % 4 || out_row_stride < L || out_row_stride % 4)
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "row strides must be multiples of 4 words covering n_indiv*(n+1)");
    if (!aligned16(d_in, 0) || !aligned16(d_out, 0))
        return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "LWE buffers must be 16-byte aligned");
    if (out_begin > out_end || out_end > m->n_out) return ctx->fail(IDASH_ERR_INVALID_ARGUMENT, "bad output range");
    if (out_begin == out_end) return IDASH_OK;
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    cudaStream_t cs = ctx->stream;
    idash_status s;
    if (user && user != cs) {
        if ((s = ctx->check_cuda(cudaEventRecord(ctx->join_in, user), "join")) != IDASH_OK) return s;
        if ((s = ctx->check_cuda(cudaStreamWaitEvent(cs, ctx->join_in, 0), "join")) != IDASH_OK) return s;
    }
    if (autotune_wanted(m)) {
        // tune on (at most) the first ~64 phase-0 blocks of this range, per output
        s = autotune(m, [&]() -> float {
            uint32_t b_lo, b_hi;
            block_range(m, 0, out_begin, out_end, &b_lo, &b_hi);
            if (b_hi == b_lo) return -1.f;
            const uint32_t hi = std::min<uint32_t>(b_hi, b_lo + 64);
            const uint64_t o_hi = std::min<uint64_t>(out_end, m->plan.blocks[hi - 1].out_hi);
            const float ms = time_candidate_lwe(m, n_indiv, d_in, in_row_stride, out_begin, o_hi, d_out,
                                                out_row_stride, cs, 2);
            return ms <= 0 ? -1.f : ms / float(o_hi - out_begin);
        });
        if (s != IDASH_OK) return s;
    }
    const uint32_t rw = row_words_of(m, n_indiv);
    const uint32_t n_slices = (rw + m->slice_words - 1) / m->slice_words;
    // split so each launch stays below 2^31 tiles; phases in order
    const uint32_t per_launch = std::max<uint32_t>(1, uint32_t((1ull << 30) / n_slices));
    for (uint32_t p = 0; p < n_phases(m); ++p) {
        uint32_t b_lo, b_hi;
        block_range(m, p, out_begin, out_end, &b_lo, &b_hi);
        for (uint32_t lo = b_lo; lo < b_hi; lo += per_launch) {
            const uint32_t hi = std::min(b_hi, lo + per_launch);
            ScoreArgs a = make_args(m, reinterpret_cast<const uint8_t *>(d_in), in_row_stride * 4,
                                    reinterpret_cast<uint8_t *>(d_out), out_row_stride * 4, rw, lo, hi, out_begin,
                                    out_end, out_begin);
            a.accumulate = p > 0 ? 1u : 0u;
            if ((s = launch(m, a, cs)) != IDASH_OK) return s;
        }
    }
    if (user && user != cs) {
        if ((s = ctx->check_cuda(cudaEventRecord(ctx->join_out, cs), "join")) != IDASH_OK) return s;
        if ((s = ctx->check_cuda(cudaStreamWaitEvent(user, ctx->join_out, 0), "join")) != IDASH_OK) return s;
    }
    return IDASH_OK;
}

}  // extern "C"
