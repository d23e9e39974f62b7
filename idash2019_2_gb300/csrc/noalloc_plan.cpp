// Host half of idash_score_trlwe_noalloc: planning and the scratch layout
// (noalloc_plan.hpp).
#include "noalloc_plan.hpp"

#include <algorithm>

namespace idash {

namespace {

constexpr size_t kSmemPerSm = 233472;  // 228 KB of shared memory per SM
constexpr size_t kSmemReserve = 1024;  // per CTA, kept by the runtime
constexpr size_t kWindowHeader = 128;  // window kernel: barrier and tile word before the buffer
constexpr uint32_t kGroups = 64;       // groups per block
// PlanBlock, PlanSlot, PlanGroup and PlanTerm sizes as the kernels read them
constexpr size_t kTermBytes = 16, kGroupBytes = 32, kBlockBytes = 32, kSlotBytes = 8;
static_assert(sizeof(PlanTerm) == kTermBytes && sizeof(PlanGroup) == kGroupBytes &&
                  sizeof(PlanBlock) == kBlockBytes && sizeof(PlanSlot) == kSlotBytes,
              "plan table layouts");

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

std::string plan_noalloc(const PlanInput &in, size_t smem_optin, bool with_variance, bool with_index,
                         NoallocPlan *out, bool *index_error) {
    *index_error = false;
    std::string err;
    out->window = false;
    for (uint32_t w : {1024u, 512u, 256u}) {
        // two CTAs per SM: half of the SM's shared memory each
        const size_t budget = std::min(kSmemPerSm / 2 - kSmemReserve, smem_optin);
        const size_t fixed = kWindowHeader + kGroups * kGroupBytes;
        PlanLimits lim;
        lim.group_size = 3;
        lim.max_groups = kGroups;
        lim.max_terms = uint32_t((budget - fixed) / 4 / kTermBytes);
        lim.max_slots = uint32_t((budget - fixed - lim.max_terms * kTermBytes) / (size_t(w) * 4));
        err = build_plan(in, lim, &out->plan, index_error);
        if (err.empty()) {
            out->window = true;
            out->slice_words = w;
            out->group_size = 3;
            break;
        }
        if (*index_error) return err;
    }
    if (!out->window) {
        // a neighbourhood larger than any window: the direct kernel, which
        // reads each term's row from global memory
        PlanLimits lim;
        lim.group_size = 1;
        lim.max_slots = lim.max_terms = 0xFFFFFFFFu;
        lim.max_groups = 8;
        err = build_plan(in, lim, &out->plan, index_error);
        if (!err.empty()) return err;
        out->slice_words = 512;
        out->group_size = 1;
    }

    const Plan &p = out->plan;
    size_t off = 256;  // error word and tile counter
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off = align256(off + std::max<size_t>(bytes, 1));
        return at;
    };
    out->o_blocks = take(p.blocks.size() * kBlockBytes);
    out->o_slots = take(p.slots.size() * kSlotBytes);
    out->o_groups = take(p.groups.size() * kGroupBytes);
    out->o_terms = take(p.terms.size() * kTermBytes);
    if (with_variance) {
        out->o_var_ptr = take(p.var_ptr.size() * 8);
        out->o_var_row = take(p.var_row.size() * 4);
        out->o_var_coef = take(p.var_coef.size() * 4);
    }
    if (with_index) out->o_out_index = take(in.n_out * 4);
    out->bytes = off;
    if (off > kNoallocScratchBytes)
        return "model needs " + std::to_string((off + (1 << 20) - 1) >> 20) +
               " MiB of scratch; the no-allocation entry point holds " +
               std::to_string(kNoallocScratchBytes >> 20) + " MiB";
    return "";
}

}  // namespace idash
