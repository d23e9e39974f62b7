// Host half of idash_score_trlwe_noalloc (noalloc.cu): the plan it runs and
// where each of the plan's tables sits in the fixed scratch array.  Free of
// CUDA, so the layout can be checked on a machine without a GPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "plan.hpp"

namespace idash {

// Size of the no-allocation entry point's scratch array, per device.  It
// holds the full-scale model (242,646 outputs, 5 neighbours, 3.9 M terms) in
// the reference's record layout, variance program included (about 52 MiB).
constexpr size_t kNoallocScratchBytes = size_t(64) << 20;

struct NoallocPlan {
    Plan plan;
    bool window = false;  // the batched window kernel; else the direct kernel
    uint32_t slice_words = 512, group_size = 1;
    // byte offsets into the scratch array; [0, 256) holds the device error
    // word (offset 0) and the tile counter (offset 4)
    size_t o_blocks = 0, o_slots = 0, o_groups = 0, o_terms = 0;
    size_t o_var_ptr = 0, o_var_row = 0, o_var_coef = 0;  // with_variance only
    size_t o_out_index = 0;                               // with_index only
    size_t bytes = 0;  // scratch the tables need, error word and counter included
};

// Plans `in` for the no-allocation path: the window kernel at the widest
// slice (1024, 512, 256 words) whose window holds every output's slots, two
// CTAs per SM within `smem_optin` bytes of shared memory per CTA, else the
// direct kernel.  with_variance adds the variance program (records with a
// variance field); with_index the output index table (record headers with
// caller-given indices).  Returns "" on success; on failure the message, with
// *index_error set when a term names a feature without an input row.  A plan
// larger than kNoallocScratchBytes is returned with out->bytes set and the
// message saying so.
std::string plan_noalloc(const PlanInput &in, size_t smem_optin, bool with_variance, bool with_index,
                         NoallocPlan *out, bool *index_error);

}  // namespace idash
