// Host planner (see plan.hpp).  Pure C++, no CUDA.
#include "plan.hpp"

#include <algorithm>
#include <cstring>

namespace idash {

namespace {

inline uint64_t make_key(uint32_t row, uint32_t rot) { return (uint64_t(row) << 32) | rot; }

// Size of the union of two sorted key lists.
size_t union_size(const uint64_t *a, size_t na, const uint64_t *b, size_t nb) {
    size_t i = 0, j = 0, n = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i;
        else if (b[j] < a[i]) ++j;
        else { ++i; ++j; }
        ++n;
    }
    return n + (na - i) + (nb - j);
}

// Step 1 of both planners: every output as (slot key, coefficient) sorted by
// key, duplicates summed mod 2^32, zero coefficients dropped, constants
// folded into the bias; the variance program and the distinct row count go
// into `plan`.
struct Normalised {
    std::vector<uint64_t> nptr, nkey;
    std::vector<uint32_t> ncoef, bias;
};

std::string normalise(const PlanInput &in, Plan *plan, Normalised *nm, bool *index_error) {
    const uint64_t n_out = in.n_out;
    plan->n_terms_in = n_out ? in.term_ptr[n_out] - in.term_ptr[0] : 0;
    std::vector<uint64_t> &nptr = nm->nptr, &nkey = nm->nkey;
    std::vector<uint32_t> &ncoef = nm->ncoef, &bias = nm->bias;
    nptr.assign(n_out + 1, 0);
    bias.assign(n_out, 0);
    nkey.reserve(plan->n_terms_in);
    ncoef.reserve(plan->n_terms_in);
    std::vector<std::pair<uint64_t, uint32_t>> tmp;
    if (in.form == Form::kTrlwe) plan->var_ptr.assign(n_out + 1, 0);
    for (uint64_t o = 0; o < n_out; ++o) {
        tmp.clear();
        if (in.term_ptr[o + 1] < in.term_ptr[o]) return "term_ptr must be non-decreasing";
        for (uint64_t t = in.term_ptr[o]; t < in.term_ptr[o + 1]; ++t) {
            const uint32_t feat = in.term_feat[t];
            const uint32_t coef = uint32_t(in.term_coef[t]);
            if (feat == kConstantFeature) {
                bias[o] += coef * uint32_t(in.one_t32);
                continue;
            }
            uint64_t row;
            uint32_t rot = 0;
            if (in.form == Form::kTrlwe) {
                const uint64_t index = feat / in.num_regions;
                const uint32_t region = feat % in.num_regions;
                if (in.row_of_index) {
                    if (index >= in.n_index) { *index_error = true; return "feature index has no input ciphertext"; }
                    row = in.row_of_index[index];
                } else {
                    row = index;
                }
                rot = region * in.region_size;
                if (region == 0) {
                    plan->var_row.push_back(uint32_t(row));
                    plan->var_coef.push_back(in.term_coef[t]);
                }
            } else {
                row = feat;
            }
            if (row >= in.n_rows || row >= 0xFFFFFFFFull) {
                *index_error = true;
                return "feature maps to an input row outside the input";
            }
            tmp.emplace_back(make_key(uint32_t(row), rot), coef);
        }
        if (in.form == Form::kTrlwe) plan->var_ptr[o + 1] = plan->var_row.size();
        std::sort(tmp.begin(), tmp.end(),
                  [](const std::pair<uint64_t, uint32_t> &x, const std::pair<uint64_t, uint32_t> &y) {
                      return x.first < y.first;
                  });
        for (size_t i = 0; i < tmp.size();) {
            size_t j = i;
            uint32_t c = 0;
            while (j < tmp.size() && tmp[j].first == tmp[i].first) c += tmp[j++].second;
            if (c != 0) {
                nkey.push_back(tmp[i].first);
                ncoef.push_back(c);
            }
            i = j;
        }
        nptr[o + 1] = nkey.size();
    }
    {
        std::vector<uint8_t> seen(in.n_rows, 0);
        for (uint64_t k : nkey) seen[k >> 32] = 1;
        uint64_t d = 0;
        for (uint8_t s : seen) d += s;
        plan->distinct_rows = d;
    }

    return "";
}

}  // namespace

std::string build_plan(const PlanInput &in, const PlanLimits &lim, Plan *plan, bool *index_error) {
    *index_error = false;
    *plan = Plan();
    if (lim.group_size != 1 && lim.group_size != 3) return "group_size must be 1 or 3";
    if (in.n_out >= kNoOutput) return "too many outputs";
    if (in.form == Form::kTrlwe) {
        if (in.num_regions == 0 || in.region_size == 0 ||
            uint64_t(in.num_regions) * in.region_size > in.N)
            return "NUM_REGIONS * REGION_SIZE must be in [1, N]";
    }
    const uint64_t n_out = in.n_out;

    // 1. Normalise every output.
    Normalised nm;
    {
        const std::string err = normalise(in, plan, &nm, index_error);
        if (!err.empty()) return err;
    }
    const std::vector<uint64_t> &nptr = nm.nptr, &nkey = nm.nkey;
    const std::vector<uint32_t> &ncoef = nm.ncoef, &bias = nm.bias;

    // 2. Groups of up to group_size consecutive outputs with (nearly) the
    //    same slot set: union no larger than 5/4 of the largest member + 1.
    //    With lim.split, a group larger than one window becomes parts.
    struct G {
        uint64_t o0;
        uint32_t n;
        uint32_t phase = 0;  // part index of a split group
        std::vector<uint64_t> keys;
        std::vector<uint32_t> c[3];
    };
    const size_t cap = std::min<size_t>(lim.max_slots, lim.max_terms);
    if (cap == 0) return "a block must hold at least one slot and one term";
    std::vector<G> groups;
    groups.reserve(n_out / lim.group_size + 1);
    for (uint64_t o = 0; o < n_out;) {
        uint32_t n = 1;
        std::vector<uint64_t> keys(nkey.begin() + nptr[o], nkey.begin() + nptr[o + 1]);
        size_t largest = keys.size();
        while (n < lim.group_size && o + n < n_out) {
            const uint64_t p = o + n;
            const size_t np = nptr[p + 1] - nptr[p];
            const size_t u = union_size(keys.data(), keys.size(), nkey.data() + nptr[p], np);
            const size_t big = std::max(largest, np);
            if (u > big + big / 4 + 1) break;
            if (!lim.split && (u > lim.max_slots || u > lim.max_terms)) break;
            std::vector<uint64_t> merged;
            merged.reserve(u);
            std::set_union(keys.begin(), keys.end(), nkey.begin() + nptr[p], nkey.begin() + nptr[p + 1],
                           std::back_inserter(merged));
            keys.swap(merged);
            largest = big;
            ++n;
        }
        G g;
        g.o0 = o;
        g.n = n;
        g.keys = keys;
        for (uint32_t m = 0; m < 3; ++m) g.c[m].assign(keys.size(), 0);
        for (uint32_t m = 0; m < n; ++m) {
            const uint64_t p = o + m;
            size_t idx = 0;
            for (uint64_t t = nptr[p]; t < nptr[p + 1]; ++t) {
                while (g.keys[idx] != nkey[t]) ++idx;
                g.c[m][idx] = ncoef[t];
            }
        }
        if (g.keys.size() <= cap) {
            groups.push_back(std::move(g));
        } else if (!lim.split) {
            return "an output needs more window slots than one block holds";
        } else {
            // parts of at most `cap` consecutive slots; part k runs in phase k
            for (size_t k0 = 0, part = 0; k0 < g.keys.size(); k0 += cap, ++part) {
                const size_t k1 = std::min(g.keys.size(), k0 + cap);
                G gp;
                gp.o0 = g.o0;
                gp.n = g.n;
                gp.phase = uint32_t(part);
                gp.keys.assign(g.keys.begin() + k0, g.keys.begin() + k1);
                for (uint32_t m = 0; m < 3; ++m) gp.c[m].assign(g.c[m].begin() + k0, g.c[m].begin() + k1);
                groups.push_back(std::move(gp));
            }
        }
        o += n;
    }
    uint32_t n_phases = 1;
    for (const G &g : groups) n_phases = std::max(n_phases, g.phase + 1);
    // per phase, its groups in output order
    std::vector<std::vector<uint32_t>> by_phase(n_phases);
    for (uint32_t q = 0; q < groups.size(); ++q) by_phase[groups[q].phase].push_back(q);

    // 3. Blocks of consecutive groups (of one phase) sharing one window of slots.
    std::vector<uint64_t> win;
    for (uint32_t ph = 0; ph < n_phases; ++ph) {
        plan->phase_begin.push_back(uint32_t(plan->blocks.size()));
        const std::vector<uint32_t> &order = by_phase[ph];
        size_t gi = 0;
        while (gi < order.size()) {
            PlanBlock b{};
            b.group_begin = uint32_t(plan->groups.size());
            b.term_begin = uint32_t(plan->terms.size());
            b.slot_begin = uint32_t(plan->slots.size());
            win.clear();
            size_t gend = gi;
            uint32_t terms = 0;
            while (gend < order.size()) {
                const G &g = groups[order[gend]];
                const size_t u = union_size(win.data(), win.size(), g.keys.data(), g.keys.size());
                if (gend > gi && (u > lim.max_slots || terms + g.keys.size() > lim.max_terms ||
                                  gend - gi + 1 > lim.max_groups))
                    break;
                std::vector<uint64_t> merged;
                merged.reserve(u);
                std::set_union(win.begin(), win.end(), g.keys.begin(), g.keys.end(), std::back_inserter(merged));
                win.swap(merged);
                terms += uint32_t(g.keys.size());
                ++gend;
            }
            if (win.size() > 0xFFFFu) return "a block window needs more than 65535 slots";
            // unrotated slots first (bulk-copied by the kernel), rotated ones
            // after (gathered with the negacyclic sign); both parts stay sorted
            const size_t n_unrot = size_t(std::count_if(win.begin(), win.end(),
                                                        [](uint64_t k) { return (k & 0xFFFFFFFFu) == 0; }));
            std::stable_partition(win.begin(), win.end(), [](uint64_t k) { return (k & 0xFFFFFFFFu) == 0; });
            auto local_of = [&](uint64_t key) -> uint32_t {
                const auto lo = (key & 0xFFFFFFFFu) == 0 ? win.begin() : win.begin() + n_unrot;
                const auto hi = (key & 0xFFFFFFFFu) == 0 ? win.begin() + n_unrot : win.end();
                return uint32_t(std::lower_bound(lo, hi, key) - win.begin());
            };
            b.n_slots = uint16_t(win.size());
            b.n_rot = uint16_t(win.size() - n_unrot);
            uint32_t max_row = 0, min_row = win.empty() ? 0u : 0xFFFFFFFFu;
            for (uint64_t k : win) {
                plan->slots.push_back(PlanSlot{uint32_t(k >> 32), uint32_t(k & 0xFFFFFFFFu)});
                max_row = std::max(max_row, uint32_t(k >> 32));
                min_row = std::min(min_row, uint32_t(k >> 32));
            }
            plan->block_max_row.push_back(max_row);
            plan->block_min_row.push_back(min_row);
            const G &first = groups[order[gi]], &last = groups[order[gend - 1]];
            b.out_lo = uint32_t(first.o0);
            b.out_hi = uint32_t(last.o0 + last.n);
            // the block's groups, most terms first: kernels that hand groups
            // out dynamically then start the long ones early (longest
            // processing time first), and the short ones fill in around them
            std::vector<uint32_t> in_block(order.begin() + gi, order.begin() + gend);
            std::stable_sort(in_block.begin(), in_block.end(), [&](uint32_t x, uint32_t y) {
                return groups[x].keys.size() > groups[y].keys.size();
            });
            for (const uint32_t gq : in_block) {
                const G &g = groups[gq];
                PlanGroup pg{};
                pg.term_begin = uint32_t(plan->terms.size()) - b.term_begin;
                pg.n_terms = uint32_t(g.keys.size());
                for (uint32_t m = 0; m < 3; ++m) {
                    pg.out[m] = m < g.n ? uint32_t(g.o0 + m) : kNoOutput;
                    // the bias goes with the first part only
                    pg.bias[m] = m < g.n && g.phase == 0 ? int32_t(bias[g.o0 + m]) : 0;
                }
                for (size_t t = 0; t < g.keys.size(); ++t)
                    plan->terms.push_back(PlanTerm{int32_t(g.c[0][t]), int32_t(g.c[1][t]), int32_t(g.c[2][t]),
                                                   local_of(g.keys[t])});
                plan->groups.push_back(pg);
            }
            b.n_groups = uint32_t(gend - gi);
            b.n_terms = uint32_t(plan->terms.size()) - b.term_begin;
            plan->max_block_slots = std::max<uint32_t>(plan->max_block_slots, b.n_slots);
            plan->max_block_terms = std::max(plan->max_block_terms, b.n_terms);
            plan->max_block_groups = std::max(plan->max_block_groups, b.n_groups);
            plan->blocks.push_back(b);
            gi = gend;
        }
    }
    plan->phase_begin.push_back(uint32_t(plan->blocks.size()));
    return "";
}

namespace {

// fp16 bit pattern of an integer that fp16 holds exactly (|v| < 65536 with
// at most 11 significant bits, e.g. every |v| <= 2048).
uint16_t half_bits(int32_t v) {
    if (v == 0) return 0;
    const uint16_t sign = v < 0 ? 0x8000u : 0u;
    const uint32_t m = uint32_t(v < 0 ? -v : v);
    const int e = 31 - __builtin_clz(m);
    const uint32_t frac = e <= 10 ? (m << (10 - e)) : (m >> (e - 10));
    return uint16_t(sign | uint32_t((e + 15) << 10) | (frac & 0x3FFu));
}

// Byte offset of element (row m, k) of one digit plane in the MMA's
// no-swizzle K-major layout: 8x8 core matrices of 16-byte rows, K-blocks of 8
// outermost (2,048 bytes each: 128 rows), then 8-row groups (128 bytes).
inline uint64_t tc_a_offset(uint32_t m, uint32_t k) {
    return uint64_t(k / 8) * 2048 + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2;
}

}  // namespace

std::string build_tc_plan(const PlanInput &in, const TcLimits &lim, Plan *plan, bool *index_error) {
    *index_error = false;
    *plan = Plan();
    if (in.n_out >= kNoOutput) return "too many outputs";
    if (in.form == Form::kIntPoly) return "the tensor-core plan serves the TRLWE and LWE forms";
    if (in.form == Form::kTrlwe && in.num_regions != 1)
        return "the tensor-core plan reads rows unrotated (NUM_REGIONS = 1)";
    const uint64_t n_out = in.n_out;
    Normalised nm;
    {
        const std::string err = normalise(in, plan, &nm, index_error);
        if (!err.empty()) return err;
    }
    // coefficient digits c = c0 + 256 c1, c0 in [-128, 127]; |c1| <= 128
    int32_t max_c1 = 0;
    for (uint32_t c : nm.ncoef) {
        const int32_t c0 = int32_t((c + 128u) & 255u) - 128;
        const int64_t c1 = (int64_t(int32_t(c)) - c0) / 256;
        if (c1 < -128 || c1 > 128) return "a coefficient needs more than two base-256 digits";
        max_c1 = std::max<int32_t>(max_c1, int32_t(c1 < 0 ? -c1 : c1));
    }
    const uint64_t per_k = uint64_t(128) * uint64_t(128 + max_c1);
    uint32_t k_max = uint32_t(((uint64_t(1) << 22) - 1) / per_k) / 16 * 16;
    k_max = std::min(k_max, lim.max_k / 16 * 16);
    if (k_max < 16) return "no K satisfies the exactness bound";

    plan->tc_bias.assign(nm.bias.begin(), nm.bias.end());
    plan->phase_begin.push_back(0);
    std::vector<uint64_t> win, merged;
    for (uint64_t o = 0; o < n_out;) {
        win.clear();
        uint64_t e = o;
        while (e < n_out && e - o < kTcRows) {
            const uint64_t *k0 = nm.nkey.data() + nm.nptr[e], *k1 = nm.nkey.data() + nm.nptr[e + 1];
            merged.clear();
            std::set_union(win.begin(), win.end(), k0, k1, std::back_inserter(merged));
            if (merged.size() > k_max) {
                if (e == o) return "an output reads more rows than one tensor-core block holds";
                break;
            }
            win.swap(merged);
            ++e;
        }
        for (uint64_t k : win)
            if ((k & 0xFFFFFFFFu) != 0) return "the tensor-core plan reads rows unrotated";
        PlanBlock b{};
        b.slot_begin = uint32_t(plan->slots.size());
        b.n_slots = uint16_t(win.size());
        b.n_rot = 0;
        const uint32_t k_pad = std::max<uint32_t>(16, uint32_t((win.size() + 15) / 16 * 16));
        b.group_begin = uint32_t(plan->tc_a.size() / 16);
        b.n_groups = k_pad;
        b.term_begin = 0;
        for (size_t c0 = 0, c = 0; c0 < win.size(); c0 += 32, ++c) {
            const size_t c1 = std::min(win.size(), c0 + 32);
            bool run = true;
            for (size_t k = c0 + 1; k < c1 && run; ++k) run = (win[k] >> 32) == (win[c0] >> 32) + (k - c0);
            if (run && c < 32) b.term_begin |= 1u << c;
        }
        b.n_terms = uint32_t(nm.nptr[e] - nm.nptr[o]);
        b.out_lo = uint32_t(o);
        b.out_hi = uint32_t(e);
        uint32_t max_row = 0, min_row = win.empty() ? 0u : 0xFFFFFFFFu;
        for (uint64_t k : win) {
            plan->slots.push_back(PlanSlot{uint32_t(k >> 32), 0});
            max_row = std::max(max_row, uint32_t(k >> 32));
            min_row = std::min(min_row, uint32_t(k >> 32));
        }
        plan->block_max_row.push_back(max_row);
        plan->block_min_row.push_back(min_row);
        // the block's coefficient digits: plane 0 holds c0, plane 1 holds c1
        const size_t a0 = plan->tc_a.size();
        const uint64_t plane = tc_a_bytes(k_pad) / 2;
        plan->tc_a.resize(a0 + tc_a_bytes(k_pad), 0);
        uint8_t *A = plan->tc_a.data() + a0;
        for (uint64_t p = o; p < e; ++p) {
            const uint32_t m = uint32_t(p - o);
            size_t idx = 0;
            for (uint64_t t = nm.nptr[p]; t < nm.nptr[p + 1]; ++t) {
                while (win[idx] != nm.nkey[t]) ++idx;
                const uint32_t c = nm.ncoef[t];
                const int32_t c0 = int32_t((c + 128u) & 255u) - 128;
                const int32_t c1 = int32_t((int64_t(int32_t(c)) - c0) / 256);
                const uint16_t h0 = half_bits(c0), h1 = half_bits(c1);
                std::memcpy(A + tc_a_offset(m, uint32_t(idx)), &h0, 2);
                std::memcpy(A + plane + tc_a_offset(m, uint32_t(idx)), &h1, 2);
            }
        }
        plan->max_block_slots = std::max<uint32_t>(plan->max_block_slots, b.n_slots);
        plan->max_block_terms = std::max(plan->max_block_terms, k_pad);
        plan->blocks.push_back(b);
        o = e;
    }
    plan->phase_begin.push_back(uint32_t(plan->blocks.size()));
    return "";
}

}  // namespace idash
