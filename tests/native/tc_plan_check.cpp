// Tensor-core planner check without a GPU (build_tc_plan, plan.cpp): random
// models with coefficients up to two base-256 digits, duplicate features and
// constants are planned; then, per block,
//   - every fp16 coefficient digit decoded from the MMA layout gives back the
//     model's (summed) coefficient as c0 + 256 c1, and rows without a term
//     hold zeros;
//   - the padded K respects the exactness bound K * 128 * (128 + max|c1|) < 2^22;
//   - each chunk flagged consecutive really has consecutive rows;
// and the kernel's digit arithmetic is restated in integers: for random
// ciphertext words, sum_s 256^s D_s with D_s = sum over i + j = s of
// A_j * B_i (balanced digits) equals sum_k coef * word mod 2^32, with every
// |D_s| below 2^22.  A model with a coefficient needing a third digit is
// refused.  Prints one line per trial; exits non-zero on a mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "plan.hpp"
using namespace idash;

static int32_t half_to_int(uint16_t h) {
    _Float16 f;
    std::memcpy(&f, &h, 2);
    return int32_t(float(f));
}

int main() {
    std::mt19937_64 rng(11);
    int failures = 0;
    for (int trial = 0; trial < 24; ++trial) {
        const uint32_t n_rows = 400;
        const uint64_t n_out = 150 + rng() % 300;
        const int32_t cmax = trial % 3 == 0 ? 32767 : 8192;
        std::vector<uint64_t> ptr{0};
        std::vector<uint32_t> feat;
        std::vector<int32_t> coef;
        for (uint64_t o = 0; o < n_out; ++o) {
            // 16-bit coefficients allow K = 112: at most 30 neighbours (90 rows) there
            const uint32_t nb = std::vector<uint32_t>{1, 5, 20, cmax > 8192 ? 30u : 40u}[rng() % 4];
            const uint32_t base = uint32_t(o * (n_rows - 3 * nb) / n_out);
            for (uint32_t k = 0; k < 3 * nb; ++k) {
                if (rng() % 50 == 0) continue;  // a dropped feature: rows no longer consecutive
                feat.push_back(base + k);
                coef.push_back(int32_t(rng() % uint64_t(2 * cmax)) - cmax);
            }
            if (rng() % 2) { feat.push_back(0xFFFFFFFFu); coef.push_back(int32_t(rng() % 1000)); }
            if (rng() % 7 == 0) { feat.push_back(base); coef.push_back(-3); }  // duplicate feature
            ptr.push_back(feat.size());
        }
        PlanInput in;
        in.form = trial % 2 ? Form::kLwe : Form::kTrlwe;
        in.n_out = n_out;
        in.term_ptr = ptr.data();
        in.term_feat = feat.data();
        in.term_coef = coef.data();
        in.n_rows = n_rows;
        Plan plan;
        bool index_error = false;
        const std::string err = build_tc_plan(in, TcLimits{}, &plan, &index_error);
        if (!err.empty()) { std::printf("trial %d FAIL plan: %s\n", trial, err.c_str()); ++failures; continue; }
        // the model's coefficients, summed per (output, row)
        std::vector<std::map<uint32_t, uint32_t>> want(n_out);
        for (uint64_t o = 0; o < n_out; ++o)
            for (uint64_t t = ptr[o]; t < ptr[o + 1]; ++t)
                if (feat[t] != 0xFFFFFFFFu) want[o][feat[t]] += uint32_t(coef[t]);
        int32_t max_c1 = 0;
        for (auto &m : want)
            for (auto &kv : m) {
                const int32_t c = int32_t(kv.second), c0 = int32_t((uint32_t(c) + 128u) & 255u) - 128;
                max_c1 = std::max(max_c1, std::abs((c - c0) / 256));
            }
        bool ok = true;
        std::vector<uint32_t> words(n_rows);
        for (auto &w : words) w = uint32_t(rng());
        int64_t worst = 0;
        for (size_t bi = 0; bi < plan.blocks.size() && ok; ++bi) {
            const PlanBlock &b = plan.blocks[bi];
            const uint32_t k_pad = b.n_groups;
            if (k_pad % 16 || uint64_t(k_pad) * 128 * (128 + max_c1) >= (1ull << 22) + 128ull * (128 + max_c1) * 15) ok = false;
            if (b.n_slots > k_pad || b.out_hi - b.out_lo > kTcRows) ok = false;
            for (uint32_t c = 0; 32 * c < b.n_slots; ++c)
                if ((b.term_begin >> c) & 1u)
                    for (uint32_t k = 32 * c + 1; k < std::min<uint32_t>(b.n_slots, 32 * c + 32); ++k)
                        if (plan.slots[b.slot_begin + k].row != plan.slots[b.slot_begin + 32 * c].row + (k - 32 * c))
                            ok = false;
            const uint8_t *A = plan.tc_a.data() + uint64_t(b.group_begin) * 16;
            const uint64_t plane = tc_a_bytes(k_pad) / 2;
            for (uint32_t m = 0; m < kTcRows && ok; ++m) {
                const uint64_t o = b.out_lo + m;
                int64_t D[4] = {0, 0, 0, 0};
                uint32_t direct = 0;
                for (uint32_t k = 0; k < k_pad; ++k) {
                    const uint64_t off = uint64_t(k / 8) * 2048 + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2;
                    uint16_t h0, h1;
                    std::memcpy(&h0, A + off, 2);
                    std::memcpy(&h1, A + plane + off, 2);
                    const int32_t a0 = half_to_int(h0), a1 = half_to_int(h1);
                    uint32_t c = 0;
                    if (o < b.out_hi && k < b.n_slots) {
                        auto it = want[o].find(plan.slots[b.slot_begin + k].row);
                        if (it != want[o].end()) c = it->second;
                    }
                    if (uint32_t(a0 + 256 * a1) != c) { ok = false; break; }
                    if (k >= b.n_slots) continue;
                    const uint32_t x = words[plan.slots[b.slot_begin + k].row], y = x + 0x80808080u;
                    int32_t d[4];
                    for (int i = 0; i < 4; ++i) d[i] = int32_t((y >> (8 * i)) & 255u) - 128;
                    D[0] += int64_t(a0) * d[0];
                    for (int s = 1; s < 4; ++s) D[s] += int64_t(a0) * d[s] + int64_t(a1) * d[s - 1];
                    direct += c * x;
                }
                uint32_t sum = 0;
                for (int s = 0; s < 4; ++s) {
                    sum += uint32_t(D[s]) << (8 * s);
                    worst = std::max<int64_t>(worst, D[s] < 0 ? -D[s] : D[s]);
                }
                if (o < b.out_hi && sum != direct) ok = false;
            }
        }
        if (worst >= (1 << 22)) ok = false;
        std::printf("trial %d %s: outputs=%llu blocks=%zu max|c1|=%d worst|D|=%lld\n", trial, ok ? "ok" : "FAIL",
                    (unsigned long long)n_out, plan.blocks.size(), max_c1, (long long)worst);
        failures += ok ? 0 : 1;
    }
    // a coefficient that needs a third digit is refused
    const uint64_t p2[2] = {0, 1};
    const uint32_t f2[1] = {0};
    const int32_t c2[1] = {2000000000};
    PlanInput in;
    in.n_out = 1;
    in.term_ptr = p2;
    in.term_feat = f2;
    in.term_coef = c2;
    in.n_rows = 1;
    Plan plan;
    bool index_error = false;
    const bool refused = !build_tc_plan(in, TcLimits{}, &plan, &index_error).empty();
    std::printf("three-digit coefficient %s\n", refused ? "refused ok" : "FAIL accepted");
    return failures == 0 && refused ? 0 : 1;
}
