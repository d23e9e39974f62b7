// Planner check without a GPU: random models (1 to 50 neighbours, duplicate
// features, constants, NUM_REGIONS 1 / 3 / 10) are planned with small windows
// and splitting on; the plan is then executed on the CPU exactly as the
// scoring kernels execute it (phase by phase, later phases adding to the
// outputs) and compared word for word with a direct evaluation of the CSR
// model, on a few columns of every output.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include "plan.hpp"
using namespace idash;

static uint32_t rowval(uint32_t row, uint32_t col) { uint64_t z = (uint64_t(row) << 32 | col) * 0x9E3779B97F4A7C15ull; z ^= z >> 29; return uint32_t(z * 0xBF58476D1CE4E5B9ull >> 32); }
static uint32_t rotated(uint32_t row, uint32_t c, uint32_t m, uint32_t N) {
    uint32_t p = c >= N, j = c - p * N, t = j + m;
    return t < N ? rowval(row, p * N + t) : 0u - rowval(row, p * N + t - N);
}

int main() {
    std::mt19937_64 rng(5);
    for (int trial = 0; trial < 40; ++trial) {
        const uint32_t R = (trial % 3 == 0) ? 1 : (trial % 3 == 1 ? 3 : 10), N = 1024, RS = N / R;
        const uint32_t n_feat = 300;
        const uint64_t n_out = 60 + rng() % 100;
        std::vector<uint64_t> ptr{0};
        std::vector<uint32_t> feat;
        std::vector<int32_t> coef;
        for (uint64_t o = 0; o < n_out; ++o) {
            const uint32_t nb = std::vector<uint32_t>{1, 5, 20, 50}[rng() % 4];
            const uint32_t base = rng() % (n_feat - 3 * nb);
            for (uint32_t k = 0; k < 3 * nb; ++k) {
                feat.push_back(base + k);
                coef.push_back(int32_t(rng() % 16384) - 8192);
            }
            if (rng() % 2) { feat.push_back(0xFFFFFFFFu); coef.push_back(int32_t(rng() % 100)); }
            if (rng() % 5 == 0) { feat.push_back(base); coef.push_back(7); }  // duplicate feature
            ptr.push_back(feat.size());
        }
        PlanInput in;
        in.form = Form::kTrlwe;
        in.n_out = n_out;
        in.term_ptr = ptr.data();
        in.term_feat = feat.data();
        in.term_coef = coef.data();
        in.num_regions = R;
        in.region_size = RS;
        in.n_rows = (n_feat + R - 1) / R;
        PlanLimits lim;
        lim.group_size = 3;
        lim.max_slots = 8 + rng() % 40;
        lim.max_terms = lim.max_slots * 4;
        lim.max_groups = 16;
        lim.split = true;
        Plan plan;
        bool ie = false;
        std::string err = build_plan(in, lim, &plan, &ie);
        if (!err.empty()) { printf("plan error %s\n", err.c_str()); return 1; }
        const uint32_t cols[] = {0, 5, 1023, 1024, 1024 + 17, 2047};
        std::vector<uint32_t> got(n_out * 6, 0xDEADBEEF);
        const uint32_t P = plan.phase_begin.size() - 1;
        for (uint32_t p = 0; p < P; ++p)
            for (uint32_t b = plan.phase_begin[p]; b < plan.phase_begin[p + 1]; ++b) {
                const PlanBlock &blk = plan.blocks[b];
                if (blk.n_slots > lim.max_slots) { printf("block over slots\n"); return 1; }
                for (uint32_t g = 0; g < blk.n_groups; ++g) {
                    const PlanGroup &gr = plan.groups[blk.group_begin + g];
                    for (int m = 0; m < 3; ++m) {
                        if (gr.out[m] == kNoOutput) continue;
                        for (int ci = 0; ci < 6; ++ci) {
                            const uint32_t c = cols[ci];
                            uint32_t acc = (c >= N && c - N < 1000) ? uint32_t(gr.bias[m]) : 0u;
                            for (uint32_t t = 0; t < gr.n_terms; ++t) {
                                const PlanTerm &tm = plan.terms[blk.term_begin + gr.term_begin + t];
                                const PlanSlot &sl = plan.slots[blk.slot_begin + tm.slot];
                                const uint32_t cc = m == 0 ? tm.c0 : m == 1 ? tm.c1 : tm.c2;
                                acc += cc * rotated(sl.row, c, sl.rot, N);
                            }
                            uint32_t &o = got[gr.out[m] * 6 + ci];
                            if (p == 0) { if (o != 0xDEADBEEF) { printf("output written twice in phase 0\n"); return 1; } o = acc; }
                            else o += acc;
                        }
                    }
                }
            }
        for (uint64_t o = 0; o < n_out; ++o)
            for (int ci = 0; ci < 6; ++ci) {
                const uint32_t c = cols[ci];
                uint32_t want = 0;
                for (uint64_t t = ptr[o]; t < ptr[o + 1]; ++t) {
                    if (feat[t] == 0xFFFFFFFFu) { if (c >= N && c - N < 1000) want += uint32_t(coef[t]) * (1u << 18); continue; }
                    want += uint32_t(coef[t]) * rotated(feat[t] / R, c, (feat[t] % R) * RS, N);
                }
                if (got[o * 6 + ci] != want) { printf("trial %d out %lu col %u: %08x vs %08x (phases %u)\n", trial, (unsigned long)o, c, got[o*6+ci], want, P); return 1; }
            }
        printf("trial %d ok: R=%u slots<=%u phases=%u blocks=%zu\n", trial, R, lim.max_slots, P, plan.blocks.size());
    }
    return 0;
}
