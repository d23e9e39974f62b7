// Host-side planner: turns a model in CSR form (the reference's
// Model::model, eval/idash.h:129-134, flattened) into the device work list
// the scoring kernels consume.
//
//   slot   one input row as seen by a term: (row, rotation m).  In the TRLWE
//          layout a feature in region r is read as X^(-r*REGION_SIZE) * row,
//          which is exactly the reference's fold of region r into region 0
//          (torusPolynomialMulByXai with exponent 2N - r*REGION_SIZE,
//          eval/idash.cpp:830-833) applied term by term (the map is linear).
//   group  up to 3 consecutive outputs (normally the 3 genotype models of one
//          target position) sharing one term list; each term carries the 3
//          coefficients, so an input word read once feeds 3 accumulators.
//   block  consecutive groups whose slots fit one shared-memory window: the
//          unit of input reuse across neighbouring targets.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace idash {

struct PlanBlock {
    uint32_t slot_begin;
    uint16_t n_slots;   // unrotated slots first, then n_rot rotated ones
    uint16_t n_rot;
    uint32_t group_begin, n_groups;
    uint32_t term_begin, n_terms;
    uint32_t out_lo, out_hi;  // outputs covered: [out_lo, out_hi)
};
static_assert(sizeof(PlanBlock) == 32, "PlanBlock layout");

struct PlanSlot {
    uint32_t row;  // input row
    uint32_t rot;  // m in [0, N): the slot holds X^(-m) * row (0 = as stored)
};

struct PlanGroup {
    uint32_t term_begin;  // relative to the block's term_begin
    uint32_t n_terms;
    uint32_t out[3];      // output ordinals, kNoOutput if unused
    int32_t bias[3];      // sum of constant coefficients * one_t32, mod 2^32
};
static_assert(sizeof(PlanGroup) == 32, "PlanGroup must stay 32 bytes (bulk-copied)");

// One term of a group: coefficients for the group's 3 outputs and the
// block-local slot index; 16 bytes so one shared-memory load fetches it.
struct PlanTerm {
    int32_t c0, c1, c2;
    uint32_t slot;
};

constexpr uint32_t kNoOutput = 0xFFFFFFFFu;
constexpr uint32_t kConstantFeature = 0xFFFFFFFFu;

enum class Form : int { kTrlwe = 0, kLwe = 1, kIntPoly = 2 };

struct PlanInput {
    Form form = Form::kTrlwe;
    uint64_t n_out = 0;
    const uint64_t *term_ptr = nullptr;
    const uint32_t *term_feat = nullptr;
    const int32_t *term_coef = nullptr;
    int32_t one_t32 = 1 << 18;
    // TRLWE: feature -> (row_of_index[feat / R], (feat % R) * region_size)
    uint32_t N = 1024, num_regions = 1, region_size = 1024;
    const uint32_t *row_of_index = nullptr;
    uint64_t n_index = 0;
    uint64_t n_rows = 0;  // valid input rows (LWE: feature rows)
};

struct PlanLimits {
    uint32_t group_size = 3;    // 1 (plain per-output) or 3 (per target)
    uint32_t max_slots = 48;    // window slots per block
    uint32_t max_terms = 2048;  // terms per block
    uint32_t max_groups = 64;   // groups per block
    // A group whose slots exceed one window is split into parts of at most
    // min(max_slots, max_terms) slots; part p is planned in phase p, whose
    // launch adds its partial sums to the outputs phase p - 1 wrote.
    bool split = false;
};

struct Plan {
    std::vector<PlanBlock> blocks;
    // Blocks of phase p are [phase_begin[p], phase_begin[p + 1]), each phase
    // in output order.  Phase 0 writes every output (with its bias); a later
    // phase holds the further parts of split groups and accumulates.
    std::vector<uint32_t> phase_begin;
    std::vector<PlanSlot> slots;
    std::vector<PlanGroup> groups;
    std::vector<PlanTerm> terms;
    // Variance program (TRLWE records): output o's region-0 terms in CSR
    // order, var_row/var_coef[var_ptr[o] .. var_ptr[o+1]).
    std::vector<uint64_t> var_ptr;
    std::vector<uint32_t> var_row;
    std::vector<int32_t> var_coef;
    uint32_t max_block_slots = 0, max_block_terms = 0, max_block_groups = 0;
    uint64_t n_terms_in = 0;       // CSR terms given
    uint64_t distinct_rows = 0;    // input rows read at least once
    uint32_t max_row_per_block_hint = 0;
    std::vector<uint32_t> block_max_row;  // per block: largest input row read
    std::vector<uint32_t> block_min_row;  // per block: smallest input row read (0 if none)
    // Tensor-core plans only (build_tc_plan): per block, the coefficient
    // digits in the MMA's shared-memory layout, and every output's bias.
    std::vector<uint8_t> tc_a;
    std::vector<uint32_t> tc_bias;
};

// Tensor-core plans (build_tc_plan).  A block is up to kTcRows consecutive
// outputs (the MMA's M, one TMEM lane each) over the sorted union of their
// input rows (the MMA's K, padded to a multiple of 16).  PlanBlock fields are
// read as: slot_begin/n_slots the rows, n_rot 0, group_begin the offset of the
// block's coefficient digits in tc_a in 16-byte units, n_groups the padded K,
// term_begin a bit mask of the block's 32-row chunks whose rows are
// consecutive (bit c: rows 32c .. min(32c + 32, n_slots) - 1; such a chunk is
// one 2D tensor copy), n_terms the block's nonzero terms, out_lo/out_hi its
// outputs.
//
// Exactness (fp16 digits, fp32 accumulation): a ciphertext word x is split
// into four balanced base-256 digits (x + 0x80808080 byte by byte, minus 128),
// a coefficient c into c0 in [-128, 127] and c1 = (c - c0) / 256; product
// digit sums for shift 8s are sums over K of at most two digit products, so
// |sum| <= K * 128 * (128 + max|c1|).  The planner keeps that below 2^22
// (where x + 1.5 * 2^23 is exact in fp32) by bounding K, and refuses models
// with a coefficient outside two digits.
constexpr uint32_t kTcRows = 128;
struct TcLimits {
    uint32_t max_k = 192;  // shared-memory bound on the padded K
};
// Bytes of one block's coefficient digits: 2 digit planes x 128 rows x k_pad fp16.
inline uint64_t tc_a_bytes(uint32_t k_pad) { return uint64_t(4) * kTcRows * k_pad; }
std::string build_tc_plan(const PlanInput &in, const TcLimits &lim, Plan *plan, bool *index_error);

// Returns "" on success, else a message; *index_error is set when a term
// names a feature without an input row (IDASH_ERR_INDEX).
std::string build_plan(const PlanInput &in, const PlanLimits &lim, Plan *plan, bool *index_error);

}  // namespace idash
