// Planner check without a GPU for idash_score_trlwe_noalloc: reads a CSR
// model from a file (u64 n_out, u64 nnz, u64 term_ptr[n_out + 1],
// u32 term_feat[nnz], i32 term_coef[nnz]) and prints, for the no-allocation
// entry point's planning limits (noalloc_plan.cpp, GB300's 227 KB of shared
// memory per CTA), the kernel it would run and the scratch bytes its tables
// take.  Arguments: file NUM_REGIONS REGION_SIZE n_rows with_variance with_index
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "noalloc_plan.hpp"

int main(int argc, char **argv) {
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s csr NUM_REGIONS REGION_SIZE n_rows with_variance with_index\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    uint64_t n_out = 0, nnz = 0;
    bool ok = std::fread(&n_out, 8, 1, f) == 1 && std::fread(&nnz, 8, 1, f) == 1;
    std::vector<uint64_t> ptr(n_out + 1);
    std::vector<uint32_t> feat(nnz);
    std::vector<int32_t> coef(nnz);
    ok = ok && std::fread(ptr.data(), 8, ptr.size(), f) == ptr.size() &&
         std::fread(feat.data(), 4, nnz, f) == nnz && std::fread(coef.data(), 4, nnz, f) == nnz;
    std::fclose(f);
    if (!ok) return 2;
    idash::PlanInput in;
    in.form = idash::Form::kTrlwe;
    in.n_out = n_out;
    in.term_ptr = ptr.data();
    in.term_feat = feat.data();
    in.term_coef = coef.data();
    in.N = 1024;
    in.num_regions = uint32_t(std::atoi(argv[2]));
    in.region_size = uint32_t(std::atoi(argv[3]));
    in.n_rows = std::strtoull(argv[4], nullptr, 10);
    idash::NoallocPlan np;
    bool index_error = false;
    const std::string err =
        idash::plan_noalloc(in, 232448, std::atoi(argv[5]) != 0, std::atoi(argv[6]) != 0, &np, &index_error);
    std::printf("bytes=%zu limit=%zu window=%d slice=%u index_error=%d err=%s\n", np.bytes,
                idash::kNoallocScratchBytes, np.window ? 1 : 0, np.slice_words, index_error ? 1 : 0,
                err.empty() ? "-" : err.c_str());
    return 0;
}
