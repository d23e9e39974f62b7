// idash_score_trlwe_noalloc: TRLWE scoring that allocates no device or
// page-locked memory.
//
// Some callers cannot call cudaMalloc.  Examples: a service whose framework
// reserves the GPU's memory for its own pool up front, a process capped by a
// per-client device-memory limit that it has already reached, or a
// latency-bound loop that cannot afford the implicit synchronisation of
// cudaMalloc/cudaFree.  They still own the input and output buffers.  This
// entry point needs nothing else from the device heap.  Its scratch is the
// array below: the planned work list (blocks, slots, groups, terms), the
// window kernel's tile counter, the device error word, the variance program
// and the output index table (noalloc_plan.cpp lays them out).  The array is
// a fixed part of the library's device image, so every GPU that loads the
// library holds it until the process exits.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "capi_internal.hpp"
#include "noalloc_plan.hpp"

namespace {

// kNoallocScratchBytes (64 MiB) per device: the full-scale model (242,646
// outputs, 5 neighbours) fits in the reference's record layout with its
// variance program.  Larger models are refused.
static __device__ __align__(256) unsigned char g_noalloc_scratch[idash::kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_addr[kMaxDevices] = {};  // device address per device, set on first call

idash_status fail(idash_status s, const std::string &msg) {
    idash_set_thread_error(msg);
    return s;
}

// First call on a device: resolve the array's device address with that
// device current, and allow the window kernels their shared memory.
idash_status setup_device(int dev, unsigned char **addr, int *sm_count, size_t *smem_optin) {
    cudaDeviceProp prop{};
    cudaError_t e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return fail(IDASH_ERR_CUDA, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
    *sm_count = prop.multiProcessorCount;
    *smem_optin = prop.sharedMemPerBlockOptin;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(IDASH_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        e = idash::configure_window_kernels(prop.sharedMemPerBlockOptin);
        if (e != cudaSuccess) return fail(IDASH_ERR_CUDA, std::string("configure kernels: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *addr = g_scratch_addr[dev];
    return IDASH_OK;
}

bool layout_ok(const void *base, const idash_row_layout *l, uint64_t payload) {
    if (!l || l->row_stride % 16 || ((reinterpret_cast<uintptr_t>(base) + l->payload_offset) & 15u)) return false;
    if (l->payload_offset + payload > l->row_stride) return false;
    auto clash = [&](int64_t off, uint64_t len) {
        return off >= 0 && (uint64_t(off) + len > l->row_stride ||
                            (uint64_t(off) < l->payload_offset + payload && uint64_t(off) + len > l->payload_offset));
    };
    if (clash(l->variance_offset, 8) || clash(l->header_offset, 8)) return false;
    if (l->variance_offset >= 0 && (reinterpret_cast<uintptr_t>(base) + l->variance_offset) % 8) return false;
    return true;
}

}  // namespace

extern "C" idash_status idash_score_trlwe_noalloc(const idash_trlwe_params *p, uint64_t n_out,
                                                  const uint32_t *out_index, const uint64_t *term_ptr,
                                                  const uint32_t *term_feat, const int32_t *term_coef,
                                                  uint64_t n_in_index, const uint32_t *in_row_of_index,
                                                  uint64_t n_in_rows, const void *d_in,
                                                  const idash_row_layout *in_layout, void *d_out,
                                                  const idash_row_layout *out_layout, void *stream) {
    using namespace idash;
    if (!p || !d_in || !d_out || !in_layout || !out_layout || (n_out && (!term_ptr || (term_ptr[n_out] &&
                                                                                      (!term_feat || !term_coef)))))
        return fail(IDASH_ERR_INVALID_ARGUMENT, "null argument");
    if (n_in_index && !in_row_of_index) return fail(IDASH_ERR_INVALID_ARGUMENT, "n_in_index without in_row_of_index");
    if (p->k != 1 || p->N == 0 || p->N % 256 || p->N > 4096)
        return fail(IDASH_ERR_UNSUPPORTED, "need k = 1 and N a multiple of 256 up to 4096");
    if (p->num_regions == 0 || p->region_size == 0 || uint64_t(p->num_regions) * p->region_size > p->N ||
        p->num_samples > p->region_size)
        return fail(IDASH_ERR_INVALID_ARGUMENT, "need NUM_REGIONS*REGION_SIZE <= N and NUM_SAMPLES <= REGION_SIZE");
    const uint64_t payload = uint64_t(2) * p->N * 4;
    if (!layout_ok(d_in, in_layout, payload) || !layout_ok(d_out, out_layout, payload))
        return fail(IDASH_ERR_INVALID_ARGUMENT, "row layout: stride, alignment or field offsets");
    if (n_out == 0) return IDASH_OK;

    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return fail(IDASH_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(ce));
    if (dev < 0 || dev >= kMaxDevices) return fail(IDASH_ERR_UNSUPPORTED, "device ordinal beyond 63");
    unsigned char *scratch = nullptr;
    int sm_count = 0;
    size_t smem_optin = 0;
    idash_status s = setup_device(dev, &scratch, &sm_count, &smem_optin);
    if (s != IDASH_OK) return s;

    // Plan on the host (ordinary heap memory).
    PlanInput in;
    in.form = Form::kTrlwe;
    in.n_out = n_out;
    in.term_ptr = term_ptr;
    in.term_feat = term_feat;
    in.term_coef = term_coef;
    in.one_t32 = p->one_t32;
    in.N = p->N;
    in.num_regions = p->num_regions;
    in.region_size = p->region_size;
    in.row_of_index = in_row_of_index;
    in.n_index = in_row_of_index ? n_in_index : 0;
    in.n_rows = n_in_rows;
    const bool want_var = out_layout->variance_offset >= 0;
    const bool want_index = out_index && out_layout->header_offset >= 0;
    NoallocPlan np;
    bool index_error = false;
    const std::string err = plan_noalloc(in, smem_optin, want_var, want_index, &np, &index_error);
    if (!err.empty())
        return fail(index_error ? IDASH_ERR_INDEX : np.bytes > kNoallocScratchBytes ? IDASH_ERR_INVALID_ARGUMENT
                                                                                    : IDASH_ERR_UNSUPPORTED,
                    err);
    const Plan &plan = np.plan;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto put = [&](size_t at, const void *src, size_t bytes) -> cudaError_t {
        return bytes ? cudaMemcpyAsync(scratch + at, src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
    };
    ce = cudaMemsetAsync(scratch, 0, 256, st);  // error word and tile counter start at zero
    if (ce == cudaSuccess) ce = put(np.o_blocks, plan.blocks.data(), plan.blocks.size() * sizeof(PlanBlock));
    if (ce == cudaSuccess) ce = put(np.o_slots, plan.slots.data(), plan.slots.size() * sizeof(PlanSlot));
    if (ce == cudaSuccess) ce = put(np.o_groups, plan.groups.data(), plan.groups.size() * sizeof(PlanGroup));
    if (ce == cudaSuccess) ce = put(np.o_terms, plan.terms.data(), plan.terms.size() * sizeof(PlanTerm));
    if (ce == cudaSuccess && want_var) {
        ce = put(np.o_var_ptr, plan.var_ptr.data(), plan.var_ptr.size() * 8);
        if (ce == cudaSuccess) ce = put(np.o_var_row, plan.var_row.data(), plan.var_row.size() * 4);
        if (ce == cudaSuccess) ce = put(np.o_var_coef, plan.var_coef.data(), plan.var_coef.size() * 4);
    }
    if (ce == cudaSuccess && want_index) ce = put(np.o_out_index, out_index, n_out * 4);
    if (ce != cudaSuccess) return fail(IDASH_ERR_CUDA, std::string("scratch upload: ") + cudaGetErrorString(ce));

    uint32_t *d_err = reinterpret_cast<uint32_t *>(scratch);
    const KernelKind kind = np.window ? KernelKind::kWindow : KernelKind::kDirect;
    const uint32_t w = np.slice_words, g = np.group_size;
    ScoreArgs a{};
    a.blocks = reinterpret_cast<const PlanBlock *>(scratch + np.o_blocks);
    a.slots = reinterpret_cast<const PlanSlot *>(scratch + np.o_slots);
    a.groups = reinterpret_cast<const PlanGroup *>(scratch + np.o_groups);
    a.terms = reinterpret_cast<const PlanTerm *>(scratch + np.o_terms);
    a.block_lo = 0;
    a.n_blocks = uint32_t(plan.blocks.size());
    a.row_words = 2 * p->N;
    a.n_slices = (a.row_words + w - 1) / w;
    a.n_tiles = a.n_blocks * a.n_slices;
    a.n_rows = uint32_t(std::min<uint64_t>(n_in_rows, 0xFFFFFFFFull));
    a.in = static_cast<const uint8_t *>(d_in) + in_layout->payload_offset;
    a.in_stride = in_layout->row_stride;
    a.out = static_cast<uint8_t *>(d_out) + out_layout->payload_offset;
    a.out_stride = out_layout->row_stride;
    a.out_lo = 0;
    a.out_hi = n_out;
    a.out_row_base = 0;
    a.out_row_map = nullptr;
    a.form = kFormTrlwe;
    a.N = p->N;
    a.num_samples = p->num_samples;
    a.region_size = p->region_size;
    a.max_slots = plan.max_block_slots;
    a.max_terms = plan.max_block_terms;
    a.max_groups = plan.max_block_groups;
    a.tile_counter = reinterpret_cast<uint32_t *>(scratch + 4);
    a.err = d_err;
    uint32_t ctas = 0;
    if (kind == KernelKind::kWindow) {
        const int occ = window_ctas_per_sm(w, g, window_smem_bytes(w, a.max_slots, a.max_terms, a.max_groups));
        if (occ <= 0) return fail(IDASH_ERR_CUDA, "window kernel cannot be resident");
        ctas = uint32_t(sm_count) * uint32_t(std::min(occ, 2));
    }
    ce = launch_score(kind, w, g, a, ctas, st);
    if (ce == cudaSuccess && (out_layout->variance_offset >= 0 || out_layout->header_offset >= 0)) {
        FinalizeArgs f{};
        f.var_ptr = reinterpret_cast<const uint64_t *>(scratch + np.o_var_ptr);
        f.var_row = reinterpret_cast<const uint32_t *>(scratch + np.o_var_row);
        f.var_coef = reinterpret_cast<const int32_t *>(scratch + np.o_var_coef);
        f.out_index = want_index ? reinterpret_cast<const uint32_t *>(scratch + np.o_out_index) : nullptr;
        f.out_row_map = nullptr;
        f.o_begin = 0;
        f.o_end = n_out;
        f.in_rows = static_cast<const uint8_t *>(d_in);
        f.in_stride = in_layout->row_stride;
        f.in_var_off = want_var ? in_layout->variance_offset : -1;
        f.out_rows = static_cast<uint8_t *>(d_out);
        f.out_stride = out_layout->row_stride;
        f.out_var_off = out_layout->variance_offset;
        f.out_hdr_off = out_layout->header_offset;
        f.tag = p->record_tag;
        ce = launch_finalize(f, st);
    }
    if (ce != cudaSuccess) return fail(IDASH_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(ce));
    // Return only once the outputs are written, with the kernels' verdict.
    ce = cudaStreamSynchronize(st);
    uint32_t word = 0;
    if (ce == cudaSuccess) ce = cudaMemcpy(&word, d_err, sizeof(word), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return fail(IDASH_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(ce));
    if (word == kDevTimeout) return fail(IDASH_ERR_DEVICE_TIMEOUT, "a device-side wait expired");
    if (word != kDevOk) return fail(IDASH_ERR_INDEX, "a kernel met an input row outside its buffer");
    return IDASH_OK;
}
