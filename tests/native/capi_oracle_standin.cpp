// TEST INFRASTRUCTURE ONLY.  A CPU stand-in for the entry points of
// include/idash_gpu.h that the reference-side adapters call
// (idash2019_2_gb300/integration/cloud_compute_score_gpu.cpp and
// party_a_gpu.cpp), computed by the oracle's restatement (oracle/oracle.c).
//
// Linked in place of libidash_gpu.so into the reference's own cloud and
// decrypt mains, it lets a machine without a GPU check the adapters' own
// logic end to end: record order, FeatIndex -> row maps, record layouts and
// the variance bookkeeping, against the files the reference writes.  "Device"
// memory is host memory here; no entry point touches a GPU.
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "idash_gpu.h"
#include "oracle.h"

struct idash_ctx {
    std::string last_error;
};

struct idash_model {
    idash_ctx *ctx = nullptr;
    idash_trlwe_params p{};
    uint64_t n_out = 0, n_in_rows = 0;
    std::vector<uint64_t> term_ptr;
    std::vector<uint32_t> term_feat, out_index, row_of_index;
    std::vector<int32_t> term_coef;
};

namespace {
std::string g_thread_error;

idash_status fail(idash_ctx *ctx, idash_status s, const char *msg) {
    (ctx ? ctx->last_error : g_thread_error) = msg;
    return s;
}
}  // namespace

extern "C" {

const char *idash_status_string(idash_status s) { return s == IDASH_OK ? "ok" : "error (oracle stand-in)"; }

idash_status idash_open(idash_ctx **ctx, int device) {
    (void)device;
    if (!ctx) return IDASH_ERR_INVALID_ARGUMENT;
    *ctx = new idash_ctx();
    return IDASH_OK;
}

void idash_close(idash_ctx *ctx) { delete ctx; }

const char *idash_last_error(const idash_ctx *ctx) { return ctx ? ctx->last_error.c_str() : g_thread_error.c_str(); }

idash_status idash_sync(idash_ctx *ctx) { return ctx ? IDASH_OK : IDASH_ERR_INVALID_ARGUMENT; }

static idash_status host_alloc(idash_ctx *ctx, size_t bytes, void **ptr) {
    if (!ctx || !ptr) return IDASH_ERR_INVALID_ARGUMENT;
    *ptr = std::aligned_alloc(64, (bytes + 63) & ~size_t(63));
    return *ptr ? IDASH_OK : fail(ctx, IDASH_ERR_OUT_OF_MEMORY, "aligned_alloc");
}
idash_status idash_host_alloc(idash_ctx *ctx, size_t bytes, void **ptr) { return host_alloc(ctx, bytes, ptr); }
idash_status idash_device_alloc(idash_ctx *ctx, size_t bytes, void **ptr) { return host_alloc(ctx, bytes, ptr); }
idash_status idash_host_free(idash_ctx *ctx, void *ptr) {
    (void)ctx;
    std::free(ptr);
    return IDASH_OK;
}
idash_status idash_device_free(idash_ctx *ctx, void *ptr) { return idash_host_free(ctx, ptr); }
idash_status idash_copy_h2d(idash_ctx *ctx, void *dst, const void *src, size_t bytes) {
    (void)ctx;
    std::memcpy(dst, src, bytes);
    return IDASH_OK;
}
idash_status idash_copy_d2h(idash_ctx *ctx, void *dst, const void *src, size_t bytes) {
    return idash_copy_h2d(ctx, dst, src, bytes);
}

idash_status idash_model_trlwe(idash_ctx *ctx, idash_model **model, const idash_trlwe_params *p, uint64_t n_out,
                               const uint32_t *out_index, const uint32_t *out_row, const uint64_t *term_ptr,
                               const uint32_t *term_feat, const int32_t *term_coef, uint64_t n_in_index,
                               const uint32_t *in_row_of_index, uint64_t n_in_rows) {
    if (!ctx || !model || !p || !term_ptr) return IDASH_ERR_INVALID_ARGUMENT;
    if (out_row) return fail(ctx, IDASH_ERR_UNSUPPORTED, "stand-in: out_row not supported");
    idash_model *m = new idash_model();
    m->ctx = ctx;
    m->p = *p;
    m->n_out = n_out;
    m->n_in_rows = n_in_rows;
    m->term_ptr.assign(term_ptr, term_ptr + n_out + 1);
    m->term_feat.assign(term_feat, term_feat + term_ptr[n_out]);
    m->term_coef.assign(term_coef, term_coef + term_ptr[n_out]);
    if (out_index) m->out_index.assign(out_index, out_index + n_out);
    if (in_row_of_index) m->row_of_index.assign(in_row_of_index, in_row_of_index + n_in_index);
    *model = m;
    return IDASH_OK;
}

void idash_model_free(idash_model *m) { delete m; }

idash_status idash_score_trlwe_host(idash_model *m, const void *h_in, const idash_row_layout *il, uint64_t n_in_rows,
                                    void *h_out, const idash_row_layout *ol) {
    if (!m || !h_in || !h_out || !il || !ol) return IDASH_ERR_INVALID_ARGUMENT;
    const uint64_t W = 2ull * m->p.N;
    const uint8_t *in = static_cast<const uint8_t *>(h_in);
    uint8_t *out = static_cast<uint8_t *>(h_out);
    std::vector<int32_t> rows(n_in_rows * W), res(m->n_out * W);
    std::vector<double> var_in(n_in_rows, 0.0), var_out(m->n_out, 0.0);
    for (uint64_t r = 0; r < n_in_rows; ++r) {
        std::memcpy(&rows[r * W], in + r * il->row_stride + il->payload_offset, W * 4);
        if (il->variance_offset >= 0) std::memcpy(&var_in[r], in + r * il->row_stride + il->variance_offset, 8);
    }
    const int rc = oracle_trlwe_score(m->p.N, m->p.num_samples, m->p.num_regions, m->p.region_size, m->p.one_t32,
                                      m->n_out, m->term_ptr.data(), m->term_feat.data(), m->term_coef.data(),
                                      m->row_of_index.empty() ? nullptr : m->row_of_index.data(),
                                      m->row_of_index.size(), n_in_rows, rows.data(),
                                      il->variance_offset >= 0 ? var_in.data() : nullptr, res.data(), var_out.data(),
                                      1);
    if (rc == -2) return fail(m->ctx, IDASH_ERR_INDEX, "a term names a feature without an input row");
    if (rc != 0) return fail(m->ctx, IDASH_ERR_INVALID_ARGUMENT, "oracle_trlwe_score refused the parameters");
    for (uint64_t o = 0; o < m->n_out; ++o) {
        uint8_t *rec = out + o * ol->row_stride;
        std::memcpy(rec + ol->payload_offset, &res[o * W], W * 4);
        if (ol->variance_offset >= 0) std::memcpy(rec + ol->variance_offset, &var_out[o], 8);
        if (ol->header_offset >= 0) {
            const uint32_t idx = m->out_index.empty() ? uint32_t(o) : m->out_index[o];
            std::memcpy(rec + ol->header_offset, &idx, 4);
            std::memcpy(rec + ol->header_offset + 4, &m->p.record_tag, 4);
        }
    }
    return IDASH_OK;
}

idash_status idash_decrypt_trlwe_device(idash_ctx *ctx, const int32_t *key, uint32_t N, const void *d_in,
                                        const idash_row_layout *in_layout, uint64_t n_rows, uint32_t num_samples,
                                        float *d_out, void *stream) {
    (void)stream;
    if (!ctx || !key || !d_in || !in_layout || !d_out) return IDASH_ERR_INVALID_ARGUMENT;
    if (in_layout->row_stride % 4 || in_layout->payload_offset % 4)
        return fail(ctx, IDASH_ERR_INVALID_ARGUMENT, "stand-in: word-aligned layouts only");
    const int32_t *rows =
        reinterpret_cast<const int32_t *>(static_cast<const uint8_t *>(d_in) + in_layout->payload_offset);
    oracle_trlwe_decrypt(N, key, n_rows, in_layout->row_stride / 4, rows, num_samples, d_out, 1);
    return IDASH_OK;
}

idash_status idash_encrypt_trlwe_device(idash_ctx *ctx, const idash_encrypt_params *, const int32_t *, uint64_t,
                                        uint64_t, const uint32_t *, const int8_t *, uint32_t, const uint32_t *,
                                        const uint32_t *, void *, const idash_row_layout *, int32_t *, void *) {
    return fail(ctx, IDASH_ERR_UNSUPPORTED, "stand-in: encryption draws fresh randomness; not restated");
}

}  // extern "C"
