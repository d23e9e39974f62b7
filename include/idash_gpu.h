/*
 * idash_gpu.h — C ABI of the GB300 party-B scoring library (libidash_gpu.so).
 *
 * The library replaces the reference's cloud step,
 *   void cloud_compute_score(EncryptedPredictions&, const EncryptedData&,
 *                            const Model&, const IdashParams&)
 * (eval/idash.h:251-252, defined at eval/idash.cpp:763-848, called once from
 * eval/cloud.cpp:17), with hand-written sm_103a CUDA behind plain C entry
 * points: no C++ or torch types cross this boundary, every function returns an
 * idash_status and none aborts (the reference aborts through
 * REQUIRE_DRAMATICALLY, eval/idash.h:12).
 *
 * Vocabulary (the reference's):
 *   input feature   FeatBigIndex of a tag SNP's one-hot bit (eval/idash.h:40)
 *   FeatIndex       which TRLWE holds the feature: bidx / NUM_REGIONS (eval/idash.h:87)
 *   region          bidx % NUM_REGIONS: the slot block [r*REGION_SIZE, ...) (eval/idash.h:89)
 *   output          one (target position, genotype) model; FeatBigIndex out (eval/idash.h:129-134)
 *   constant        the model's "Constant" entry, feature 0xFFFFFFFF (eval/idash.h:93)
 * All ciphertext arithmetic is on Torus32 = Z/2^32 with wrap-around.
 */
#ifndef IDASH_GPU_H
#define IDASH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IDASH_GPU_ABI_VERSION 1
#define IDASH_CONSTANT_FEATURE 0xFFFFFFFFu

typedef enum {
    IDASH_OK = 0,
    IDASH_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, alignment or parameter */
    IDASH_ERR_CUDA = 2,             /* a CUDA runtime call failed (see idash_last_error) */
    IDASH_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed */
    IDASH_ERR_INDEX = 4,            /* a model term names a feature with no input ciphertext
                                       (the reference aborts here: eval/idash.h:164) */
    IDASH_ERR_DEVICE_TIMEOUT = 5,   /* a bounded device-side wait expired; results invalid */
    IDASH_ERR_IO = 6,               /* file could not be opened, read or written */
    IDASH_ERR_FORMAT = 7,           /* malformed params.bin / model / ciphertext file */
    IDASH_ERR_UNSUPPORTED = 8,      /* parameter outside what the kernels implement (k != 1 ...) */
    IDASH_ERR_ADMISSION = 9,        /* serving: request can never fit the HBM budget */
    IDASH_ERR_STATE = 10,           /* call out of order (e.g. score before a model is loaded) */
    IDASH_PENDING = 11              /* serving: the request is still in flight (idash_server_poll) */
} idash_status;

typedef struct idash_ctx idash_ctx;     /* one device, one stream, scratch, error word */
typedef struct idash_model idash_model; /* a resident, planned model (one layout) */

/* ---------------------------------------------------------------- context */
const char *idash_status_string(idash_status s);
int idash_abi_version(void);

/* Opens `device` and creates the context's stream.  Replaces nothing in the
 * reference (its only "context" is the OpenMP team, eval/idash.cpp:779). */
idash_status idash_open(idash_ctx **ctx, int device);
/* Waits for the context's work, frees every model still open on it, then the
 * context.  Models of a closed context must not be used or freed again. */
void idash_close(idash_ctx *ctx);
/* Human-readable detail of the last failure on this context ("" if none);
 * with ctx == NULL, why the last idash_open on this thread failed. */
const char *idash_last_error(const idash_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order work on it. */
void *idash_stream(idash_ctx *ctx);
/* Blocks until the context's stream is idle, then reads and clears the device
 * error word.  Returns IDASH_ERR_DEVICE_TIMEOUT / IDASH_ERR_INDEX if a kernel
 * reported one since the last check. */
idash_status idash_sync(idash_ctx *ctx);

/* Tunables: "kernel" (0 batched: autotuned among the persistent kernels,
 * 1 plain per-output kernel, 2 single-buffer persistent only, 3 double-buffer
 * persistent only, 4 warp-specialised producer/consumer ring only),
 * "slice_words" (0 = autotune; 128..2048), "ctas_per_sm",
 * "graph" (0/1: replay launches from a CUDA graph), "max_window_slots",
 * "max_group_terms", "split" (1, the default: the batched kernels take
 * neighbourhoods larger than one shared-memory window in parts, later parts
 * adding to the outputs in follow-up launches; 0: such models fall back to
 * the plain kernel). */
idash_status idash_set_option(idash_ctx *ctx, const char *name, int64_t value);
idash_status idash_get_option(const idash_ctx *ctx, const char *name, int64_t *value);

typedef struct {
    uint64_t kernel_launches;   /* scoring kernels launched by this context */
    uint64_t graph_launches;    /* CUDA-graph replays */
    uint64_t h2d_bytes, d2h_bytes;
} idash_stats;
idash_status idash_get_stats(const idash_ctx *ctx, idash_stats *out);

/* ------------------------------------------------------------ memory helpers
 * Device and page-locked host buffers owned by the caller (freed with the
 * matching *_free).  Copies are ordered on the context's stream. */
idash_status idash_device_alloc(idash_ctx *ctx, size_t bytes, void **ptr);
idash_status idash_device_free(idash_ctx *ctx, void *ptr);
idash_status idash_host_alloc(idash_ctx *ctx, size_t bytes, void **ptr);
idash_status idash_host_free(idash_ctx *ctx, void *ptr);
idash_status idash_copy_h2d(idash_ctx *ctx, void *dst, const void *src, size_t bytes);
idash_status idash_copy_d2h(idash_ctx *ctx, void *dst, const void *src, size_t bytes);
idash_status idash_memset_device(idash_ctx *ctx, void *dst, int value, size_t bytes);

/* ------------------------------------------------------------- row layouts
 * Ciphertexts live in rows.  A TRLWE row (k = 1) is 2N int32 coefficients:
 * the mask a[0..N) then the body b[0..N).  A row may sit inside a larger
 * record, e.g. one entry of encrypted_data.bin / encrypted_prediction.bin
 * (eval/idash.cpp:540-556, :596-613):
 *   uint32 FeatIndex/FeatBigIndex | int32 record tag | 2N int32 | double variance
 * which is 8208 bytes: layout {8208, 8, 8200, 0} with `base` = file image + 8. */
typedef struct {
    uint64_t row_stride;     /* bytes between consecutive rows; multiple of 16 */
    uint64_t payload_offset; /* bytes from row start to coefficient 0; base+offset 16-byte aligned */
    int64_t variance_offset; /* bytes to the double current_variance, or -1 */
    int64_t header_offset;   /* outputs: bytes to (uint32 index, int32 tag), or -1 */
} idash_row_layout;

/* ------------------------------------------- TRLWE-packed scoring (drop-in)
 * Parameters of IdashParams that the scoring step reads (eval/idash.h:45-80,
 * eval/idash.cpp:766-770). */
typedef struct {
    uint32_t N;           /* TRLWE polynomial size, IdashParams::N (1024) */
    uint32_t k;           /* must be 1 (eval/idash.cpp:768) */
    uint32_t num_samples; /* NUM_SAMPLES: individuals packed per region */
    uint32_t num_regions; /* NUM_REGIONS */
    uint32_t region_size; /* REGION_SIZE; num_regions*region_size <= N */
    int32_t one_t32;      /* ONE_IN_T32 = dtot32(2^-14) = 2^18 (eval/idash.cpp:39) */
    int32_t record_tag;   /* tag written into output record headers */
} idash_trlwe_params;

/* Loads a Model (eval/idash.h:129-134) flattened to CSR and plans it for the
 * device: output o's terms are term_feat/term_coef[term_ptr[o] .. term_ptr[o+1]),
 * in the order the caller iterates the model (that order only matters for the
 * double variance bookkeeping).  Outputs should be numbered so that
 * neighbouring targets are adjacent (FeatBigIndex order is): consecutive
 * outputs share input windows.  out_index[o] is the output's FeatBigIndex,
 * written into record headers (NULL: o).  out_row[o] is the output row that
 * receives output o (NULL: row o; must be a permutation of [0, n_out)); the
 * host-memory path requires NULL.  in_row_of_index maps FeatIndex to the
 * input row that holds it (NULL: identity); n_in_rows bounds it.
 * Replaces the setup half of cloud_compute_score (eval/idash.cpp:772-777). */
idash_status idash_model_trlwe(idash_ctx *ctx, idash_model **model, const idash_trlwe_params *params,
                               uint64_t n_out, const uint32_t *out_index, const uint32_t *out_row,
                               const uint64_t *term_ptr, const uint32_t *term_feat, const int32_t *term_coef,
                               uint64_t n_in_index, const uint32_t *in_row_of_index, uint64_t n_in_rows);

/* Scores every output of a TRLWE model: the hot loop of cloud_compute_score
 * (eval/idash.cpp:779-842).  d_in / d_out are device pointers to row 0 of the
 * input and output rows; output o goes to row o.  Asynchronous on `stream`
 * (NULL = the context's stream). */
idash_status idash_score_trlwe_device(idash_model *model, const void *d_in, const idash_row_layout *in_layout,
                                      void *d_out, const idash_row_layout *out_layout, void *stream);

/* Same, end to end from host memory: copies the input rows in, scores, and
 * copies the output rows back, overlapping the copies with the kernels in
 * chunks.  Host buffers should be page-locked (idash_host_alloc).  Returns
 * after the outputs are in h_out. */
idash_status idash_score_trlwe_host(idash_model *model, const void *h_in, const idash_row_layout *in_layout,
                                    uint64_t n_in_rows, void *h_out, const idash_row_layout *out_layout);

/* Scores outputs [out_begin, out_end) only (e.g. the contiguous targets of
 * one serving request): output o goes to row (o - out_begin) of d_out.  The
 * input holds n_in_rows rows; plan row r (FeatIndex, or in_row_of_index's
 * value) is read from row (r - in_row_base).  num_samples (0 = the model's)
 * is the number of packed individuals that receive the bias.  Asynchronous
 * on `stream` (NULL: the context's stream); no graph, no autotuning. */
idash_status idash_score_trlwe_range(idash_model *model, uint64_t out_begin, uint64_t out_end, uint32_t num_samples,
                                     const void *d_in, const idash_row_layout *in_layout, uint64_t in_row_base,
                                     uint64_t n_in_rows, void *d_out, const idash_row_layout *out_layout,
                                     void *stream);
/* The input rows [row_begin, row_end) that outputs [out_begin, out_end) read. */
idash_status idash_model_input_rows(const idash_model *model, uint64_t out_begin, uint64_t out_end,
                                    uint64_t *row_begin, uint64_t *row_end);

/* ------------------------------------------- serving (continuous batching)
 * No counterpart in the reference (its cloud binary scores one batch per
 * process, eval/cloud.cpp:3-28).  A server keeps one model resident (TRLWE
 * planned with NUM_REGIONS = 1, or LWE; planned for the warp-specialised
 * kernel, "kernel" option 4 or autotuned to it) and serves imputation
 * requests submitted at any time, from any thread, while others run.
 *
 * A request is n_indiv individuals and the contiguous targets
 * [target_begin, target_end): outputs 3*target_begin .. 3*target_end, which
 * read the input rows [row_begin, row_end) of idash_model_input_rows.
 *   TRLWE: individuals packed REGION_SIZE per block, ceil(n_indiv /
 *     REGION_SIZE) blocks; input: blocks x (row_end - row_begin) rows, output:
 *     blocks x (3 * targets) rows, dense 2N int32 rows (block-major).
 *   LWE: input: (row_end - row_begin) rows, output: 3 * targets rows, each of
 *     n_indiv samples of n+1 int32 at a stride of n_indiv*(n+1) rounded up to
 *     a multiple of 4 words; n_indiv at most the model's.
 * h_in NULL: the inputs are generated on the device from `seed` (TRLWE
 * block b: idash_synth_uniform_device with seed * 0x9E3779B97F4A7C15 + b; LWE
 * the same with b = 0, row_words n_indiv*(n+1)); h_out NULL: only the digest
 * is kept.  Host buffers should be page-locked (idash_host_alloc) for
 * full-speed copies, and stay untouched until the request completes.
 *
 * The scheduler admits requests in submission order while fewer than
 * max_inflight are admitted and the HBM budget holds their inputs and one
 * output segment (segment_outputs outputs; 0 = all of a TRLWE request, 2,048
 * for LWE).  Every launch scores the staged segments of all admitted
 * requests together (onto an idle device, about half of them, so that the
 * next launch is queued behind it): one persistent kernel over a job table.  Inputs are
 * copied in and outputs out on their own streams, overlapped with the
 * launches.  A request's outputs and digest do not depend on what else runs
 * beside it.  While a server runs on a model, use the model only through it. */
typedef struct idash_server idash_server;
typedef struct {
    uint64_t hbm_budget;      /* device bytes the admitted requests may hold together */
    uint32_t max_inflight;    /* requests admitted at once, 1 .. 4096 */
    uint32_t segment_outputs; /* outputs per segment (0: the form's default) */
} idash_serve_config;
typedef struct {
    uint32_t n_indiv;                  /* individuals in the request */
    uint32_t reserved;
    uint64_t target_begin, target_end; /* contiguous target SNPs */
    const void *h_in;                  /* host input rows, or NULL: generated from seed */
    void *h_out;                       /* host output rows, or NULL: digest only */
    uint64_t seed;
} idash_serve_request;
typedef struct {
    double admit_s;        /* admission, seconds after idash_server_open (host clock) */
    double done_s;         /* completion: outputs in h_out (or scored), seconds after open (CUDA events) */
    uint64_t device_bytes; /* HBM the request held at admission (inputs + one output segment) */
    uint64_t digest;       /* sum mod 2^64, over the aligned quads of its output words (word
                              positions 4Q .. 4Q+3 in the output layout above), of a 32-bit hash
                              of (Q, the quad's words); idash_digest_host restates it */
} idash_request_result;

idash_status idash_server_open(idash_model *model, const idash_serve_config *config, idash_server **server);
/* Queues a request; *ticket names it.  Fails with IDASH_ERR_ADMISSION when
 * the request could never fit the budget, IDASH_ERR_INVALID_ARGUMENT when it
 * is empty or out of range. */
idash_status idash_server_submit(idash_server *server, const idash_serve_request *request, uint64_t *ticket);
/* IDASH_OK and *result when the request is complete, IDASH_PENDING while it
 * is in flight, or the request's error. */
idash_status idash_server_poll(idash_server *server, uint64_t ticket, idash_request_result *result);
/* Blocks until the request completes (or fails). */
idash_status idash_server_wait(idash_server *server, uint64_t ticket, idash_request_result *result);
/* Kernel launches so far (each scores the segments staged at that time). */
uint64_t idash_server_launches(const idash_server *server);
typedef struct {
    uint64_t launches;       /* scoring launches issued */
    uint64_t requests_done;  /* requests completed */
    double busy_s;           /* device time of the completed scoring launches, summed (CUDA events) */
    uint64_t h2d_bytes;      /* request input bytes copied in from host memory */
    uint64_t d2h_bytes;      /* request output bytes copied out to host memory */
} idash_server_stats;
/* Counters since idash_server_open; busy_s / elapsed time is the share of the
 * time the device spent scoring. */
idash_status idash_server_get_stats(idash_server *server, idash_server_stats *stats);
/* Finishes every submitted request, then frees the server. */
idash_status idash_server_close(idash_server *server);
/* Why the server failed, else why the last refused submit was refused ("" if neither). */
const char *idash_server_last_error(const idash_server *server);

/* The whole stream in one call, on a server opened for it: request i is
 * submitted at arrival_s seconds after the start (synthetic inputs from
 * seed, outputs to host_out[i] when non-NULL) and results[i] filled.  A
 * request larger than the budget fails with IDASH_ERR_ADMISSION before
 * anything runs.  TRLWE models only. */
typedef struct {
    double arrival_s;                  /* seconds after the run starts */
    uint32_t n_indiv;                  /* individuals in the request */
    uint32_t reserved;
    uint64_t target_begin, target_end; /* contiguous target SNPs */
    uint64_t seed;                     /* the request's synthetic ciphertexts */
} idash_request;
idash_status idash_serve_trlwe(idash_model *model, const idash_serve_config *config, const idash_request *requests,
                               uint64_t n_requests, idash_request_result *results, void *const *host_out);
/* Host restatement of the serving digest, for checking results. */
uint64_t idash_digest_host(const uint32_t *words, uint64_t n_words, uint64_t index_base);

/* ------------------------------------------- per-individual LWE scoring
 * Each individual's one-hot bit is its own LWE sample (n mask words + body).
 * Input row f holds n_indiv samples of (n+1) int32, row stride in words a
 * multiple of 4.  Output o, row (o - out_begin) of d_out, same layout.  The
 * result for individual i equals SampleExtract_i of the TRLWE form. */
typedef struct {
    uint32_t n;       /* LWE dimension (1024) */
    uint32_t n_indiv; /* individuals per row */
    int32_t one_t32;  /* constant scaling (2^18) */
} idash_lwe_params;

idash_status idash_model_lwe(idash_ctx *ctx, idash_model **model, const idash_lwe_params *params,
                             uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                             const int32_t *term_coef, uint64_t n_feat_rows);
/* Scores outputs [out_begin, out_end) (any range; outputs beyond HBM are
 * produced range by range).  n_indiv may be smaller than the model's (serving
 * requests of fewer individuals); strides are in int32 words. */
idash_status idash_score_lwe_device(idash_model *model, uint32_t n_indiv, const int32_t *d_in,
                                    uint64_t in_row_stride, uint64_t out_begin, uint64_t out_end,
                                    int32_t *d_out, uint64_t out_row_stride, void *stream);

/* ------------------------------------------- integer-polynomial x TRLWE
 * The generalisation of the TRLWE form to dense integer-polynomial weights:
 * out_o = sum_f W_{o,f}(X) * C_f(X) mod (X^N + 1, 2^32) on both polynomials,
 * then b[s] += bias_o * one_t32 for s < num_samples, b[j] = 0 for
 * j >= region_size.  The reference's terms are W = coef * X^(-r*REGION_SIZE)
 * (eval/idash.cpp:817, 830-833).  Exact: two-prime NTT + CRT, no floating
 * point.  Terms per output must satisfy terms * max_abs_coef * N * 2^31 <
 * p1*p2/2 (about 127 terms at |W| <= 8192); checked at model creation. */
typedef struct {
    uint32_t N;            /* 1024 */
    uint32_t num_samples;  /* b slots that receive the bias */
    uint32_t region_size;  /* b[j] = 0 for j >= region_size (N: none) */
    int32_t one_t32;       /* bias scaling (2^18) */
    int32_t max_abs_coef;  /* bound on |W| coefficients (8192) */
} idash_intpoly_params;
/* term_poly: [nnz][N] int16 weight polynomials (host, or device when
 * term_poly_on_device); term_feat: the input TRLWE row of each term; bias:
 * one integer per output (NULL: 0).  The weights are transformed once and
 * kept resident (nnz * 8 KiB of HBM at N = 1024). */
idash_status idash_model_intpoly(idash_ctx *ctx, idash_model **model, const idash_intpoly_params *params,
                                 uint64_t n_out, const uint64_t *term_ptr, const uint32_t *term_feat,
                                 const int32_t *bias, uint64_t n_in_rows, const int16_t *term_poly,
                                 int term_poly_on_device);
/* Replaces the model's weights in place: d_term_poly holds new [nnz][N]
 * int16 polynomials (device memory) for the same terms; they are
 * transformed into the resident form on `stream` (NULL: the context's),
 * asynchronously.  A coefficient beyond max_abs_coef is reported by the next
 * synchronising call as IDASH_ERR_INDEX; that term's resident weights are
 * then undefined until replaced again. */
idash_status idash_model_intpoly_set_weights(idash_model *model, const int16_t *d_term_poly, void *stream);
/* Scores outputs [out_begin, out_end) (output o -> row o - out_begin) from
 * the n_in_rows input TRLWE rows at d_in.  Asynchronous on `stream`. */
idash_status idash_score_intpoly_device(idash_model *model, const void *d_in, const idash_row_layout *in_layout,
                                        uint64_t out_begin, uint64_t out_end, void *d_out,
                                        const idash_row_layout *out_layout, void *stream);
/* Seeded int16 weights uniform in [-max_abs, max_abs) on the device. */
idash_status idash_synth_int16_device(idash_ctx *ctx, uint64_t seed, uint64_t n, int32_t max_abs, int16_t *d_out,
                                      void *stream);

/* Model facts: outputs, total terms, planned blocks, slice width chosen.
 * kernel: 0 window, 1 direct (plain), 2 pipe, 3 warp-specialised, 4 tensor
 * cores.  dense_k: tensor-core plans only, the sum over blocks of the padded
 * K (each block multiplies a 128 x dense_k coefficient matrix per column
 * slice; 0 for the other kernels). */
typedef struct {
    uint64_t n_out, n_terms, n_groups, n_blocks, n_slots;
    uint32_t slice_words, max_window_slots, kernel;
    uint64_t algorithmic_in_rows; /* distinct input rows the model reads */
    uint64_t dense_k;
} idash_model_info;
idash_status idash_model_get_info(const idash_model *model, idash_model_info *info);
/* Re-plans the model for a new kernel / slice choice (after idash_set_option). */
idash_status idash_model_replan(idash_model *model);
void idash_model_free(idash_model *model);

/* ------------------------------------------- scoring without allocation
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a service whose framework reserves the GPU's memory for its own pool, a
 * process at its per-client device-memory limit, or a latency-bound loop
 * that cannot take the implicit synchronisation of cudaMalloc/cudaFree.  The
 * caller passes the model as host CSR with the same arguments and meaning as
 * idash_model_trlwe (out_index: FeatBigIndex per output for record headers,
 * NULL: o; in_row_of_index: FeatIndex -> input row, NULL: identity), and
 * device input and output rows as idash_score_trlwe_device (output o -> row
 * o); nothing else comes from the device heap.  The plan, tile counter, error
 * word, variance program and output index table live in a fixed 64 MiB array
 * that every GPU loading the library holds until the process exits (the
 * full-scale model, 242,646 outputs with 5 neighbours in the reference's
 * record layout, needs about 52 MiB); a model whose tables do not fit is
 * refused with IDASH_ERR_INVALID_ARGUMENT before anything is launched.
 * Runs on the calling thread's current device, on `stream` (NULL: the legacy
 * default stream), and returns after the outputs are written.  The first call
 * on a device resolves the array's address with that device current; make
 * that first call before any stream capture.  Every call reuses the same
 * array (it keeps the last call's contents; what must start at zero is
 * cleared by each call): calls that overlap on one GPU, from several threads
 * or streams, race and must be serialised by the caller.  Host-side planning
 * uses ordinary heap memory; no device or page-locked memory is allocated. */
idash_status idash_score_trlwe_noalloc(const idash_trlwe_params *params, uint64_t n_out, const uint32_t *out_index,
                                       const uint64_t *term_ptr, const uint32_t *term_feat,
                                       const int32_t *term_coef, uint64_t n_in_index,
                                       const uint32_t *in_row_of_index, uint64_t n_in_rows, const void *d_in,
                                       const idash_row_layout *in_layout, void *d_out,
                                       const idash_row_layout *out_layout, void *stream);

/* ------------------------------------------- the cloud step on files
 * eval/cloud.cpp:3-28 as one call: reads params.bin (eval/idash.cpp:200-261),
 * the model directory of <pos>_<snp>.hr files (eval/idash.cpp:66-114) and
 * encrypted_data.bin (:513-535), scores on `device`, and writes
 * encrypted_prediction.bin (:596-613) with the records in the order the
 * reference writes them.  Ciphertext files move as single bulk images.
 * With IDASH_MODEL_CACHE=<file> in the environment the flattened model is
 * read from that file when it matches params.bin and the model directory,
 * and written there otherwise (remove it when the .hr files change). */
typedef struct {
    double read_s;   /* params + model + ciphertext file reads */
    double plan_s;   /* model flattening and device planning */
    double score_s;  /* host->device copy, kernels, device->host copy */
    double write_s;  /* prediction file write */
    uint64_t n_in_records, n_out_records;
    uint32_t model_from_cache; /* 1: the model came from the IDASH_MODEL_CACHE file */
    uint32_t reserved;
} idash_cloud_report;
idash_status idash_cloud_files(int device, const char *params_file, const char *model_dir, const char *data_file,
                               const char *pred_file, idash_cloud_report *report, char *errbuf, size_t errbuf_len);

/* ------------------------------------------- encryption (party A)
 * encrypt_data_ph1 + encrypt_data_ph2 (eval/idash.cpp:615-679) on the
 * device.  Row r (of n_rows) becomes a fresh TRLWE encryption of zero under
 * `key` (tLweSymEncryptZero, :625): mask a uniform, noise e Gaussian with
 * standard deviation alpha on the torus (truncated as dtot32), b = a*s + e;
 * then the one-hot messages are added as setScore does (eval/idash.h:152-156):
 * for region g < num_regions and sample s < num_samples, coefficient
 * b[g*region_size + s] gains the value of plaintext feature
 * src = d_slot_src[r*num_regions + g] (3p + v: genotype row p, genotype
 * value v; 0xFFFFFFFF: none): one_t32 when d_geno[p*geno_stride + s] == v,
 * nan_t32[v] when that genotype is not 0, 1 or 2 (missing), else 0.
 * Row r is written at output row d_row_out[r] (NULL: r); with a header in
 * out_layout it gets index d_row_index[r] (NULL: r) and record_tag, and the
 * variance field gets alpha^2.  Masks and noise come from a counter-based
 * generator keyed by `seed` (a statistical generator, as TFHE's is, not a
 * cryptographic one).  d_noise (optional, n_rows * N int32) receives e.
 * key: N integer coefficients in host memory; N a power of two in [4, 2048].
 * Asynchronous on `stream` once the key has been staged. */
typedef struct {
    uint32_t N, k;          /* k must be 1 */
    uint32_t num_samples;   /* NUM_SAMPLES */
    uint32_t num_regions;   /* NUM_REGIONS */
    uint32_t region_size;   /* REGION_SIZE */
    int32_t one_t32;        /* ONE_IN_T32 = dtot32(2^-14) (eval/idash.cpp:39) */
    int32_t nan_t32[3];     /* NAN_{0,1,2}_IN_T32 = dtot32({3,2,1}/6 * 2^-14) (:40-45) */
    int32_t record_tag;     /* tag written into record headers */
    double alpha;           /* noise standard deviation on the torus (IdashParams::alpha = 2^-25) */
} idash_encrypt_params;
idash_status idash_encrypt_trlwe_device(idash_ctx *ctx, const idash_encrypt_params *params, const int32_t *key,
                                        uint64_t seed, uint64_t n_rows, const uint32_t *d_slot_src,
                                        const int8_t *d_geno, uint32_t geno_stride, const uint32_t *d_row_index,
                                        const uint32_t *d_row_out, void *d_out, const idash_row_layout *out_layout,
                                        int32_t *d_noise, void *stream);

/* eval/encrypt.cpp:14-38 as one call: reads keys.bin and the challenge file
 * of tag genotypes (read_plaintext_data, eval/idash.cpp:280-309: lines
 * "22 <pos> <pos> <name> <g_0> ... <g_{NUM_SAMPLES-1}>", a genotype other than
 * 0/1/2 counts as missing), encrypts on `device`, and writes
 * encrypted_data.bin with the records (FeatIndex, tag, TRLWE, variance) in the
 * order the reference writes them (:536-556).  The ciphertexts differ from
 * the reference's (another random generator); they decrypt to the same
 * messages.  seed 0 draws a fresh seed from the operating system. */
typedef struct {
    double read_s;     /* key + challenge file reads */
    double encrypt_s;  /* planning, kernel, device->host copy */
    double write_s;    /* encrypted_data.bin write */
    uint64_t n_positions, n_records;
} idash_encrypt_report;
idash_status idash_encrypt_files(int device, const char *keys_file, const char *challenge_file, const char *data_file,
                                 uint64_t seed, idash_encrypt_report *report, char *errbuf, size_t errbuf_len);

/* ------------------------------------------- decryption (party A)
 * decrypt_predictions (eval/idash.cpp:682-761) on the device: for each of
 * n_rows TRLWE rows (k = 1, layout in_layout), the phase b - a*s (tLwePhase,
 * an exact negacyclic product mod X^N + 1 over Z/2^32 with the integer key s)
 * at coefficients [0, num_samples), converted as t32tod to float:
 * d_out[r * num_samples + j] = float(phase_r[j] / 2^32).  key: the key's N
 * integer coefficients in host memory (binary for TFHE keys; any integers
 * are accepted).  N a power of two in [4, 2048].  Asynchronous on `stream`
 * once the key has been staged (the call synchronises with `stream` first). */
idash_status idash_decrypt_trlwe_device(idash_ctx *ctx, const int32_t *key, uint32_t N, const void *d_in,
                                        const idash_row_layout *in_layout, uint64_t n_rows, uint32_t num_samples,
                                        float *d_out, void *stream);

/* eval/decrypt.cpp:13-48 as one call: reads keys.bin (read_key,
 * eval/idash.cpp:488-502: params.bin's content followed by the key record)
 * and encrypted_prediction.bin, decrypts on `device`, and writes the CSV of
 * write_decrypted_predictions (eval/idash.cpp:436-469) byte for byte: header
 * "Subject ID,target SNP,0,1,2", then one line per (sample, output position)
 * with the position's name (by_position = 0) or number (by_position = 1) and
 * the three scores printed as an iostream prints a float (6 significant
 * digits).  Key record: int32 tag, int32 N, int32 k, double alpha_min,
 * double alpha_max, k * N int32 coefficients. */
typedef struct {
    double read_s;     /* key + prediction file reads */
    double decrypt_s;  /* host->device copy, phase kernel, device->host copy */
    double write_s;    /* CSV formatting and write */
    uint64_t n_records, n_lines;
} idash_decrypt_report;
idash_status idash_decrypt_files(int device, const char *keys_file, const char *pred_file, const char *csv_file,
                                 int by_position, idash_decrypt_report *report, char *errbuf, size_t errbuf_len);

/* ------------------------------------------- synthetic workloads (host)
 * Seeded synthetic imputation models with the reference's shapes: tag SNPs at
 * sorted positions, targets at sorted random positions, each target's
 * neighbours = its k nearest tags (train/to_vw.py:33-34), 3 outputs per target
 * with coefficients uniform in [-8192, 8191] (zeros dropped,
 * train/test_vw_hr.py:44) and an integer bias.  Features are numbered as the
 * reference's keygen numbers them: tag p owns 3p, 3p+1, 3p+2
 * (eval/idash.cpp:388-390); target t owns outputs 3t..3t+2 (:337-339). */
typedef struct {
    uint64_t seed;
    uint32_t n_tags, n_targets;
    uint32_t neighbours;          /* fixed neighbour count, or 0 to draw from choices[] */
    uint32_t n_choices;
    uint32_t choices[8];          /* e.g. {5,10,20,30,50} */
} idash_synth_spec;

typedef struct {
    uint64_t n_out, n_terms;
    uint64_t *term_ptr;     /* n_out + 1 */
    uint32_t *term_feat;    /* n_terms */
    int32_t *term_coef;     /* n_terms */
    uint64_t *tag_pos;      /* n_tags positions (sorted) */
    uint64_t *target_pos;   /* n_targets positions (sorted) */
    uint32_t *window_start; /* per target: first neighbour tag */
    uint32_t *window_len;   /* per target: neighbour count */
} idash_synth_model_t;

idash_status idash_synth_model(const idash_synth_spec *spec, idash_synth_model_t *out);
void idash_synth_model_free(idash_synth_model_t *m);

/* Device generators of synthetic ciphertexts (valid encryptions under a
 * seeded binary key, one-hot genotypes, noise sd ~2^-25): per-individual LWE
 * rows, and TRLWE rows packing num_samples individuals per region. */
idash_status idash_synth_lwe_device(idash_ctx *ctx, uint64_t seed, uint32_t n, uint32_t n_indiv,
                                    uint64_t n_feat_rows, int32_t *d_out, uint64_t row_stride, void *stream);
idash_status idash_synth_trlwe_device(idash_ctx *ctx, uint64_t seed, const idash_trlwe_params *params,
                                      uint32_t n_tags, void *d_out, const idash_row_layout *layout, void *stream);
/* The binary key those generators encrypt under: N coefficients in {0, 1}. */
void idash_synth_key(uint64_t seed, uint32_t N, int32_t *out);
/* Uniformly random ciphertext rows (statistically the same as encryptions):
 * word j of global row r = hash(seed, r * row_words + j); rows
 * [row_begin, row_begin + n_rows) are written from d_out on. */
idash_status idash_synth_uniform_device(idash_ctx *ctx, uint64_t seed, uint64_t row_begin, uint64_t n_rows,
                                        uint32_t row_words, void *d_out, uint64_t row_stride, void *stream);

#ifdef __cplusplus
}
#endif

#endif
