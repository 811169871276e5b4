/*
 * gsea103.h -- C ABI of libgsea103.so, the GB300 (sm_103a) implementation of
 * cudaGSEA's GSEA permutation pipeline.
 *
 * Every entry point returns a gsea_status (0 = success) and never exits the
 * process; the reference instead calls exit() on CUDA errors and unknown
 * metrics (src/include/cuda_helpers.cuh:10-17, correlate_genes.cuh:292-295).
 * A human-readable message for the last failure on the calling thread is
 * available from gsea_last_error().
 *
 * Layouts (identical to the reference's R path):
 *   exprs   patient-major [num_samples][num_genes]
 *           (src/cudaGSEA_wrapper.cu:229-236 keeps R's column-major table as is)
 *   labels  uint8 [num_samples], 0 = class A, 1 = class B
 *   sets    CSR over gene indices: set k = set_genes[set_offsets[k] ..
 *           set_offsets[k+1]); indices outside [0, num_genes) are ignored and
 *           duplicates collapse, as create_bitmaps does for unknown symbols
 *           (src/include/create_bitmaps.cuh:13-65)
 *   es      [num_sets][num_perms] row-major, permutation 0 = observed labels
 *           (the .es dump layout, src/include/dump_binary.cuh:10-30)
 *   stats   struct of arrays [5][num_sets]: ES, NES, NP, FWER, FDR
 *           (src/include/statistics.cuh:46-117; FDR is filled here, the
 *           reference leaves it NaN)
 */
#ifndef GSEA103_H
#define GSEA103_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSEA103_VERSION_MAJOR 0
#define GSEA103_VERSION_MINOR 1

typedef enum {
    GSEA_OK = 0,
    GSEA_ERR_INVALID_ARGUMENT = 1,
    GSEA_ERR_UNKNOWN_METRIC = 2,      /* reference: exit(1), correlate_genes.cuh:292-295 */
    GSEA_ERR_CUDA = 3,                /* reference: CUERR -> exit(1)                    */
    GSEA_ERR_OUT_OF_MEMORY = 4,
    GSEA_ERR_NO_DEVICE = 5,
    GSEA_ERR_IO = 6,                  /* reference: exit codes 2-9, error_codes.cuh     */
    GSEA_ERR_UNSUPPORTED = 7,
    GSEA_ERR_INJECTED = 8,            /* host-side fault injection (GSEA_FAULT)         */
    GSEA_ERR_INVALID_INPUT = 9        /* data checks of checkInput (cudaGSEA_wrapper.cpp:156-227) */
} gsea_status;

/* metric ids in the order of the reference's dispatch (correlate_genes.cuh:166-291) */
typedef enum {
    GSEA_NAIVE_DIFF_OF_CLASSES = 0,
    GSEA_NAIVE_RATIO_OF_CLASSES = 1,
    GSEA_NAIVE_LOG2_RATIO_OF_CLASSES = 2,
    GSEA_STABLE_DIFF_OF_CLASSES = 3,
    GSEA_STABLE_RATIO_OF_CLASSES = 4,
    GSEA_STABLE_LOG2_RATIO_OF_CLASSES = 5,
    GSEA_ONEPASS_SIGNAL2NOISE = 6,
    GSEA_ONEPASS_T_TEST = 7,
    GSEA_TWOPASS_SIGNAL2NOISE = 8,
    GSEA_TWOPASS_T_TEST = 9,
    GSEA_STABLE_SIGNAL2NOISE = 10,
    GSEA_STABLE_T_TEST = 11,
    GSEA_OVERKILL_SIGNAL2NOISE = 12,
    GSEA_OVERKILL_T_TEST = 13,
    GSEA_NUM_METRICS = 14
} gsea_metric;

/* pipeline form */
typedef enum {
    GSEA_FORM_PLAIN = 0,       /* bit-exact SIMT class statistics in the reference's operation order */
    GSEA_FORM_CHOSEN = 1,      /* tensor-core (tcgen05) class statistics; variance subtraction as an
                                  error-free FP32 transformation (FP32 inputs only)               */
    GSEA_FORM_CHOSEN_FP64 = 2  /* tensor-core class statistics, variance subtraction in FP64      */
} gsea_form;

typedef struct {
    int64_t num_genes;     /* G */
    int64_t num_samples;   /* S */
    int64_t num_sets;      /* K */
    int64_t num_perms;     /* P, permutation 0 = observed labels */
    int32_t metric;        /* gsea_metric */
    int32_t precision;     /* 32 (float, like gsea_single_proxy) or 64 (double) */
    int32_t ascending;     /* 0 = descending ranking (reference default), 1 = ascending */
    int32_t form;          /* gsea_form */
    int64_t perm_offset;   /* global index of this plan's first permutation (sharding) */
    int64_t perm_batch;    /* permutations per device batch (at most 262,140), 0 = automatic */
    uint32_t seed;         /* permutation seed, 42 in the reference (configuration.cuh:29) */
    int32_t device;        /* CUDA device ordinal, -1 = current device */
} gsea_config;

typedef struct gsea_plan_s* gsea_plan;

/* ---- errors / metadata ----------------------------------------------------- */
const char* gsea_status_string(int status);
/* message of the last failure on this thread ("" if none) */
const char* gsea_last_error(void);
/* "naive_diff_of_classes" ... -> id, -1 if unknown.
 * Replaces the string dispatch of correllate_genes_gpu (correlate_genes.cuh:166-295). */
int gsea_metric_id(const char* metric_string);
const char* gsea_metric_name(int metric_id);
/* default configuration: precision 32, descending, plain form, seed 42 */
void gsea_config_init(gsea_config* cfg);

/* ---- CUDA devices (replace listCudaDevices_proxy / getCudaDevice_proxy /
 *      setCudaDevice_proxy, src/cudaGSEA_wrapper.cuh:31-33) ---------------- */
int gsea_device_count(int* count);
/* "device <id>: <name> with <n> GiB RAM", as create_device_string_helper
 * (src/cudaGSEA_wrapper.cu:87-104) */
int gsea_device_string(int device, char* buf, size_t buflen);
int gsea_get_device(int* device);
/* returns the active device in *active (falls back like setCudaDevice_proxy) */
int gsea_set_device(int device, int* active);

/* ---- one-shot host API (replaces gsea_proxy<>, src/cudaGSEA_wrapper.cu:179-401)
 * Host buffers in, host buffers out; device memory is allocated and freed
 * inside the call.  es_out may be NULL; stats_out (5*K) may be NULL.  A
 * non-empty dump_prefix writes <prefix>_<K>_<P>_<32|64>.es before the
 * statistics, as gsea_proxy does (cudaGSEA_wrapper.cu:384-390).           */
int gsea_run(const gsea_config* cfg, const void* exprs, const uint8_t* labels,
             const int64_t* set_offsets, const int32_t* set_genes,
             void* es_out, void* stats_out, const char* dump_prefix);
int gsea_run_f32(const float* exprs, int64_t num_genes, int64_t num_samples,
                 const uint8_t* labels, const int64_t* set_offsets,
                 const int32_t* set_genes, int64_t num_sets, int64_t num_perms,
                 int metric, int ascending, float* es_out, float* stats_out,
                 const char* dump_prefix);
int gsea_run_f64(const double* exprs, int64_t num_genes, int64_t num_samples,
                 const uint8_t* labels, const int64_t* set_offsets,
                 const int32_t* set_genes, int64_t num_sets, int64_t num_perms,
                 int metric, int ascending, double* es_out, double* stats_out,
                 const char* dump_prefix);

/* ---- flat form of the C++ proxies gsea_single_proxy / gsea_double_proxy
 * (src/cudaGSEA_wrapper.cuh:39-61) for callers without C++: gene symbols
 * and gene-set symbols as C strings (unknown symbols ignored, duplicates
 * collapse), sort_direction 1 = descending, swap_labels flips the classes.
 * result_out receives 5*num_sets values of the chosen precision.        */
int gsea_proxy_run(int precision, const void* exprs, int64_t num_genes, int64_t num_samples,
                   const char* const* gene_symbols, const uint8_t* labels, int64_t num_sets,
                   const int64_t* set_symbol_offsets, const char* const* set_symbols,
                   const char* metric, int64_t num_perms, int sort_direction, int swap_labels,
                   const char* dump_filename, void* result_out);

/* ---- statistics of a run split over ranks (permutation shards) --------
 *      The reference computes final_statistics once on the whole [K][P]
 *      matrix (src/include/statistics.cuh:46-117).  A rank holding
 *      permutations [first, first + count) (device ES columns, row stride ld)
 *      contributes O(K) partial results instead, and the merged statistics
 *      are bit-identical to a single run's:
 *        1. gsea_shard_sum: continues the sequential sum of |ES| over its
 *           columns from `init` (the previous rank's result; NULL on the rank
 *           holding permutation 0) -- chained over the ranks in order;
 *        2. gsea_shard_head: head = [ES, NES, fac] (3K) from the observed
 *           scores (column 0 of the first rank) and the chained total;
 *        3. gsea_shard_partial: counts = [NP counts (K), FWER counts (K)] and
 *           hist = FDR null histograms [2(K+2)] + null totals [2] of its
 *           columns -- summed over the ranks (integers: exact);
 *        4. gsea_shard_finish: stats [5K] from head and the summed counts.
 *      Device pointers; `stream` a cudaStream_t (NULL = default stream).   */
int gsea_shard_sum(const void* es, int64_t num_sets, int64_t count, int64_t ld, int precision, const void* init,
                   void* sum, void* stream);
int gsea_shard_head(const void* es_obs, const void* sum, int64_t num_sets, int64_t num_perms, int precision,
                    void* head, void* stream);
int gsea_shard_partial(const void* es, int64_t num_sets, int64_t count, int64_t ld, int precision, int64_t first_perm,
                       const void* head, uint64_t* counts, double* hist, void* stream);
int gsea_shard_finish(const void* head, int64_t num_sets, int64_t num_perms, int precision, const uint64_t* counts,
                      double* hist, void* stats, void* stream);

/* ---- gene-set membership on the device (replaces create_bitmaps,
 *      src/include/create_bitmaps.cuh:13-65, which rebuilds host bitmaps for
 *      every 32/64-set batch of every permutation batch).  Gene symbols are
 *      hashed once into a device table, set members looked up (exact byte
 *      comparison), per-set membership bitmasks built and compacted into CSR:
 *      unknown symbols dropped, duplicates collapsed, genes ascending; a
 *      repeated gene symbol maps to its first gene.  set_offsets_out gets
 *      num_sets + 1 entries; set_genes_out (may be NULL to size the call)
 *      the *nnz_out members if capacity >= *nnz_out.                       */
int gsea_map_sets(int64_t num_genes, const char* const* gene_symbols, int64_t num_sets,
                  const int64_t* set_symbol_offsets, const char* const* set_symbols, int64_t* set_offsets_out,
                  int32_t* set_genes_out, int64_t capacity, int64_t* nnz_out);

/* ---- plan API: device-resident inputs, repeated execution.  Splits
 *      gsea_proxy<> (src/cudaGSEA_wrapper.cu:179-401), which allocates, runs
 *      and frees per call (:229-372), into create / set_inputs / execute /
 *      read, so inputs and buffers stay resident across executes. -------- */
int gsea_plan_create(const gsea_config* cfg, gsea_plan* out);
int gsea_plan_destroy(gsea_plan plan);
/* copy inputs from host memory (synchronous) */
int gsea_plan_set_inputs(gsea_plan plan, const void* exprs, const uint8_t* labels,
                         const int64_t* set_offsets, const int32_t* set_genes);
/* run permutation -> metric -> sort -> ES -> statistics on `stream`
 * (a cudaStream_t, NULL = the plan's own stream); asynchronous.  The first
 * execute (and the first after new set buffers, a tuning or debug change)
 * captures the launches into a CUDA graph on the plan's stream; later ones
 * replay it.  With stage profiling on, the launches are issued directly. */
int gsea_plan_execute(gsea_plan plan, void* stream);
/* one call = upload of all inputs from host + execute + download of the
 * results to host, ordered on the plan's stream and synchronised at the end
 * (the end-to-end path; pinned host buffers make the copies asynchronous) */
int gsea_plan_run_host(gsea_plan plan, const void* exprs, const uint8_t* labels,
                       const int64_t* set_offsets, const int32_t* set_genes,
                       void* es_out, void* stats_out);
/* wait for the plan's stream, then copy results to host (either may be NULL) */
int gsea_plan_read(gsea_plan plan, void* es_out, void* stats_out);
int gsea_plan_synchronize(gsea_plan plan);

/* device buffers of a plan, for zero-copy consumers and parity tests.
 * Per-permutation buffers hold the LAST permutation batch of the last
 * execute (P_batch = the plan's batch size, see gsea_plan_info). */
typedef enum {
    GSEA_BUF_EXPRS = 0,       /* [S][G] T                                      */
    GSEA_BUF_LABEL_MASKS = 1, /* [P_batch][W] uint32, bit s set = class A      */
    GSEA_BUF_KEYS = 2,        /* [P_batch][G] T, metric per (perm, gene)       */
    GSEA_BUF_RANKS = 3,       /* [P_batch][G] uint16 (G <= 65536) or uint32    */
    GSEA_BUF_ORDER = 4,       /* [P_batch][G] uint32, gene at each position    */
    GSEA_BUF_ES = 5,          /* [K][P] T                                      */
    GSEA_BUF_STATS = 6,       /* [5][K] T                                      */
    GSEA_BUF_SORTED = 7       /* [P_batch][G] T, |metric| at each position     */
} gsea_buffer;
int gsea_plan_buffer(gsea_plan plan, int which, void** dev_ptr, size_t* bytes);
/* synchronise and copy min(bytes, buffer size) bytes of a plan buffer to host */
int gsea_plan_read_buffer(gsea_plan plan, int which, void* host_dst, size_t bytes);
/* permutations per device batch and whether ranks are stored as uint16 */
int gsea_plan_info(gsea_plan plan, int64_t* perm_batch, int* ranks16);
/* keep_intermediates != 0 also materialises GSEA_BUF_ORDER on execute */
int gsea_plan_set_debug(gsea_plan plan, int keep_intermediates);
/* kernel launches issued by the last execute */
int gsea_plan_last_launches(gsea_plan plan, int64_t* launches);
/* stage timing: with profiling on, execute records CUDA events between the
 * stages on its stream (the reference's TIMERSTART/TIMERSTOP, cuda_helpers.cuh:
 * 20-32); gsea_plan_stage_times waits for them and returns the device time of
 * each stage of the last execute in milliseconds, summed over batches */
typedef enum {
    GSEA_STAGE_PERMUTE = 0, GSEA_STAGE_METRIC = 1, GSEA_STAGE_SORT = 2,
    GSEA_STAGE_ES = 3, GSEA_STAGE_STATS = 4, GSEA_NUM_STAGES = 5
} gsea_stage;
int gsea_plan_set_profiling(gsea_plan plan, int on);
int gsea_plan_stage_times(gsea_plan plan, double* ms /* [GSEA_NUM_STAGES] */);

/* Final statistics of a device ES matrix [K][P] (row-major, permutation 0 =
 * observed) into a device buffer of 5*K values with the caller's own working
 * memory: the statistics stage of a plan, on any device matrix (e.g. the
 * columns of a sharded run gathered on one rank).  Replaces the host-side
 * final_statistics (src/include/statistics.cuh:46-117).
 * gsea_stats_scratch_bytes gives the bytes of `scratch` (256-byte aligned,
 * contents need not be cleared) that gsea_stats_device needs; the library
 * allocates nothing.  `stream` a cudaStream_t (NULL = default); asynchronous. */
int gsea_stats_scratch_bytes(int64_t num_sets, int64_t num_perms, int precision, size_t* bytes);
int gsea_stats_device(const void* es, int64_t num_sets, int64_t num_perms, int precision, void* stats,
                      void* scratch, size_t scratch_bytes, void* stream);

/* Final statistics of a device ES matrix [K][P] into a device buffer of 5*K
 * values, allocating no device memory at all.  No counterpart in the
 * reference.  For hosts that cannot let a library allocate (an application
 * that gives all device memory to its own pool, or a loop that must not call
 * cudaMalloc/cudaFree because they can synchronise the device).  The working
 * memory is a fixed 4 MiB array inside the library, held by every GPU that
 * loads it; sizes whose scratch exceeds it are rejected with
 * GSEA_ERR_INVALID_ARGUMENT.  The scratch is sizeof(T)*(3K+2P) + 8*(4K+12)
 * + 320 bytes, plus the FDR histogram's per-block rows (up to 1 MiB:
 * floor(2^20 / (4W)) * 4W + 16 bytes, W = 2K + 6) when K <= 6,142 (fp32) /
 * 4,095 (fp64); gsea_stats_scratch_bytes gives the exact figure.  The first
 * call on a device -- and the first after that device's context was reset
 * and re-created -- looks the array up for the current context (make it
 * before any stream capture); calls share the array, so calls that overlap
 * on the GPU race.
 * `stream` is a cudaStream_t (NULL = default stream); asynchronous.        */
int gsea_stats_device_noalloc(const void* es, int64_t num_sets, int64_t num_perms, int precision,
                              void* stats, void* stream);

/* ---- launch configuration and autotuner ---------------------------------
 *      No counterpart in the reference (its launch shapes are constants).
 *      Every setting computes identical results; only the speed differs.
 *      0 / -1 leave a choice automatic.                                    */
typedef struct gsea_tuning {
    int32_t metric_pb;    /* plain fp32 metric: permutations per thread, 4 or 8 */
    int32_t chosen_tile;  /* tensor-core form: permutations per tile, 128 (the automatic choice: one
                             persistent CTA per SM walking the tiles, the copies, MMAs and
                             epilogue on separate warps) or 256 (one tile per CTA) */
    int32_t sort_variant; /* 1 register radix sort (fp32, G <= 40,960: one CTA up to 20,480, a two-CTA
                             cluster exchanging through distributed shared memory beyond; fp64,
                             G <= 20,480: one CTA up to 10,240, a two-CTA cluster beyond), 2 tiled */
    int32_t es_warps;     /* warps per CTA of the enrichment kernel: 8, 16, 24 or 32 (24: with
                             es_stage 2 or 3 only) */
    int32_t es_stage;     /* 1 stage the permutation's ranks and weights in shared memory, 2 its ranks
                             only, 3 its weights only (2 and 3: 24-64 bitmap words per lane,
                             20,481-65,536 genes), 0 read it from L2, -1 automatic */
} gsea_tuning;
/* all automatic */
void gsea_tuning_init(gsea_tuning* t);
int gsea_plan_set_tuning(gsea_plan plan, const gsea_tuning* t);
int gsea_plan_get_tuning(gsea_plan plan, gsea_tuning* t);
/* Times every candidate of every stage on the plan's inputs (sample_perms
 * permutations, at most one device batch; 0 = the plan's device batch up to
 * 1,024 permutations, at least 2 x the SM count), keeps the
 * fastest of each stage in the plan and returns it in *best (may be NULL).
 * ms_out (may be NULL) receives the fastest time of the metric, sort and ES
 * stages on the sample.  Overwrites the first sample_perms columns of the
 * plan's ES matrix; needs gsea_plan_set_inputs first.                     */
int gsea_plan_autotune(gsea_plan plan, int64_t sample_perms, gsea_tuning* best, double* ms_out);

/* ---- batched instances -------------------------------------------------
 *      Many independent GSEA problems run together.  No counterpart in the
 *      reference (one problem per call).  Instances share precision and
 *      form; each has its own genes, samples, sets, permutations and metric
 *      (num_genes <= 65,536).  An execute runs each stage as one launch
 *      over every instance (one device batch: num_perms x num_genes buffers
 *      per instance): the permutations; the metric (tensor-core form: one
 *      launch set per metric family; plain form: one launch per metric and
 *      kernel path); the sort (one launch per
 *      register-resident class; instances beyond the register forms sort on
 *      their own); one persistent enrichment launch per size class (bitmap
 *      words per lane) whose CTAs pull (instance, permutation) items,
 *      largest instances first; the statistics (nine launches).  Every
 *      instance's results are its solo plan's bit for bit.  The first
 *      execute captures all of it into one CUDA graph; later executes
 *      replay that graph (gsea_batch_set_inputs or gsea_batch_autotune make
 *      the next execute capture again).  gsea_batch_autotune tunes every
 *      instance's plain metric (permutations per thread, which picks its
 *      launch group) and the enrichment launch per size class.            */
typedef struct gsea_batch_s* gsea_batch;
/* streams: size of the stream pool (0 = 16) over which an execute spreads
 * the sort classes and the enrichment size classes */
int gsea_batch_create(int64_t num_instances, const gsea_config* cfgs, int streams, gsea_batch* out);
int gsea_batch_destroy(gsea_batch b);
int gsea_batch_set_inputs(gsea_batch b, int64_t instance, const void* exprs, const uint8_t* labels,
                          const int64_t* set_offsets, const int32_t* set_genes);
/* tunes every instance's metric and sort stages and every size class's
 * enrichment launch on sample_perms permutations (0 = 2 x the SM count);
 * runs one full pass of the first stage to have real data to time on */
int gsea_batch_autotune(gsea_batch b, int64_t sample_perms);
/* asynchronous on `stream` (NULL: the batch's own stream) */
int gsea_batch_execute(gsea_batch b, void* stream);
int gsea_batch_synchronize(gsea_batch b);
int gsea_batch_read(gsea_batch b, int64_t instance, void* es_out, void* stats_out);
/* the plan holding an instance's buffers (owned by the batch) */
int gsea_batch_plan(gsea_batch b, int64_t instance, gsea_plan* plan);
/* nodes of the captured graph, enrichment size classes, kernel launches in
 * one execute (any output may be NULL; 0 before the first execute)        */
int gsea_batch_info(gsea_batch b, int64_t* graph_nodes, int64_t* es_classes, int64_t* launches);

/* ---- learned permutation allocator -----------------------------------
 *      No counterpart in the reference, which gives every set the same
 *      number of permutations.  A small network (5 -> 64 -> 64 -> 2, tanh,
 *      BF16 parameters, FP32 accumulation) maps per-set features
 *        x = [log n_k, |ES_k| / m_k, mu/sd, skewness, cv of |metric|]
 *      (n_k members, ES_k observed score, m_k the mean |ES| of the set's
 *      scores so far, moments of the observed ranking metric) to the null
 *      tail P(|ES_null| >= |ES_k|) and the null mean E|ES_null| of the set.  It is trained on the GPU (own forward and
 *      backward kernels, Adam) on null scores that a plan produced, and it
 *      is used only as a prior of the sequential stopping rule of
 *      gsea_plan_execute_adaptive: every reported p, NES, FWER and FDR is
 *      still counted from permutations.                                   */
#define GSEA_MODEL_INPUTS 5
#define GSEA_MODEL_HIDDEN 64
#define GSEA_MODEL_OUTPUTS 2
/* parameter vector: W1[64][5] b1[64] W2[64][64] b2[64] W3[2][64] b3[2] */
#define GSEA_MODEL_PARAMS 4674
/* normaliser vector: x_mean[5] x_scale[5] (x_n = (x - mean) * scale,
 * clamped to [-8, 8]; training sets scale 0 for a feature that is constant
 * over its samples),
 * y_mean y_std (log null mean = z1 * y_std + y_mean), sigma_tail (sd of the
 * logit error of the tail on held-out sets), sigma_mean (sd of the log error
 * of the null mean), trained (0/1) */
#define GSEA_MODEL_NORMS 15
typedef struct gsea_model_s* gsea_model;
/* parameters drawn from `seed` (Glorot-uniform weights, zero biases) on the
 * current device (device < 0) or on `device` */
int gsea_model_create(uint32_t seed, int device, gsea_model* out);
int gsea_model_destroy(gsea_model m);
/* FP32 master parameters and normalisers (either pointer may be NULL) */
int gsea_model_get(gsea_model m, float* params, float* norms);
int gsea_model_set(gsea_model m, const float* params, const float* norms);
/* inference on device arrays: x [n][5] raw features -> y [n][2] =
 * (predicted tail probability, predicted null mean) */
int gsea_model_predict(gsea_model m, const float* x, int64_t n, float* y, void* stream);
/* mean loss over n device samples and its gradient with respect to the
 * parameters (device grad [GSEA_MODEL_PARAMS], device loss [1]); targets
 * t [n][2] = (tail probability, log null mean).  Loss per sample:
 * 0.5 w (z0 - logit(tc))^2 + 0.5 (z1 - (t1 - y_mean) / y_std)^2 with
 * tc = clamp(t0, 1e-4, 1 - 1e-4), w = min(1, 400 tc (1 - tc)), evaluated with
 * the BF16-rounded parameters. */
int gsea_model_loss_grad(gsea_model m, const float* x, const float* t, int64_t n, float* grad, float* loss,
                         void* stream);
/* sets the normalisers from the samples, then `steps` Adam steps (minibatch
 * `batch`, cosine-decayed learning rate `lr`) captured in a CUDA graph;
 * loss_curve (host, may be NULL) receives the loss of every step */
int gsea_model_train(gsea_model m, const float* x, const float* t, int64_t n, int steps, int batch, float lr,
                     float* loss_curve);
/* held-out calibration: sigma_tail / sigma_mean from n device samples */
int gsea_model_calibrate(gsea_model m, const float* x, const float* t, int64_t n);

/* Training samples from a plan's last execute (dense ES of all sets,
 * permutation 0 observed, plan perm_offset 0): for every set, `queries`
 * thresholds u_j = m_k f_j (m_k = mean |ES| of the set; f_j stratified over
 * [0.25, 9) in log scale, jittered by a hash of (k, j)) with targets
 * (#{p: |ES_p| >= u_j} / P, log m_k), plus the observed score.
 * x [K*(queries+1)][5], t [..][2] device arrays of the caller.  Sets with
 * k % holdout == holdout - 1 (holdout > 0) go to the second pair of arrays
 * (x_val, t_val), the rest to the first; counts returned in n_train / n_val. */
int gsea_plan_model_samples(gsea_plan p, int queries, int holdout, float* x, float* t, int64_t* n_train,
                            float* x_val, float* t_val, int64_t* n_val);

typedef struct gsea_adaptive_params {
    int64_t pilot_perms; /* permutations every set gets, perm 0 included (default 1000) */
    double growth;       /* factor of the permutation count between rounds (2) */
    double z;            /* stop when posterior mean - z * sd >= stop_p (3) */
    double q_call;       /* FDR level of the calls the rule protects (0.25) */
    double margin;       /* stop_p = margin * largest pilot p among pilot calls (2) */
    double p_floor;      /* lower bound of stop_p (0.01) */
    double prior_cap;    /* prior pseudo-permutations <= prior_cap * pilot_perms (4) */
    double fallback_tol; /* model dropped if its median |log m~ - log m^| on the pilot exceeds (0.25) */
    double q_margin;     /* also stop a set once a lower bound of its FDR q (NES pushed z standard
                            errors outward) is >= q_margin * q_call; 0 turns this rule off (1.5) */
    double sig_margin;   /* also stop a set as clearly significant once an upper bound of its FDR q
                            (NES pulled z standard errors inward) is <= q_call / sig_margin and the
                            upper bound of its nominal p (posterior mean + z sd, with the model's prior
                            where it applies) is <= p_sig = (smallest pilot p among the pilot's
                            non-calls) / sig_margin; its reported NES, NP and FDR then come from the
                            permutations it received; 0 turns this rule off (2) */
} gsea_adaptive_params;
void gsea_adaptive_params_init(gsea_adaptive_params* ap);
typedef struct gsea_adaptive_report {
    int64_t rounds;          /* permutation rounds run, pilot included */
    int64_t scores;          /* enrichment scores computed (sum of the set counts) */
    int64_t stopped_pilot;   /* sets stopped after the pilot */
    int64_t full_sets;       /* sets that reached num_perms */
    double stop_p;           /* p threshold of the stopping rule */
    int32_t model_used;      /* 1 if the model's prior was applied */
    double model_mean_err;   /* median |log m~ - log m^| on the pilot */
    int64_t prior_sets;      /* sets with a finite model prior (model_used) */
    int64_t prior_agreed;    /* of those, sets whose pilot agreed with the prior (kept at the pilot decision) */
    int64_t stopped_q;       /* sets stopped by the FDR bound (q_margin), any round */
    int64_t stopped_sig;     /* sets stopped as clearly significant (sig_margin), any round */
    double p_sig;            /* p threshold of the significance rule (0: rule off) */
} gsea_adaptive_report;
/* Adaptive permutation test on the plan's inputs, num_perms permutations at
 * most per set: a pilot of pilot_perms permutations for every set, then
 * rounds of growing permutation counts for the sets the rules keep (the p
 * rule, the FDR bound q_margin, the significance rule sig_margin).  The
 * plan's ES rows hold counts[k] scores each (the rest of a row is left as
 * it was); its statistics are the ragged statistics of those rows (FWER over
 * the pilot permutations).  model may be NULL (empirical rule only).
 * counts (host, K) and report may be NULL.  Requires perm_offset 0.  The
 * whole test runs as one CUDA graph on the plan's stream (recorded on the
 * first call with given parameters and model, replayed after): the
 * decisions are kernels and the host waits only for the report.  The first
 * call therefore belongs outside any stream capture of the caller's. */
int gsea_plan_execute_adaptive(gsea_plan p, gsea_model model, const gsea_adaptive_params* ap, int64_t* counts,
                               gsea_adaptive_report* report);
/* The p rule alone (host arrays, no device): set k (counts[k] scores,
 * exceed[k] of them with |S| >= |ES_k|) stops when the Beta posterior
 * Beta(a0 + exceed, b0 + counts - exceed) has mean - z * sd >= stop_p, with
 * a0 = 0.5 + p_model[k] * prior[k], b0 = 0.5 + (1 - p_model[k]) * prior[k]
 * (p_model / prior NULL: Jeffreys prior alone).  The prior is dropped for a
 * set whose exceed/counts lies more than z sd from the prior predictive
 * (sd^2 = p (1 - p) (prior + counts) / (counts (prior + 1))).  stop[k] = 1 / 0. */
int gsea_adaptive_decide(int64_t num_sets, const int64_t* counts, const int64_t* exceed, const float* p_model,
                         const float* prior, double stop_p, double z, uint8_t* stop);
/* Ragged statistics (ES, NES, NP, FWER, FDR) of a device ES matrix whose row
 * k (stride ld) holds counts[k] scores (device int64 array); FWER over the
 * first p_fwer columns.  Allocates its scratch; synchronous.               */
int gsea_stats_ragged(const void* es, int64_t num_sets, int64_t ld, const int64_t* counts, int64_t p_fwer,
                      int precision, void* stats, void* stream);
/* The adaptive test's FDR stopping bound on its own: the ragged statistics
 * (as gsea_stats_ragged, into stats) and, per set, a lower bound of its FDR
 * q with |NES| pushed z standard errors outward (qlow, device float [K]).
 * sums: device double [2K], sum |S| then sum S^2 over each set's counts[k]
 * scores.  With z = 0 and untied NES the bound is the FDR q itself.
 * Allocates its scratch; synchronous.                                      */
int gsea_fdr_lower_bound(const void* es, int64_t num_sets, int64_t ld, const int64_t* counts, int64_t p_fwer,
                         const double* sums, double z, int precision, void* stats, float* qlow, void* stream);

/* ---- Broad files (replace read_gct / read_cls / read_gmt,
 *      src/include/read_data_files.cuh:46-321, and the loader proxies
 *      src/cudaGSEA_wrapper.cuh:15-25): parse a .gct / .cls / .gmt triple,
 *      map gene-set symbols to gene indices (unknown dropped, duplicates
 *      collapsed) and hand out the arrays gsea_run takes.  Parse errors return
 *      GSEA_ERR_IO with the reference's message in gsea_last_error().       */
typedef struct gsea_dataset_s* gsea_dataset;
int gsea_dataset_load(const char* gct_path, const char* cls_path, const char* gmt_path, gsea_dataset* out);
int gsea_dataset_dims(gsea_dataset ds, int64_t* num_genes, int64_t* num_samples, int64_t* num_sets,
                      int64_t* num_members);
/* exprs patient-major in the given precision (32: values parsed as float,
 * like the reference's single-precision reader; 64: as double); any output
 * may be NULL */
int gsea_dataset_arrays(gsea_dataset ds, int precision, void* exprs_pm, uint8_t* labels,
                        int64_t* set_offsets, int32_t* set_genes);
const char* gsea_dataset_gene(gsea_dataset ds, int64_t gene);
const char* gsea_dataset_set_name(gsea_dataset ds, int64_t set);
void gsea_dataset_free(gsea_dataset ds);

/* pinned (page-locked) host memory for asynchronous copies */
int gsea_host_alloc(size_t bytes, void** ptr);
int gsea_host_free(void* ptr);

/* ---- .es dump (src/include/dump_binary.cuh:10-30 and naming at
 *      src/cudaGSEA_wrapper.cu:384-390) --------------------------------- */
int gsea_write_es_dump(const char* prefix, const void* es, int64_t num_sets,
                       int64_t num_perms, int precision, char* path_out,
                       size_t path_len);

#ifdef __cplusplus
}
#endif
#endif /* GSEA103_H */
