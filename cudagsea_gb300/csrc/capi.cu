// capi.cu -- the C ABI of libgsea103 (include/gsea103.h): plans, one-shot
// runs, devices, errors and the .es dump.
//
// The pipeline orchestration replaces gsea_proxy<> (src/cudaGSEA_wrapper.cu:
// 179-401).  Differences by design:
//   * inputs stay resident on the device; permutations run in batches sized
//     by a memory budget rather than by free RAM (batch_scheduler.cuh:24-33),
//     and gene sets are not batched at all: every set of a permutation batch is
//     scored by one kernel from the CSR membership lists;
//   * the statistics run on the device;
//   * errors are returned as status codes with a per-thread message instead of
//     exit().
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gsea103.h"
#include "kernels.h"
#include "plan.h"

namespace gsea {
static std::atomic<long long> g_launches{0};
int64_t launches_take() { return g_launches.exchange(0); }
void launches_add(int64_t n) { g_launches.fetch_add(n); }
}  // namespace gsea

namespace {

thread_local std::string t_error;
using gsea::fail;
using gsea::cuda_fail;

// Host-side fault injection for the error paths: GSEA_FAULT=alloc|launch|d2h
// makes the matching step of the next call fail with GSEA_ERR_INJECTED.  No
// device fault is ever provoked.
bool injected(const char* stage) {
    const char* f = std::getenv("GSEA_FAULT");
    return f && std::strcmp(f, stage) == 0;
}

const char* const kMetricNames[GSEA_NUM_METRICS] = {
    "naive_diff_of_classes",   "naive_ratio_of_classes",      "naive_log2_ratio_of_classes",
    "stable_diff_of_classes",  "stable_ratio_of_classes",     "stable_log2_ratio_of_classes",
    "onepass_signal2noise",    "onepass_t_test",              "twopass_signal2noise",
    "twopass_t_test",          "stable_signal2noise",         "stable_t_test",
    "overkill_signal2noise",   "overkill_t_test"};

constexpr size_t kBatchBudget = size_t(4) << 30;  // bytes of per-permutation buffers

}  // namespace

namespace gsea {
void set_last_error(const char* msg) { t_error = msg ? msg : ""; }
}  // namespace gsea


namespace {

int validate_config(const gsea_config* c) {
    if (!c) return fail(GSEA_ERR_INVALID_ARGUMENT, "null config");
    if (c->num_genes < 1 || c->num_genes > (int64_t)1 << 30)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "num_genes out of range");
    if (c->num_samples < 2 || c->num_samples > 6400)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "num_samples must be in [2, 6400]");
    if (c->num_sets < 1 || c->num_sets > (int64_t)1 << 30)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "num_sets must be >= 1");
    if (c->num_perms < 1 || c->num_perms > (int64_t)1 << 31)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "num_perms must be >= 1");
    if (c->metric < 0 || c->metric >= GSEA_NUM_METRICS)
        return fail(GSEA_ERR_UNKNOWN_METRIC, "unknown metric id");
    if (c->precision != 32 && c->precision != 64)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "precision must be 32 or 64");
    if (c->form != GSEA_FORM_PLAIN && c->form != GSEA_FORM_CHOSEN && c->form != GSEA_FORM_CHOSEN_FP64)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "unknown form");
    if (c->perm_offset < 0 || c->perm_batch < 0)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "negative perm_offset / perm_batch");
    return GSEA_OK;
}

// record a stage-boundary event (no-op unless profiling)
int mark(gsea_plan_s* p, int stage, cudaStream_t st) {
    if (!p->profile) return GSEA_OK;
    if (p->events_used == p->events.size()) {
        cudaEvent_t e;
        GSEA_CUDA(cudaEventCreate(&e), "cudaEventCreate");
        p->events.push_back(e);
        p->event_stage.push_back(0);
    }
    p->event_stage[p->events_used] = stage;
    GSEA_CUDA(cudaEventRecord(p->events[p->events_used++], st), "cudaEventRecord");
    return GSEA_OK;
}

void free_plan_buffers(gsea_plan_s* p) {
    void* bufs[] = {p->exprs, p->labels, p->set_off, p->set_genes, p->set_order, p->masks, p->fast_ok, p->decay, p->gene_mu,
                    p->gene_t1, p->gene_t2, p->opA1, p->opA2, p->opB, p->dev_error, p->keys,
                    p->ranks, p->sorted, p->order, p->sort_scratch, p->es, p->stats, p->stats_scratch,
                    p->moments, p->active, p->counts, p->exceed, p->sumabs, p->qlow, p->feat, p->pred,
                    p->stop, p->ad_err, p->ad_ctl, p->qhigh};
    for (void* b : bufs)
        if (b) cudaFree(b);
    p->exprs = p->labels = nullptr;
    p->set_off = nullptr;
    p->set_genes = nullptr;
    p->set_order = nullptr;
    p->masks = nullptr;
    p->fast_ok = nullptr;
    p->decay = nullptr;
    p->gene_mu = nullptr;
    p->gene_t1 = p->gene_t2 = nullptr;
    p->opA1 = p->opA2 = p->opB = nullptr;
    p->dev_error = nullptr;
    p->keys = p->ranks = p->sorted = nullptr;
    p->order = nullptr;
    p->sort_scratch = p->es = p->stats = p->stats_scratch = nullptr;
    p->moments = nullptr;
    p->active = nullptr;
    p->counts = nullptr;
    p->exceed = nullptr;
    p->sumabs = nullptr;
    p->qlow = nullptr;
    p->feat = p->pred = nullptr;
    p->stop = nullptr;
    p->ad_err = nullptr;
    p->ad_ctl = nullptr;
    p->qhigh = nullptr;
}

void drop_graph(gsea_plan_s* p) {
    if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->graph_exec = nullptr;
    p->graph = nullptr;
    if (p->ad_exec) cudaGraphExecDestroy(p->ad_exec);  // the adaptive test's graph holds the same launches
    if (p->ad_graph) cudaGraphDestroy(p->ad_graph);
    p->ad_exec = nullptr;
    p->ad_graph = nullptr;
    p->ad_key.clear();
}

template <class Ptr>
int dev_alloc(Ptr** ptr, size_t bytes, const char* what) {
    if (injected("alloc")) return fail(GSEA_ERR_INJECTED, std::string("injected allocation failure: ") + what);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(e, what);
    }
    *ptr = static_cast<Ptr*>(p);
    return GSEA_OK;
}

int use_device(const gsea_plan_s* p) {
    GSEA_CUDA(cudaSetDevice(p->device), "cudaSetDevice");
    return GSEA_OK;
}

int alloc_order(gsea_plan_s* p) {
    if (p->order) return GSEA_OK;
    return dev_alloc(&p->order, sizeof(uint32_t) * (size_t)p->pb * p->cfg.num_genes, "order buffer");
}

int upload_sets(gsea_plan_s* p, const int64_t* off, const int32_t* genes, cudaStream_t st, bool async) {
    const int64_t K = p->cfg.num_sets;
    if (!off || !genes) return fail(GSEA_ERR_INVALID_ARGUMENT, "null gene-set arrays");
    if (off[0] != 0) return fail(GSEA_ERR_INVALID_INPUT, "set_offsets[0] must be 0");
    for (int64_t k = 0; k < K; k++)
        if (off[k + 1] < off[k]) return fail(GSEA_ERR_INVALID_INPUT, "set_offsets must be non-decreasing");
    const int64_t nnz = off[K];
    if (nnz > p->nnz_cap) {
        drop_graph(p);  // the captured launches point at the old buffer
        if (p->set_genes) cudaFree(p->set_genes);
        p->set_genes = nullptr;
        int rc = dev_alloc(&p->set_genes, sizeof(int32_t) * (size_t)nnz, "set genes");
        if (rc) return rc;
        p->nnz_cap = nnz;
    }
    p->nnz = nnz;
    // largest sets first: the ES kernel's warps take sets in this order
    p->h_set_order.resize((size_t)K);
    p->h_set_size.resize((size_t)K);
    for (int64_t k = 0; k < K; k++) {
        p->h_set_order[k] = (int32_t)k;
        p->h_set_size[k] = off[k + 1] - off[k];
    }
    std::stable_sort(p->h_set_order.begin(), p->h_set_order.end(),
                     [off](int32_t x, int32_t y) { return off[x + 1] - off[x] > off[y + 1] - off[y]; });
    if (async) {
        GSEA_CUDA(cudaMemcpyAsync(p->set_order, p->h_set_order.data(), sizeof(int32_t) * K, cudaMemcpyHostToDevice, st),
                  "copy set order");
        GSEA_CUDA(cudaMemcpyAsync(p->set_off, off, sizeof(int64_t) * (K + 1), cudaMemcpyHostToDevice, st), "copy set offsets");
        if (nnz) GSEA_CUDA(cudaMemcpyAsync(p->set_genes, genes, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st), "copy set genes");
    } else {
        GSEA_CUDA(cudaMemcpy(p->set_order, p->h_set_order.data(), sizeof(int32_t) * K, cudaMemcpyHostToDevice),
                  "copy set order");
        GSEA_CUDA(cudaMemcpy(p->set_off, off, sizeof(int64_t) * (K + 1), cudaMemcpyHostToDevice), "copy set offsets");
        if (nnz) GSEA_CUDA(cudaMemcpy(p->set_genes, genes, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice), "copy set genes");
    }
    return GSEA_OK;
}

int count_labels(gsea_plan_s* p, const uint8_t* labels) {
    int64_t a = 0, b = 0;
    for (int64_t s = 0; s < p->cfg.num_samples; s++) {
        if (labels[s] == 0) a++;
        else if (labels[s] == 1) b++;
        else return fail(GSEA_ERR_INVALID_INPUT, "labels must be 0 or 1");
    }
    if (a == 0 || b == 0) return fail(GSEA_ERR_INVALID_INPUT, "both classes need at least one sample");
    p->nA = a;
    p->nB = b;
    return GSEA_OK;
}

// device-side preparation of freshly uploaded inputs, on `st`: the check of
// the expression table (sets p->fast_ok) and, for the chosen form, the split
// tensor-core operands
int check_inputs(gsea_plan_s* p, cudaStream_t st) {
    const int64_t n = p->cfg.num_genes * p->cfg.num_samples;
    cudaError_t e = p->cfg.precision == 64
                        ? gsea::launch_finite_check<double>(static_cast<const double*>(p->exprs), n, p->fast_ok, st)
                        : gsea::launch_finite_check<float>(static_cast<const float*>(p->exprs), n, p->fast_ok, st);
    if (e != cudaSuccess) return cuda_fail(e, "input check kernel");
    if (p->cfg.form != GSEA_FORM_PLAIN) {
        e = gsea::launch_chosen_prepare<float>(static_cast<const float*>(p->exprs), (int)p->cfg.num_genes,
                                               (int)p->cfg.num_samples, p->gene_mu, p->gene_t1, p->gene_t2, p->opA1,
                                               p->opA2, st);
        if (e != cudaSuccess) return cuda_fail(e, "tensor operand preparation");
    }
    return GSEA_OK;
}

// error flag raised by a kernel whose bounded wait expired (after a sync)
int check_device_error(gsea_plan_s* p) {
    int flag = 0;
    GSEA_CUDA(cudaMemcpy(&flag, p->dev_error, sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (flag) {
        cudaMemset(p->dev_error, 0, sizeof(int));
        return fail(GSEA_ERR_CUDA, "a tensor-core kernel gave up waiting for its data (bounded wait expired)");
    }
    return GSEA_OK;
}

template <class T>
int run_range_t(gsea_plan_s* p, cudaStream_t st, int64_t lo, int64_t hi, const int32_t* set_list, int n_sets,
                bool with_es = true, const int* n_dev = nullptr) {
    const gsea_config& c = p->cfg;
    const int G = (int)c.num_genes, S = (int)c.num_samples;
    const int64_t P = c.num_perms;
    gsea::SortBuffers sb;
    sb.ranks = p->ranks;
    sb.ranks16 = p->ranks16;
    sb.sorted_abs = p->sorted;
    sb.order = p->debug ? p->order : nullptr;
    sb.scratch = p->sort_scratch;
    sb.scratch_bytes = p->sort_scratch_bytes;
    sb.error_flag = p->dev_error;
    sb.variant = p->tuning.sort_variant;
    gsea::EsTuning et;
    et.warps = p->tuning.es_warps;
    et.stage = p->tuning.es_stage;
    int rc;
    for (int64_t b0 = lo; b0 < hi; b0 += p->pb) {
        const int nb = (int)(hi - b0 < p->pb ? hi - b0 : p->pb);
        GSEA_CUDA(gsea::launch_permute(p->labels, S, nb, c.perm_offset + b0, c.seed, p->masks, p->words, st),
                  "permute kernel");
        if ((rc = mark(p, 0, st))) return rc;
        if (c.form != GSEA_FORM_PLAIN) {
            GSEA_CUDA(gsea::launch_chosen_metric(c.metric, c.form == GSEA_FORM_CHOSEN_FP64, p->masks, p->words, G, S,
                                                 nb, p->nA, p->nB, p->gene_mu,
                                                 p->gene_t1, p->gene_t2, p->opA1, p->opA2, p->opB,
                                                 static_cast<float*>(p->keys), p->dev_error, st,
                                                 p->tuning.chosen_tile),
                      "tensor-core class statistics");
        } else {
            GSEA_CUDA(gsea::launch_metric<T>(c.metric, static_cast<const T*>(p->exprs), G, S, p->masks, p->words,
                                             nb, p->nA, p->nB, static_cast<T*>(p->keys), p->fast_ok, st,
                                             p->tuning.metric_pb),
                      "metric kernel");
        }
        if ((rc = mark(p, 1, st))) return rc;
        GSEA_CUDA(gsea::launch_sort<T>(static_cast<const T*>(p->keys), G, nb, c.ascending != 0, sb, st),
                  "sort kernel");
        if ((rc = mark(p, 2, st))) return rc;
        if (!with_es) continue;
        GSEA_CUDA(gsea::launch_es<T>(p->ranks, p->ranks16, static_cast<const T*>(p->sorted), G, nb, p->set_off,
                                     p->set_genes, set_list, static_cast<const T*>(p->decay), n_sets,
                                     static_cast<T*>(p->es), P, b0, st, et, n_dev),
                  "enrichment kernel");
        if ((rc = mark(p, 3, st))) return rc;
    }
    return GSEA_OK;
}

template <class T>
int record_t(gsea_plan_s* p, cudaStream_t st) {
    const int K = (int)p->cfg.num_sets;
    const int64_t P = p->cfg.num_perms;
    int rc = mark(p, -1, st);
    if (rc) return rc;
    if ((rc = run_range_t<T>(p, st, 0, P, p->set_order, K))) return rc;
    GSEA_CUDA(gsea::launch_stats<T>(static_cast<const T*>(p->es), K, P, static_cast<T*>(p->stats),
                                    p->stats_scratch, st),
              "statistics kernels");
    return mark(p, 4, st);
}

// One execute.  With stage profiling off, the launches are captured into a
// CUDA graph on the plan's stream the first time and the graph is replayed
// on `st` afterwards (one launch instead of ~12).
template <class T>
int execute_t(gsea_plan_s* p, cudaStream_t st) {
    if (injected("launch")) return fail(GSEA_ERR_INJECTED, "injected launch failure");
    gsea::launches_take();
    p->events_used = 0;
    if (p->profile || !p->use_graph) {
        drop_graph(p);
        const int rc = record_t<T>(p, st);
        p->last_launches = gsea::launches_take();
        return rc;
    }
    if (!p->graph_exec) {
        GSEA_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        const int rc = record_t<T>(p, p->stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(p->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return rc;
        }
        GSEA_CUDA(e, "end capture");
        p->graph = g;
        p->graph_launches = gsea::launches_take();
        GSEA_CUDA(cudaGraphInstantiate(&p->graph_exec, g, 0), "graph instantiate");
    }
    GSEA_CUDA(cudaGraphLaunch(p->graph_exec, st), "graph launch");
    p->last_launches = p->graph_launches;
    return GSEA_OK;
}

int write_dump(const char* prefix, const void* es, int64_t K, int64_t P, int precision, char* path_out,
               size_t path_len) {
    if (!prefix || !*prefix) return fail(GSEA_ERR_INVALID_ARGUMENT, "empty dump prefix");
    std::string name = std::string(prefix) + "_" + std::to_string(K) + "_" + std::to_string(P) + "_" +
                       std::to_string(precision) + ".es";
    FILE* f = std::fopen(name.c_str(), "wb");
    if (!f) return fail(GSEA_ERR_IO, "cannot open " + name);
    const size_t bytes = (size_t)K * (size_t)P * (precision / 8);
    const size_t wrote = std::fwrite(es, 1, bytes, f);
    std::fclose(f);
    if (wrote != bytes) return fail(GSEA_ERR_IO, "short write to " + name);
    if (path_out && path_len) {
        std::strncpy(path_out, name.c_str(), path_len - 1);
        path_out[path_len - 1] = 0;
    }
    return GSEA_OK;
}

}  // namespace

namespace gsea {
int plan_run_range(gsea_plan_s* p, cudaStream_t st, int64_t lo, int64_t hi, const int32_t* set_list, int n_sets,
                   const int* n_dev) {
    if (injected("launch")) return fail(GSEA_ERR_INJECTED, "injected launch failure");
    return p->cfg.precision == 64 ? run_range_t<double>(p, st, lo, hi, set_list, n_sets, true, n_dev)
                                  : run_range_t<float>(p, st, lo, hi, set_list, n_sets, true, n_dev);
}
int plan_dev_alloc(void** ptr, size_t bytes, const char* what) { return dev_alloc(ptr, bytes, what); }
void plan_drop_graph(gsea_plan_s* p) { drop_graph(p); }
int plan_check_error(gsea_plan_s* p) { return p->cfg.form != GSEA_FORM_PLAIN ? check_device_error(p) : GSEA_OK; }
int plan_run_stage1(gsea_plan_s* p, cudaStream_t st) {
    return p->cfg.precision == 64 ? run_range_t<double>(p, st, 0, p->cfg.num_perms, nullptr, 0, false)
                                  : run_range_t<float>(p, st, 0, p->cfg.num_perms, nullptr, 0, false);
}
int plan_run_metric(gsea_plan_s* p, cudaStream_t st) {
    const gsea_config& c = p->cfg;
    const int G = (int)c.num_genes, S = (int)c.num_samples, n = (int)p->pb;
    if (c.form != GSEA_FORM_PLAIN) {
        GSEA_CUDA(gsea::launch_chosen_metric(c.metric, c.form == GSEA_FORM_CHOSEN_FP64, p->masks, p->words, G, S, n,
                                             p->nA, p->nB, p->gene_mu, p->gene_t1, p->gene_t2, p->opA1, p->opA2,
                                             p->opB, static_cast<float*>(p->keys), p->dev_error, st,
                                             p->tuning.chosen_tile),
                  "tensor-core class statistics");
        return GSEA_OK;
    }
    cudaError_t e = c.precision == 64
                        ? gsea::launch_metric<double>(c.metric, static_cast<const double*>(p->exprs), G, S, p->masks,
                                                      p->words, n, p->nA, p->nB, static_cast<double*>(p->keys),
                                                      p->fast_ok, st, p->tuning.metric_pb)
                        : gsea::launch_metric<float>(c.metric, static_cast<const float*>(p->exprs), G, S, p->masks,
                                                     p->words, n, p->nA, p->nB, static_cast<float*>(p->keys),
                                                     p->fast_ok, st, p->tuning.metric_pb);
    GSEA_CUDA(e, "metric kernel");
    return GSEA_OK;
}
int plan_run_sort(gsea_plan_s* p, cudaStream_t st) {
    const gsea_config& c = p->cfg;
    gsea::SortBuffers sb;
    sb.ranks = p->ranks;
    sb.ranks16 = p->ranks16;
    sb.sorted_abs = p->sorted;
    sb.order = p->debug ? p->order : nullptr;
    sb.scratch = p->sort_scratch;
    sb.scratch_bytes = p->sort_scratch_bytes;
    sb.error_flag = p->dev_error;
    sb.variant = p->tuning.sort_variant;
    const int G = (int)c.num_genes, n = (int)p->pb;
    cudaError_t e = c.precision == 64
                        ? gsea::launch_sort<double>(static_cast<const double*>(p->keys), G, n, c.ascending != 0, sb, st)
                        : gsea::launch_sort<float>(static_cast<const float*>(p->keys), G, n, c.ascending != 0, sb, st);
    GSEA_CUDA(e, "sort kernel");
    return GSEA_OK;
}
int plan_run_stats(gsea_plan_s* p, cudaStream_t st) {
    const int K = (int)p->cfg.num_sets;
    const int64_t P = p->cfg.num_perms;
    cudaError_t e = p->cfg.precision == 64
                        ? gsea::launch_stats<double>(static_cast<const double*>(p->es), K, P,
                                                     static_cast<double*>(p->stats), p->stats_scratch, st)
                        : gsea::launch_stats<float>(static_cast<const float*>(p->es), K, P,
                                                    static_cast<float*>(p->stats), p->stats_scratch, st);
    GSEA_CUDA(e, "statistics kernels");
    return GSEA_OK;
}
}  // namespace gsea

extern "C" {

const char* gsea_status_string(int s) {
    switch (s) {
        case GSEA_OK: return "success";
        case GSEA_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GSEA_ERR_UNKNOWN_METRIC: return "unknown metric";
        case GSEA_ERR_CUDA: return "CUDA error";
        case GSEA_ERR_OUT_OF_MEMORY: return "out of device memory";
        case GSEA_ERR_NO_DEVICE: return "no CUDA device";
        case GSEA_ERR_IO: return "I/O error";
        case GSEA_ERR_UNSUPPORTED: return "unsupported";
        case GSEA_ERR_INJECTED: return "injected fault";
        case GSEA_ERR_INVALID_INPUT: return "invalid input data";
        default: return "unknown status";
    }
}

const char* gsea_last_error(void) { return t_error.c_str(); }

int gsea_metric_id(const char* m) {
    if (!m) return -1;
    for (int i = 0; i < GSEA_NUM_METRICS; i++)
        if (std::strcmp(m, kMetricNames[i]) == 0) return i;
    return -1;
}

const char* gsea_metric_name(int id) {
    return (id >= 0 && id < GSEA_NUM_METRICS) ? kMetricNames[id] : nullptr;
}

void gsea_config_init(gsea_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->metric = GSEA_ONEPASS_SIGNAL2NOISE;  // CLI default (src/cudaGSEA.cu:90-94)
    c->precision = 32;
    c->seed = 42;
    c->device = -1;
    c->form = GSEA_FORM_PLAIN;
}

int gsea_device_count(int* count) {
    if (!count) return fail(GSEA_ERR_INVALID_ARGUMENT, "null count");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *count = 0;
        return cuda_fail(e, "cudaGetDeviceCount");
    }
    *count = n;
    return GSEA_OK;
}

int gsea_device_string(int device, char* buf, size_t len) {
    if (!buf || !len) return fail(GSEA_ERR_INVALID_ARGUMENT, "null buffer");
    cudaDeviceProp prop;
    GSEA_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    const size_t gib = ((size_t)prop.totalGlobalMem + (1ull << 30) - 1) >> 30;
    std::snprintf(buf, len, "device %d: %s with %zu GiB RAM", device, prop.name, gib);
    return GSEA_OK;
}

int gsea_get_device(int* device) {
    if (!device) return fail(GSEA_ERR_INVALID_ARGUMENT, "null device");
    GSEA_CUDA(cudaGetDevice(device), "cudaGetDevice");
    return GSEA_OK;
}

int gsea_set_device(int device, int* active) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) cudaGetLastError();  // fall back to the current device
    int cur = 0;
    GSEA_CUDA(cudaGetDevice(&cur), "cudaGetDevice");
    if (active) *active = cur;
    if (cur != device) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid device id, staying on device " + std::to_string(cur));
    return GSEA_OK;
}

int gsea_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(GSEA_ERR_INVALID_ARGUMENT, "null pointer");
    GSEA_CUDA(cudaMallocHost(ptr, bytes ? bytes : 16), "cudaMallocHost");
    return GSEA_OK;
}

int gsea_host_free(void* ptr) {
    if (ptr) GSEA_CUDA(cudaFreeHost(ptr), "cudaFreeHost");
    return GSEA_OK;
}

int gsea_plan_create(const gsea_config* cfg, gsea_plan* out) {
    if (!out) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan pointer");
    *out = nullptr;
    int rc = validate_config(cfg);
    if (rc) return rc;
    if (injected("alloc")) return fail(GSEA_ERR_INJECTED, "injected allocation failure: plan");
    if (cfg->form != GSEA_FORM_PLAIN && cfg->precision != 32)
        return fail(GSEA_ERR_UNSUPPORTED, "the tensor-core form computes from fp32 inputs (precision 32)");
    gsea_plan_s* p = new (std::nothrow) gsea_plan_s();
    if (!p) return fail(GSEA_ERR_OUT_OF_MEMORY, "host allocation");
    p->cfg = *cfg;
    if (cfg->device >= 0) {
        cudaError_t e = cudaSetDevice(cfg->device);
        if (e != cudaSuccess) { delete p; return cuda_fail(e, "cudaSetDevice"); }
    }
    cudaError_t e = cudaGetDevice(&p->device);
    if (e != cudaSuccess) { cudaGetLastError(); delete p; return cuda_fail(e, "cudaGetDevice"); }
    const int64_t G = cfg->num_genes, S = cfg->num_samples, K = cfg->num_sets, P = cfg->num_perms;
    p->tsize = cfg->precision == 64 ? 8 : 4;
    p->words = (int)((S + 31) / 32);
    p->ranks16 = G <= 65536;
    const size_t per_perm = (size_t)G * (2 * p->tsize + (p->ranks16 ? 2 : 4)) + 4 * (size_t)p->words;
    int64_t pb = cfg->perm_batch > 0 ? cfg->perm_batch : (int64_t)(kBatchBudget / per_perm);
    if (pb < 1) pb = 1;
    // the metric kernels' second grid dimension is one block per 4 or 8
    // permutations of a batch and may not exceed 65,535
    constexpr int64_t kMaxBatch = (int64_t)4 * 65535;
    if (pb > kMaxBatch) pb = kMaxBatch;
    if (pb > P) pb = P;
    p->pb = pb;
    e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete p; return cuda_fail(e, "cudaStreamCreate"); }
    const size_t T = p->tsize;
    if ((rc = dev_alloc(&p->exprs, T * G * S, "expression table")) ||
        (rc = dev_alloc(&p->labels, (size_t)S, "labels")) ||
        (rc = dev_alloc(&p->set_off, sizeof(int64_t) * (K + 1), "set offsets")) ||
        (rc = dev_alloc(&p->set_order, sizeof(int32_t) * K, "set order")) ||
        (rc = dev_alloc(&p->masks, 4 * (size_t)p->words * pb, "label masks")) ||
        (rc = dev_alloc(&p->fast_ok, sizeof(int), "input flags")) ||
        (rc = dev_alloc(&p->decay, T * ((size_t)G + 1), "decay table")) ||
        (rc = dev_alloc(&p->dev_error, sizeof(int), "error flag")) ||
        (rc = dev_alloc(&p->keys, T * (size_t)G * pb, "metric keys")) ||
        (rc = dev_alloc(&p->ranks, (p->ranks16 ? 2 : 4) * (size_t)G * pb, "ranks")) ||
        (rc = dev_alloc(&p->sorted, T * (size_t)G * pb, "sorted weights")) ||
        (rc = dev_alloc(&p->es, T * (size_t)K * P, "enrichment scores")) ||
        (rc = dev_alloc(&p->stats, T * 5 * (size_t)K, "statistics"))) {
        free_plan_buffers(p);
        cudaStreamDestroy(p->stream);
        delete p;
        return rc;
    }
    p->sort_scratch_bytes = cfg->precision == 64 ? gsea::sort_scratch_bytes<double>((int)G, (int)pb)
                                                 : gsea::sort_scratch_bytes<float>((int)G, (int)pb);
    p->stats_scratch_bytes = cfg->precision == 64 ? gsea::stats_scratch_bytes<double>((int)K, P)
                                                  : gsea::stats_scratch_bytes<float>((int)K, P);
    if (cfg->form != GSEA_FORM_PLAIN &&
        ((rc = dev_alloc(&p->gene_mu, sizeof(float) * (size_t)G, "gene means")) ||
         (rc = dev_alloc(&p->gene_t1, sizeof(double) * (size_t)G, "gene totals")) ||
         (rc = dev_alloc(&p->gene_t2, sizeof(double) * (size_t)G, "gene totals")) ||
         (rc = dev_alloc(&p->opA1, gsea::chosen_a_bytes((int)G, (int)S), "tensor operand A")) ||
         (rc = dev_alloc(&p->opA2, gsea::chosen_a_bytes((int)G, (int)S), "tensor operand A2")) ||
         (rc = dev_alloc(&p->opB, gsea::chosen_b_bytes((int)pb, (int)S), "tensor operand B")))) {
        free_plan_buffers(p);
        cudaStreamDestroy(p->stream);
        delete p;
        return rc;
    }
    if ((p->sort_scratch_bytes && (rc = dev_alloc(&p->sort_scratch, p->sort_scratch_bytes, "sort scratch"))) ||
        (rc = dev_alloc(&p->stats_scratch, p->stats_scratch_bytes, "statistics scratch"))) {
        free_plan_buffers(p);
        cudaStreamDestroy(p->stream);
        delete p;
        return rc;
    }
    cudaError_t de = cfg->precision == 64
                         ? gsea::launch_decay_table<double>((int)G, static_cast<double*>(p->decay), p->stream)
                         : gsea::launch_decay_table<float>((int)G, static_cast<float*>(p->decay), p->stream);
    if (de == cudaSuccess) de = cudaMemsetAsync(p->dev_error, 0, sizeof(int), p->stream);
    if (de == cudaSuccess) de = cudaStreamSynchronize(p->stream);
    if (de != cudaSuccess) {
        free_plan_buffers(p);
        cudaStreamDestroy(p->stream);
        delete p;
        return cuda_fail(de, "decay table");
    }
    *out = p;
    return GSEA_OK;
}

int gsea_plan_destroy(gsea_plan p) {
    if (!p) return GSEA_OK;
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    for (cudaEvent_t e : p->events) cudaEventDestroy(e);
    drop_graph(p);
    free_plan_buffers(p);
    cudaStreamDestroy(p->stream);
    delete p;
    return GSEA_OK;
}

int gsea_plan_set_inputs(gsea_plan p, const void* exprs, const uint8_t* labels, const int64_t* set_offsets,
                         const int32_t* set_genes) {
    if (!p || !exprs || !labels) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    int rc = use_device(p);
    if (rc) return rc;
    if ((rc = count_labels(p, labels))) return rc;
    GSEA_CUDA(cudaStreamSynchronize(p->stream), "stream sync");
    const size_t xbytes = p->tsize * (size_t)p->cfg.num_genes * p->cfg.num_samples;
    GSEA_CUDA(cudaMemcpy(p->exprs, exprs, xbytes, cudaMemcpyHostToDevice), "copy expression table");
    GSEA_CUDA(cudaMemcpy(p->labels, labels, (size_t)p->cfg.num_samples, cudaMemcpyHostToDevice), "copy labels");
    if ((rc = upload_sets(p, set_offsets, set_genes, p->stream, false))) return rc;
    if ((rc = check_inputs(p, p->stream))) return rc;
    GSEA_CUDA(cudaStreamSynchronize(p->stream), "stream sync");
    p->inputs_set = true;
    p->moments_ready = false;
    return GSEA_OK;
}

int gsea_plan_execute(gsea_plan p, void* stream) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    if (!p->inputs_set) return fail(GSEA_ERR_INVALID_ARGUMENT, "plan inputs were not set");
    int rc = use_device(p);
    if (rc) return rc;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : p->stream;
    return p->cfg.precision == 64 ? execute_t<double>(p, st) : execute_t<float>(p, st);
}

int gsea_plan_synchronize(gsea_plan p) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    int rc = use_device(p);
    if (rc) return rc;
    GSEA_CUDA(cudaStreamSynchronize(p->stream), "stream sync");
    GSEA_CUDA(cudaDeviceSynchronize(), "device sync");
    return check_device_error(p);
}

int gsea_plan_read(gsea_plan p, void* es_out, void* stats_out) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    int rc = use_device(p);
    if (rc) return rc;
    GSEA_CUDA(cudaDeviceSynchronize(), "device sync");
    if ((rc = check_device_error(p))) return rc;
    if (injected("d2h")) return fail(GSEA_ERR_INJECTED, "injected device-to-host failure");
    const size_t T = p->tsize;
    if (es_out)
        GSEA_CUDA(cudaMemcpy(es_out, p->es, T * (size_t)p->cfg.num_sets * p->cfg.num_perms, cudaMemcpyDeviceToHost),
                  "copy enrichment scores");
    if (stats_out)
        GSEA_CUDA(cudaMemcpy(stats_out, p->stats, T * 5 * (size_t)p->cfg.num_sets, cudaMemcpyDeviceToHost),
                  "copy statistics");
    return GSEA_OK;
}

int gsea_plan_run_host(gsea_plan p, const void* exprs, const uint8_t* labels, const int64_t* set_offsets,
                       const int32_t* set_genes, void* es_out, void* stats_out) {
    if (!p || !exprs || !labels) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    int rc = use_device(p);
    if (rc) return rc;
    if ((rc = count_labels(p, labels))) return rc;
    cudaStream_t st = p->stream;
    const size_t T = p->tsize;
    const size_t xbytes = T * (size_t)p->cfg.num_genes * p->cfg.num_samples;
    GSEA_CUDA(cudaMemcpyAsync(p->exprs, exprs, xbytes, cudaMemcpyHostToDevice, st), "copy expression table");
    GSEA_CUDA(cudaMemcpyAsync(p->labels, labels, (size_t)p->cfg.num_samples, cudaMemcpyHostToDevice, st), "copy labels");
    if ((rc = upload_sets(p, set_offsets, set_genes, st, true))) return rc;
    if ((rc = check_inputs(p, st))) return rc;
    p->inputs_set = true;
    p->moments_ready = false;
    rc = p->cfg.precision == 64 ? execute_t<double>(p, st) : execute_t<float>(p, st);
    if (rc) return rc;
    if (injected("d2h")) return fail(GSEA_ERR_INJECTED, "injected device-to-host failure");
    if (es_out)
        GSEA_CUDA(cudaMemcpyAsync(es_out, p->es, T * (size_t)p->cfg.num_sets * p->cfg.num_perms,
                                  cudaMemcpyDeviceToHost, st), "copy enrichment scores");
    if (stats_out)
        GSEA_CUDA(cudaMemcpyAsync(stats_out, p->stats, T * 5 * (size_t)p->cfg.num_sets, cudaMemcpyDeviceToHost, st),
                  "copy statistics");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    return p->cfg.form != GSEA_FORM_PLAIN ? check_device_error(p) : GSEA_OK;
}

int gsea_plan_buffer(gsea_plan p, int which, void** dev_ptr, size_t* bytes) {
    if (!p || !dev_ptr) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    const size_t T = p->tsize, G = (size_t)p->cfg.num_genes, pb = (size_t)p->pb;
    void* ptr = nullptr;
    size_t n = 0;
    switch (which) {
        case GSEA_BUF_EXPRS: ptr = p->exprs; n = T * G * p->cfg.num_samples; break;
        case GSEA_BUF_LABEL_MASKS: ptr = p->masks; n = 4 * (size_t)p->words * pb; break;
        case GSEA_BUF_KEYS: ptr = p->keys; n = T * G * pb; break;
        case GSEA_BUF_RANKS: ptr = p->ranks; n = (p->ranks16 ? 2 : 4) * G * pb; break;
        case GSEA_BUF_ORDER: ptr = p->order; n = p->order ? 4 * G * pb : 0; break;
        case GSEA_BUF_ES: ptr = p->es; n = T * (size_t)p->cfg.num_sets * p->cfg.num_perms; break;
        case GSEA_BUF_STATS: ptr = p->stats; n = T * 5 * (size_t)p->cfg.num_sets; break;
        case GSEA_BUF_SORTED: ptr = p->sorted; n = T * G * pb; break;
        default: return fail(GSEA_ERR_INVALID_ARGUMENT, "unknown buffer id");
    }
    *dev_ptr = ptr;
    if (bytes) *bytes = n;
    return GSEA_OK;
}

int gsea_plan_read_buffer(gsea_plan p, int which, void* host_dst, size_t bytes) {
    if (!host_dst) return fail(GSEA_ERR_INVALID_ARGUMENT, "null destination");
    void* src = nullptr;
    size_t n = 0;
    int rc = gsea_plan_buffer(p, which, &src, &n);
    if (rc) return rc;
    if ((rc = use_device(p))) return rc;
    GSEA_CUDA(cudaDeviceSynchronize(), "device sync");
    if (!src || n == 0) return fail(GSEA_ERR_INVALID_ARGUMENT, "buffer not allocated");
    GSEA_CUDA(cudaMemcpy(host_dst, src, bytes < n ? bytes : n, cudaMemcpyDeviceToHost), "copy buffer");
    return GSEA_OK;
}

int gsea_plan_info(gsea_plan p, int64_t* perm_batch, int* ranks16) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    if (perm_batch) *perm_batch = p->pb;
    if (ranks16) *ranks16 = p->ranks16 ? 1 : 0;
    return GSEA_OK;
}

int gsea_plan_set_debug(gsea_plan p, int keep) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    int rc = use_device(p);
    if (rc) return rc;
    p->debug = keep != 0;
    drop_graph(p);
    if (p->debug) return alloc_order(p);
    return GSEA_OK;
}

int gsea_plan_set_profiling(gsea_plan p, int on) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    p->profile = on != 0;
    return GSEA_OK;
}

int gsea_plan_stage_times(gsea_plan p, double* ms) {
    if (!p || !ms) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    for (int i = 0; i < GSEA_NUM_STAGES; i++) ms[i] = 0.0;
    if (!p->profile || p->events_used < 2) return fail(GSEA_ERR_INVALID_ARGUMENT, "no profiled execute");
    int rc = use_device(p);
    if (rc) return rc;
    GSEA_CUDA(cudaEventSynchronize(p->events[p->events_used - 1]), "cudaEventSynchronize");
    for (size_t i = 1; i < p->events_used; i++) {
        float t = 0.f;
        GSEA_CUDA(cudaEventElapsedTime(&t, p->events[i - 1], p->events[i]), "cudaEventElapsedTime");
        const int stage = p->event_stage[i];
        if (stage >= 0 && stage < GSEA_NUM_STAGES) ms[stage] += t;
    }
    return GSEA_OK;
}

int gsea_plan_last_launches(gsea_plan p, int64_t* launches) {
    if (!p || !launches) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    *launches = p->last_launches;
    return GSEA_OK;
}

int gsea_write_es_dump(const char* prefix, const void* es, int64_t K, int64_t P, int precision, char* path_out,
                       size_t path_len) {
    if (!es || K < 1 || P < 1 || (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid dump arguments");
    return write_dump(prefix, es, K, P, precision, path_out, path_len);
}

int gsea_run(const gsea_config* cfg, const void* exprs, const uint8_t* labels, const int64_t* set_offsets,
             const int32_t* set_genes, void* es_out, void* stats_out, const char* dump_prefix) {
    gsea_plan p = nullptr;
    int rc = gsea_plan_create(cfg, &p);
    if (rc) return rc;
    std::vector<unsigned char> es_tmp;
    const bool dump = dump_prefix && *dump_prefix;
    void* es_dst = es_out;
    if (dump && !es_dst) {
        es_tmp.resize(p->tsize * (size_t)cfg->num_sets * cfg->num_perms);
        es_dst = es_tmp.data();
    }
    rc = gsea_plan_run_host(p, exprs, labels, set_offsets, set_genes, es_dst, stats_out);
    if (!rc && dump) rc = write_dump(dump_prefix, es_dst, cfg->num_sets, cfg->num_perms, cfg->precision, nullptr, 0);
    const std::string keep = t_error;
    gsea_plan_destroy(p);
    t_error = keep;
    return rc;
}

int gsea_run_f32(const float* exprs, int64_t G, int64_t S, const uint8_t* labels, const int64_t* off,
                 const int32_t* genes, int64_t K, int64_t P, int metric, int ascending, float* es_out,
                 float* stats_out, const char* dump_prefix) {
    gsea_config c;
    gsea_config_init(&c);
    c.num_genes = G; c.num_samples = S; c.num_sets = K; c.num_perms = P;
    c.metric = metric; c.ascending = ascending; c.precision = 32;
    return gsea_run(&c, exprs, labels, off, genes, es_out, stats_out, dump_prefix);
}

int gsea_run_f64(const double* exprs, int64_t G, int64_t S, const uint8_t* labels, const int64_t* off,
                 const int32_t* genes, int64_t K, int64_t P, int metric, int ascending, double* es_out,
                 double* stats_out, const char* dump_prefix) {
    gsea_config c;
    gsea_config_init(&c);
    c.num_genes = G; c.num_samples = S; c.num_sets = K; c.num_perms = P;
    c.metric = metric; c.ascending = ascending; c.precision = 64;
    return gsea_run(&c, exprs, labels, off, genes, es_out, stats_out, dump_prefix);
}

}  // extern "C"
