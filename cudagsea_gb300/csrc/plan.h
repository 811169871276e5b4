// plan.h -- the plan object behind gsea_plan and helpers shared by the
// translation units of the C ABI (capi.cu, adaptive.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gsea103.h"

namespace gsea {
void set_last_error(const char* msg);  // capi.cu

inline int fail(int status, const std::string& msg) {
    set_last_error(msg.c_str());
    return status;
}

inline int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(GSEA_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return fail(GSEA_ERR_NO_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(GSEA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace gsea

#define GSEA_CUDA(call, what)                                      \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return gsea::cuda_fail(e_, what);   \
    } while (0)

struct gsea_plan_s {
    gsea_config cfg;
    gsea_tuning tuning{0, 0, 0, 0, -1};
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t tsize = 4;
    int words = 0;
    int64_t pb = 0;  // permutations per batch
    bool ranks16 = true;
    bool debug = false;
    bool inputs_set = false;
    int64_t nA = 0, nB = 0;
    int64_t nnz = 0, nnz_cap = 0;
    int64_t last_launches = 0;
    // device buffers
    void* exprs = nullptr;
    uint8_t* labels = nullptr;
    int64_t* set_off = nullptr;
    int32_t* set_genes = nullptr;
    int32_t* set_order = nullptr;      // sets by decreasing size, for the ES kernel
    std::vector<int32_t> h_set_order;  // host staging of set_order
    std::vector<int64_t> h_set_size;   // members of each set (after mapping)
    uint32_t* masks = nullptr;
    int* fast_ok = nullptr;            // expression values allow the packed metric form
    void* decay = nullptr;             // [G+1] T: miss step per hit count
    // chosen form (tensor-core class statistics)
    float* gene_mu = nullptr;
    double* gene_t1 = nullptr;
    double* gene_t2 = nullptr;
    unsigned char* opA1 = nullptr;
    unsigned char* opA2 = nullptr;
    unsigned char* opB = nullptr;
    int* dev_error = nullptr;          // set by kernels whose bounded waits expired
    void* keys = nullptr;
    void* ranks = nullptr;
    void* sorted = nullptr;
    uint32_t* order = nullptr;
    void* sort_scratch = nullptr;
    size_t sort_scratch_bytes = 0;
    void* es = nullptr;
    void* stats = nullptr;
    void* stats_scratch = nullptr;
    size_t stats_scratch_bytes = 0;
    // the execute captured as a CUDA graph (replayed until buffers, tuning or
    // debug change)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int64_t graph_launches = 0;
    bool use_graph = true;
    // adaptive allocation / model features
    double* moments = nullptr;         // mean, sd, skewness of the observed ranking metric
    bool moments_ready = false;        // moments hold the current inputs' values
    int32_t* active = nullptr;         // [K] set list of the current adaptive round
    int64_t* counts = nullptr;         // [K] scores held per set (ragged statistics)
    unsigned long long* exceed = nullptr;  // [K] #{|S| >= |ES|} per set
    double* sumabs = nullptr;          // [2K] sum of |S| per set, then sum of S^2 per set
    float* qlow = nullptr;             // [K] lower bound of each set's FDR q (adaptive stopping)
    float* qhigh = nullptr;            // [K] upper bound of each set's FDR q (significance stopping)
    float* feat = nullptr;             // [K][5] model features
    float* pred = nullptr;             // [K][2] model predictions
    // the adaptive test on the device: per-set stop flags, the model's error
    // per set, the decision record (gsea::AdaptiveCtl) and the captured graph
    // of the whole test with what it was captured for (parameters, model)
    uint8_t* stop = nullptr;           // [K]
    double* ad_err = nullptr;          // [K] |log m~ - log m^| of the model, NaN where undefined
    void* ad_ctl = nullptr;
    cudaGraph_t ad_graph = nullptr;
    cudaGraphExec_t ad_exec = nullptr;
    std::vector<unsigned char> ad_key;
    int64_t ad_launches = 0;
    // stage timing (gsea_plan_set_profiling): events recorded at every stage
    // boundary of the last execute, tagged with the stage they close
    bool profile = false;
    std::vector<cudaEvent_t> events;
    std::vector<int> event_stage;
    size_t events_used = 0;
};

namespace gsea {
// Scores permutations [lo, hi) (global indices perm_offset + lo ...) of the
// sets set_list[0..n_sets) into columns lo..hi-1 of the plan's ES matrix
// (row stride num_perms).  No statistics.
// n_dev (may be null): the list holds min(n_sets, *n_dev) sets, read on the device.
int plan_run_range(gsea_plan_s* p, cudaStream_t st, int64_t lo, int64_t hi, const int32_t* set_list, int n_sets,
                   const int* n_dev = nullptr);
int plan_dev_alloc(void** ptr, size_t bytes, const char* what);
// forget the captured execute graph (buffers, tuning or debug changed)
void plan_drop_graph(gsea_plan_s* p);
// after a synchronisation: GSEA_ERR_CUDA if a tensor-core kernel's bounded wait expired
int plan_check_error(gsea_plan_s* p);
// permutation, metric and sort of every permutation (one device batch) without
// the enrichment kernel; and the statistics of the plan's ES matrix
int plan_run_stage1(gsea_plan_s* p, cudaStream_t st);
int plan_run_stats(gsea_plan_s* p, cudaStream_t st);
// the metric (plain or tensor-core form) and the sort of every permutation
// of a plan with one device batch, each on its own (batched-form fallbacks)
int plan_run_metric(gsea_plan_s* p, cudaStream_t st);
int plan_run_sort(gsea_plan_s* p, cudaStream_t st);
// autotune the metric and sort stages of a plan on n permutations (tune.cu)
int plan_autotune_front(gsea_plan_s* p, int64_t n);
}  // namespace gsea
