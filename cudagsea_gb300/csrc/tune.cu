// tune.cu -- launch configuration of a plan and the autotuner that picks it.
//
// No counterpart in the reference, whose launch shapes are constants
// (correlate_genes.cuh:128-300 launches 256 threads per permutation;
// batched_sort.cuh:91-269 sorts 128 segments per CUB call;
// enrichment_scores.cuh:218-256 launches 32 threads per permutation).
//
// Tunables (every choice computes identical results):
//   metric      plain fp32 packed form: 4 or 8 permutations per thread;
//               tensor-core form: 128- or 256-permutation tiles (the GEMM's N)
//   sort        register-resident radix sort or the tiled one
//   enrichment  8 / 16 / 24 / 32 warps per CTA; the permutation's ranks and
//               weights staged in shared memory, its ranks only, its
//               weights only, or read from L2
// The autotuner runs each stage's candidates on a sample of the plan's own
// permutations (CUDA events on the plan's stream, best of three after one
// warm-up run) stage by stage -- metric, then sort on that stage's keys, then
// enrichment on the sort's output -- and keeps the fastest of each.
#include <algorithm>
#include <vector>

#include "kernels.h"
#include "plan.h"

namespace {
using gsea::fail;

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    Timer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~Timer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// best of 3 timed runs after one warm-up; a negative time if the candidate
// cannot run (configuration does not fit)
template <class F>
float time_best(F run, cudaStream_t st, Timer& t) {
    cudaError_t e = run();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return -1.f;
    }
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(t.a, st);
        if (run() != cudaSuccess) {
            cudaGetLastError();
            return -1.f;
        }
        cudaEventRecord(t.b, st);
        if (cudaEventSynchronize(t.b) != cudaSuccess) return -1.f;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t.a, t.b);
        best = std::min(best, ms);
    }
    return best;
}

constexpr unsigned kMetric = 1, kSort = 2, kEs = 4;

template <class T>
int autotune_t(gsea_plan_s* p, int64_t n64, unsigned stages, gsea_tuning* best_out, double* ms_out) {
    const gsea_config& c = p->cfg;
    const int G = (int)c.num_genes, S = (int)c.num_samples, K = (int)c.num_sets;
    const int n = (int)n64;
    cudaStream_t st = p->stream;
    Timer t;
    gsea_tuning best = p->tuning;
    GSEA_CUDA(gsea::launch_permute(p->labels, S, n, c.perm_offset, c.seed, p->masks, p->words, st), "permute kernel");
    // metric
    std::vector<int> mc;
    if (c.form != GSEA_FORM_PLAIN) mc = {256, 128};
    else mc = {8, 4};
    float mbest = 1e30f;
    if (!(stages & kMetric)) mc = {c.form != GSEA_FORM_PLAIN ? best.chosen_tile : best.metric_pb};
    for (int v : mc) {
        auto run = [&]() -> cudaError_t {
            if (c.form != GSEA_FORM_PLAIN)
                return gsea::launch_chosen_metric(c.metric, c.form == GSEA_FORM_CHOSEN_FP64, p->masks, p->words, G, S,
                                                  n, p->nA, p->nB, p->gene_mu, p->gene_t1, p->gene_t2, p->opA1,
                                                  p->opA2, p->opB, static_cast<float*>(p->keys), p->dev_error, st, v);
            return gsea::launch_metric<T>(c.metric, static_cast<const T*>(p->exprs), G, S, p->masks, p->words, n,
                                          p->nA, p->nB, static_cast<T*>(p->keys), p->fast_ok, st, v);
        };
        const float ms = time_best(run, st, t);
        if (ms >= 0.f && ms < mbest) {
            mbest = ms;
            if (c.form != GSEA_FORM_PLAIN) best.chosen_tile = v;
            else best.metric_pb = v;
        }
    }
    // leave the keys of the chosen metric configuration in place (identical
    // for every candidate, but make the buffer state independent of order)
    // sort
    gsea::SortBuffers sb;
    sb.ranks = p->ranks;
    sb.ranks16 = p->ranks16;
    sb.sorted_abs = p->sorted;
    sb.order = nullptr;
    sb.scratch = p->sort_scratch;
    sb.scratch_bytes = p->sort_scratch_bytes;
    sb.error_flag = p->dev_error;
    float sbest = 1e30f;
    std::vector<int> sc = {1, 2};
    if (!(stages & kSort)) sc = {best.sort_variant};
    for (int v : sc) {
        sb.variant = v;
        const float ms = time_best(
            [&]() { return gsea::launch_sort<T>(static_cast<const T*>(p->keys), G, n, c.ascending != 0, sb, st); }, st,
            t);
        if (ms >= 0.f && ms < sbest) {
            sbest = ms;
            best.sort_variant = v;
        }
    }
    // enrichment (on the last sort's output: identical for every variant)
    float ebest = 1e30f;
    for (int w : {32, 24, 16, 8}) {
        for (int stage : {1, 3, 2, 0}) {
            if (!(stages & kEs)) break;
            gsea::EsTuning et;
            et.warps = w;
            et.stage = stage;
            const float ms = time_best(
                [&]() {
                    return gsea::launch_es<T>(p->ranks, p->ranks16, static_cast<const T*>(p->sorted), G, n, p->set_off,
                                              p->set_genes, p->set_order, static_cast<const T*>(p->decay), K,
                                              static_cast<T*>(p->es), c.num_perms, 0, st, et);
                },
                st, t);
            if (ms >= 0.f && ms < ebest) {
                ebest = ms;
                best.es_warps = w;
                best.es_stage = stage;
            }
        }
    }
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    GSEA_CUDA(cudaGetLastError(), "autotune");
    if ((ebest >= 1e30f && (stages & kEs)) || sbest >= 1e30f || mbest >= 1e30f)
        return fail(GSEA_ERR_CUDA, "no launch configuration ran");
    p->tuning = best;
    gsea::plan_drop_graph(p);
    if (best_out) *best_out = best;
    if (ms_out) {
        ms_out[0] = mbest;
        ms_out[1] = sbest;
        ms_out[2] = ebest;
    }
    gsea::launches_take();
    return GSEA_OK;
}

bool valid(const gsea_tuning* t) {
    return (t->metric_pb == 0 || t->metric_pb == 4 || t->metric_pb == 8) &&
           (t->chosen_tile == 0 || t->chosen_tile == 128 || t->chosen_tile == 256) &&
           (t->sort_variant >= 0 && t->sort_variant <= 2) &&
           (t->es_warps == 0 || t->es_warps == 8 || t->es_warps == 16 || t->es_warps == 24 ||
            t->es_warps == 32) &&
           (t->es_stage >= -1 && t->es_stage <= 3);
}

}  // namespace

namespace gsea {
// the metric and sort stages only (the batch tunes its ES kernels per class)
int plan_autotune_front(gsea_plan_s* p, int64_t n) {
    n = std::min(n, p->pb);
    return p->cfg.precision == 64 ? autotune_t<double>(p, n, kMetric | kSort, nullptr, nullptr)
                                  : autotune_t<float>(p, n, kMetric | kSort, nullptr, nullptr);
}
}  // namespace gsea

extern "C" {

void gsea_tuning_init(gsea_tuning* t) {
    if (!t) return;
    t->metric_pb = 0;
    t->chosen_tile = 0;
    t->sort_variant = 0;
    t->es_warps = 0;
    t->es_stage = -1;
}

int gsea_plan_set_tuning(gsea_plan p, const gsea_tuning* t) {
    if (!p || !t) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    if (!valid(t)) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid tuning value");
    p->tuning = *t;
    gsea::plan_drop_graph(p);
    return GSEA_OK;
}

int gsea_plan_get_tuning(gsea_plan p, gsea_tuning* t) {
    if (!p || !t) return fail(GSEA_ERR_INVALID_ARGUMENT, "null argument");
    *t = p->tuning;
    return GSEA_OK;
}

int gsea_plan_autotune(gsea_plan p, int64_t sample_perms, gsea_tuning* best, double* ms_out) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    if (!p->inputs_set) return fail(GSEA_ERR_INVALID_ARGUMENT, "plan inputs were not set");
    if (sample_perms < 0) return fail(GSEA_ERR_INVALID_ARGUMENT, "negative sample");
    GSEA_CUDA(cudaSetDevice(p->device), "cudaSetDevice");
    int sms = 1;
    GSEA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device), "device attribute");
    // default sample: the plan's own batch (launch shapes depend on it), at
    // most 1,024 permutations and at least two per SM
    int64_t n = sample_perms ? sample_perms : std::max<int64_t>(2 * (int64_t)sms, std::min<int64_t>(p->pb, 1024));
    n = std::min(n, p->pb);
    return p->cfg.precision == 64 ? autotune_t<double>(p, n, kMetric | kSort | kEs, best, ms_out)
                                  : autotune_t<float>(p, n, kMetric | kSort | kEs, best, ms_out);
}

}  // extern "C"
