// adaptive.cu -- adaptive permutation allocation with the learned prior, the
// training-sample builder and the ragged statistics entry point.  No
// counterpart in the reference (every set gets num_perms permutations there,
// src/cudaGSEA_wrapper.cu:300-372).
//
// Sequential rule.  After r rounds set k holds n_k scores, c_k of them with
// |S| >= |ES_k| (permutation 0 counts itself, as NP does).  Its nominal p has
// the posterior Beta(a0 + c_k, b0 + n_k - c_k); the set stops when the
// posterior mean - z * sd >= stop_p, i.e. when it is confidently less
// significant than anything the FDR call at q_call could keep:
//   stop_p = max(p_floor, margin * max{NP_k^pilot : FDR_k^pilot < q_call}).
// Without a model the prior is Jeffreys' (a0 = b0 = 1/2).  With a trained
// model the prior adds w_k pseudo-permutations at the predicted tail p~_k:
//   a0 += p~_k w_k, b0 += (1 - p~_k) w_k,
//   w_k = min(1 / (sigma_tail^2 p~_k (1 - p~_k)), prior_cap * pilot_perms)
// (a Beta with that many pseudo-counts has the logit spread sigma_tail the
// model showed on held-out sets).  A set whose observed fraction c_k / n_k
// lies more than z sd from the prior predictive (beta-binomial: variance
// p~ (1 - p~) (w + n) / (n (w + 1))) ignores the prior: the permutations
// overrule the model.  The model is dropped for the run if the
// median |log m~_k - log m^_k| between its predicted and the pilot's
// measured null mean exceeds fallback_tol.  Two rules on the set's FDR q,
// from bounds over its NES uncertainty (z standard errors of its normalising
// mean): a set whose q lower bound is >= q_margin * q_call stops as clearly
// non-significant; a set whose q upper bound is <= q_call / sig_margin and
// whose p upper bound (posterior mean + z sd, the same posterior, model prior
// included) is <= p_sig = min{NP_k^pilot : FDR_k^pilot >= q_call} / sig_margin
// stops as clearly significant -- the permutations go to the sets near the
// call level.  Sets that never stop run all num_perms permutations, the full
// test; every reported statistic is counted from the permutations a set
// received.
//
// The whole test -- pilot, decisions, rounds, statistics -- is recorded once
// into a CUDA graph and replayed: the decisions are kernels and the rounds
// read the number of sets still running on the device, so the host waits
// only for the final report.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "plan.h"

namespace {
using gsea::fail;

int ensure_buffers(gsea_plan_s* p) {
    const size_t K = (size_t)p->cfg.num_sets;
    int rc = GSEA_OK;
    if (!p->moments && (rc = gsea::plan_dev_alloc((void**)&p->moments, sizeof(double) * 8, "moments"))) return rc;
    if (!p->active && (rc = gsea::plan_dev_alloc((void**)&p->active, sizeof(int32_t) * K, "active sets"))) return rc;
    if (!p->counts && (rc = gsea::plan_dev_alloc((void**)&p->counts, sizeof(int64_t) * K, "set counts"))) return rc;
    if (!p->exceed && (rc = gsea::plan_dev_alloc((void**)&p->exceed, sizeof(unsigned long long) * K, "exceedances")))
        return rc;
    if (!p->sumabs && (rc = gsea::plan_dev_alloc((void**)&p->sumabs, sizeof(double) * 2 * K, "score sums"))) return rc;
    if (!p->qlow && (rc = gsea::plan_dev_alloc((void**)&p->qlow, sizeof(float) * K, "q bounds"))) return rc;
    if (!p->feat && (rc = gsea::plan_dev_alloc((void**)&p->feat, sizeof(float) * 5 * K, "features"))) return rc;
    if (!p->pred && (rc = gsea::plan_dev_alloc((void**)&p->pred, sizeof(float) * 2 * K, "predictions"))) return rc;
    return GSEA_OK;
}

// moments of the observed ranking metric: permutation 0 alone through the
// plan's permute + metric kernels, then the moments kernel
template <class T>
int compute_moments(gsea_plan_s* p, cudaStream_t st) {
    const gsea_config& c = p->cfg;
    const int G = (int)c.num_genes, S = (int)c.num_samples;
    GSEA_CUDA(gsea::launch_permute(p->labels, S, 1, 0, c.seed, p->masks, p->words, st), "permute kernel");
    if (c.form != GSEA_FORM_PLAIN) {
        GSEA_CUDA(gsea::launch_chosen_metric(c.metric, c.form == GSEA_FORM_CHOSEN_FP64, p->masks, p->words, G, S, 1,
                                             p->nA, p->nB, p->gene_mu, p->gene_t1, p->gene_t2, p->opA1, p->opA2,
                                             p->opB, static_cast<float*>(p->keys), p->dev_error, st),
                  "tensor-core class statistics");
    } else {
        GSEA_CUDA(gsea::launch_metric<T>(c.metric, static_cast<const T*>(p->exprs), G, S, p->masks, p->words, 1, p->nA,
                                         p->nB, static_cast<T*>(p->keys), p->fast_ok, st),
                  "metric kernel");
    }
    GSEA_CUDA(gsea::launch_moments<T>(static_cast<const T*>(p->keys), G, p->moments, st), "moments kernel");
    return GSEA_OK;
}

double median(std::vector<double> v) {
    if (v.empty()) return INFINITY;
    std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
    return v[v.size() / 2];
}

template <class T>
int model_samples_t(gsea_plan_s* p, int queries, int holdout, float* x, float* t, int64_t* n_train, float* xv,
                    float* tv, int64_t* n_val) {
    const int K = (int)p->cfg.num_sets;
    const int64_t P = p->cfg.num_perms;
    cudaStream_t st = p->stream;
    int rc = ensure_buffers(p);
    if (rc || (rc = compute_moments<T>(p, st))) return rc;
    p->moments_ready = true;
    GSEA_CUDA(gsea::launch_set_means<T>(static_cast<const T*>(p->es), P, P, K, p->sumabs, st), "set means");
    std::vector<double> means((size_t)K);
    GSEA_CUDA(cudaMemcpyAsync(means.data(), p->sumabs, sizeof(double) * K, cudaMemcpyDeviceToHost, st), "copy means");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    // deterministic sample rows: sets in index order, invalid sets skipped
    std::vector<int64_t> slot((size_t)K, -1);
    int64_t nt = 0, nv = 0;
    const int per = queries + 1;
    for (int k = 0; k < K; k++) {
        if (!(std::isfinite(means[k]) && means[k] > 0.0)) continue;
        if (holdout > 0 && k % holdout == holdout - 1) {
            slot[k] = -(nv + 2);
            nv += per;
        } else {
            slot[k] = nt;
            nt += per;
        }
    }
    int64_t* dslot = nullptr;
    GSEA_CUDA(cudaMalloc((void**)&dslot, sizeof(int64_t) * K), "slots");
    cudaError_t e = cudaMemcpyAsync(dslot, slot.data(), sizeof(int64_t) * K, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = gsea::launch_model_samples<T>(static_cast<const T*>(p->es), P, P, p->set_off, K, p->moments, p->sumabs,
                                          queries, dslot, x, t, xv, tv, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dslot);
    GSEA_CUDA(e, "model samples");
    if (n_train) *n_train = nt;
    if (n_val) *n_val = nv;
    return GSEA_OK;
}

}  // namespace

namespace gsea {
// prior-data conflict check: the observed fraction c / n within z sd of the
// prior predictive (beta-binomial with mean pm and pm * w + (1 - pm) * w
// pseudo-counts) keeps the prior for the set
bool prior_agrees(double pm, double w, double n, double c, double z) {
    const double sd_pp = std::sqrt(pm * (1.0 - pm) * (w + n) / (n * (w + 1.0)));
    return std::fabs(c / n - pm) <= z * sd_pp;
}
}  // namespace gsea

namespace {

// Records the whole adaptive test on `st`: the pilot over every set, the
// decisions (kernels: stop_p, model fallback test, stopping rule, active
// list), then every round of the fixed schedule over the sets a kernel left
// active -- the set count is read on the device, so nothing waits for the
// host -- and the final ragged statistics.
template <class T>
int record_adaptive(gsea_plan_s* p, gsea_model model, bool use_model, const gsea::AdaptiveRule& rule, bool bounds_on,
                    const std::vector<std::pair<int64_t, int64_t>>& schedule, cudaStream_t st) {
    const int K = (int)p->cfg.num_sets;
    const int64_t P = p->cfg.num_perms, P0 = rule.P0;
    const T* es = static_cast<const T*>(p->es);
    T* stats = static_cast<T*>(p->stats);
    auto* ctl = static_cast<gsea::AdaptiveCtl*>(p->ad_ctl);
    const float* pred = use_model ? p->pred : nullptr;
    int rc;
    GSEA_CUDA(cudaMemsetAsync(p->exceed, 0, sizeof(unsigned long long) * K, st), "clear exceedances");
    GSEA_CUDA(cudaMemsetAsync(p->sumabs, 0, sizeof(double) * 2 * K, st), "clear sums");
    GSEA_CUDA(gsea::launch_adaptive_reset(K, P0, p->counts, ctl, st), "adaptive reset");
    // pilot: every set, permutations [0, P0)
    if ((rc = gsea::plan_run_range(p, st, 0, P0, p->set_order, K))) return rc;
    GSEA_CUDA(gsea::launch_exceed<T>(es, P, K, nullptr, K, 0, P0, p->exceed, p->sumabs, st), "exceedance kernel");
    GSEA_CUDA(gsea::launch_stats_ragged<T>(es, K, P, p->counts, P0, stats, p->stats_scratch, st), "pilot statistics");
    const bool bound0 = bounds_on && P0 < P;
    if (bound0)
        GSEA_CUDA(gsea::launch_fdr_bound<T>(K, P0, stats, p->counts, p->sumabs, rule.z, p->stats_scratch, p->qlow, st,
                                            p->qhigh),
                  "FDR bound kernel");
    if (use_model) {
        GSEA_CUDA(gsea::launch_model_features<T>(es, P, p->set_off, K, p->moments, p->sumabs, P0, p->feat, st),
                  "features");
        if ((rc = gsea_model_predict(model, p->feat, K, p->pred, st))) return rc;
    }
    GSEA_CUDA(gsea::launch_adaptive_prepare<T>(K, stats, pred, p->sumabs, rule, p->ad_err, ctl, st),
              "adaptive pilot decisions");
    GSEA_CUDA(gsea::launch_adaptive_decide(K, nullptr, nullptr, p->counts, p->exceed, pred, p->qlow, p->qhigh, bound0,
                                           true, rule, p->stop, ctl, st),
              "stopping rule");
    GSEA_CUDA(gsea::launch_adaptive_compact(K, p->set_order, p->stop, p->active, ctl, st), "active sets");
    for (const auto& r : schedule) {
        const int64_t cur = r.first, next = r.second;
        if ((rc = gsea::plan_run_range(p, st, cur, next, p->active, K, &ctl->n_active))) return rc;
        GSEA_CUDA(gsea::launch_exceed<T>(es, P, K, p->active, K, cur, next, p->exceed, p->sumabs, st, &ctl->n_active),
                  "exceedances");
        GSEA_CUDA(gsea::launch_adaptive_counts(K, p->active, ctl, next, p->counts, st), "set counts");
        const bool bound_now = bounds_on && next < P;
        if (bound_now) {  // statistics at the new counts, then the bounds
            // the stopping bound's null histogram: the pilot columns of
            // every set (the final statistics use every score)
            GSEA_CUDA(gsea::launch_stats_ragged<T>(es, K, P, p->counts, P0, stats, p->stats_scratch, st, P0),
                      "round statistics");
            GSEA_CUDA(gsea::launch_fdr_bound<T>(K, P0, stats, p->counts, p->sumabs, rule.z, p->stats_scratch, p->qlow,
                                                st, p->qhigh),
                      "FDR bound kernel");
        }
        GSEA_CUDA(gsea::launch_adaptive_decide(K, p->active, &ctl->n_active, p->counts, p->exceed, pred, p->qlow,
                                               p->qhigh, bound_now, false, rule, p->stop, ctl, st),
                  "stopping rule");
        GSEA_CUDA(gsea::launch_adaptive_compact(K, p->set_order, p->stop, p->active, ctl, st), "active sets");
    }
    GSEA_CUDA(gsea::launch_stats_ragged<T>(es, K, P, p->counts, P0, stats, p->stats_scratch, st),
              "statistics kernels");
    return GSEA_OK;
}

template <class T>
int execute_adaptive_t(gsea_plan_s* p, gsea_model model, const gsea_adaptive_params& ap, int64_t* counts_out,
                       gsea_adaptive_report* report) {
    const int K = (int)p->cfg.num_sets;
    const int64_t P = p->cfg.num_perms;
    const int64_t P0 = std::min<int64_t>(std::max<int64_t>(ap.pilot_perms, 2), P);
    cudaStream_t st = p->stream;
    int rc = ensure_buffers(p);
    if (rc) return rc;
    if (!p->stop && (rc = gsea::plan_dev_alloc((void**)&p->stop, (size_t)K, "stop flags"))) return rc;
    if (!p->ad_err && (rc = gsea::plan_dev_alloc((void**)&p->ad_err, sizeof(double) * K, "model errors"))) return rc;
    if (!p->qhigh && (rc = gsea::plan_dev_alloc((void**)&p->qhigh, sizeof(float) * K, "q upper bounds"))) return rc;
    if (!p->ad_ctl && (rc = gsea::plan_dev_alloc(&p->ad_ctl, sizeof(gsea::AdaptiveCtl), "adaptive record")))
        return rc;
    // the learned prior: only a trained model (norms[14] set by calibration)
    float norms[GSEA_MODEL_NORMS] = {};
    bool use_model = false;
    if (model) {
        if ((rc = gsea_model_get(model, nullptr, norms))) return rc;
        use_model = norms[14] != 0.f;
    }
    if (use_model && !p->moments_ready) {  // a property of the inputs: computed once per upload
        if ((rc = compute_moments<T>(p, st))) return rc;
        p->moments_ready = true;
    }
    gsea::AdaptiveRule rule;
    rule.q_call = ap.q_call;
    rule.margin = ap.margin;
    rule.p_floor = ap.p_floor;
    rule.z = ap.z;
    rule.q_stop = ap.q_margin * ap.q_call;
    rule.tol = ap.fallback_tol;
    rule.cap = ap.prior_cap * (double)P0;
    rule.s2 = (double)norms[12] * (double)norms[12];
    rule.sig_margin = ap.sig_margin;
    rule.P = P;
    rule.P0 = P0;
    const bool bounds_on = ap.q_margin > 0.0 || ap.sig_margin > 0.0;  // either rule needs the q bounds
    std::vector<std::pair<int64_t, int64_t>> schedule;
    for (int64_t cur = P0; cur < P;) {
        const int64_t next = std::min<int64_t>(P, std::max<int64_t>(cur + 1, (int64_t)std::ceil((double)cur * ap.growth)));
        schedule.emplace_back(cur, next);
        cur = next;
    }
    // what a captured graph was recorded for: the parameters and the model
    std::vector<unsigned char> key(sizeof(ap) + sizeof(model) + sizeof(norms) + 1);
    std::memcpy(key.data(), &ap, sizeof(ap));
    std::memcpy(key.data() + sizeof(ap), &model, sizeof(model));
    std::memcpy(key.data() + sizeof(ap) + sizeof(model), norms, sizeof(norms));
    key.back() = use_model ? 1 : 0;
    gsea::launches_take();
    int64_t launches = 0;
    if (p->profile) {  // stage events between the launches: issued one by one
        p->events_used = 0;
        if ((rc = record_adaptive<T>(p, model, use_model, rule, bounds_on, schedule, st))) return rc;
        launches = gsea::launches_take();
    } else {
        if (!p->ad_exec || p->ad_key != key) {
            if (p->ad_exec) cudaGraphExecDestroy(p->ad_exec);
            if (p->ad_graph) cudaGraphDestroy(p->ad_graph);
            p->ad_exec = nullptr;
            p->ad_graph = nullptr;
            GSEA_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            rc = record_adaptive<T>(p, model, use_model, rule, bounds_on, schedule, st);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return rc;
            }
            GSEA_CUDA(e, "end capture");
            p->ad_graph = g;
            p->ad_launches = gsea::launches_take();
            GSEA_CUDA(cudaGraphInstantiate(&p->ad_exec, g, 0), "graph instantiate");
            p->ad_key = key;
        }
        GSEA_CUDA(cudaGraphLaunch(p->ad_exec, st), "graph launch");
        launches = p->ad_launches;
    }
    std::vector<int64_t> counts((size_t)K);
    gsea::AdaptiveCtl ctl{};
    std::vector<double> err(use_model ? (size_t)K : 0);
    GSEA_CUDA(cudaMemcpyAsync(counts.data(), p->counts, sizeof(int64_t) * K, cudaMemcpyDeviceToHost, st),
              "copy counts");
    GSEA_CUDA(cudaMemcpyAsync(&ctl, p->ad_ctl, sizeof(ctl), cudaMemcpyDeviceToHost, st), "copy decisions");
    if (use_model)
        GSEA_CUDA(cudaMemcpyAsync(err.data(), p->ad_err, sizeof(double) * K, cudaMemcpyDeviceToHost, st),
                  "copy model errors");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    if ((rc = gsea::plan_check_error(p))) return rc;
    p->last_launches = launches;
    if (counts_out) std::copy(counts.begin(), counts.end(), counts_out);
    if (report) {
        int64_t total = 0, full = 0;
        for (int64_t c : counts) {
            total += c;
            full += c == P;
        }
        std::vector<double> valid;
        for (double e : err)
            if (std::isfinite(e)) valid.push_back(e);
        report->rounds = (int64_t)ctl.rounds;
        report->scores = total;
        report->stopped_pilot = (int64_t)ctl.stopped_pilot;
        report->full_sets = full;
        report->stop_p = ctl.stop_p;
        report->model_used = ctl.model_used;
        report->model_mean_err = use_model ? median(valid) : NAN;
        report->prior_sets = (int64_t)ctl.prior_sets;
        report->prior_agreed = (int64_t)ctl.prior_agreed;
        report->stopped_q = (int64_t)ctl.stopped_q;
        report->stopped_sig = (int64_t)ctl.stopped_sig;
        report->p_sig = ctl.p_sig;
    }
    return GSEA_OK;
}

}  // namespace

extern "C" {

void gsea_adaptive_params_init(gsea_adaptive_params* ap) {
    if (!ap) return;
    ap->pilot_perms = 1000;
    ap->growth = 2.0;
    ap->z = 3.0;
    ap->q_call = 0.25;
    ap->margin = 2.0;
    ap->p_floor = 0.01;
    ap->prior_cap = 4.0;
    ap->fallback_tol = 0.25;
    ap->q_margin = 1.5;
    ap->sig_margin = 2.0;
}

int gsea_adaptive_decide(int64_t num_sets, const int64_t* counts, const int64_t* exceed, const float* p_model,
                         const float* prior, double stop_p, double z, uint8_t* stop) {
    using gsea::prior_agrees;
    if (num_sets < 0 || (num_sets > 0 && (!counts || !exceed || !stop)))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    for (int64_t k = 0; k < num_sets; k++) {
        const double n = (double)counts[k], c = (double)exceed[k];
        if (!(n > 0) || c < 0 || c > n) {
            stop[k] = 0;
            continue;
        }
        double a = 0.5 + c, b = 0.5 + (n - c);
        if (p_model && prior && std::isfinite(p_model[k]) && std::isfinite(prior[k]) && prior[k] > 0) {
            const double pm = std::min(std::max((double)p_model[k], 1e-6), 1.0 - 1e-6), w = prior[k];
            if (prior_agrees(pm, w, n, c, z)) {
                a += pm * w;
                b += (1.0 - pm) * w;
            }
        }
        const double s = a + b, mean = a / s, sd = std::sqrt(a * b / (s * s * (s + 1.0)));
        stop[k] = mean - z * sd >= stop_p ? 1 : 0;
    }
    return GSEA_OK;
}

int gsea_plan_model_samples(gsea_plan p, int queries, int holdout, float* x, float* t, int64_t* n_train,
                            float* x_val, float* t_val, int64_t* n_val) {
    if (!p || !x || !t || queries < 1 || queries > gsea::model_max_queries() || holdout < 0 ||
        (holdout > 0 && (!x_val || !t_val)))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    if (!p->inputs_set) return fail(GSEA_ERR_INVALID_ARGUMENT, "plan inputs were not set");
    if (p->cfg.perm_offset != 0) return fail(GSEA_ERR_INVALID_ARGUMENT, "training samples need perm_offset 0");
    GSEA_CUDA(cudaSetDevice(p->device), "cudaSetDevice");
    return p->cfg.precision == 64 ? model_samples_t<double>(p, queries, holdout, x, t, n_train, x_val, t_val, n_val)
                                  : model_samples_t<float>(p, queries, holdout, x, t, n_train, x_val, t_val, n_val);
}

int gsea_plan_execute_adaptive(gsea_plan p, gsea_model model, const gsea_adaptive_params* ap, int64_t* counts,
                               gsea_adaptive_report* report) {
    if (!p) return fail(GSEA_ERR_INVALID_ARGUMENT, "null plan");
    if (!p->inputs_set) return fail(GSEA_ERR_INVALID_ARGUMENT, "plan inputs were not set");
    if (p->cfg.perm_offset != 0) return fail(GSEA_ERR_INVALID_ARGUMENT, "adaptive runs need perm_offset 0");
    gsea_adaptive_params def;
    gsea_adaptive_params_init(&def);
    const gsea_adaptive_params& a = ap ? *ap : def;
    if (a.pilot_perms < 2 || !(a.growth > 1.0) || !(a.z >= 0.0) || !(a.margin > 0.0) || !(a.p_floor >= 0.0) ||
        !(a.prior_cap >= 0.0) || !(a.q_call > 0.0) || !(a.q_margin >= 0.0) || !(a.sig_margin >= 0.0))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid adaptive parameters");
    GSEA_CUDA(cudaSetDevice(p->device), "cudaSetDevice");
    return p->cfg.precision == 64 ? execute_adaptive_t<double>(p, model, a, counts, report)
                                  : execute_adaptive_t<float>(p, model, a, counts, report);
}

int gsea_stats_ragged(const void* es, int64_t num_sets, int64_t ld, const int64_t* counts, int64_t p_fwer,
                      int precision, void* stats, void* stream) {
    if (!es || !stats || num_sets < 1 || num_sets > (int64_t)1 << 30 || ld < 1 || p_fwer < 1 || p_fwer > ld ||
        (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = precision == 64 ? gsea::stats_scratch_bytes<double>((int)num_sets, ld)
                                         : gsea::stats_scratch_bytes<float>((int)num_sets, ld);
    void* scratch = nullptr;
    GSEA_CUDA(cudaMalloc(&scratch, bytes), "statistics scratch");
    cudaError_t e = precision == 64
                        ? gsea::launch_stats_ragged<double>(static_cast<const double*>(es), (int)num_sets, ld, counts,
                                                            p_fwer, static_cast<double*>(stats), scratch, st)
                        : gsea::launch_stats_ragged<float>(static_cast<const float*>(es), (int)num_sets, ld, counts,
                                                           p_fwer, static_cast<float*>(stats), scratch, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(scratch);
    GSEA_CUDA(e, "ragged statistics");
    return GSEA_OK;
}

int gsea_fdr_lower_bound(const void* es, int64_t num_sets, int64_t ld, const int64_t* counts, int64_t p_fwer,
                         const double* sums, double z, int precision, void* stats, float* qlow, void* stream) {
    if (!es || !stats || !counts || !sums || !qlow || num_sets < 1 || num_sets > (int64_t)1 << 30 || ld < 1 ||
        p_fwer < 1 || p_fwer > ld || !(z >= 0.0) || (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int K = (int)num_sets;
    const size_t bytes = precision == 64 ? gsea::stats_scratch_bytes<double>(K, ld)
                                         : gsea::stats_scratch_bytes<float>(K, ld);
    void* scratch = nullptr;
    GSEA_CUDA(cudaMalloc(&scratch, bytes), "statistics scratch");
    cudaError_t e;
    if (precision == 64) {
        e = gsea::launch_stats_ragged<double>(static_cast<const double*>(es), K, ld, counts, p_fwer,
                                              static_cast<double*>(stats), scratch, st);
        if (e == cudaSuccess)
            e = gsea::launch_fdr_bound<double>(K, p_fwer, static_cast<const double*>(stats), counts, sums, z, scratch,
                                               qlow, st);
    } else {
        e = gsea::launch_stats_ragged<float>(static_cast<const float*>(es), K, ld, counts, p_fwer,
                                             static_cast<float*>(stats), scratch, st);
        if (e == cudaSuccess)
            e = gsea::launch_fdr_bound<float>(K, p_fwer, static_cast<const float*>(stats), counts, sums, z, scratch,
                                              qlow, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(scratch);
    GSEA_CUDA(e, "FDR bound");
    return GSEA_OK;
}

}  // extern "C"
