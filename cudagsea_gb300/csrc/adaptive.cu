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
// measured null mean exceeds fallback_tol.  Sets that never stop run all
// num_perms permutations, the full test; every reported statistic is counted
// from the permutations a set received.
#include <algorithm>
#include <cmath>
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

template <class T>
int execute_adaptive_t(gsea_plan_s* p, gsea_model model, const gsea_adaptive_params& ap, int64_t* counts_out,
                       gsea_adaptive_report* report) {
    const int K = (int)p->cfg.num_sets;
    const int64_t P = p->cfg.num_perms;
    const int64_t P0 = std::min<int64_t>(std::max<int64_t>(ap.pilot_perms, 2), P);
    cudaStream_t st = p->stream;
    const T* es = static_cast<const T*>(p->es);
    int rc = ensure_buffers(p);
    if (rc) return rc;
    gsea::launches_take();
    p->events_used = 0;
    GSEA_CUDA(cudaMemsetAsync(p->exceed, 0, sizeof(unsigned long long) * K, st), "clear exceedances");
    GSEA_CUDA(cudaMemsetAsync(p->sumabs, 0, sizeof(double) * 2 * K, st), "clear sums");
    // pilot: every set, permutations [0, P0)
    if ((rc = gsea::plan_run_range(p, st, 0, P0, p->set_order, K))) return rc;
    GSEA_CUDA(gsea::launch_exceed<T>(es, P, K, nullptr, K, 0, P0, p->exceed, p->sumabs, st), "exceedance kernel");
    std::vector<int64_t> counts((size_t)K, P0);
    GSEA_CUDA(cudaMemcpyAsync(p->counts, counts.data(), sizeof(int64_t) * K, cudaMemcpyHostToDevice, st),
              "copy counts");
    GSEA_CUDA(gsea::launch_stats_ragged<T>(es, K, P, p->counts, P0, static_cast<T*>(p->stats), p->stats_scratch, st),
              "pilot statistics");
    // FDR rule: lower bounds of the sets' q from the statistics just computed
    // (launched before the host synchronises, copied back with the rest)
    const bool q_on = ap.q_margin > 0.0;
    std::vector<float> qlow((size_t)K);
    auto launch_bound = [&]() -> int {
        GSEA_CUDA(gsea::launch_fdr_bound<T>(K, P0, static_cast<const T*>(p->stats), p->counts, p->sumabs, ap.z,
                                            p->stats_scratch, p->qlow, st),
                  "FDR bound kernel");
        GSEA_CUDA(cudaMemcpyAsync(qlow.data(), p->qlow, sizeof(float) * K, cudaMemcpyDeviceToHost, st), "copy bounds");
        return GSEA_OK;
    };
    if (q_on && P0 < P && (rc = launch_bound())) return rc;
    std::vector<T> stats((size_t)5 * K);
    std::vector<unsigned long long> exceed((size_t)K);
    std::vector<double> sumabs((size_t)K);
    GSEA_CUDA(cudaMemcpyAsync(stats.data(), p->stats, sizeof(T) * 5 * K, cudaMemcpyDeviceToHost, st), "copy stats");
    GSEA_CUDA(cudaMemcpyAsync(exceed.data(), p->exceed, sizeof(unsigned long long) * K, cudaMemcpyDeviceToHost, st),
              "copy exceedances");
    GSEA_CUDA(cudaMemcpyAsync(sumabs.data(), p->sumabs, sizeof(double) * K, cudaMemcpyDeviceToHost, st), "copy sums");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    double pstar = 0.0;
    for (int k = 0; k < K; k++) {
        const double q = (double)stats[4 * (size_t)K + k], np = (double)stats[2 * (size_t)K + k];
        if (q < ap.q_call && np > pstar) pstar = np;
    }
    const double stop_p = std::min(1.0, std::max(ap.p_floor, ap.margin * pstar));
    // learned prior
    std::vector<float> pm, prior;
    int32_t model_used = 0;
    double mean_err = NAN;
    if (model) {
        float norms[GSEA_MODEL_NORMS];
        if ((rc = gsea_model_get(model, nullptr, norms))) return rc;
        if (norms[14] != 0.f) {
            if (!p->moments_ready) {  // a property of the inputs: computed once per upload
                if ((rc = compute_moments<T>(p, st))) return rc;
                p->moments_ready = true;
            }
            GSEA_CUDA(gsea::launch_model_features<T>(es, P, p->set_off, K, p->moments, p->sumabs, P0, p->feat, st),
                      "features");
            if ((rc = gsea_model_predict(model, p->feat, K, p->pred, st))) return rc;
            std::vector<float> pred((size_t)2 * K);
            GSEA_CUDA(cudaMemcpyAsync(pred.data(), p->pred, sizeof(float) * 2 * K, cudaMemcpyDeviceToHost, st),
                      "copy predictions");
            GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
            std::vector<double> errs;
            for (int k = 0; k < K; k++) {
                const double mt = pred[2 * (size_t)k + 1], mh = sumabs[k] / (double)P0;
                if (std::isfinite(mt) && mt > 0 && std::isfinite(mh) && mh > 0) errs.push_back(std::fabs(std::log(mt / mh)));
            }
            mean_err = median(errs);
            if (mean_err <= ap.fallback_tol) {
                model_used = 1;
                const double s2 = (double)norms[12] * (double)norms[12];
                const double cap = ap.prior_cap * (double)P0;
                pm.resize((size_t)K);
                prior.resize((size_t)K);
                for (int k = 0; k < K; k++) {
                    const double v = std::min(std::max((double)pred[2 * (size_t)k], 1e-6), 1.0 - 1e-6);
                    pm[k] = (float)v;
                    prior[k] = (float)std::min(1.0 / (s2 * v * (1.0 - v)), cap);
                }
            }
        }
    }
    std::vector<int64_t> ex64((size_t)K);
    std::vector<uint8_t> stop((size_t)K), now((size_t)K);
    auto decide = [&](std::vector<uint8_t>& out) {
        for (int k = 0; k < K; k++) ex64[k] = (int64_t)exceed[k];
        return gsea_adaptive_decide(K, counts.data(), ex64.data(), model_used ? pm.data() : nullptr,
                                    model_used ? prior.data() : nullptr, stop_p, ap.z, out.data());
    };
    if ((rc = decide(stop))) return rc;
    int64_t stopped_q = 0;
    const double q_stop = ap.q_margin * ap.q_call;
    auto apply_bound = [&](std::vector<uint8_t>& st_out) {  // after the synchronisation that brought qlow
        for (int k = 0; k < K; k++)
            if (!st_out[k] && counts[k] < P && (double)qlow[k] >= q_stop) {
                st_out[k] = 1;
                stopped_q++;
            }
    };
    if (q_on && P0 < P) apply_bound(stop);
    int64_t prior_sets = 0, prior_agreed = 0;
    if (model_used) {
        for (int k = 0; k < K; k++) {
            if (!(std::isfinite(pm[k]) && std::isfinite(prior[k]) && prior[k] > 0)) continue;
            prior_sets++;
            const double v = std::min(std::max((double)pm[k], 1e-6), 1.0 - 1e-6);
            prior_agreed += gsea::prior_agrees(v, prior[k], (double)P0, (double)exceed[k], ap.z) ? 1 : 0;
        }
    }
    int64_t stopped_pilot = 0;
    for (int k = 0; k < K; k++) stopped_pilot += stop[k];
    int64_t cur = P0, rounds = 1;
    std::vector<int32_t> active;
    active.reserve((size_t)K);
    while (cur < P) {
        const int64_t next = std::min<int64_t>(P, std::max<int64_t>(cur + 1, (int64_t)std::ceil((double)cur * ap.growth)));
        active.clear();
        for (int32_t k : p->h_set_order)
            if (!stop[k]) active.push_back(k);
        if (active.empty()) break;
        const int n = (int)active.size();
        GSEA_CUDA(cudaMemcpyAsync(p->active, active.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st),
                  "copy active sets");
        if ((rc = gsea::plan_run_range(p, st, cur, next, p->active, n))) return rc;
        GSEA_CUDA(gsea::launch_exceed<T>(es, P, K, p->active, n, cur, next, p->exceed, p->sumabs, st), "exceedances");
        for (int32_t k : active) counts[k] = next;
        const bool bound_now = q_on && next < P;
        if (bound_now) {  // statistics at the new counts, then the bounds: one synchronisation per round
            GSEA_CUDA(cudaMemcpyAsync(p->counts, counts.data(), sizeof(int64_t) * K, cudaMemcpyHostToDevice, st),
                      "copy counts");
            // the stopping bound's null histogram: the pilot columns of
            // every set (the final statistics use every score)
            GSEA_CUDA(gsea::launch_stats_ragged<T>(es, K, P, p->counts, P0, static_cast<T*>(p->stats),
                                                   p->stats_scratch, st, P0),
                      "round statistics");
            if ((rc = launch_bound())) return rc;
        }
        GSEA_CUDA(cudaMemcpyAsync(exceed.data(), p->exceed, sizeof(unsigned long long) * K, cudaMemcpyDeviceToHost, st),
                  "copy exceedances");
        GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
        if ((rc = decide(now))) return rc;
        for (int32_t k : active) stop[k] = now[k];
        if (bound_now) apply_bound(stop);
        cur = next;
        rounds++;
    }
    GSEA_CUDA(cudaMemcpyAsync(p->counts, counts.data(), sizeof(int64_t) * K, cudaMemcpyHostToDevice, st),
              "copy counts");
    GSEA_CUDA(gsea::launch_stats_ragged<T>(es, K, P, p->counts, P0, static_cast<T*>(p->stats), p->stats_scratch, st),
              "statistics kernels");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    p->last_launches = gsea::launches_take();
    if (counts_out) std::copy(counts.begin(), counts.end(), counts_out);
    if (report) {
        report->rounds = rounds;
        int64_t total = 0, full = 0;
        for (int64_t c : counts) {
            total += c;
            full += c == P;
        }
        report->scores = total;
        report->stopped_pilot = stopped_pilot;
        report->full_sets = full;
        report->stop_p = stop_p;
        report->model_used = model_used;
        report->model_mean_err = mean_err;
        report->prior_sets = prior_sets;
        report->prior_agreed = prior_agreed;
        report->stopped_q = stopped_q;
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
        !(a.prior_cap >= 0.0) || !(a.q_call > 0.0) || !(a.q_margin >= 0.0))
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
