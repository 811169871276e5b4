// batch.cu -- many independent GSEA instances in one CUDA graph.
//
// No counterpart in the reference, which runs one problem per call
// (src/cudaGSEA_wrapper.cu:179-401).  Per execute, every stage is one launch
// over all instances (each instance's plan holds num_perms x num_genes
// buffers), blockIdx.z naming the instance where the work is a grid:
//   1. the label permutations of every instance: one launch;
//   2. the metric: in the tensor-core form one launch each of the label
//      operand and the tcgen05 class statistics per metric family (one
//      family when all instances share a metric); in the plain form one
//      launch per metric and kernel path (exact, or packed with 4 or 8
//      permutations per thread);
//   3. the sort: one launch per register-resident class (ITEMS keys per
//      thread, one CTA or a two-CTA cluster per permutation); instances
//      beyond the register forms (G > 40,960 fp32 / 20,480 fp64) sort on
//      their own;
//   4. one persistent enrichment launch per size class (the bitmap words per
//      lane of the register procedure, fixed by G): its CTAs pull
//      (instance, permutation) items from a global counter, heaviest
//      instances first, so uneven instances keep every SM busy to the end;
//   5. the statistics of every instance: one launch per step (nine), the
//      instances whose FDR histogram does not fit shared memory on their own.
// Every instance's results are those of its solo plan bit for bit.  The
// first execute captures the stages into one CUDA graph; later executes
// replay it.
#include <algorithm>
#include <map>
#include <new>
#include <numeric>
#include <vector>

#include "kernels.h"
#include "plan.h"

namespace {
using gsea::fail;

// one multi-instance launch: its device task table and a host copy
template <class Task>
struct Multi {
    int key = 0;                 // metric family / sort class
    std::vector<Task> h;
    Task* d = nullptr;
};

struct EsClass {
    int wpl = 0;
    int Gmax = 0;
    std::vector<int64_t> inst;  // instances, heaviest first
    void* d_tasks = nullptr;
    int64_t* d_item_end = nullptr;
    int64_t nitems = 0;
};

}  // namespace

struct gsea_batch_s {
    int device = 0;
    int precision = 32;
    std::vector<gsea_plan> plans;
    std::vector<char> ready;
    cudaStream_t main = nullptr;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    std::vector<EsClass> classes;
    std::map<int, gsea::EsTuning> es_tuning;  // per size class
    unsigned long long* d_counters = nullptr;
    // the multi-instance launches of the other stages (built with the classes)
    Multi<gsea::PermTask> perm;
    std::vector<Multi<gsea::ChosenTask>> chosen;
    std::vector<Multi<gsea::MetricTask<float>>> metric32;   // plain form
    std::vector<Multi<gsea::MetricTask<double>>> metric64;
    std::vector<Multi<gsea::SortTask>> sorts;
    std::vector<int64_t> solo_sort;   // instances sorted on their own (tiled sort)
    Multi<gsea::StatsTask<float>> stats32;
    Multi<gsea::StatsTask<double>> stats64;
    std::vector<int64_t> solo_stats;  // instances whose statistics run on their own
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t nodes = 0;
    int64_t launches = 0;
};

namespace {

void drop_graph(gsea_batch_s* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->nodes = 0;
}

template <class Task>
void free_multi(Multi<Task>& m) {
    if (m.d) cudaFree(m.d);
    m.d = nullptr;
    m.h.clear();
}

template <class Task>
cudaError_t upload_multi(Multi<Task>& m) {
    if (m.h.empty()) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&m.d, sizeof(Task) * m.h.size());
    if (e == cudaSuccess) e = cudaMemcpy(m.d, m.h.data(), sizeof(Task) * m.h.size(), cudaMemcpyHostToDevice);
    return e;
}

void drop_classes(gsea_batch_s* b) {
    for (EsClass& c : b->classes) {
        if (c.d_tasks) cudaFree(c.d_tasks);
        if (c.d_item_end) cudaFree(c.d_item_end);
    }
    b->classes.clear();
    if (b->d_counters) cudaFree(b->d_counters);
    b->d_counters = nullptr;
    free_multi(b->perm);
    for (auto& m : b->chosen) free_multi(m);
    b->chosen.clear();
    for (auto& m : b->metric32) free_multi(m);
    b->metric32.clear();
    for (auto& m : b->metric64) free_multi(m);
    b->metric64.clear();
    for (auto& m : b->sorts) free_multi(m);
    b->sorts.clear();
    b->solo_sort.clear();
    free_multi(b->stats32);
    free_multi(b->stats64);
    b->solo_stats.clear();
}

template <class T>
std::vector<Multi<gsea::MetricTask<T>>>& metric_groups(gsea_batch_s* b) {
    if constexpr (sizeof(T) == 8) return b->metric64;
    else return b->metric32;
}

// the task tables of the multi-instance stages
template <class T>
int build_multi(gsea_batch_s* b, Multi<gsea::StatsTask<T>>& stats) {
    const bool fp64 = b->precision == 64;
    std::map<int, size_t> chosen_at, sort_at, metric_at;
    auto& metrics = metric_groups<T>(b);
    for (int64_t i = 0; i < (int64_t)b->plans.size(); i++) {
        gsea_plan_s* p = b->plans[i];
        const gsea_config& c = p->cfg;
        gsea::PermTask pt;
        pt.labels = p->labels;
        pt.masks = p->masks;
        pt.perm_offset = c.perm_offset;
        pt.num_perms = c.num_perms;
        pt.seed = c.seed;
        pt.S = (int)c.num_samples;
        pt.words = p->words;
        b->perm.h.push_back(pt);
        if (c.form != GSEA_FORM_PLAIN) {
            gsea::ChosenTask ct;
            ct.A1 = p->opA1;
            ct.A2 = p->opA2;
            ct.Bm = p->opB;
            ct.mu = p->gene_mu;
            ct.t1 = p->gene_t1;
            ct.t2 = p->gene_t2;
            ct.keys = static_cast<float*>(p->keys);
            ct.masks = p->masks;
            ct.error_flag = p->dev_error;
            ct.nA = (float)p->nA;
            ct.nB = (float)p->nB;
            ct.G = (int)c.num_genes;
            ct.S = (int)c.num_samples;
            ct.num_perms = (int)c.num_perms;
            ct.chunks = gsea::chosen_chunks(ct.S);
            ct.words = p->words;
            ct.comb = gsea::chosen_comb(c.metric);
            auto it = chosen_at.find(ct.comb);
            if (it == chosen_at.end()) {
                it = chosen_at.emplace(ct.comb, b->chosen.size()).first;
                b->chosen.emplace_back();
                b->chosen.back().key = ct.comb;
            }
            b->chosen[it->second].h.push_back(ct);
        } else {
            gsea::MetricTask<T> mt;
            mt.X = static_cast<const T*>(p->exprs);
            mt.masks = p->masks;
            mt.keys = static_cast<T*>(p->keys);
            mt.fast_ok = p->fast_ok;
            mt.G = (int)c.num_genes;
            mt.S = (int)c.num_samples;
            mt.words = p->words;
            mt.num_perms = (int)p->pb;
            mt.nA = (T)p->nA;
            mt.nB = (T)p->nB;
            const int key = gsea::metric_multi_key<T>(c.metric, mt.S, mt.words, p->fast_ok != nullptr,
                                                      p->tuning.metric_pb);
            auto it = metric_at.find(key);
            if (it == metric_at.end()) {
                it = metric_at.emplace(key, metrics.size()).first;
                metrics.emplace_back();
                metrics.back().key = key;
            }
            metrics[it->second].h.push_back(mt);
        }
        const int cls = gsea::sort_multi_class((int)c.num_genes, fp64);
        if (cls == 0 || !p->ranks16) {
            b->solo_sort.push_back(i);
        } else {
            gsea::SortTask st;
            st.keys = p->keys;
            st.ranks = p->ranks;
            st.sorted = p->sorted;
            st.order = p->debug ? p->order : nullptr;
            st.G = (int)c.num_genes;
            st.num_perms = (int)c.num_perms;
            st.descending = c.ascending ? 0 : 1;
            auto it = sort_at.find(cls);
            if (it == sort_at.end()) {
                it = sort_at.emplace(cls, b->sorts.size()).first;
                b->sorts.emplace_back();
                b->sorts.back().key = cls;
            }
            b->sorts[it->second].h.push_back(st);
        }
        const int rows = gsea::stats_multi_rows<T>((int)c.num_sets, c.num_perms);
        if (rows <= 0) {
            b->solo_stats.push_back(i);
        } else {
            gsea::StatsTask<T> t;
            t.es = static_cast<const T*>(p->es);
            t.stats = static_cast<T*>(p->stats);
            t.scratch = p->stats_scratch;
            t.K = (int)c.num_sets;
            t.rows = rows;
            t.P = c.num_perms;
            stats.h.push_back(t);
        }
    }
    cudaError_t e = upload_multi(b->perm);
    for (auto& m : b->chosen)
        if (e == cudaSuccess) e = upload_multi(m);
    for (auto& m : metrics)
        if (e == cudaSuccess) e = upload_multi(m);
    for (auto& m : b->sorts)
        if (e == cudaSuccess) e = upload_multi(m);
    if (e == cudaSuccess) e = upload_multi(stats);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gsea::cuda_fail(e, "batch task tables");
    }
    return GSEA_OK;
}

// enrichment cost of an instance (G*K*P), for the order of the persistent launch
double es_cost(const gsea_config& c) {
    return (double)c.num_perms * c.num_sets * (double)(c.num_genes / 32 + 64);
}

template <class T>
int build_classes(gsea_batch_s* b) {
    drop_classes(b);
    std::map<int, EsClass> by;
    for (int64_t i = 0; i < (int64_t)b->plans.size(); i++) {
        const gsea_config& c = b->plans[i]->cfg;
        const int w = gsea::es_size_class((int)c.num_genes);
        EsClass& cl = by[w];
        cl.wpl = w;
        cl.Gmax = std::max(cl.Gmax, (int)c.num_genes);
        cl.inst.push_back(i);
    }
    for (auto& kv : by) {
        EsClass cl = kv.second;
        std::stable_sort(cl.inst.begin(), cl.inst.end(), [b](int64_t x, int64_t y) {
            return es_cost(b->plans[x]->cfg) > es_cost(b->plans[y]->cfg);
        });
        std::vector<gsea::EsTask<T>> tasks;
        std::vector<int64_t> item_end;
        int64_t items = 0;
        for (int64_t i : cl.inst) {
            gsea_plan_s* p = b->plans[i];
            gsea::EsTask<T> t;
            t.ranks = p->ranks;
            t.sorted = static_cast<const T*>(p->sorted);
            t.off = p->set_off;
            t.genes = p->set_genes;
            t.order = p->set_order;
            t.decay = static_cast<const T*>(p->decay);
            t.es = static_cast<T*>(p->es);
            t.col0 = 0;
            t.stride = p->cfg.num_perms;
            t.G = (int)p->cfg.num_genes;
            t.K = (int)p->cfg.num_sets;
            tasks.push_back(t);
            items += p->cfg.num_perms;
            item_end.push_back(items);
        }
        cl.nitems = items;
        cudaError_t e = cudaMalloc(&cl.d_tasks, sizeof(gsea::EsTask<T>) * tasks.size());
        if (e == cudaSuccess) e = cudaMalloc((void**)&cl.d_item_end, sizeof(int64_t) * item_end.size());
        if (e == cudaSuccess)
            e = cudaMemcpy(cl.d_tasks, tasks.data(), sizeof(gsea::EsTask<T>) * tasks.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(cl.d_item_end, item_end.data(), sizeof(int64_t) * item_end.size(), cudaMemcpyHostToDevice);
        b->classes.push_back(cl);
        if (e != cudaSuccess) {
            cudaGetLastError();
            drop_classes(b);
            return gsea::cuda_fail(e, "batch task tables");
        }
    }
    GSEA_CUDA(cudaMalloc((void**)&b->d_counters, sizeof(unsigned long long) * b->classes.size()), "batch counters");
    if constexpr (sizeof(T) == 8) return build_multi<double>(b, b->stats64);
    return build_multi<float>(b, b->stats32);
}

template <class T>
cudaError_t launch_class(gsea_batch_s* b, size_t ci, int64_t nitems, gsea::EsTuning tune, cudaStream_t st) {
    const EsClass& cl = b->classes[ci];
    return gsea::launch_es_batch<T>(static_cast<const gsea::EsTask<T>*>(cl.d_tasks), cl.d_item_end,
                                    (int)cl.inst.size(), nitems, b->d_counters + ci, cl.Gmax, cl.wpl, tune, st);
}

// the whole execute on `main`: one launch per stage over all instances
template <class T>
int record(gsea_batch_s* b) {
    const bool fp64 = b->precision == 64;
    cudaStream_t st = b->main;
    int rc;
    GSEA_CUDA(gsea::launch_permute_multi(b->perm.d, b->perm.h.data(), (int)b->perm.h.size(), st), "batched permute");
    if (b->plans[0]->cfg.form != GSEA_FORM_PLAIN) {
        const bool fp64var = b->plans[0]->cfg.form == GSEA_FORM_CHOSEN_FP64;
        for (auto& m : b->chosen)
            GSEA_CUDA(gsea::launch_chosen_metric_multi(m.d, m.h.data(), (int)m.h.size(), fp64var, st),
                      "batched tensor-core class statistics");
    } else {
        for (auto& m : metric_groups<T>(b))
            GSEA_CUDA(gsea::launch_metric_multi<T>(m.key, m.d, m.h.data(), (int)m.h.size(), st), "batched metric");
    }
    // the sort classes (and the instances that sort on their own), then the
    // enrichment size classes, each set of launches spread over the stream
    // pool so that one launch's tail overlaps the next one's start
    const size_t ns = b->streams.size();
    cudaEvent_t* ev = b->events.data();  // [0] fork 1, [1..ns] join 1, [ns+1] fork 2, [ns+2..2ns+1] join 2
    auto fork = [&](cudaEvent_t e) -> int {
        GSEA_CUDA(cudaEventRecord(e, st), "fork");
        for (size_t k = 0; k < ns; k++) GSEA_CUDA(cudaStreamWaitEvent(b->streams[k], e, 0), "fork");
        return GSEA_OK;
    };
    auto join = [&](cudaEvent_t* es) -> int {
        for (size_t k = 0; k < ns; k++) {
            GSEA_CUDA(cudaEventRecord(es[k], b->streams[k]), "join");
            GSEA_CUDA(cudaStreamWaitEvent(st, es[k], 0), "join");
        }
        return GSEA_OK;
    };
    if ((rc = fork(ev[0]))) return rc;
    size_t lane = 0;
    for (auto& m : b->sorts)
        GSEA_CUDA(gsea::launch_sort_multi(m.d, (int)m.h.size(), m.key, fp64, b->streams[lane++ % ns]),
                  "batched sort");
    for (int64_t i : b->solo_sort)
        if ((rc = gsea::plan_run_sort(b->plans[i], b->streams[lane++ % ns]))) return rc;
    if ((rc = join(ev + 1))) return rc;
    if ((rc = fork(ev[ns + 1]))) return rc;
    for (size_t ci = 0; ci < b->classes.size(); ci++) {
        const auto it = b->es_tuning.find(b->classes[ci].wpl);
        const gsea::EsTuning tune = it == b->es_tuning.end() ? gsea::EsTuning() : it->second;
        GSEA_CUDA(launch_class<T>(b, ci, b->classes[ci].nitems, tune, b->streams[ci % ns]),
                  "batched enrichment kernel");
    }
    if ((rc = join(ev + ns + 2))) return rc;
    if constexpr (sizeof(T) == 8)
        GSEA_CUDA(gsea::launch_stats_multi<double>(b->stats64.d, b->stats64.h.data(), (int)b->stats64.h.size(), st),
                  "batched statistics");
    else
        GSEA_CUDA(gsea::launch_stats_multi<float>(b->stats32.d, b->stats32.h.data(), (int)b->stats32.h.size(), st),
                  "batched statistics");
    for (int64_t i : b->solo_stats)
        if ((rc = gsea::plan_run_stats(b->plans[i], st))) return rc;
    return GSEA_OK;
}

template <class T>
int capture(gsea_batch_s* b) {
    drop_graph(b);
    int rc = build_classes<T>(b);
    if (rc) return rc;
    gsea::launches_take();
    GSEA_CUDA(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal), "begin capture");
    rc = record<T>(b);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->main, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc;
    }
    GSEA_CUDA(e, "end capture");
    b->graph = g;
    b->launches = gsea::launches_take();
    GSEA_CUDA(cudaGraphGetNodes(g, nullptr, &b->nodes), "graph nodes");
    GSEA_CUDA(cudaGraphInstantiate(&b->exec, g, 0), "graph instantiate");
    return GSEA_OK;
}

template <class T>
int autotune_b(gsea_batch_s* b, int64_t n) {
    int rc;
    for (gsea_plan p : b->plans)
        if ((rc = gsea::plan_autotune_front(p, n))) return rc;
    drop_graph(b);
    if ((rc = build_classes<T>(b))) return rc;
    // real data for the enrichment candidates: one pass of the first stage
    for (gsea_plan p : b->plans)
        if ((rc = gsea::plan_run_stage1(p, b->main))) return rc;
    cudaEvent_t t0, t1;
    GSEA_CUDA(cudaEventCreate(&t0), "event");
    GSEA_CUDA(cudaEventCreate(&t1), "event");
    for (size_t ci = 0; ci < b->classes.size(); ci++) {
        const int64_t items = std::min<int64_t>(b->classes[ci].nitems, std::max<int64_t>(n, 1) * 4);
        float best = 1e30f;
        gsea::EsTuning pick;
        for (int w : {32, 24, 16, 8}) {
            for (int stage : {1, 3, 2, 0}) {
                gsea::EsTuning t;
                t.warps = w;
                t.stage = stage;
                if (launch_class<T>(b, ci, items, t, b->main) != cudaSuccess) {  // warm-up, or does not fit
                    cudaGetLastError();
                    continue;
                }
                float ms_best = 1e30f;
                for (int r = 0; r < 3; r++) {
                    cudaEventRecord(t0, b->main);
                    launch_class<T>(b, ci, items, t, b->main);
                    cudaEventRecord(t1, b->main);
                    cudaEventSynchronize(t1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, t0, t1);
                    ms_best = std::min(ms_best, ms);
                }
                if (ms_best < best) {
                    best = ms_best;
                    pick = t;
                }
            }
        }
        b->es_tuning[b->classes[ci].wpl] = pick;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    GSEA_CUDA(cudaStreamSynchronize(b->main), "stream sync");
    GSEA_CUDA(cudaGetLastError(), "batch autotune");
    gsea::launches_take();
    return GSEA_OK;
}

bool check_instance(const gsea_batch_s* b, int64_t i) { return b && i >= 0 && i < (int64_t)b->plans.size(); }

}  // namespace

extern "C" {

int gsea_batch_create(int64_t n, const gsea_config* cfgs, int streams, gsea_batch* out) {
    if (!out || !cfgs || n < 1 || streams < 0 || streams > 128)
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    *out = nullptr;
    for (int64_t i = 0; i < n; i++) {
        if (cfgs[i].precision != cfgs[0].precision || cfgs[i].form != cfgs[0].form)
            return fail(GSEA_ERR_INVALID_ARGUMENT, "batch instances must share precision and form");
        if (cfgs[i].num_genes > 65536) return fail(GSEA_ERR_UNSUPPORTED, "batch instances need num_genes <= 65536");
    }
    gsea_batch_s* b = new (std::nothrow) gsea_batch_s();
    if (!b) return fail(GSEA_ERR_OUT_OF_MEMORY, "host allocation");
    b->precision = cfgs[0].precision;
    int rc = GSEA_OK;
    for (int64_t i = 0; i < n && rc == GSEA_OK; i++) {
        gsea_config c = cfgs[i];
        c.perm_batch = c.num_perms;  // every permutation in one device batch
        if (i > 0) c.device = b->device;
        gsea_plan p = nullptr;
        rc = gsea_plan_create(&c, &p);
        if (rc == GSEA_OK) {
            b->plans.push_back(p);
            b->ready.push_back(0);
            if (i == 0) b->device = p->device;
        }
    }
    const int ns = streams ? streams : 16;
    cudaError_t e = cudaSuccess;
    if (rc == GSEA_OK) e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking);
    for (int s = 0; s < ns && rc == GSEA_OK && e == cudaSuccess; s++) {
        cudaStream_t st;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) b->streams.push_back(st);
    }
    for (int k = 0; k < 2 * ns + 2 && rc == GSEA_OK && e == cudaSuccess; k++) {
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) b->events.push_back(ev);
    }
    if (rc == GSEA_OK && e != cudaSuccess) rc = gsea::cuda_fail(e, "batch streams");
    if (rc) {
        gsea_batch_destroy(b);
        return rc;
    }
    *out = b;
    return GSEA_OK;
}

int gsea_batch_destroy(gsea_batch b) {
    if (!b) return GSEA_OK;
    cudaSetDevice(b->device);
    if (b->main) cudaStreamSynchronize(b->main);
    drop_graph(b);
    drop_classes(b);
    for (cudaEvent_t e : b->events) cudaEventDestroy(e);
    for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
    if (b->main) cudaStreamDestroy(b->main);
    for (gsea_plan p : b->plans) gsea_plan_destroy(p);
    delete b;
    return GSEA_OK;
}

int gsea_batch_set_inputs(gsea_batch b, int64_t i, const void* exprs, const uint8_t* labels,
                          const int64_t* set_offsets, const int32_t* set_genes) {
    if (!check_instance(b, i)) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid batch instance");
    GSEA_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    if (b->main) GSEA_CUDA(cudaStreamSynchronize(b->main), "stream sync");
    const int rc = gsea_plan_set_inputs(b->plans[i], exprs, labels, set_offsets, set_genes);
    if (rc) return rc;
    b->ready[i] = 1;
    drop_graph(b);  // buffers of the sets may have moved
    return GSEA_OK;
}

int gsea_batch_autotune(gsea_batch b, int64_t sample_perms) {
    if (!b) return fail(GSEA_ERR_INVALID_ARGUMENT, "null batch");
    for (char r : b->ready)
        if (!r) return fail(GSEA_ERR_INVALID_ARGUMENT, "batch inputs were not all set");
    if (sample_perms < 0) return fail(GSEA_ERR_INVALID_ARGUMENT, "negative sample");
    GSEA_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    int sms = 1;
    GSEA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device), "device attribute");
    const int64_t n = sample_perms ? sample_perms : 2 * (int64_t)sms;
    return b->precision == 64 ? autotune_b<double>(b, n) : autotune_b<float>(b, n);
}

int gsea_batch_execute(gsea_batch b, void* stream) {
    if (!b) return fail(GSEA_ERR_INVALID_ARGUMENT, "null batch");
    for (char r : b->ready)
        if (!r) return fail(GSEA_ERR_INVALID_ARGUMENT, "batch inputs were not all set");
    GSEA_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    if (!b->exec) {
        const int rc = b->precision == 64 ? capture<double>(b) : capture<float>(b);
        if (rc) return rc;
    }
    GSEA_CUDA(cudaGraphLaunch(b->exec, stream ? static_cast<cudaStream_t>(stream) : b->main), "graph launch");
    return GSEA_OK;
}

int gsea_batch_synchronize(gsea_batch b) {
    if (!b) return fail(GSEA_ERR_INVALID_ARGUMENT, "null batch");
    GSEA_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    GSEA_CUDA(cudaDeviceSynchronize(), "device sync");
    for (gsea_plan p : b->plans) {
        const int rc = gsea_plan_synchronize(p);  // surfaces a kernel's error flag
        if (rc) return rc;
    }
    return GSEA_OK;
}

int gsea_batch_read(gsea_batch b, int64_t i, void* es_out, void* stats_out) {
    if (!check_instance(b, i)) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid batch instance");
    return gsea_plan_read(b->plans[i], es_out, stats_out);
}

int gsea_batch_plan(gsea_batch b, int64_t i, gsea_plan* plan) {
    if (!check_instance(b, i) || !plan) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid batch instance");
    *plan = b->plans[i];
    return GSEA_OK;
}

int gsea_batch_info(gsea_batch b, int64_t* graph_nodes, int64_t* es_classes, int64_t* launches) {
    if (!b) return fail(GSEA_ERR_INVALID_ARGUMENT, "null batch");
    if (graph_nodes) *graph_nodes = (int64_t)b->nodes;
    if (es_classes) *es_classes = (int64_t)b->classes.size();
    if (launches) *launches = b->exec ? b->launches : 0;
    return GSEA_OK;
}

}  // extern "C"
