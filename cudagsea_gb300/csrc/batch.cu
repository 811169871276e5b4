// batch.cu -- many independent GSEA instances in one CUDA graph.
//
// No counterpart in the reference, which runs one problem per call
// (src/cudaGSEA_wrapper.cu:179-401).  Per execute:
//   1. every instance's permutation, metric and sort over all its
//      permutations (its plan holds num_perms x num_genes buffers), the
//      instances spread over a pool of streams, heaviest first on the least
//      loaded stream;
//   2. one persistent enrichment launch per size class (the bitmap words per
//      lane of the register procedure, fixed by G): its CTAs pull
//      (instance, permutation) items from a global counter, heaviest
//      instances first, so uneven instances keep every SM busy to the end;
//   3. every instance's statistics, again over the stream pool.
// The first execute captures the three phases into one CUDA graph (fork and
// join through events); later executes replay the instantiated graph.
#include <algorithm>
#include <map>
#include <new>
#include <numeric>
#include <vector>

#include "kernels.h"
#include "plan.h"

namespace {
using gsea::fail;

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

void drop_classes(gsea_batch_s* b) {
    for (EsClass& c : b->classes) {
        if (c.d_tasks) cudaFree(c.d_tasks);
        if (c.d_item_end) cudaFree(c.d_item_end);
    }
    b->classes.clear();
    if (b->d_counters) cudaFree(b->d_counters);
    b->d_counters = nullptr;
}

// stage-1 cost model (metric ~ G*S*P, sort ~ G*P*passes) and ES cost (G*K*P)
double front_cost(const gsea_config& c) {
    return (double)c.num_genes * c.num_perms * ((double)c.num_samples / 8.0 + (c.precision == 64 ? 8.0 : 4.0));
}
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
    return GSEA_OK;
}

template <class T>
cudaError_t launch_class(gsea_batch_s* b, size_t ci, int64_t nitems, gsea::EsTuning tune, cudaStream_t st) {
    const EsClass& cl = b->classes[ci];
    return gsea::launch_es_batch<T>(static_cast<const gsea::EsTask<T>*>(cl.d_tasks), cl.d_item_end,
                                    (int)cl.inst.size(), nitems, b->d_counters + ci, cl.Gmax, cl.wpl, tune, st);
}

// the whole execute on `main`, forking to and joining from the stream pool
template <class T>
int record(gsea_batch_s* b) {
    const size_t ns = b->streams.size();
    const int64_t n = (int64_t)b->plans.size();
    cudaEvent_t* ev = b->events.data();  // [0] fork 1, [1..ns] join 1, [ns+1] fork 2, [ns+2..2ns+1] join 2
    int rc;
    GSEA_CUDA(cudaEventRecord(ev[0], b->main), "fork");
    for (size_t s = 0; s < ns; s++) GSEA_CUDA(cudaStreamWaitEvent(b->streams[s], ev[0], 0), "fork");
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [b](int64_t x, int64_t y) {
        return front_cost(b->plans[x]->cfg) > front_cost(b->plans[y]->cfg);
    });
    std::vector<double> load(ns, 0.0);
    for (int64_t i : order) {
        const size_t s = std::min_element(load.begin(), load.end()) - load.begin();
        load[s] += front_cost(b->plans[i]->cfg);
        if ((rc = gsea::plan_run_stage1(b->plans[i], b->streams[s]))) return rc;
    }
    for (size_t s = 0; s < ns; s++) {
        GSEA_CUDA(cudaEventRecord(ev[1 + s], b->streams[s]), "join");
        GSEA_CUDA(cudaStreamWaitEvent(b->main, ev[1 + s], 0), "join");
    }
    for (size_t ci = 0; ci < b->classes.size(); ci++) {
        const auto it = b->es_tuning.find(b->classes[ci].wpl);
        const gsea::EsTuning tune = it == b->es_tuning.end() ? gsea::EsTuning() : it->second;
        GSEA_CUDA(launch_class<T>(b, ci, b->classes[ci].nitems, tune, b->main), "batched enrichment kernel");
    }
    GSEA_CUDA(cudaEventRecord(ev[ns + 1], b->main), "fork");
    for (size_t s = 0; s < ns; s++) GSEA_CUDA(cudaStreamWaitEvent(b->streams[s], ev[ns + 1], 0), "fork");
    for (int64_t i = 0; i < n; i++)
        if ((rc = gsea::plan_run_stats(b->plans[i], b->streams[i % ns]))) return rc;
    for (size_t s = 0; s < ns; s++) {
        GSEA_CUDA(cudaEventRecord(ev[ns + 2 + s], b->streams[s]), "join");
        GSEA_CUDA(cudaStreamWaitEvent(b->main, ev[ns + 2 + s], 0), "join");
    }
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
