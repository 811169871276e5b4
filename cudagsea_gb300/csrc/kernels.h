// kernels.h -- host-side launchers of the libgsea103 kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace gsea {

// Label permutation: masks[p][w] bit s == 1 <=> permuted label of sample s is
// 0 (class A) for global permutation perm_offset + p.
cudaError_t launch_permute(const uint8_t* labels, int S, int64_t num_perms, int64_t perm_offset,
                           uint32_t seed, uint32_t* masks, int words, cudaStream_t st);

// Plain-form class statistics + metric: keys[p][g] for p < num_perms.
// fast_ok (device int, may be null): set by launch_finite_check; non-zero lets
// the fp32 kernels use the packed form (bit-identical for finite inputs).
template <class T>
cudaError_t launch_metric(int metric, const T* exprs, int G, int S, const uint32_t* masks,
                          int words, int num_perms, int64_t nA, int64_t nB, T* keys,
                          const int* fast_ok, cudaStream_t st, int pb = 0);
// (pb: permutations per thread of the packed fp32 form, 4 or 8; 0 = 8)

// Batched instances: one launch of the metric over every instance of a group
// (blockIdx.z = instance), keys bit-identical to launch_metric's.  Instances
// share a group when metric_multi_key agrees (metric, and the path -- exact or
// packed with pb permutations per thread -- that launch_metric takes; fast_ok:
// the instance has a finite-check flag).  At most 65,535 instances and
// 524,280 permutations per instance.
template <class T>
struct MetricTask {
    const T* X;
    const uint32_t* masks;
    T* keys;
    const int* fast_ok;
    int G, S, words, num_perms;
    T nA, nB;
};
template <class T>
int metric_multi_key(int metric, int S, int words, bool fast_ok, int pb);
template <class T>
cudaError_t launch_metric_multi(int key, const MetricTask<T>* d_tasks, const MetricTask<T>* h_tasks, int n,
                                cudaStream_t st);

// fast_ok = 1 if every expression value is finite with |x| < 2^60, else 0
template <class T>
cudaError_t launch_finite_check(const T* exprs, int64_t n, int* fast_ok, cudaStream_t st);

// Per-permutation stable sort of keys (descending unless ascending):
//   ranks[p][g]   position of gene g (uint16 when G <= 65536, else uint32)
//   sorted[p][r]  |key| of the gene at position r
//   order[p][r]   gene at position r (optional, may be null)
struct SortBuffers {
    void* ranks;          // uint16_t* or uint32_t*
    bool ranks16;
    void* sorted_abs;     // T*
    uint32_t* order;      // optional
    void* scratch;        // per-CTA ping-pong buffers for the tiled variant
    size_t scratch_bytes;
    int variant = 0;      // 0 automatic, 1 register radix sort (fp32, G <= 40,960; two-CTA clusters above 20,480), 2 tiled
    int* error_flag = nullptr;  // set to 1 when a bounded wait of the tiled sort expires
};
template <class T>
size_t sort_scratch_bytes(int G, int num_perms);
template <class T>
cudaError_t launch_sort(const T* keys, int G, int num_perms, bool ascending, const SortBuffers& out,
                        cudaStream_t st);

// Enrichment scores es[k][perm_col0 + p] (row stride es_stride) from ranks and
// sorted |keys| of num_perms permutations.
// set_order (optional) lists the sets in the order warps should take them
// (largest first balances the warps of a CTA).
// decay (G+1 entries, from launch_decay_table) holds the miss step per hit count.
// ES launch configuration: warps per CTA (8, 16, 32; 0 = the most that fit)
// and whether a CTA stages its permutation's ranks and weights in shared
// memory (1), reads them from L2 (0) or takes the first that fits (-1).
// Every configuration gives identical scores.
struct EsTuning {
    int warps = 0;
    int stage = -1;
};
template <class T>
cudaError_t launch_es(const void* ranks, bool ranks16, const T* sorted_abs, int G, int num_perms,
                      const int64_t* set_offsets, const int32_t* set_genes, const int32_t* set_order,
                      const T* decay, int K, T* es, int64_t es_stride, int64_t perm_col0, cudaStream_t st,
                      EsTuning tune = EsTuning(), const int* K_dev = nullptr);
// (K_dev: when not null, the number of sets is min(K, *K_dev), read on the
// device -- a set list whose length a kernel decided)
template <class T>
cudaError_t launch_decay_table(int G, T* decay, cudaStream_t st);

// One instance of a multi-instance ES launch: scores es[k][col0 + p] (row
// stride `stride`) of its P permutations from ranks (uint16, G <= 65536) and
// sorted |keys|.
template <class T>
struct EsTask {
    const void* ranks;
    const T* sorted;
    const int64_t* off;
    const int32_t* genes;
    const int32_t* order;
    const T* decay;
    T* es;
    int64_t col0;
    int64_t stride;
    int G;
    int K;
};
// bitmap words per lane of the register procedure for G (0: general procedure)
int es_size_class(int G);
// Persistent ES over every (task, permutation) item of one size class (all
// tasks with es_size_class(G) == wpl, G <= Gmax), items taken from *counter
// (zeroed here); tasks and item_end (inclusive item prefix) in device memory.
template <class T>
cudaError_t launch_es_batch(const EsTask<T>* tasks, const int64_t* item_end, int ntasks, int64_t nitems,
                            unsigned long long* counter, int Gmax, int wpl, EsTuning tune, cudaStream_t st);

// Final statistics (ES, NES, NP, FWER, FDR) from es[K][P]; scratch sized by
// stats_scratch_bytes.
template <class T>
size_t stats_scratch_bytes(int K, int64_t P);
template <class T>
cudaError_t launch_stats(const T* es, int K, int64_t P, T* stats, void* scratch, cudaStream_t st);
// Ragged form: row k of es (stride ld) holds counts[k] scores (device array;
// null means ld for every set); FWER over the first p_fwer columns.  Scratch
// of stats_scratch_bytes<T>(K, ld) suffices.
// hist_cols > 0: the FDR null histogram uses each set's first
// min(n_k, hist_cols) columns only (an estimate of the same pooled null)
template <class T>
cudaError_t launch_stats_ragged(const T* es, int K, int64_t ld, const int64_t* counts, int64_t p_fwer, T* stats,
                                void* scratch, cudaStream_t st, int64_t hist_cols = 0);

// Sorts of many instances at once (batched form): all instances of one
// register-resident class (sort_multi_class of their G and precision; 0: the
// class has no multi form, the instance takes its solo launch_sort), one
// launch, blockIdx.z = instance; ranks (16-bit), weights and order those of
// the solo sort.
struct SortTask {
    const void* keys;   // [P][G] T
    void* ranks;        // [P][G] uint16
    void* sorted;       // [P][G] T
    uint32_t* order;    // [P][G] or null
    int G;
    int num_perms;
    int descending;
};
int sort_multi_class(int G, bool fp64);
cudaError_t launch_sort_multi(const SortTask* d_tasks, int n, int cls, bool fp64, cudaStream_t st);

// Label permutations of many instances at once (batched form), blockIdx.z =
// instance; each instance's masks those of its solo launch_permute.
struct PermTask {
    const uint8_t* labels;
    uint32_t* masks;
    int64_t perm_offset;
    int64_t num_perms;
    uint32_t seed;
    int S;
    int words;
};
cudaError_t launch_permute_multi(const PermTask* d_tasks, const PermTask* h_tasks, int n, cudaStream_t st);

// Statistics of many instances at once (batched form): one launch per step
// over all instances (blockIdx.z = instance), each instance's results those
// of its solo launch_stats bit for bit.  Dense form only: every instance has
// P >= 2 columns and rows = stats_multi_rows<T>(K, P) > 0 (its FDR
// histogram fits shared memory).
template <class T>
struct StatsTask {
    const T* es;    // [K][P]
    T* stats;       // [5][K]
    void* scratch;  // stats_scratch_bytes<T>(K, P)
    int K;
    int rows;       // stats_multi_rows<T>(K, P)
    int64_t P;
};
template <class T>
int stats_multi_rows(int K, int64_t P);
template <class T>
cudaError_t launch_stats_multi(const StatsTask<T>* d_tasks, const StatsTask<T>* h_tasks, int n, cudaStream_t st);

// Chosen form (tcgen05 class statistics, fp32 inputs).  Operand buffers:
// A1/A2 chosen_a_bytes(G, S) each, B chosen_b_bytes(P_batch, S).
int chosen_chunks(int S);
size_t chosen_a_bytes(int G, int S);
size_t chosen_b_bytes(int P, int S);
// once per upload: gene means / centred totals and the split operands
template <class T>
cudaError_t launch_chosen_prepare(const T* X, int G, int S, float* mu, double* t1, double* t2,
                                  unsigned char* A1, unsigned char* A2, cudaStream_t st);
// per permutation batch: label operand + GEMM + metric epilogue -> keys[p][g];
// error_flag is set if a bounded wait expired
cudaError_t launch_chosen_metric(int metric, bool fp64_variance, const uint32_t* masks, int words, int G, int S,
                                 int num_perms, int64_t nA, int64_t nB, const float* mu, const double* t1,
                                 const double* t2, const unsigned char* A1, const unsigned char* A2,
                                 unsigned char* Bm, float* keys, int* error_flag, cudaStream_t st,
                                 int tile_n = 0);
// (tile_n: permutations per tensor-core tile, 128 or 256; 0 = 256.  The B
// buffer of chosen_b_bytes fits either.)
// metric id -> its combiner family (the class statistics kernel's template)
int chosen_comb(int metric);
// Many instances at once (batched form): one launch each of the B clearing,
// the label operand and the tensor-core class statistics (128-permutation
// tiles) over every instance, blockIdx.z = instance; all tasks of one call
// share `comb`.  Keys identical to the solo launch_chosen_metric's.
struct ChosenTask {
    const unsigned char* A1;
    const unsigned char* A2;
    unsigned char* Bm;
    const float* mu;
    const double* t1;
    const double* t2;
    float* keys;
    const uint32_t* masks;
    int* error_flag;
    float nA, nB;
    int G, S, num_perms, chunks, words, comb;
};
cudaError_t launch_chosen_metric_multi(const ChosenTask* d_tasks, const ChosenTask* h_tasks, int n,
                                       bool fp64_variance, cudaStream_t st);

// mean, standard deviation and skewness (biased, in double) of keys[0..G)
template <class T>
cudaError_t launch_moments(const T* keys, int G, double* moments, cudaStream_t st);

// Learned-allocator helpers (k_adaptive.cu)
template <class T>
cudaError_t launch_set_means(const T* es, int64_t ld, int64_t P, int K, double* means, cudaStream_t st);
int model_max_queries();
template <class T>
cudaError_t launch_model_samples(const T* es, int64_t ld, int64_t P, const int64_t* off, int K, const double* mom,
                                 const double* means, int queries, const int64_t* slot, float* x, float* t,
                                 float* xv, float* tv, cudaStream_t st);
template <class T>
cudaError_t launch_model_features(const T* es, int64_t ld, const int64_t* off, int K, const double* mom,
                                  const double* sumabs, int64_t n, float* x, cudaStream_t st);
// sumabs: [2K], sum of |S| then sum of S^2 per set
// (n_dev: when not null, the list holds min(n_list, *n_dev) sets, read on the device)
template <class T>
cudaError_t launch_exceed(const T* es, int64_t ld, int K, const int32_t* list, int n_list, int64_t lo, int64_t hi,
                          unsigned long long* exceed, double* sumabs, cudaStream_t st, const int* n_dev = nullptr);
// after launch_stats_ragged with the same (K, p_fwer, scratch): a lower bound
// of every set's FDR q with its NES pushed z standard errors outward
template <class T>
cudaError_t launch_fdr_bound(int K, int64_t p_fwer, const T* stats, const int64_t* counts, const double* sums,
                             double z, const void* scratch, float* qlow, cudaStream_t st, float* qhigh = nullptr);
// (qhigh, may be null: an upper bound of every set's q with its NES pulled z
// standard errors inward)

// The adaptive test's decisions on the device (k_adaptive.cu): the pilot's
// p threshold and model fallback test, the stopping rule per round, the list
// of sets still running.  Counters for the report.
struct AdaptiveCtl {
    double stop_p;                    // p threshold of the stopping rule
    int n_active;                     // sets still running (length of the active list)
    int model_used;                   // 1: the model's prior enters the rule
    unsigned long long stopped_pilot;  // sets stopped after the pilot
    unsigned long long stopped_q;      // sets stopped by the FDR bound, any round
    unsigned long long stopped_sig;    // sets stopped as clearly significant, any round
    double p_sig;                      // p threshold of the significance rule (0: off)
    unsigned long long prior_sets;     // sets with a usable model prior
    unsigned long long prior_agreed;   // of those, pilots within z sd of the prior predictive
    unsigned long long rounds;         // rounds run, the pilot included
    unsigned long long valid;          // sets whose model error is defined
    unsigned long long within_tol;     // of those, error <= the fallback tolerance
};
struct AdaptiveRule {  // the rule's constants
    double q_call, margin, p_floor, z, q_stop, tol, cap, s2;  // s2: sigma_tail^2 of the model
    double sig_margin;  // significance rule: q_high <= q_call / sig_margin, p_high <= p_sig (0: off)
    int64_t P, P0;
};
// pilot: stop_p = min(1, max(p_floor, margin * max{NP_k : FDR_k < q_call}))
// and the model fallback test (pred may be null: no model)
template <class T>
cudaError_t launch_adaptive_prepare(int K, const T* stats, const float* pred, const double* sumabs,
                                    const AdaptiveRule& rule, double* err, AdaptiveCtl* ctl, cudaStream_t st);
// the stopping rule over the sets of `list` (n_dev entries; list null: all K
// sets), optionally the FDR bound (qlow); pilot != 0 also counts the prior's
// agreement and the sets stopped after the pilot
cudaError_t launch_adaptive_decide(int K, const int32_t* list, const int* n_dev, const int64_t* counts,
                                   const unsigned long long* exceed, const float* pred, const float* qlow,
                                   const float* qhigh, bool bound_on, bool pilot, const AdaptiveRule& rule,
                                   uint8_t* stop, AdaptiveCtl* ctl, cudaStream_t st);
// active list (ctl->n_active) = sets of `order` not stopped, in that order
cudaError_t launch_adaptive_compact(int K, const int32_t* order, const uint8_t* stop, int32_t* active,
                                    AdaptiveCtl* ctl, cudaStream_t st);
// counts[active[i]] = next for the active sets; counts the round if any ran
cudaError_t launch_adaptive_counts(int K, const int32_t* active, AdaptiveCtl* ctl, int64_t next,
                                   int64_t* counts, cudaStream_t st);
// counts[k] = v for every set, and the decision record cleared (rounds = 1)
cudaError_t launch_adaptive_reset(int K, int64_t v, int64_t* counts, AdaptiveCtl* ctl, cudaStream_t st);

// number of kernel launches issued by the launchers above since the last reset
int64_t launches_take();
void launches_add(int64_t n);

}  // namespace gsea
