// shard_stats.cu -- the final statistics of a permutation run split over
// ranks, merged from O(K) partial results instead of the K x P matrix.
//
// final_statistics (src/include/statistics.cuh:46-117) needs, per set, the
// sequential sum of |S| over all P permutations, the observed score (column
// 0) and counts over every permutation.  A rank holding permutations
// [first, first + count):
//   gsea_shard_sum      continues the sequential sum of |S| from the value the
//                       previous rank handed on (so the chain over ranks adds
//                       in exactly the single run's order: bit-identical);
//   gsea_shard_head     fac = P / sum, NES = ES * fac (once the chain is done);
//   gsea_shard_partial  its NP counts, FWER counts (per-permutation extrema of
//                       its columns) and FDR null histogram (its null scores
//                       binned against the sorted observed NES);
//   gsea_shard_finish   ES, NES, NP, FWER, FDR from the summed counts and
//                       histograms.
// Counts and histogram bins are integers (weights 1.0 in double), so their
// sums over ranks are exact and the merged statistics are bit-identical to a
// single run's.
#include "common.cuh"
#include "kernels.h"
#include "plan.h"

namespace gsea {
namespace {

// warp per set: s = init[k] (or 0) + sum_p |es[k][p]| in column order, in T
template <class T>
__global__ void shard_sum_kernel(const T* __restrict__ es, int K, int64_t count, int64_t ld,
                                 const T* __restrict__ init, T* __restrict__ out) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= K) return;
    const T* row = es + (int64_t)k * ld;
    T sum = init ? init[k] : T(0);
    for (int64_t p0 = 0; p0 < count; p0 += 32) {
        const int64_t p = p0 + lane;
        const T av = p < count ? fabs(row[p]) : T(0);
        const int n = (int)(count - p0 < 32 ? count - p0 : 32);
        for (int i = 0; i < n; i++) sum = Exact<T>::add(sum, __shfl_sync(kFullMask, av, i));
    }
    if (lane == 0) out[k] = sum;
}

// head = [ES (K), NES (K), fac (K)]
template <class T>
__global__ void shard_head_kernel(const T* __restrict__ es_obs, const T* __restrict__ sum, int K, int64_t P,
                                  T* __restrict__ head) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const T f = Exact<T>::div((T)P, sum[k]);
    head[k] = es_obs[k];
    head[K + k] = Exact<T>::mul(es_obs[k], f);
    head[2 * K + k] = f;
}

// warp per set: NP count over the local columns
template <class T>
__global__ void shard_np_kernel(const T* __restrict__ es, int K, int64_t count, int64_t ld, const T* __restrict__ head,
                                unsigned long long* __restrict__ np) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= K) return;
    const T a0 = fabs(head[k]);
    unsigned long long c = 0;
    for (int64_t p = lane; p < count; p += 32) c += fabs(es[(int64_t)k * ld + p]) >= a0;
    for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(kFullMask, c, o);
    if (lane == 0) np[k] = c;
}

// per local column: the extrema of S * fac over the sets (NaN skipped), as
// order-preserving radix images (the same rule as the single run)
template <class T>
__global__ void shard_extrema_kernel(const T* __restrict__ es, int K, int64_t count, int64_t ld,
                                     const T* __restrict__ fac, typename RadixKey<T>::U* __restrict__ mx,
                                     typename RadixKey<T>::U* __restrict__ mn) {
    using U = typename RadixKey<T>::U;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    T hi = -INFINITY, lo = INFINITY;
    for (int k = 0; k < K; k++) {
        const T v = Exact<T>::mul(es[(int64_t)k * ld + p], fac[k]);
        hi = hi < v ? v : hi;
        lo = lo > v ? v : lo;
    }
    mx[p] = (U)RadixKey<T>::from(hi, false);
    mn[p] = (U)RadixKey<T>::from(lo, false);
}

template <class T>
__device__ __forceinline__ T radix_val(typename RadixKey<T>::U u);
template <>
__device__ __forceinline__ float radix_val<float>(uint32_t u) {
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(u);
}
template <>
__device__ __forceinline__ double radix_val<double>(unsigned long long u) {
    u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)u);
}

// warp per set: FWER count over the local columns
template <class T>
__global__ void shard_fwer_kernel(int K, int64_t count, const typename RadixKey<T>::U* __restrict__ mx,
                                  const typename RadixKey<T>::U* __restrict__ mn, const T* __restrict__ head,
                                  unsigned long long* __restrict__ fw) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= K) return;
    const T score = head[K + k];
    unsigned long long c = 0;
    if (score > T(0)) {
        for (int64_t p = lane; p < count; p += 32) c += radix_val<T>(mx[p]) >= score;
    } else {
        for (int64_t p = lane; p < count; p += 32) c += radix_val<T>(mn[p]) <= score;
    }
    for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(kFullMask, c, o);
    if (lane == 0) fw[k] = c;
}

// warp per set: position of its NES among the same-side observed keys and
// the sorted key arrays (the single run's stats_fdr_obs rule)
template <class T>
__global__ void shard_obs_kernel(int K, const T* __restrict__ head, unsigned long long* __restrict__ cnt_obs,
                                 unsigned long long* __restrict__ lcount, T* __restrict__ sorted_pos,
                                 T* __restrict__ sorted_neg, unsigned long long* __restrict__ side_tot) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= K) return;
    const T* nes = head + K;
    const T s = nes[k];
    for (int side = 0; side < 2; side++) {
        const bool in = side == 0 ? (s >= T(0)) : (s <= T(0));
        if (!in) continue;
        const T key = side == 0 ? s : -s;
        unsigned long long less = 0, eq_before = 0;
        for (int j = lane; j < K; j += 32) {
            const T o = nes[j];
            const bool jin = side == 0 ? (o >= T(0)) : (o <= T(0));
            if (!jin) continue;
            const T oj = side == 0 ? o : -o;
            less += oj < key;
            eq_before += (oj == key) && (j < k);
        }
        for (int o = 16; o >= 1; o >>= 1) {
            less += __shfl_xor_sync(kFullMask, less, o);
            eq_before += __shfl_xor_sync(kFullMask, eq_before, o);
        }
        if (lane == 0) {
            (side == 0 ? sorted_pos : sorted_neg)[less + eq_before] = key;
            atomicAdd(&side_tot[side], 1ull);
            const int sd = s > T(0) ? 0 : 1;
            if (sd == side) lcount[k] = less;
        }
    }
    const int sd = s > T(0) ? 0 : (s <= T(0) ? 1 : -1);
    if (sd >= 0) {
        const T key = sd == 0 ? s : -s;
        unsigned long long ge = 0;
        for (int j = lane; j < K; j += 32) {
            const T o = nes[j];
            const bool jin = sd == 0 ? (o >= T(0)) : (o <= T(0));
            ge += jin && ((sd == 0 ? o : -o) >= key);
        }
        for (int o = 16; o >= 1; o >>= 1) ge += __shfl_xor_sync(kFullMask, ge, o);
        if (lane == 0) cnt_obs[k] = ge;
    }
}

template <class T>
__device__ __forceinline__ unsigned ub(const T* a, unsigned n, T v) {
    unsigned lo = 0, hi = n;
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// block per set: its null scores (global permutation index >= 1) binned
// against the sorted observed keys; hist = [hpos K+2 | hneg K+2 | null pos, null neg]
template <class T>
__global__ void shard_hist_kernel(const T* __restrict__ es, int K, int64_t count, int64_t ld, int64_t c0,
                                  const T* __restrict__ head, const T* __restrict__ sorted_pos,
                                  const T* __restrict__ sorted_neg, const unsigned long long* __restrict__ side_tot,
                                  double* __restrict__ hist) {
    const int64_t k = blockIdx.x;
    const unsigned npos = (unsigned)side_tot[0], nneg = (unsigned)side_tot[1];
    const T f = head[2 * K + k];
    double* hpos = hist;
    double* hneg = hist + (K + 2);
    double* tot = hist + 2 * (K + 2);
    double cpos = 0.0, cneg = 0.0;
    for (int64_t p = c0 + threadIdx.x; p < count; p += blockDim.x) {
        const T v = Exact<T>::mul(es[k * ld + p], f);
        if (v >= T(0)) {
            cpos += 1.0;
            atomicAdd(&hpos[ub(sorted_pos, npos, v)], 1.0);
        }
        if (v <= T(0)) {
            cneg += 1.0;
            atomicAdd(&hneg[ub(sorted_neg, nneg, -v)], 1.0);
        }
    }
    for (int o = 16; o >= 1; o >>= 1) {
        cpos += __shfl_xor_sync(kFullMask, cpos, o);
        cneg += __shfl_xor_sync(kFullMask, cneg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cpos != 0.0) atomicAdd(&tot[0], cpos);
        if (cneg != 0.0) atomicAdd(&tot[1], cneg);
    }
}

// suffix sums of the two histograms (one block each), in place
__global__ void shard_suffix_kernel(double* __restrict__ hist, int K, const unsigned long long* __restrict__ side_tot) {
    double* h = hist + (size_t)blockIdx.x * (K + 2);
    const unsigned n = (unsigned)side_tot[blockIdx.x] + 1;
    if (threadIdx.x == 0) {
        double run = 0.0;
        for (int64_t i = (int64_t)n - 1; i >= 0; i--) {
            run += h[i];
            h[i] = run;
        }
    }
}

template <class T>
__global__ void shard_final_kernel(int K, int64_t P, const T* __restrict__ head,
                                   const unsigned long long* __restrict__ counts, const double* __restrict__ hist,
                                   const unsigned long long* __restrict__ cnt_obs,
                                   const unsigned long long* __restrict__ lcount,
                                   const unsigned long long* __restrict__ side_tot, T* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const T s = head[K + k];
    out[k] = head[k];
    out[K + k] = s;
    out[2 * K + k] = Exact<T>::div((T)counts[k], (T)P);
    out[3 * K + k] = Exact<T>::div((T)counts[K + k], (T)P);
    T q;
    if (!(s == s)) {
        q = s;
    } else {
        const bool up = s > T(0);
        const unsigned long long L = lcount[k];
        const unsigned long long m = up ? side_tot[0] : side_tot[1];
        const double* S = hist + (up ? 0 : (K + 2));
        const double c_null = L + 1 <= m ? S[L + 1] : 0.0;
        const double null_side = hist[2 * (K + 2) + (up ? 0 : 1)];
        const double fn = null_side > 0 ? c_null / null_side : 0.0;
        const double fo = (double)cnt_obs[k] / (double)m;
        const double r = fn / fo;
        q = (T)(r < 1.0 ? r : 1.0);
    }
    out[4 * K + k] = q;
}

struct Scratch {
    void* p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

template <class T>
int partial_t(const T* es, int K, int64_t count, int64_t ld, int64_t first, const T* head,
              unsigned long long* counts, double* hist, cudaStream_t st) {
    using U = typename RadixKey<T>::U;
    const size_t bytes = sizeof(U) * 2 * (size_t)(count > 0 ? count : 1) + sizeof(T) * 2 * (size_t)K +
                         sizeof(unsigned long long) * (2 * (size_t)K + 2) + 64;
    Scratch s;
    GSEA_CUDA(cudaMalloc(&s.p, bytes), "shard scratch");
    U* mx = static_cast<U*>(s.p);
    U* mn = mx + (count > 0 ? count : 1);
    T* sorted_pos = reinterpret_cast<T*>(mn + (count > 0 ? count : 1));
    T* sorted_neg = sorted_pos + K;
    unsigned long long* cnt_obs = reinterpret_cast<unsigned long long*>(sorted_neg + K);
    unsigned long long* lcount = cnt_obs + K;
    unsigned long long* side_tot = lcount + K;
    GSEA_CUDA(cudaMemsetAsync(side_tot, 0, 2 * sizeof(unsigned long long), st), "clear");
    GSEA_CUDA(cudaMemsetAsync(hist, 0, sizeof(double) * (2 * ((size_t)K + 2) + 2), st), "clear");
    const int wpb = 8;
    shard_np_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(es, K, count, ld, head, counts);
    if (count > 0) {
        shard_extrema_kernel<T><<<(unsigned)((count + 127) / 128), 128, 0, st>>>(es, K, count, ld, head + 2 * K, mx,
                                                                                 mn);
        shard_fwer_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(K, count, mx, mn, head, counts + K);
    } else {
        GSEA_CUDA(cudaMemsetAsync(counts + K, 0, sizeof(unsigned long long) * K, st), "clear");
    }
    shard_obs_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(K, head, cnt_obs, lcount, sorted_pos, sorted_neg,
                                                                  side_tot);
    const int64_t c0 = first == 0 ? 1 : 0;  // global permutation 0 is observed, not null
    if (count > c0)
        shard_hist_kernel<T><<<K, 256, 0, st>>>(es, K, count, ld, c0, head, sorted_pos, sorted_neg, side_tot, hist);
    GSEA_CUDA(cudaGetLastError(), "shard partial kernels");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");  // the scratch is freed on return
    launches_add(5);
    return GSEA_OK;
}

template <class T>
int finish_t(const T* head, int K, int64_t P, const unsigned long long* counts, double* hist, T* stats,
             cudaStream_t st) {
    const size_t bytes = sizeof(T) * 2 * (size_t)K + sizeof(unsigned long long) * (2 * (size_t)K + 2) + 64;
    Scratch s;
    GSEA_CUDA(cudaMalloc(&s.p, bytes), "shard scratch");
    T* sorted_pos = static_cast<T*>(s.p);
    T* sorted_neg = sorted_pos + K;
    unsigned long long* cnt_obs = reinterpret_cast<unsigned long long*>(sorted_neg + K);
    unsigned long long* lcount = cnt_obs + K;
    unsigned long long* side_tot = lcount + K;
    GSEA_CUDA(cudaMemsetAsync(side_tot, 0, 2 * sizeof(unsigned long long), st), "clear");
    const int wpb = 8;
    shard_obs_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(K, head, cnt_obs, lcount, sorted_pos, sorted_neg,
                                                                  side_tot);
    shard_suffix_kernel<<<2, 32, 0, st>>>(hist, K, side_tot);
    shard_final_kernel<T><<<(K + 255) / 256, 256, 0, st>>>(K, P, head, counts, hist, cnt_obs, lcount, side_tot, stats);
    GSEA_CUDA(cudaGetLastError(), "shard finish kernels");
    GSEA_CUDA(cudaStreamSynchronize(st), "stream sync");
    launches_add(3);
    return GSEA_OK;
}

}  // namespace
}  // namespace gsea

using gsea::fail;

extern "C" {

int gsea_shard_sum(const void* es, int64_t K, int64_t count, int64_t ld, int precision, const void* init, void* sum,
                   void* stream) {
    if (!es || !sum || K < 1 || K > INT32_MAX || count < 0 || ld < count || (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int wpb = 8;
    if (precision == 64)
        gsea::shard_sum_kernel<double><<<(unsigned)((K + wpb - 1) / wpb), wpb * 32, 0, st>>>(
            static_cast<const double*>(es), (int)K, count, ld, static_cast<const double*>(init),
            static_cast<double*>(sum));
    else
        gsea::shard_sum_kernel<float><<<(unsigned)((K + wpb - 1) / wpb), wpb * 32, 0, st>>>(
            static_cast<const float*>(es), (int)K, count, ld, static_cast<const float*>(init),
            static_cast<float*>(sum));
    GSEA_CUDA(cudaGetLastError(), "shard sum kernel");
    gsea::launches_add(1);
    return GSEA_OK;
}

int gsea_shard_head(const void* es_obs, const void* sum, int64_t K, int64_t num_perms, int precision, void* head,
                    void* stream) {
    if (!es_obs || !sum || !head || K < 1 || K > INT32_MAX || num_perms < 1 || (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((K + 255) / 256);
    if (precision == 64)
        gsea::shard_head_kernel<double><<<blocks, 256, 0, st>>>(static_cast<const double*>(es_obs),
                                                                static_cast<const double*>(sum), (int)K, num_perms,
                                                                static_cast<double*>(head));
    else
        gsea::shard_head_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(es_obs),
                                                               static_cast<const float*>(sum), (int)K, num_perms,
                                                               static_cast<float*>(head));
    GSEA_CUDA(cudaGetLastError(), "shard head kernel");
    gsea::launches_add(1);
    return GSEA_OK;
}

int gsea_shard_partial(const void* es, int64_t K, int64_t count, int64_t ld, int precision, int64_t first_perm,
                       const void* head, uint64_t* counts, double* hist, void* stream) {
    if (!es || !head || !counts || !hist || K < 1 || K > INT32_MAX || count < 0 || ld < count || first_perm < 0 ||
        (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto* c = reinterpret_cast<unsigned long long*>(counts);
    return precision == 64 ? gsea::partial_t<double>(static_cast<const double*>(es), (int)K, count, ld, first_perm,
                                                      static_cast<const double*>(head), c, hist, st)
                           : gsea::partial_t<float>(static_cast<const float*>(es), (int)K, count, ld, first_perm,
                                                     static_cast<const float*>(head), c, hist, st);
}

int gsea_shard_finish(const void* head, int64_t K, int64_t num_perms, int precision, const uint64_t* counts,
                      double* hist, void* stats, void* stream) {
    if (!head || !counts || !hist || !stats || K < 1 || K > INT32_MAX || num_perms < 1 ||
        (precision != 32 && precision != 64))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto* c = reinterpret_cast<const unsigned long long*>(counts);
    return precision == 64 ? gsea::finish_t<double>(static_cast<const double*>(head), (int)K, num_perms, c, hist,
                                                     static_cast<double*>(stats), st)
                           : gsea::finish_t<float>(static_cast<const float*>(head), (int)K, num_perms, c, hist,
                                                    static_cast<float*>(stats), st);
}

}  // extern "C"
