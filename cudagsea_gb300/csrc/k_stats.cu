// k_stats.cu -- NES, nominal p, FWER and FDR on the device.
//
// final_statistics (src/include/statistics.cuh:46-117) runs on the host in
// the reference, in the enrichment precision T.  The same arithmetic runs here
// on the GPU:
//   ES_k    = S[k][0]
//   fac_k   = (T)P / sum_p |S[k][p]|        (sequential sum over p, in T,
//                                            statistics.cuh:60-70)
//   NES_k   = ES_k * fac_k
//   NP_k    = #{p : |S[k][p]| >= |ES_k|} / P          (statistics.cuh:72-77)
//   max_p   = max_k S[k][p]*fac_k, min_p likewise     (statistics.cuh:84-97)
//   FWER_k  = #{p : max_p >= NES_k} / P  if NES_k > 0,
//             #{p : min_p <= NES_k} / P  otherwise    (statistics.cuh:99-110)
// so the results are bit-identical to the reference's for identical ES.
//
// FDR (statistics.cuh:112-114 leaves NaN): q-value of the normalised score
// against the null of permutations 1..P-1 of all sets, per sign side:
//   NES* > 0: q = [#{null >= NES*} / #{null >= 0}] / [#{obs >= NES*} / #{obs >= 0}]
//   NES* <= 0: mirrored with <=, capped at 1.
//
// Ragged form (adaptive permutation allocation): set k holds n_k scores in
// row k of a matrix with row stride ld.  fac, NES and NP use the set's own
// n_k columns; FWER uses the first p_fwer columns (those every set has);
// in the FDR null every set carries the same total weight, each of its
// n_k - 1 null scores counting (ld - 1) / (n_k - 1).  With n_k = ld for all
// sets the weights are exactly 1 and the ragged form is the dense one.
#include <algorithm>
#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace {

struct StatsScratch {
    // fac[K] mx[P] mn[P] (T) | cnt_obs[K] lcount[K] (u64) | sorted_pos[K]
    // sorted_neg[K] (T) | hpos[K+2] hneg[K+2] (f64) | totals[8] (u64 / f64)
    static size_t bytes(int K, int64_t P, size_t tsize) {
        return tsize * ((size_t)3 * K + 2 * (size_t)P) + sizeof(unsigned long long) * (4 * (size_t)K + 12) + 64;
    }
};

// one warp per set: factor, NES, NP
template <class T>
__device__ __forceinline__ void stats_set_kernel_body(int bx, const T* __restrict__ es, int K, int64_t ld, const int64_t* __restrict__ counts,
                                 T* __restrict__ out, T* __restrict__ fac) {
    const int warp = (bx * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= K) return;
    const T* row = es + (int64_t)warp * ld;
    const int64_t P = counts ? counts[warp] : ld;
    const T es0 = row[0];
    T sum = T(0);
    unsigned long long np = 0;
    const T aes0 = fabs(es0);
    // blocks of 4 x 32 columns; the next block's loads are in flight while
    // this block is summed
    constexpr int kB = 4;
    T cur[kB];
#pragma unroll
    for (int j = 0; j < kB; j++) cur[j] = j * 32 + lane < P ? row[j * 32 + lane] : T(0);
    for (int64_t p0 = 0; p0 < P; p0 += kB * 32) {
        T nxt[kB];
#pragma unroll
        for (int j = 0; j < kB; j++) {
            const int64_t q = p0 + kB * 32 + j * 32 + lane;
            nxt[j] = q < P ? row[q] : T(0);
        }
#pragma unroll
        for (int j = 0; j < kB; j++) {
            const int64_t b = p0 + j * 32;
            if (b >= P) break;  // warp-uniform
            const T av = fabs(cur[j]);
            if (b + lane < P && av >= aes0) np++;
            const int n = (int)(P - b < 32 ? P - b : 32);
            // sequential sum in index order, as the reference's host loop
            for (int i = 0; i < n; i++) {
                const T x = __shfl_sync(kFullMask, av, i);
                sum = Exact<T>::add(sum, x);
            }
        }
#pragma unroll
        for (int j = 0; j < kB; j++) cur[j] = nxt[j];
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) np += __shfl_xor_sync(kFullMask, np, o);
    if (lane == 0) {
        const T f = Exact<T>::div((T)P, sum);
        fac[warp] = f;
        out[warp] = es0;
        out[K + warp] = Exact<T>::mul(es0, f);
        out[2 * K + warp] = Exact<T>::div((T)np, (T)P);
    }
}

// extrema of the normalised scores per permutation column.  Each thread folds
// a chunk of sets for one column and merges it with an atomic max / min on
// the order-preserving radix image of the value (NaN skipped, as the
// reference's `<` / `>` updates skip it).  Radix image 0 ("empty" for the
// max) and all-ones ("empty" for the min) belong only to NaN bit patterns.
constexpr int kExtremaSets = 16;
template <class T>
__device__ __forceinline__ void stats_extrema_kernel_body(int bx, int by, const T* __restrict__ es, int K, int64_t ld, int64_t P, const T* __restrict__ fac,
                                     typename RadixKey<T>::U* __restrict__ mx,
                                     typename RadixKey<T>::U* __restrict__ mn) {
    using U = typename RadixKey<T>::U;
    const int64_t p = (int64_t)bx * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int k0 = by * kExtremaSets, k1 = min(K, k0 + kExtremaSets);
    T hi = -INFINITY, lo = INFINITY;
    for (int k = k0; k < k1; k++) {
        const T v = Exact<T>::mul(es[(int64_t)k * ld + p], fac[k]);
        hi = hi < v ? v : hi;
        lo = lo > v ? v : lo;
    }
    atomicMax(&mx[p], (U)RadixKey<T>::from(hi, false));
    atomicMin(&mn[p], (U)RadixKey<T>::from(lo, false));
}

template <class T>
__device__ __forceinline__ T radix_value(typename RadixKey<T>::U u);
template <>
__device__ __forceinline__ float radix_value<float>(uint32_t u) {
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(u);
}
template <>
__device__ __forceinline__ double radix_value<double>(unsigned long long u) {
    u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)u);
}

// one warp per set: FWER
template <class T>
__device__ __forceinline__ void stats_fwer_kernel_body(int bx, int K, int64_t P, const typename RadixKey<T>::U* __restrict__ mx,
                                  const typename RadixKey<T>::U* __restrict__ mn, T* __restrict__ out) {
    const int warp = (bx * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= K) return;
    const T score = out[K + warp];
    unsigned long long c = 0;
    if (score > T(0)) {
        for (int64_t p = lane; p < P; p += 32) c += radix_value<T>(mx[p]) >= score;
    } else {
        for (int64_t p = lane; p < P; p += 32) c += radix_value<T>(mn[p]) <= score;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(kFullMask, c, o);
    if (lane == 0) out[3 * K + warp] = Exact<T>::div((T)c, (T)P);
}

// ---------------------------------------------------------------------------
// FDR counts, exact and O(K*P*log K).  Each side is handled as "key >= key*":
// positive side keys are the scores themselves (observed NES >= 0, null
// scores >= 0), negative side keys their negations (scores <= 0); a zero is on
// both sides, NaN on neither.
//   1. stats_fdr_obs_kernel: for every set, L = #{same-side observed keys <
//      its key} and the observed count #{>= key}; the observed keys are
//      scattered into ascending order at L + (#equal keys of lower index).
//   2. stats_fdr_hist_kernel: every null score is binary-searched into the
//      sorted observed keys of its side: t = #{observed keys <= it}, H[t]++.
//   3. stats_fdr_suffix_kernel: S[i] = sum_{t >= i} H[t].
//   4. stats_fdr_final_kernel: #{null keys >= key*} = S[L + 1] (a null key v
//      satisfies v >= key* exactly when t(v) >= L + 1).
// Layout of the FDR part of the scratch (unsigned long long):
//   cnt_obs[K] | L[K] | sorted_pos[K] (T) | sorted_neg[K] (T) |
//   H_pos[K+2] | H_neg[K+2] (double weights) | totals[8]: [2], [3] observed
//   counts per side (u64), [4], [5] null weight per side (double)

template <class T>
__device__ __forceinline__ int side_of(T s) { return s > T(0) ? 0 : (s <= T(0) ? 1 : -1); }

// one warp per set; the lanes stride over the other sets and the counts are
// warp-reduced
template <class T>
__device__ __forceinline__ void stats_fdr_obs_kernel_body(int bx, int K, const T* __restrict__ out, unsigned long long* __restrict__ cnt_obs,
                                     unsigned long long* __restrict__ lcount, T* __restrict__ sorted_pos,
                                     T* __restrict__ sorted_neg, unsigned long long* __restrict__ totals) {
    const int k = (bx * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= K) return;
    const T s = out[K + k];
    // membership in the two sorted arrays: o >= 0 (positive), o <= 0 (negative)
    for (int side = 0; side < 2; side++) {
        const bool in = side == 0 ? (s >= T(0)) : (s <= T(0));
        if (!in) continue;  // warp-uniform
        const T key = side == 0 ? s : -s;
        unsigned long long less = 0, eq_before = 0;
        for (int j = lane; j < K; j += 32) {
            const T o = out[K + j];
            const bool jin = side == 0 ? (o >= T(0)) : (o <= T(0));
            if (!jin) continue;
            const T oj = side == 0 ? o : -o;
            less += oj < key;
            eq_before += (oj == key) && (j < k);
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            less += __shfl_xor_sync(kFullMask, less, o);
            eq_before += __shfl_xor_sync(kFullMask, eq_before, o);
        }
        if (lane == 0) {
            (side == 0 ? sorted_pos : sorted_neg)[less + eq_before] = key;
            atomicAdd(&totals[2 + side], 1ull);
            // observed count on the set's own side: #{keys >= key} = m - less
            if (side_of(s) == side) lcount[k] = less;
        }
    }
    const int sd = side_of(s);
    if (sd >= 0) {
        const T key = sd == 0 ? s : -s;
        unsigned long long ge = 0;
        for (int j = lane; j < K; j += 32) {
            const T o = out[K + j];
            const bool jin = sd == 0 ? (o >= T(0)) : (o <= T(0));
            ge += jin && ((sd == 0 ? o : -o) >= key);
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) ge += __shfl_xor_sync(kFullMask, ge, o);
        if (lane == 0) cnt_obs[k] = ge;
    }
}

template <class T>
__device__ __forceinline__ unsigned upper_bound_t(const T* a, unsigned n, T v) {
    unsigned lo = 0, hi = n;
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

constexpr int kHistThreads = 256;
constexpr int kHistCols = kHistThreads * 8;  // null columns per block
// grid (sets, column chunks): block (b, c) bins the null scores of the sets
// b, b + gridDim.x, ... in the chunks c, c + gridDim.y, ... of kHistCols
// columns of each set's columns 1..m_k-1, m_k = min(n_k, hist_cols) (the
// adaptive test's intermediate rounds bin only the pilot columns: the same
// pooled null, each set's nulls weighted to equal total weight).  With
// stage_obs the sorted observed keys are copied to shared memory once per
// block (one resident block per SM with THREADS = 1024 when they need more
// than the default 48 KB).
template <class T, int THREADS>
__global__ void __launch_bounds__(THREADS)
stats_fdr_hist_kernel(const T* __restrict__ es, int K, int64_t ld, const int64_t* __restrict__ counts,
                      int64_t hist_cols, const T* __restrict__ fac, const T* sorted_pos, const T* sorted_neg,
                      double* __restrict__ hpos, double* __restrict__ hneg, unsigned long long* __restrict__ totals,
                      bool stage_obs) {
    extern __shared__ __align__(16) unsigned char hist_smem[];  // [2K] T when staged (dynamic size > 0)
    constexpr int kCols = THREADS * 8;
    const unsigned npos = (unsigned)totals[2], nneg = (unsigned)totals[3];
    if (stage_obs) {  // the binary searches then run in shared memory
        T* s_pos = reinterpret_cast<T*>(hist_smem);
        T* s_neg = s_pos + npos;
        for (unsigned i = threadIdx.x; i < npos; i += THREADS) s_pos[i] = sorted_pos[i];
        for (unsigned i = threadIdx.x; i < nneg; i += THREADS) s_neg[i] = sorted_neg[i];
        __syncthreads();
        sorted_pos = s_pos;
        sorted_neg = s_neg;
    }
    double* wtot = reinterpret_cast<double*>(totals + 4);
    double cpos = 0.0, cneg = 0.0;
    for (int64_t k = blockIdx.x; k < K; k += gridDim.x) {
        const int64_t n0 = counts ? counts[k] : ld;
        const int64_t n = n0 < hist_cols ? n0 : hist_cols;
        if (n < 2) continue;
        const double w = counts ? (double)(ld - 1) / (double)(n - 1) : 1.0;
        const T f = fac[k];
        const T* row = es + k * ld;
        for (int64_t c0 = 1 + (int64_t)blockIdx.y * kCols; c0 < n; c0 += (int64_t)gridDim.y * kCols) {
            const int64_t c1 = c0 + kCols < n ? c0 + kCols : n;
            for (int64_t p = c0 + threadIdx.x; p < c1; p += THREADS) {
                const T v = Exact<T>::mul(row[p], f);
                if (v >= T(0)) {
                    cpos += w;
                    atomicAdd(&hpos[upper_bound_t(sorted_pos, npos, v)], w);
                }
                if (v <= T(0)) {
                    cneg += w;
                    atomicAdd(&hneg[upper_bound_t(sorted_neg, nneg, -v)], w);
                }
            }
        }
    }
    for (int o = 16; o >= 1; o >>= 1) {
        cpos += __shfl_xor_sync(kFullMask, cpos, o);
        cneg += __shfl_xor_sync(kFullMask, cneg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cpos != 0.0) atomicAdd(&wtot[0], cpos);
        if (cneg != 0.0) atomicAdd(&wtot[1], cneg);
    }
}

// Dense form (every set has all ld columns, unit weights): block b bins an
// equal contiguous share of the K x (ld - 1) null scores (row-major, column
// 0 excluded) into shared-memory integer histograms of both sides, against
// the sorted observed keys staged beside them, and writes them as row b of
// `partial` (width 2(K+2) + 2: H_pos | H_neg | #null >= 0 | #null <= 0).
// stats_fdr_hist_sum_kernel adds the rows up column by column: exact integer
// counts, no global atomics, the same result in any order.
constexpr int kDenseHistThreads = 512;
constexpr size_t kDenseHistPartialBytes = size_t(1) << 20;
constexpr size_t kDenseHistSmemMax = 96 * 1024;
template <class T>
__device__ __forceinline__ void
stats_fdr_hist_dense_kernel_body(int bx, int gx, const T* __restrict__ es, int K, int64_t ld, const T* __restrict__ fac,
                            const T* __restrict__ sorted_pos, const T* __restrict__ sorted_neg,
                            const unsigned long long* __restrict__ totals, unsigned* __restrict__ partial) {
    extern __shared__ __align__(16) unsigned char dense_smem[];
    const int W = 2 * (K + 2) + 2;
    unsigned* h = reinterpret_cast<unsigned*>(dense_smem);  // W counters
    T* s_pos = reinterpret_cast<T*>(dense_smem + (((size_t)W * 4 + 15) & ~(size_t)15));
    const unsigned npos = (unsigned)totals[2], nneg = (unsigned)totals[3];
    T* s_neg = s_pos + npos;
    for (int i = threadIdx.x; i < W; i += kDenseHistThreads) h[i] = 0u;
    for (unsigned i = threadIdx.x; i < npos; i += kDenseHistThreads) s_pos[i] = sorted_pos[i];
    for (unsigned i = threadIdx.x; i < nneg; i += kDenseHistThreads) s_neg[i] = sorted_neg[i];
    __syncthreads();
    const int64_t cols = ld - 1;
    const int64_t total = (int64_t)K * cols;
    const int64_t lo = total * bx / gx, hi = total * (bx + 1) / gx;
    unsigned cpos = 0, cneg = 0;
    int64_t k = lo / cols;
    int64_t c = lo - k * cols;  // column - 1 within row k
    for (int64_t i = lo; i < hi;) {
        const int64_t run = (cols - c) < (hi - i) ? (cols - c) : (hi - i);  // rest of row k in the share
        const T f = fac[k];
        const T* row = es + k * ld + 1 + c;
        for (int64_t j = threadIdx.x; j < run; j += kDenseHistThreads) {
            const T v = Exact<T>::mul(row[j], f);
            if (v >= T(0)) {
                cpos++;
                atomicAdd(&h[upper_bound_t(s_pos, npos, v)], 1u);
            }
            if (v <= T(0)) {
                cneg++;
                atomicAdd(&h[(K + 2) + upper_bound_t(s_neg, nneg, -v)], 1u);
            }
        }
        i += run;
        k++;
        c = 0;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        cpos += __shfl_xor_sync(kFullMask, cpos, o);
        cneg += __shfl_xor_sync(kFullMask, cneg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cpos) atomicAdd(&h[W - 2], cpos);
        if (cneg) atomicAdd(&h[W - 1], cneg);
    }
    __syncthreads();
    unsigned* out = partial + (size_t)bx * W;
    for (int i = threadIdx.x; i < W; i += kDenseHistThreads) out[i] = h[i];
}

// column sums of the partial histograms: H_pos, H_neg (contiguous, 2(K+2)
// doubles) and the null counts per side (totals[4], [5] as doubles)
__device__ __forceinline__ void stats_fdr_hist_sum_kernel_body(int bx, const unsigned* __restrict__ partial, int rows, int K,
                                          double* __restrict__ hist, unsigned long long* __restrict__ totals) {
    const int W = 2 * (K + 2) + 2;
    const int j = bx * blockDim.x + threadIdx.x;
    if (j >= W) return;
    unsigned long long s = 0;
    for (int r = 0; r < rows; r++) s += partial[(size_t)r * W + j];
    if (j < W - 2) hist[j] = (double)s;
    else reinterpret_cast<double*>(totals + 4)[j - (W - 2)] = (double)s;
}

template <class T>
size_t dense_hist_smem(int K) {
    const size_t W = 2 * ((size_t)K + 2) + 2;
    return ((W * 4 + 15) & ~(size_t)15) + 2 * sizeof(T) * (size_t)K;
}
// rows of the partial histograms (0: the dense form does not apply)
template <class T>
int dense_hist_rows(int K, int sms) {
    if (dense_hist_smem<T>(K) > kDenseHistSmemMax) return 0;
    const size_t W = 2 * ((size_t)K + 2) + 2;
    const size_t cap = kDenseHistPartialBytes / (4 * W);
    const size_t want = 2 * (size_t)(sms > 0 ? sms : 1);
    return (int)(cap < want ? cap : want);
}

// in-place suffix sums of the two histograms (one block each)
__device__ __forceinline__ void stats_fdr_suffix_kernel_body(int bx, double* __restrict__ hpos, double* __restrict__ hneg,
                                        const unsigned long long* __restrict__ totals) {
    double* h = bx == 0 ? hpos : hneg;
    const unsigned n = (unsigned)totals[2 + bx] + 1;  // bins 0..m
    __shared__ double carry;
    __shared__ double wsum[32];
    if (threadIdx.x == 0) carry = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // walk from the top bin down in chunks of blockDim.x
    for (int64_t top = (int64_t)n - 1; top >= 0; top -= blockDim.x) {
        const int64_t i = top - threadIdx.x;
        double v = i >= 0 ? h[i] : 0.0;
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(kFullMask, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) wsum[warp] = v;
        __syncthreads();
        double before = carry;
        for (int w = 0; w < warp; w++) before += wsum[w];
        if (i >= 0) h[i] = v + before;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < nw; w++) t += wsum[w];
            carry += t;
        }
        __syncthreads();
    }
}

template <class T>
__device__ __forceinline__ void stats_fdr_final_kernel_body(int bx, int K, const unsigned long long* __restrict__ cnt_obs,
                                       const unsigned long long* __restrict__ lcount,
                                       const double* __restrict__ spos, const double* __restrict__ sneg,
                                       const unsigned long long* __restrict__ totals, T* __restrict__ out) {
    const int k = bx * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const T s = out[K + k];
    T q;
    if (!(s == s)) {
        q = s;
    } else {
        const bool up = s > T(0);
        const unsigned long long L = lcount[k];
        const unsigned long long m = up ? totals[2] : totals[3];
        const double* wtot = reinterpret_cast<const double*>(totals + 4);
        const double c_null = L + 1 <= m ? (up ? spos : sneg)[L + 1] : 0.0;
        const double null_side = up ? wtot[0] : wtot[1];
        const double obs_side = (double)m;
        const double fn = null_side > 0 ? c_null / null_side : 0.0;
        const double fo = (double)cnt_obs[k] / obs_side;
        const double r = fn / fo;
        q = (T)(r < 1.0 ? r : 1.0);
    }
    out[4 * K + k] = q;
}

// the statistics scratch of K sets with FWER over p_fwer columns
template <class T>
struct RaggedLayout {
    using U = typename RadixKey<T>::U;
    T* fac;
    U* mx;
    U* mn;
    unsigned long long* cnt_obs;
    unsigned long long* lcount;
    T* sorted_pos;
    T* sorted_neg;
    double* hpos;
    double* hneg;
    unsigned long long* totals;
    unsigned* partial;
    __host__ __device__ RaggedLayout(void* scratch, int K, int64_t p_fwer) {
        unsigned char* s = static_cast<unsigned char*>(scratch);
        auto align16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
        fac = reinterpret_cast<T*>(s);
        mx = reinterpret_cast<U*>(fac + K);
        mn = mx + p_fwer;
        size_t off = align16(sizeof(T) * ((size_t)K + 2 * (size_t)p_fwer));
        cnt_obs = reinterpret_cast<unsigned long long*>(s + off);
        lcount = cnt_obs + K;
        off = align16(off + sizeof(unsigned long long) * 2 * (size_t)K);
        sorted_pos = reinterpret_cast<T*>(s + off);
        sorted_neg = sorted_pos + K;
        off = align16(off + sizeof(T) * 2 * (size_t)K);
        hpos = reinterpret_cast<double*>(s + off);
        hneg = hpos + (K + 2);
        totals = reinterpret_cast<unsigned long long*>(hneg + (K + 2));
        partial = reinterpret_cast<unsigned*>(s + align16(off + sizeof(double) * (2 * ((size_t)K + 2) + 8)));
    }
};

// ---- the kernels of one statistics run (solo) --------------------------------
template <class T>
__global__ void stats_set_kernel(const T* __restrict__ es, int K, int64_t ld, const int64_t* __restrict__ counts,
                                 T* __restrict__ out, T* __restrict__ fac) {
    stats_set_kernel_body<T>(blockIdx.x, es, K, ld, counts, out, fac);
}
template <class T>
__global__ void stats_extrema_kernel(const T* __restrict__ es, int K, int64_t ld, int64_t P, const T* __restrict__ fac,
                                     typename RadixKey<T>::U* __restrict__ mx, typename RadixKey<T>::U* __restrict__ mn) {
    stats_extrema_kernel_body<T>(blockIdx.x, blockIdx.y, es, K, ld, P, fac, mx, mn);
}
template <class T>
__global__ void stats_fwer_kernel(int K, int64_t P, const typename RadixKey<T>::U* __restrict__ mx,
                                  const typename RadixKey<T>::U* __restrict__ mn, T* __restrict__ out) {
    stats_fwer_kernel_body<T>(blockIdx.x, K, P, mx, mn, out);
}
template <class T>
__global__ void stats_fdr_obs_kernel(int K, const T* __restrict__ out, unsigned long long* __restrict__ cnt_obs,
                                     unsigned long long* __restrict__ lcount, T* __restrict__ sorted_pos,
                                     T* __restrict__ sorted_neg, unsigned long long* __restrict__ totals) {
    stats_fdr_obs_kernel_body<T>(blockIdx.x, K, out, cnt_obs, lcount, sorted_pos, sorted_neg, totals);
}
template <class T>
__global__ void __launch_bounds__(kDenseHistThreads)
stats_fdr_hist_dense_kernel(const T* __restrict__ es, int K, int64_t ld, const T* __restrict__ fac,
                            const T* __restrict__ sorted_pos, const T* __restrict__ sorted_neg,
                            const unsigned long long* __restrict__ totals, unsigned* __restrict__ partial) {
    stats_fdr_hist_dense_kernel_body<T>(blockIdx.x, gridDim.x, es, K, ld, fac, sorted_pos, sorted_neg, totals, partial);
}
__global__ void stats_fdr_hist_sum_kernel(const unsigned* __restrict__ partial, int rows, int K,
                                          double* __restrict__ hist, unsigned long long* __restrict__ totals) {
    stats_fdr_hist_sum_kernel_body(blockIdx.x, partial, rows, K, hist, totals);
}
__global__ void stats_fdr_suffix_kernel(double* __restrict__ hpos, double* __restrict__ hneg,
                                        const unsigned long long* __restrict__ totals) {
    stats_fdr_suffix_kernel_body(blockIdx.x, hpos, hneg, totals);
}
template <class T>
__global__ void stats_fdr_final_kernel(int K, const unsigned long long* __restrict__ cnt_obs,
                                       const unsigned long long* __restrict__ lcount,
                                       const double* __restrict__ spos, const double* __restrict__ sneg,
                                       const unsigned long long* __restrict__ totals, T* __restrict__ out) {
    stats_fdr_final_kernel_body<T>(blockIdx.x, K, cnt_obs, lcount, spos, sneg, totals, out);
}

// ---- the same kernels over many instances at once ----------------------------
// blockIdx.z = the instance; every instance has all its columns (the dense
// form); grids are sized for the largest instance and the blocks beyond an
// instance's own extent return at once.  Each instance's results are those
// of its solo run bit for bit: the same bodies, the same block decomposition.
template <class T>
__global__ void stats_init_multi(const StatsTask<T>* __restrict__ tasks) {
    using U = typename RadixKey<T>::U;
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 2 * ((int64_t)t.K + 2) + 8) L.hpos[i] = 0.0;  // H_pos | H_neg | totals
    if (i < t.P) {
        L.mx[i] = U(0);
        L.mn[i] = ~U(0);
    }
}
template <class T>
__global__ void stats_set_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_set_kernel_body<T>(blockIdx.x, t.es, t.K, t.P, nullptr, t.stats, L.fac);
}
template <class T>
__global__ void stats_extrema_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_extrema_kernel_body<T>(blockIdx.x, blockIdx.y, t.es, t.K, t.P, t.P, L.fac, L.mx, L.mn);
}
template <class T>
__global__ void stats_fwer_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_fwer_kernel_body<T>(blockIdx.x, t.K, t.P, L.mx, L.mn, t.stats);
}
template <class T>
__global__ void stats_fdr_obs_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_fdr_obs_kernel_body<T>(blockIdx.x, t.K, t.stats, L.cnt_obs, L.lcount, L.sorted_pos, L.sorted_neg, L.totals);
}
template <class T>
__global__ void __launch_bounds__(kDenseHistThreads) stats_fdr_hist_dense_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    if ((int)blockIdx.x >= t.rows) return;  // the whole block: before any barrier
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_fdr_hist_dense_kernel_body<T>(blockIdx.x, t.rows, t.es, t.K, t.P, L.fac, L.sorted_pos, L.sorted_neg,
                                        L.totals, L.partial);
}
template <class T>
__global__ void stats_fdr_hist_sum_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_fdr_hist_sum_kernel_body(blockIdx.x, L.partial, t.rows, t.K, L.hpos, L.totals);
}
template <class T>
__global__ void stats_fdr_suffix_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_fdr_suffix_kernel_body(blockIdx.x, L.hpos, L.hneg, L.totals);
}
template <class T>
__global__ void stats_fdr_final_multi(const StatsTask<T>* __restrict__ tasks) {
    const StatsTask<T> t = tasks[blockIdx.z];
    const RaggedLayout<T> L(t.scratch, t.K, t.P);
    stats_fdr_final_kernel_body<T>(blockIdx.x, t.K, L.cnt_obs, L.lcount, L.hpos, L.hneg, L.totals, t.stats);
}

// Lower bound of every set's FDR q after the statistics (adaptive stopping):
// the set's |NES| may lie anywhere in [|NES|, key], key = |NES| (1 + z cv /
// sqrt(n)) -- z standard errors of its normalising mean, cv the coefficient
// of variation of its n scores |S| (sums[k] = sum |S|, sums[K + k] = sum
// S^2).  q(x) = (null weight >= x / null weight of the side) / (#observed >=
// x / m) is not monotone in x, so the bound takes the least numerator and
// the largest denominator over the interval: with i_up observed keys below
// key, at least S[i_up + 1] null weight lies at or above key (the nulls at or
// above the next observed key); with i_lo observed keys below |NES|, at most
// m - i_lo observed keys lie at or above |NES|:
//   q >= (S[i_up + 1] / null weight of the side) / (max(m - i_lo, 1) / m).
// NaN or zero NES: 0 (no bound).
template <class T>
__global__ void stats_fdr_bound_kernel(int K, const T* __restrict__ stats, const int64_t* __restrict__ counts,
                                       const double* __restrict__ sums, double z, const T* __restrict__ sorted_pos,
                                       const T* __restrict__ sorted_neg, const double* __restrict__ spos,
                                       const double* __restrict__ sneg, const unsigned long long* __restrict__ totals,
                                       float* __restrict__ qlow, float* __restrict__ qhigh) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const double s = (double)stats[K + k];
    float out = 0.f, out_hi = 1.f;
    const double n = (double)counts[k];
    if (s == s && s != 0.0 && n > 0) {
        const bool up = s > 0.0;
        const double m = sums[k] / n;
        const double var = fmax(sums[K + k] / n - m * m, 0.0);
        const double cv = m > 0.0 ? sqrt(var) / m : INFINITY;
        const double key = fabs(s) * (1.0 + z * cv / sqrt(n));
        const unsigned mcount = (unsigned)(up ? totals[2] : totals[3]);
        if (key < INFINITY && mcount > 0) {
            const T* keys = up ? sorted_pos : sorted_neg;
            auto below = [&](double x) {  // #{keys < x}
                unsigned lo = 0, hi = mcount;
                while (lo < hi) {
                    const unsigned mid = (lo + hi) >> 1;
                    if ((double)keys[mid] < x) lo = mid + 1; else hi = mid;
                }
                return lo;
            };
            const unsigned i_up = below(key), i_lo = below(fabs(s));
            const double c_null = i_up + 1 <= mcount ? (up ? spos : sneg)[i_up + 1] : 0.0;
            const double wtot = reinterpret_cast<const double*>(totals + 4)[up ? 0 : 1];
            const double fn = wtot > 0.0 ? c_null / wtot : 0.0;
            const double obs = (double)(mcount - i_lo > 0 ? mcount - i_lo : 1u);
            const double r = fn / (obs / (double)mcount);
            out = (float)(r < 1.0 ? r : 1.0);
            if (qhigh) {
                // upper bound: the most null weight (at the interval's bottom,
                // |NES| pulled inward) over the fewest observed keys (at or
                // above its top; the set's own key is one of them)
                const double key_in = fabs(s) * fmax(1.0 - z * cv / sqrt(n), 0.0);
                const unsigned j_in = below(key_in);
                const double c_in = j_in <= mcount ? (up ? spos : sneg)[j_in] : 0.0;
                const double fn_hi = wtot > 0.0 ? c_in / wtot : 1.0;
                const double obs_hi = (double)(mcount - i_up > 0 ? mcount - i_up : 1u);
                const double rh = fn_hi / (obs_hi / (double)mcount);
                out_hi = (float)(rh < 1.0 ? rh : 1.0);
            }
        }
    }
    qlow[k] = out;
    if (qhigh) qhigh[k] = out_hi;
}

}  // namespace

template <class T>
cudaError_t launch_fdr_bound(int K, int64_t p_fwer, const T* stats, const int64_t* counts, const double* sums,
                             double z, const void* scratch, float* qlow, cudaStream_t st, float* qhigh) {
    if (K <= 0) return cudaSuccess;
    const RaggedLayout<T> L(const_cast<void*>(scratch), K, p_fwer);
    stats_fdr_bound_kernel<T><<<(K + 255) / 256, 256, 0, st>>>(K, stats, counts, sums, z, L.sorted_pos, L.sorted_neg,
                                                               L.hpos, L.hneg, L.totals, qlow, qhigh);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_fdr_bound<float>(int, int64_t, const float*, const int64_t*, const double*, double,
                                             const void*, float*, cudaStream_t, float*);
template cudaError_t launch_fdr_bound<double>(int, int64_t, const double*, const int64_t*, const double*, double,
                                              const void*, float*, cudaStream_t, float*);

template <class T>
size_t stats_scratch_bytes(int K, int64_t P) {
    // + the dense histograms' partial rows (at most kDenseHistPartialBytes)
    const size_t W = 2 * ((size_t)K + 2) + 2;
    const size_t dense = dense_hist_smem<T>(K) <= kDenseHistSmemMax
                             ? (kDenseHistPartialBytes / (4 * W)) * 4 * W + 16 : 0;
    return StatsScratch::bytes(K, P, sizeof(T)) + 256 + dense;
}
template size_t stats_scratch_bytes<float>(int, int64_t);
template size_t stats_scratch_bytes<double>(int, int64_t);

template <class T>
cudaError_t launch_stats_ragged(const T* es, int K, int64_t ld, const int64_t* counts, int64_t p_fwer, T* stats,
                                void* scratch, cudaStream_t st, int64_t hist_cols) {
    if (hist_cols <= 0 || hist_cols > ld) hist_cols = ld;
    if (K <= 0 || ld <= 0 || p_fwer <= 0 || p_fwer > ld) return K <= 0 ? cudaSuccess : cudaErrorInvalidValue;
    using U = typename RadixKey<T>::U;
    const RaggedLayout<T> L(scratch, K, p_fwer);
    T* fac = L.fac;
    U* mx = L.mx;
    U* mn = L.mn;
    unsigned long long* cnt_obs = L.cnt_obs;
    unsigned long long* lcount = L.lcount;
    T* sorted_pos = L.sorted_pos;
    T* sorted_neg = L.sorted_neg;
    double* hpos = L.hpos;
    double* hneg = L.hneg;
    unsigned long long* totals = L.totals;
    unsigned* partial = L.partial;
    cudaError_t e = cudaMemsetAsync(hpos, 0, sizeof(double) * (2 * ((size_t)K + 2) + 8), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(mx, 0x00, sizeof(U) * (size_t)p_fwer, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(mn, 0xff, sizeof(U) * (size_t)p_fwer, st);
    if (e != cudaSuccess) return e;
    const int wpb = 8;  // warps per block
    stats_set_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(es, K, ld, counts, stats, fac);
    stats_extrema_kernel<T><<<dim3((unsigned)((p_fwer + 127) / 128), (K + kExtremaSets - 1) / kExtremaSets), 128, 0,
                              st>>>(es, K, ld, p_fwer, fac, mx, mn);
    stats_fwer_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(K, p_fwer, mx, mn, stats);
    stats_fdr_obs_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(K, stats, cnt_obs, lcount, sorted_pos,
                                                                       sorted_neg, totals);
    int rows = 0;
    if (!counts && ld > 1 && hist_cols == ld) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        rows = dense_hist_rows<T>(K, sms);
    }
    if (rows > 0) {
        const size_t smem = dense_hist_smem<T>(K);
        e = cudaFuncSetAttribute(stats_fdr_hist_dense_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        stats_fdr_hist_dense_kernel<T><<<rows, kDenseHistThreads, smem, st>>>(es, K, ld, fac, sorted_pos, sorted_neg,
                                                                            totals, partial);
        const int W = 2 * (K + 2) + 2;
        stats_fdr_hist_sum_kernel<<<(W + 255) / 256, 256, 0, st>>>(partial, rows, K, hpos, totals);
    } else if (ld > 1) {
        // the sorted observed keys (at most 2K values) in shared memory: per
        // block (set x column chunk) when they fit the default 48 KB, else
        // once per resident 1,024-thread block looping over the sets
        const size_t obs_bytes = 2 * sizeof(T) * (size_t)K;
        int dev = 0, max_smem = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (obs_bytes > 48 * 1024 && obs_bytes + 1024 <= (size_t)max_smem) {
            auto kern = stats_fdr_hist_kernel<T, 1024>;
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)obs_bytes);
            if (e != cudaSuccess) return e;
            kern<<<dim3((unsigned)(K < sms ? K : sms), 1), 1024, obs_bytes, st>>>(
                es, K, ld, counts, hist_cols, fac, sorted_pos, sorted_neg, hpos, hneg, totals, true);
        } else {
            const int64_t need = (hist_cols - 1 + kHistCols - 1) / kHistCols;
            const unsigned chunks = (unsigned)(need < 65535 ? need : 65535);
            const bool stage = obs_bytes <= 48 * 1024;
            stats_fdr_hist_kernel<T, kHistThreads><<<dim3((unsigned)K, chunks), kHistThreads, stage ? obs_bytes : 0,
                                                      st>>>(es, K, ld, counts, hist_cols, fac, sorted_pos, sorted_neg,
                                                            hpos, hneg, totals, stage);
        }
    }
    stats_fdr_suffix_kernel<<<2, 1024, 0, st>>>(hpos, hneg, totals);
    stats_fdr_final_kernel<T><<<(K + 255) / 256, 256, 0, st>>>(K, cnt_obs, lcount, hpos, hneg, totals, stats);
    launches_add(rows > 0 ? 8 : (ld > 1 ? 7 : 6));
    return cudaGetLastError();
}
template cudaError_t launch_stats_ragged<float>(const float*, int, int64_t, const int64_t*, int64_t, float*, void*,
                                                cudaStream_t, int64_t);
template cudaError_t launch_stats_ragged<double>(const double*, int, int64_t, const int64_t*, int64_t, double*, void*,
                                                 cudaStream_t, int64_t);

template <class T>
int stats_multi_rows(int K, int64_t P) {
    if (K <= 0 || P < 2) return 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return dense_hist_rows<T>(K, sms);
}
template int stats_multi_rows<float>(int, int64_t);
template int stats_multi_rows<double>(int, int64_t);

template <class T>
cudaError_t launch_stats_multi(const StatsTask<T>* d_tasks, const StatsTask<T>* h_tasks, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > 65535) return cudaErrorInvalidValue;
    int Kmax = 0, rows = 0;
    int64_t Pmax = 0, init = 0;
    size_t smem = 0;
    for (int i = 0; i < n; i++) {
        const StatsTask<T>& t = h_tasks[i];
        if (t.rows <= 0 || t.P < 2) return cudaErrorInvalidValue;  // the dense form only
        Kmax = std::max(Kmax, t.K);
        Pmax = std::max(Pmax, t.P);
        rows = std::max(rows, t.rows);
        init = std::max(init, std::max(2 * ((int64_t)t.K + 2) + 8, t.P));
        smem = std::max(smem, dense_hist_smem<T>(t.K));
    }
    const unsigned z = (unsigned)n;
    const int wpb = 8;
    const unsigned set_blocks = (unsigned)((Kmax + wpb - 1) / wpb);
    stats_init_multi<T><<<dim3((unsigned)((init + 255) / 256), 1, z), 256, 0, st>>>(d_tasks);
    stats_set_multi<T><<<dim3(set_blocks, 1, z), wpb * 32, 0, st>>>(d_tasks);
    stats_extrema_multi<T><<<dim3((unsigned)((Pmax + 127) / 128), (unsigned)((Kmax + kExtremaSets - 1) / kExtremaSets), z),
                             128, 0, st>>>(d_tasks);
    stats_fwer_multi<T><<<dim3(set_blocks, 1, z), wpb * 32, 0, st>>>(d_tasks);
    stats_fdr_obs_multi<T><<<dim3(set_blocks, 1, z), wpb * 32, 0, st>>>(d_tasks);
    cudaError_t e = cudaFuncSetAttribute(stats_fdr_hist_dense_multi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    stats_fdr_hist_dense_multi<T><<<dim3((unsigned)rows, 1, z), kDenseHistThreads, smem, st>>>(d_tasks);
    const int Wmax = 2 * (Kmax + 2) + 2;
    stats_fdr_hist_sum_multi<T><<<dim3((unsigned)((Wmax + 255) / 256), 1, z), 256, 0, st>>>(d_tasks);
    stats_fdr_suffix_multi<T><<<dim3(2, 1, z), 1024, 0, st>>>(d_tasks);
    stats_fdr_final_multi<T><<<dim3((unsigned)((Kmax + 255) / 256), 1, z), 256, 0, st>>>(d_tasks);
    launches_add(9);
    return cudaGetLastError();
}
template cudaError_t launch_stats_multi<float>(const StatsTask<float>*, const StatsTask<float>*, int, cudaStream_t);
template cudaError_t launch_stats_multi<double>(const StatsTask<double>*, const StatsTask<double>*, int, cudaStream_t);

template <class T>
cudaError_t launch_stats(const T* es, int K, int64_t P, T* stats, void* scratch, cudaStream_t st) {
    if (K <= 0 || P <= 0) return cudaSuccess;
    return launch_stats_ragged<T>(es, K, P, nullptr, P, stats, scratch, st);
}
template cudaError_t launch_stats<float>(const float*, int, int64_t, float*, void*, cudaStream_t);
template cudaError_t launch_stats<double>(const double*, int, int64_t, double*, void*, cudaStream_t);

}  // namespace gsea
