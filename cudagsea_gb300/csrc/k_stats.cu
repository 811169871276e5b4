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
#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace {

struct StatsScratch {
    // laid out in the scratch buffer
    static size_t bytes(int K, int64_t P, size_t tsize) {
        return tsize * ((size_t)K + 2 * (size_t)P) + sizeof(unsigned long long) * (3 * (size_t)K + 8);
    }
};

// one warp per set: factor, NES, NP
template <class T>
__global__ void stats_set_kernel(const T* __restrict__ es, int K, int64_t P, T* __restrict__ out,
                                 T* __restrict__ fac) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= K) return;
    const T* row = es + (int64_t)warp * P;
    const T es0 = row[0];
    T sum = T(0);
    unsigned long long np = 0;
    const T aes0 = fabs(es0);
    for (int64_t p0 = 0; p0 < P; p0 += 32) {
        const int64_t p = p0 + lane;
        const T v = p < P ? row[p] : T(0);
        const T av = fabs(v);
        if (p < P && av >= aes0) np++;
        const int n = (int)(P - p0 < 32 ? P - p0 : 32);
        // sequential sum in index order, as the reference's host loop
        for (int i = 0; i < n; i++) {
            const T x = __shfl_sync(kFullMask, av, i);
            sum = Exact<T>::add(sum, x);
        }
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

// one thread per permutation column: extrema of normalised scores
template <class T>
__global__ void stats_extrema_kernel(const T* __restrict__ es, int K, int64_t P,
                                     const T* __restrict__ fac, T* __restrict__ mx, T* __restrict__ mn) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    T hi = -INFINITY, lo = INFINITY;
    for (int k = 0; k < K; k++) {
        const T v = Exact<T>::mul(es[(int64_t)k * P + p], fac[k]);
        hi = hi < v ? v : hi;
        lo = lo > v ? v : lo;
    }
    mx[p] = hi;
    mn[p] = lo;
}

// one warp per set: FWER; also the observed-side totals for FDR
template <class T>
__global__ void stats_fwer_kernel(int K, int64_t P, const T* __restrict__ mx, const T* __restrict__ mn,
                                  T* __restrict__ out, unsigned long long* __restrict__ totals) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= K) return;
    const T score = out[K + warp];
    unsigned long long c = 0;
    if (score > T(0)) {
        for (int64_t p = lane; p < P; p += 32) c += mx[p] >= score;
    } else {
        for (int64_t p = lane; p < P; p += 32) c += mn[p] <= score;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(kFullMask, c, o);
    if (lane == 0) {
        out[3 * K + warp] = Exact<T>::div((T)c, (T)P);
        if (score >= T(0)) atomicAdd(&totals[2], 1ull);   // observed >= 0
        if (score <= T(0)) atomicAdd(&totals[3], 1ull);   // observed <= 0
    }
}

// FDR counts: each block takes a chunk of null scores (all sets, perms >= 1)
// into shared memory; each thread owns sets and counts the chunk's scores
// beyond its set's NES.  Also counts the null scores on each side.
constexpr int kFdrChunk = 4096;
template <class T>
__global__ void stats_fdr_count_kernel(const T* __restrict__ es, int K, int64_t P,
                                       const T* __restrict__ fac, const T* __restrict__ out,
                                       unsigned long long* __restrict__ cnt_null,
                                       unsigned long long* __restrict__ totals) {
    __shared__ T chunk[kFdrChunk];
    const int64_t total = (int64_t)K * (P - 1);
    const int64_t c0 = (int64_t)blockIdx.x * kFdrChunk;
    const int n = (int)(total - c0 < kFdrChunk ? total - c0 : kFdrChunk);
    unsigned long long pos = 0, neg = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int64_t q = c0 + i;
        const int64_t k = q / (P - 1), p = 1 + q % (P - 1);
        const T v = Exact<T>::mul(es[k * P + p], fac[k]);
        chunk[i] = v;
        pos += v >= T(0);
        neg += v <= T(0);
    }
    __syncthreads();
    for (int o = 16; o >= 1; o >>= 1) {
        pos += __shfl_xor_sync(kFullMask, pos, o);
        neg += __shfl_xor_sync(kFullMask, neg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (pos) atomicAdd(&totals[0], pos);
        if (neg) atomicAdd(&totals[1], neg);
    }
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const T s = out[K + k];
        unsigned long long c = 0;
        if (s > T(0)) {
            for (int i = 0; i < n; i++) c += chunk[i] >= s;
        } else {
            for (int i = 0; i < n; i++) c += chunk[i] <= s;
        }
        if (c) atomicAdd(&cnt_null[k], c);
    }
}

// observed counts: #{observed NES beyond NES*} on the same side
template <class T>
__global__ void stats_fdr_obs_kernel(int K, const T* __restrict__ out, unsigned long long* __restrict__ cnt_obs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const T s = out[K + k];
    unsigned long long co = 0;
    if (s > T(0)) {
        for (int j = 0; j < K; j++) co += out[K + j] >= s;
    } else {
        for (int j = 0; j < K; j++) co += out[K + j] <= s;
    }
    cnt_obs[k] = co;
}

template <class T>
__global__ void stats_fdr_final_kernel(int K, const unsigned long long* __restrict__ cnt_null,
                                       const unsigned long long* __restrict__ cnt_obs,
                                       const unsigned long long* __restrict__ totals, T* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const T s = out[K + k];
    T q;
    if (!(s == s)) {
        q = s;
    } else {
        const bool up = s > T(0);
        const double null_side = (double)(up ? totals[0] : totals[1]);
        const double obs_side = (double)(up ? totals[2] : totals[3]);
        const double fn = null_side > 0 ? (double)cnt_null[k] / null_side : 0.0;
        const double fo = (double)cnt_obs[k] / obs_side;
        const double r = fn / fo;
        q = (T)(r < 1.0 ? r : 1.0);
    }
    out[4 * K + k] = q;
}

}  // namespace

template <class T>
size_t stats_scratch_bytes(int K, int64_t P) {
    return StatsScratch::bytes(K, P, sizeof(T)) + 256;
}
template size_t stats_scratch_bytes<float>(int, int64_t);
template size_t stats_scratch_bytes<double>(int, int64_t);

template <class T>
cudaError_t launch_stats(const T* es, int K, int64_t P, T* stats, void* scratch, cudaStream_t st) {
    if (K <= 0 || P <= 0) return cudaSuccess;
    unsigned char* s = static_cast<unsigned char*>(scratch);
    T* fac = reinterpret_cast<T*>(s);
    T* mx = fac + K;
    T* mn = mx + P;
    size_t off = sizeof(T) * ((size_t)K + 2 * (size_t)P);
    off = (off + 15) & ~(size_t)15;
    unsigned long long* cnt_null = reinterpret_cast<unsigned long long*>(s + off);
    unsigned long long* cnt_obs = cnt_null + K;
    unsigned long long* totals = cnt_obs + K;
    cudaError_t e = cudaMemsetAsync(cnt_null, 0, sizeof(unsigned long long) * (2 * (size_t)K + 8), st);
    if (e != cudaSuccess) return e;
    const int wpb = 8;  // warps per block
    stats_set_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(es, K, P, stats, fac);
    stats_extrema_kernel<T><<<(unsigned)((P + 255) / 256), 256, 0, st>>>(es, K, P, fac, mx, mn);
    stats_fwer_kernel<T><<<(K + wpb - 1) / wpb, wpb * 32, 0, st>>>(K, P, mx, mn, stats, totals);
    int launches = 4;
    const int64_t total = P > 1 ? (int64_t)K * (P - 1) : 0;
    const unsigned blocks = total > 0 ? (unsigned)((total + kFdrChunk - 1) / kFdrChunk) : 1u;
    stats_fdr_count_kernel<T><<<blocks, 256, 0, st>>>(es, K, P, fac, stats, cnt_null, totals);
    stats_fdr_obs_kernel<T><<<(K + 255) / 256, 256, 0, st>>>(K, stats, cnt_obs);
    launches++;
    stats_fdr_final_kernel<T><<<(K + 255) / 256, 256, 0, st>>>(K, cnt_null, cnt_obs, totals, stats);
    launches_add(launches + 1);
    return cudaGetLastError();
}
template cudaError_t launch_stats<float>(const float*, int, int64_t, float*, void*, cudaStream_t);
template cudaError_t launch_stats<double>(const double*, int, int64_t, double*, void*, cudaStream_t);

}  // namespace gsea
