// k_es.cu -- enrichment scores for gene sets x permutations.
//
// The reference (score_kernel_shared, src/include/enrichment_scores.cuh:91-206)
// walks the whole ranked list of every (set, permutation) twice: pass 1 sums
// N_R = sum |metric| over hits and counts N_H, pass 2 runs the Kahan running
// sum (hit: +|metric|/N_R, miss: -1/(G-N_H)) and keeps the first value of
// largest magnitude, sign included.  That is K*P*G*2 steps.
//
// Here the running sum is evaluated in closed form at its only possible
// extrema: just before and just after each hit (the sum falls monotonically
// between hits).  With hits at positions r_1 < ... < r_n, weights w_j and
// m_j = r_j - (j-1) misses before hit j:
//     before hit j:  W_{j-1}/N_R - m_j * d        (position r_j - 1)
//     after  hit j:  W_j    /N_R - m_j * d        (position r_j)
//     end of list :  W_n    /N_R - (G-n) * d      (position G-1)
// with W_j the prefix sum of weights in rank order and d = (T)(1/(G-N_H)) the
// reference's decay.  The winner is the largest |value|, earliest position on
// ties, exactly the reference's strict `|Res| > |Bsf|` update; NaN weights
// propagate the same way (the reference's Res stays NaN after the first NaN
// step, and so does every later candidate here).
//
// Per permutation one CTA stages the gene ranks and the rank-ordered weights
// in shared memory; a warp per set marks the members' ranks in a bitmap,
// enumerates hits in rank order from it (each lane a contiguous word range),
// scans hit counts and weight sums across lanes and evaluates the candidates.
// Work per (set, permutation) is O(G/32 + n) instead of O(G).
//
// Rounding: the fp32 path accumulates weights as float-float pairs, so its
// ES differ from the reference's Kahan running sum by a few ulp; the fp64
// path is double throughout.
#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace {

// compensated accumulator: float-float for fp32, plain double for fp64
template <class T> struct Acc;
template <> struct Acc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float b) {
        const float s = __fadd_rn(hi, b);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
        hi = s;
        lo = __fadd_rn(lo, err);
    }
    __device__ __forceinline__ void add(const Acc& o) { add(o.hi); lo = __fadd_rn(lo, o.lo); }
    __device__ __forceinline__ float scaled(float inv) const { return fmaf(hi, inv, lo * inv); }
    __device__ __forceinline__ float total() const { return __fadd_rn(hi, lo); }
    __device__ __forceinline__ Acc shfl_up(int o) const {
        Acc r;
        r.hi = __shfl_up_sync(kFullMask, hi, o);
        r.lo = __shfl_up_sync(kFullMask, lo, o);
        return r;
    }
    __device__ __forceinline__ Acc shfl(int src) const {
        Acc r;
        r.hi = __shfl_sync(kFullMask, hi, src);
        r.lo = __shfl_sync(kFullMask, lo, src);
        return r;
    }
};
template <> struct Acc<double> {
    double v = 0.0;
    __device__ __forceinline__ void add(double b) { v += b; }
    __device__ __forceinline__ void add(const Acc& o) { v += o.v; }
    __device__ __forceinline__ double scaled(double inv) const { return v * inv; }
    __device__ __forceinline__ double total() const { return v; }
    __device__ __forceinline__ Acc shfl_up(int o) const {
        Acc r;
        r.v = __shfl_up_sync(kFullMask, v, o);
        return r;
    }
    __device__ __forceinline__ Acc shfl(int src) const {
        Acc r;
        r.v = __shfl_sync(kFullMask, v, src);
        return r;
    }
};

template <class T>
__device__ __forceinline__ T fma_t(T a, T b, T c);
template <> __device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }

// candidate (val, pos) replaces (best, bpos) when |val| > |best| or equal
// magnitude at an earlier position; NaN never replaces
template <class T>
__device__ __forceinline__ void consider(T val, int pos, T& best, int& bpos) {
    const T a = fabs(val), b = fabs(best);
    if (a > b || (a == b && pos < bpos)) {
        best = val;
        bpos = pos;
    }
}

template <class T, class RankT, int WARPS, bool STAGE>
__global__ void __launch_bounds__(WARPS * 32)
es_kernel(const RankT* __restrict__ ranks, const T* __restrict__ sorted_abs, int G, int num_perms,
          const int64_t* __restrict__ set_off, const int32_t* __restrict__ set_genes, int K,
          T* __restrict__ es, int64_t es_stride, int64_t col0) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int words = (G + 31) >> 5;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // layout: [T w[G]] [RankT rank[G]] (when staged), then per-warp bitmaps
    T* s_w = reinterpret_cast<T*>(smem);
    RankT* s_rank = reinterpret_cast<RankT*>(smem + (STAGE ? sizeof(T) * (size_t)G : 0));
    size_t bm_off = STAGE ? (sizeof(T) + sizeof(RankT)) * (size_t)G : 0;
    bm_off = (bm_off + 15) & ~(size_t)15;
    uint32_t* bm = reinterpret_cast<uint32_t*>(smem + bm_off) + (size_t)warp * words;
    for (int w = lane; w < words; w += 32) bm[w] = 0u;

    const int wpl = (words + 31) >> 5;  // words per lane
    const int w0 = min(lane * wpl, words), w1 = min(w0 + wpl, words);

    for (int p = blockIdx.x; p < num_perms; p += gridDim.x) {
        const RankT* rk = ranks + (int64_t)p * G;
        const T* wt = sorted_abs + (int64_t)p * G;
        if (STAGE) {
            __syncthreads();
            for (int i = tid; i < G; i += WARPS * 32) {
                s_w[i] = wt[i];
                s_rank[i] = rk[i];
            }
            __syncthreads();
            rk = s_rank;
            wt = s_w;
        }
        for (int k = warp; k < K; k += WARPS) {
            const int64_t a = set_off[k], b = set_off[k + 1];
            // A: mark member ranks
            for (int64_t i = a + lane; i < b; i += 32) {
                const int g = set_genes[i];
                if (g >= 0 && g < G) {
                    const uint32_t r = (uint32_t)rk[g];
                    atomicOr(&bm[r >> 5], 1u << (r & 31));
                }
            }
            __syncwarp();
            // B: hits and weight sums of this lane's word range
            int h = 0;
            Acc<T> W;
            for (int w = w0; w < w1; w++) {
                uint32_t word = bm[w];
                h += __popc(word);
                while (word) {
                    const int bit = __ffs(word) - 1;
                    word &= word - 1;
                    W.add(wt[(w << 5) + bit]);
                }
            }
            // C: exclusive scans across lanes
            int h_incl = h;
            Acc<T> W_incl = W;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int hy = __shfl_up_sync(kFullMask, h_incl, o);
                const Acc<T> wy = W_incl.shfl_up(o);
                if (lane >= o) {
                    h_incl += hy;
                    W_incl.add(wy);
                }
            }
            const int n_hits = __shfl_sync(kFullMask, h_incl, 31);
            const Acc<T> W_tot = W_incl.shfl(31);
            int j = h_incl - h;               // hits before this lane's range
            Acc<T> Wr = W_incl.shfl_up(1);    // weight before this lane's range
            if (lane == 0) Wr = Acc<T>();
            const T N_R = W_tot.total();
            const T inv = n_hits > 0 ? T(1) / N_R : T(0);
            const T d = n_hits < G ? (T)(1.0 / (double)(G - n_hits)) : T(0);
            // D: candidates in rank order
            T best = T(0);
            int bpos = -1;
            for (int w = w0; w < w1; w++) {
                uint32_t word = bm[w];
                if (word) bm[w] = 0u;
                while (word) {
                    const int bit = __ffs(word) - 1;
                    word &= word - 1;
                    const int r = (w << 5) + bit;
                    const T miss = (T)(r - j);
                    const T hit_before = j > 0 ? Wr.scaled(inv) : T(0);
                    consider<T>(fma_t<T>(-miss, d, hit_before), r - 1, best, bpos);
                    Wr.add(wt[r]);
                    j++;
                    consider<T>(fma_t<T>(-miss, d, Wr.scaled(inv)), r, best, bpos);
                }
            }
            if (lane == 31) {
                const T hits_end = n_hits > 0 ? W_tot.scaled(inv) : T(0);
                consider<T>(fma_t<T>(-(T)(G - n_hits), d, hits_end), G - 1, best, bpos);
            }
            // E: reduce (largest magnitude, earliest position)
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) {
                const T ob = __shfl_xor_sync(kFullMask, best, o);
                const int op = __shfl_xor_sync(kFullMask, bpos, o);
                consider<T>(ob, op, best, bpos);
            }
            if (lane == 0) es[(int64_t)k * es_stride + col0 + p] = best;
            __syncwarp();
        }
    }
}

constexpr int kWarps32 = 16;
constexpr int kWarps64 = 8;

template <class T, class RankT, int WARPS>
cudaError_t launch_es_t(const RankT* ranks, const T* sorted_abs, int G, int P, const int64_t* off,
                        const int32_t* genes, int K, T* es, int64_t stride, int64_t col0,
                        cudaStream_t st) {
    int dev = 0, max_smem = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int words = (G + 31) >> 5;
    const size_t bm_bytes = sizeof(uint32_t) * (size_t)words * WARPS;
    size_t staged = (((sizeof(T) + sizeof(RankT)) * (size_t)G + 15) & ~(size_t)15) + bm_bytes;
    const int grid = P < 2 * sms ? P : 2 * sms;
    if (staged <= (size_t)max_smem) {
        auto kern = es_kernel<T, RankT, WARPS, true>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)staged);
        if (e != cudaSuccess) return e;
        kern<<<grid, WARPS * 32, staged, st>>>(ranks, sorted_abs, G, P, off, genes, K, es, stride, col0);
    } else {
        if (bm_bytes > (size_t)max_smem) return cudaErrorInvalidValue;
        auto kern = es_kernel<T, RankT, WARPS, false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bm_bytes);
        if (e != cudaSuccess) return e;
        kern<<<grid, WARPS * 32, bm_bytes, st>>>(ranks, sorted_abs, G, P, off, genes, K, es, stride, col0);
    }
    launches_add(1);
    return cudaGetLastError();
}

}  // namespace

template <class T>
cudaError_t launch_es(const void* ranks, bool ranks16, const T* sorted_abs, int G, int num_perms,
                      const int64_t* set_offsets, const int32_t* set_genes, int K, T* es,
                      int64_t es_stride, int64_t perm_col0, cudaStream_t st) {
    if (num_perms <= 0 || K <= 0) return cudaSuccess;
    constexpr int WARPS = sizeof(T) == 4 ? kWarps32 : kWarps64;
    if (ranks16)
        return launch_es_t<T, uint16_t, WARPS>(static_cast<const uint16_t*>(ranks), sorted_abs, G,
                                               num_perms, set_offsets, set_genes, K, es, es_stride,
                                               perm_col0, st);
    return launch_es_t<T, uint32_t, WARPS>(static_cast<const uint32_t*>(ranks), sorted_abs, G,
                                           num_perms, set_offsets, set_genes, K, es, es_stride,
                                           perm_col0, st);
}
template cudaError_t launch_es<float>(const void*, bool, const float*, int, int, const int64_t*,
                                      const int32_t*, int, float*, int64_t, int64_t, cudaStream_t);
template cudaError_t launch_es<double>(const void*, bool, const double*, int, int, const int64_t*,
                                       const int32_t*, int, double*, int64_t, int64_t, cudaStream_t);

}  // namespace gsea
