// k_es.cuh -- enrichment scores for gene sets x permutations (included by
// k_es_f32.cu and k_es_f64.cu, one translation unit per precision).
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
// Work per (set, permutation) is O(G/32 + n) instead of O(G):
//   * one CTA per permutation stages the rank of every gene and the weight at
//     every position in shared memory (or, when the bitmaps of large G leave
//     no room, the ranks only, the weights then read through L1 / L2);
//   * a warp takes the next set from a CTA-wide counter (largest sets first),
//     marks its members' ranks in a per-warp bitmap (duplicates collapse) and
//     sums the weights of the marked ranks (N_R);
//   * each lane owns a contiguous range of bitmap words: their popcounts and
//     one warp scan give the global index of the lane's first hit, and the
//     lane walks its hits once, in rank order, with a lane-local prefix of the
//     weights; its largest and smallest candidates are shifted afterwards by
//     the weight of the hits before the lane (a second warp scan);
//   * a warp reduction picks the winner.
//   With 32-bit ranks (G > 65,536) a general procedure walks each lane's
//   word range twice from shared memory instead.
//
// Rounding: fp32 sums are compensated (Kahan in a lane, float-float across
// lanes), so the fp32 ES stay within a few ulp of the reference's Kahan
// running sum (the shift adds one rounding); the fp64 path is double
// throughout.
#pragma once
#include <climits>
#include <type_traits>

#include <math_constants.h>

#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace {

// compensated accumulator: float-float for fp32, plain double for fp64
template <class T> struct Acc;
template <> struct Acc<float> {
    float hi = 0.f, lo = 0.f;
    // Kahan step (the running sum of one lane grows monotonically)
    __device__ __forceinline__ void add(float b) {
        const float y = __fsub_rn(b, lo);
        const float t = __fadd_rn(hi, y);
        lo = __fsub_rn(__fsub_rn(t, hi), y);
        hi = t;
    }
    // merge another accumulator: two-sum of the main terms, the rounding
    // error folded into the (negated) compensation
    __device__ __forceinline__ void merge(const Acc& o) {
        const float s = __fadd_rn(hi, o.hi);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(o.hi, bb));
        hi = s;
        lo = __fsub_rn(__fadd_rn(lo, o.lo), err);
    }
    __device__ __forceinline__ float value() const { return __fsub_rn(hi, lo); }
    // (hi - lo) * inv + c, with one rounding of the product's main term
    __device__ __forceinline__ float scaled_plus(float inv, float c) const {
        return fmaf(hi, inv, fmaf(-lo, inv, c));
    }
    __device__ __forceinline__ Acc shfl_up(int o) const {
        Acc r;
        r.hi = __shfl_up_sync(kFullMask, hi, o);
        r.lo = __shfl_up_sync(kFullMask, lo, o);
        return r;
    }
    __device__ __forceinline__ Acc shfl_xor(int o) const {
        Acc r;
        r.hi = __shfl_xor_sync(kFullMask, hi, o);
        r.lo = __shfl_xor_sync(kFullMask, lo, o);
        return r;
    }
};
template <> struct Acc<double> {
    double hi = 0.0, lo = 0.0;  // lo unused
    __device__ __forceinline__ void add(double b) { hi += b; }
    __device__ __forceinline__ void merge(const Acc& o) { hi += o.hi; }
    __device__ __forceinline__ double value() const { return hi; }
    __device__ __forceinline__ double scaled_plus(double inv, double c) const { return fma(hi, inv, c); }
    __device__ __forceinline__ Acc shfl_up(int o) const {
        Acc r;
        r.hi = __shfl_up_sync(kFullMask, hi, o);
        return r;
    }
    __device__ __forceinline__ Acc shfl_xor(int o) const {
        Acc r;
        r.hi = __shfl_xor_sync(kFullMask, hi, o);
        return r;
    }
};

// candidate (val, pos) replaces (best, bpos) when |val| > |best|, or equal
// magnitude at an earlier position; NaN never replaces
template <class T>
__device__ __forceinline__ void consider(T val, int pos, T& best, int& bpos) {
    const T a = fabs(val), b = fabs(best);
    if (a > b || (a == b && pos < bpos)) {
        best = val;
        bpos = pos;
    }
}

// ---------------------------------------------------------------------------
// Per-set procedures.  Both run on one warp with the set's member ranks marked
// in the warp's bitmap `bm` (G bits) and leave the bitmap all zero.

// Direct procedure (G <= 1024*WPL): the lane's bitmap words (WPL, a multiple
// of 4, loaded as 16-byte vectors) give its hit count and a mask of its
// nonzero words; a warp scan of the counts gives the global index of each
// lane's first hit.  Every lane then walks its own hits once, in rank order,
// with a lane-local compensated prefix of the weights, and keeps its largest
// value after a hit and smallest value before one; the weight of the hits in
// the lanes before it (a second warp scan, after the walk) shifts both by a
// constant, which leaves their positions unchanged.  The set's total weight
// `Wt` (every lane) comes from the marking.  Each word is cleared as it is
// read.  `w0` = lane*WPL: the lane's first word, 16-byte aligned inside the
// warp's region of WPL*32 words (bits at positions >= G are never set).
// order-preserving signed 64-bit key of a double (an involution): the
// integer order of the keys is the numeric order of non-NaN doubles, -0
// below +0
__device__ __forceinline__ long long okey(double v) {
    const long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double okey_value(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

// One lane's walk over its hits in rank order (the direct procedure below):
// its largest value after a hit (mx at pmx) and smallest before one (mn at
// pmn) with the lane-local prefix Wl.  IKEY (doubles whose candidates are all
// finite): the running extrema are compared as integer keys, on the integer
// pipe instead of the FP64 pipe that bounds the FP64 kernel -- the same
// results, since the keys order finite doubles as they compare except -0 /
// +0, and a zero never decides a score (only a positive maximum or a
// negative minimum counts).
template <class T, int WPL, bool IKEY, class Mask>
__device__ __forceinline__ void walk_hits(uint32_t* bm, int w0, Mask nzm, int cnt, int excl, const T* wt, T inv,
                                          T d, Acc<T>& Wl, T& mx, int& pmx, T& mn, int& pmn) {
    uint32_t cur = 0u;
    int wi = 0;
    long long kmx = 0, kmn = 0;
    if constexpr (IKEY) {
        kmx = okey(mx);
        kmn = okey(mn);
    }
    for (int t = 0; t < cnt; t++) {
        if (cur == 0u) {  // next nonzero word of the lane
            wi = (WPL > 32 ? __ffsll((long long)nzm) : __ffs((int)nzm)) - 1;
            nzm &= nzm - 1;
            cur = bm[w0 + wi];
            bm[w0 + wi] = 0u;
        }
        const int bit = __ffs(cur) - 1;
        cur &= cur - 1;
        const int r = ((w0 + wi) << 5) + bit;
        const T md = -(T)(r - (excl + t)) * d;  // misses before this hit, times the decay
        const T before = t > 0 ? Wl.scaled_plus(inv, md) : md;
        Wl.add(wt[r]);
        const T after = Wl.scaled_plus(inv, md);
        if constexpr (IKEY) {
            const long long kb = okey(before), ka = okey(after);
            if (kb < kmn) { kmn = kb; pmn = r - 1; }
            if (ka > kmx) { kmx = ka; pmx = r; }
        } else {
            if (before < mn) { mn = before; pmn = r - 1; }
            if (after > mx) { mx = after; pmx = r; }
        }
    }
    if constexpr (IKEY) {
        mx = okey_value(kmx);
        mn = okey_value(kmn);
    }
}

template <class T, int WPL>
__device__ __forceinline__ T set_score_direct(uint32_t* bm, int w0, const T* wt, const T* __restrict__ decay, int G,
                                              int lane, const Acc<T>& Wt) {
    using Mask = typename std::conditional<(WPL > 32), unsigned long long, uint32_t>::type;
    Mask nzm = 0;  // bit i: word w0 + i holds hits
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < WPL; i += 4) {
        const uint4 v = *reinterpret_cast<const uint4*>(bm + w0 + i);
        cnt += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        nzm |= (Mask)(((v.x != 0u) ? 1u : 0u) | ((v.y != 0u) ? 2u : 0u) | ((v.z != 0u) ? 4u : 0u) |
                      ((v.w != 0u) ? 8u : 0u)) << i;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += y;
    }
    const int n = __shfl_sync(kFullMask, incl, 31);
    const int excl = incl - cnt;  // hits in the lanes before
    const T inv = n > 0 ? T(1) / Wt.value() : T(0);
    const T d = decay[n];
    Acc<T> Wl;  // weight of this lane's hits so far
    T mx = -CUDART_INF, mn = CUDART_INF;
    int pmx = -1, pmn = -1;
    if constexpr (std::is_same<T, double>::value) {
        if (isfinite(Wt.value()) && isfinite(inv))  // warp-uniform: every candidate is finite
            walk_hits<T, WPL, true>(bm, w0, nzm, cnt, excl, wt, inv, d, Wl, mx, pmx, mn, pmn);
        else
            walk_hits<T, WPL, false>(bm, w0, nzm, cnt, excl, wt, inv, d, Wl, mx, pmx, mn, pmn);
    } else {
        walk_hits<T, WPL, false>(bm, w0, nzm, cnt, excl, wt, inv, d, Wl, mx, pmx, mn, pmn);
    }
    Acc<T> W_incl = Wl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Acc<T> y = W_incl.shfl_up(o);
        if (lane >= o) W_incl.merge(y);
    }
    const Acc<T> W_pre = W_incl.shfl_up(1);  // weight of the hits before this lane's
    const T shift = excl > 0 ? W_pre.scaled_plus(inv, T(0)) : T(0);
    mx += shift;
    mn += shift;
    if (lane == 31) {  // end of the list, after the trailing misses
        const T tail = -(T)(G - n) * d;
        const T end = n > 0 ? Wt.scaled_plus(inv, tail) : tail;
        if (end < mn) { mn = end; pmn = G - 1; }
    }
    // the largest value is always just after a hit and the smallest just
    // before one (or at the end): only a positive maximum and a negative
    // minimum are candidates
    T best = T(0);
    int bpos = -1;
    if (pmx >= 0 && mx > T(0)) consider<T>(mx, pmx, best, bpos);
    if (pmn >= 0 && mn < T(0)) consider<T>(mn, pmn, best, bpos);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const T ob = __shfl_xor_sync(kFullMask, best, o);
        const int op = __shfl_xor_sync(kFullMask, bpos, o);
        consider<T>(ob, op, best, bpos);
    }
    return best;
}

// General procedure (any G, any set size): each lane walks its own word range
// twice -- weights first, then candidates with the exact prefix from a scan.
template <class T>
__device__ __noinline__ T set_score_walk(uint32_t* bm, int w0, int w1, const T* wt, const T* __restrict__ decay,
                                         int G, int lane) {
    int h = 0;
    Acc<T> Wl;
    for (int w = w0; w < w1; w++) {
        uint32_t word = bm[w];
        h += __popc(word);
        while (word) {
            const int bit = __ffs(word) - 1;
            word &= word - 1;
            Wl.add(wt[(w << 5) + bit]);
        }
    }
    int h_incl = h;
    Acc<T> W_incl = Wl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int hy = __shfl_up_sync(kFullMask, h_incl, o);
        const Acc<T> wy = W_incl.shfl_up(o);
        if (lane >= o) {
            h_incl += hy;
            W_incl.merge(wy);
        }
    }
    const int n = __shfl_sync(kFullMask, h_incl, 31);
    Acc<T> Wt;
    Wt.hi = __shfl_sync(kFullMask, W_incl.hi, 31);
    Wt.lo = __shfl_sync(kFullMask, W_incl.lo, 31);
    const T N_R = Wt.value();
    const T inv = n > 0 ? T(1) / N_R : T(0);
    const T d = decay[n];
    Acc<T> W = W_incl.shfl_up(1);
    if (lane == 0) W = Acc<T>();
    int j = h_incl - h;
    T best = T(0);
    int bpos = -1;
    for (int w = w0; w < w1; w++) {
        uint32_t word = bm[w];
        if (!word) continue;
        bm[w] = 0u;
        while (word) {
            const int bit = __ffs(word) - 1;
            word &= word - 1;
            const int r = (w << 5) + bit;
            const T m = (T)(r - j);
            const T before = j > 0 ? W.scaled_plus(inv, -m * d) : -m * d;
            consider<T>(before, r - 1, best, bpos);
            W.add(wt[r]);
            j++;
            consider<T>(W.scaled_plus(inv, -m * d), r, best, bpos);
        }
    }
    if (lane == 31) {
        const T tail = -(T)(G - n) * d;
        consider<T>(n > 0 ? Wt.scaled_plus(inv, tail) : tail, G - 1, best, bpos);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const T ob = __shfl_xor_sync(kFullMask, best, o);
        const int op = __shfl_xor_sync(kFullMask, bpos, o);
        consider<T>(ob, op, best, bpos);
    }
    return best;
}

// One permutation on the calling CTA: stage its ranks and weights (STAGE 1),
// its ranks only (STAGE 2, the weights then gathered through L1 / L2), its
// weights only (STAGE 3, the ranks gathered) or nothing (STAGE 0),
// then warps take sets from the CTA-wide counter until the CTA's share is
// scored.  The share is parts [part_lo, part_hi) of `parts` interleaved parts
// of the set order (part j: slots j, j + parts, j + 2*parts, ...), so that
// every part mixes large and small sets; parts = 1 takes every set.
// s_w / s_rank: staging (STAGE), bm: this warp's zeroed bitmap region.
// Begins and ends with the CTA in step (the staging may be reused after).
template <class T, class RankT, int WARPS, int STAGE, int WPL>
__device__ __forceinline__ void es_one_perm(const RankT* rk, const T* wt, int G, const int64_t* __restrict__ set_off,
                                            const int32_t* __restrict__ set_genes,
                                            const int32_t* __restrict__ set_order, const T* __restrict__ decay, int K,
                                            T* __restrict__ es_col, int64_t es_stride, T* s_w, RankT* s_rank,
                                            uint32_t* bm, int* next_set, int part_lo = 0, int part_hi = 1,
                                            int parts = 1) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int words = (G + 31) >> 5;
    const int wpl = WPL > 0 ? WPL : (words + 31) >> 5;  // bitmap words per lane
    const int w0 = min(lane * wpl, words), w1 = min(w0 + wpl, words);
    __syncthreads();  // previous permutation finished with the staging and the counter
    if (tid == 0) *next_set = 0;
    if (STAGE) {
        for (int i = tid; i < G; i += WARPS * 32) {
            if (STAGE == 1 || STAGE == 3) s_w[i] = wt[i];
            if (STAGE == 1 || STAGE == 2) s_rank[i] = rk[i];
        }
        if (STAGE == 1 || STAGE == 2) rk = s_rank;
        if (STAGE == 1 || STAGE == 3) wt = s_w;
    }
    __syncthreads();
    while (true) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(next_set, 1);
        slot = __shfl_sync(kFullMask, slot, 0);
        if (parts > 1) {  // i-th set of the share: slots grow with i
            const int m = part_hi - part_lo;
            slot = (slot / m) * parts + part_lo + slot % m;
        }
        if (slot >= K) break;
        const int k = set_order ? set_order[slot] : slot;
        const int64_t a = set_off[k];
        const int m = (int)(set_off[k + 1] - a);  // a set lists fewer than 2^31 members
        const int32_t* __restrict__ sg = set_genes + a;
        // mark the members' ranks (duplicates and unknown ids fall away); the
        // direct procedure also sums the weights of the newly marked ranks
        Acc<T> Wm;
        for (int base = 0; base < m; base += 128) {
            int g[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int idx = base + lane + 32 * i;
                g[i] = idx < m ? __ldg(sg + idx) : -1;
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                if (g[i] >= 0 && g[i] < G) {
                    const uint32_t r = (uint32_t)rk[g[i]];
                    const uint32_t bit = 1u << (r & 31);
                    if (WPL > 0) {
                        if (!(atomicOr(&bm[r >> 5], bit) & bit)) Wm.add(wt[r]);
                    } else {
                        atomicOr(&bm[r >> 5], bit);
                    }
                }
            }
        }
        __syncwarp();
        T score;
        if (WPL > 0) {
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) Wm.merge(Wm.shfl_xor(o));  // the set's weight, every lane
            score = set_score_direct<T, (WPL > 0 ? WPL : 4)>(bm, lane * WPL, wt, decay, G, lane, Wm);
        } else {
            score = set_score_walk<T>(bm, w0, w1, wt, decay, G, lane);
        }
        if (lane == 0) es_col[(int64_t)k * es_stride] = score;
        __syncwarp();
    }
}

// bytes of a CTA's staging: weights + ranks (1), ranks (2), weights (3), none (0)
template <class T, class RankT, int STAGE>
__host__ __device__ __forceinline__ size_t es_stage_bytes(int G) {
    return STAGE == 1   ? (sizeof(T) + sizeof(RankT)) * (size_t)G
           : STAGE == 2 ? sizeof(RankT) * (size_t)G
           : STAGE == 3 ? sizeof(T) * (size_t)G
                        : 0;
}

// shared memory of a CTA: staging for G genes (STAGE) + WARPS bitmap regions
template <class T, class RankT, int STAGE>
__device__ __forceinline__ void es_smem_layout(unsigned char* smem, int G, int region, T*& s_w, RankT*& s_rank,
                                               uint32_t*& bm) {
    const int warp = threadIdx.x >> 5;
    s_w = reinterpret_cast<T*>(smem);
    s_rank = reinterpret_cast<RankT*>(smem + (STAGE == 1 ? sizeof(T) * (size_t)G : 0));
    size_t bm_off = es_stage_bytes<T, RankT, STAGE>(G);
    bm_off = (bm_off + 15) & ~(size_t)15;
    bm = reinterpret_cast<uint32_t*>(smem + bm_off) + (size_t)warp * region;
}

// WPL > 0: bitmap words per lane held in registers by the list procedure
// (G <= 1024*WPL, ranks < 65536); WPL == 0: general procedure only.
template <class T, class RankT, int WARPS, int STAGE, int WPL>
__global__ void __launch_bounds__(WARPS * 32)
es_kernel(const RankT* __restrict__ ranks, const T* __restrict__ sorted_abs, int G, int num_perms,
          const int64_t* __restrict__ set_off, const int32_t* __restrict__ set_genes,
          const int32_t* __restrict__ set_order, const T* __restrict__ decay, int K, T* __restrict__ es,
          int64_t es_stride, int64_t col0, const int* __restrict__ K_dev) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int next_set;
    if (K_dev) K = min(K, *K_dev);  // a set list whose length a kernel decided
    if (K <= 0) return;
    const int words = (G + 31) >> 5;
    const int region = WPL > 0 ? WPL * 32 : words;  // per-warp bitmap words
    T* s_w;
    RankT* s_rank;
    uint32_t* bm;
    es_smem_layout<T, RankT, STAGE>(smem, G, region, s_w, s_rank, bm);
    for (int w = threadIdx.x & 31; w < region; w += 32) bm[w] = 0u;
    // whole permutations in rounds of gridDim.x ...
    const int grid = gridDim.x;
    const int full = num_perms / grid;
    for (int i = 0; i < full; i++) {
        const int p = blockIdx.x + i * grid;
        es_one_perm<T, RankT, WARPS, STAGE, WPL>(ranks + (int64_t)p * G, sorted_abs + (int64_t)p * G, G, set_off,
                                                  set_genes, set_order, decay, K, es + col0 + p, es_stride, s_w,
                                                  s_rank, bm, &next_set);
    }
    // ... then the rem < gridDim.x left over, each cut into `parts` parts
    // (parts * rem a multiple of gridDim.x where K allows); every CTA takes an
    // equal contiguous run of the (permutation, part) items, which spans at
    // most a few permutations, so the last round ends evenly
    const int rem = num_perms - full * grid;
    if (rem == 0) return;
    int a = rem, b = grid;
    while (b) { const int t = a % b; a = b; b = t; }
    const int parts = min(grid / a, K);
    const int64_t items = (int64_t)rem * parts;
    int64_t lo = items * blockIdx.x / grid;
    const int64_t hi = items * (blockIdx.x + 1) / grid;
    while (lo < hi) {
        const int64_t q = lo / parts;
        const int j0 = (int)(lo - q * parts);
        const int64_t left = hi - lo;
        const int j1 = left < (int64_t)(parts - j0) ? j0 + (int)left : parts;
        const int p = full * grid + (int)q;
        es_one_perm<T, RankT, WARPS, STAGE, WPL>(ranks + (int64_t)p * G, sorted_abs + (int64_t)p * G, G, set_off,
                                                  set_genes, set_order, decay, K, es + col0 + p, es_stride, s_w,
                                                  s_rank, bm, &next_set, j0, j1, parts);
        lo += j1 - j0;
    }
}

// Persistent multi-instance form: every CTA takes (instance, permutation)
// items from a global counter until all are done; items run in task order
// (tasks sorted by decreasing cost by the caller) and a task's permutations
// in order.  item_end[t] = items of tasks 0..t; Gmax sizes the staging and
// the bitmap regions of the size class (every task: G <= Gmax, and
// G <= 1024*WPL for WPL > 0).
template <class T, class RankT, int WARPS, int STAGE, int WPL>
__global__ void __launch_bounds__(WARPS * 32)
es_batch_kernel(const EsTask<T>* __restrict__ tasks, const int64_t* __restrict__ item_end, int ntasks,
                int64_t nitems, unsigned long long* __restrict__ counter, int Gmax) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int next_set;
    __shared__ long long s_item;
    const int region = WPL > 0 ? WPL * 32 : (Gmax + 31) >> 5;
    T* s_w;
    RankT* s_rank;
    uint32_t* bm;
    es_smem_layout<T, RankT, STAGE>(smem, Gmax, region, s_w, s_rank, bm);
    for (int w = threadIdx.x & 31; w < region; w += 32) bm[w] = 0u;
    while (true) {
        __syncthreads();  // everyone read s_item of the previous round
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const int64_t item = s_item;
        if (item >= nitems) break;
        int lo = 0, hi = ntasks - 1;  // first task with item_end > item
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (item_end[mid] > item) hi = mid; else lo = mid + 1;
        }
        const EsTask<T>& tk = tasks[lo];
        const int64_t p = item - (lo > 0 ? item_end[lo - 1] : 0);
        const RankT* rk = static_cast<const RankT*>(tk.ranks) + p * tk.G;
        es_one_perm<T, RankT, WARPS, STAGE, WPL>(rk, tk.sorted + p * tk.G, tk.G, tk.off, tk.genes, tk.order,
                                                  tk.decay, tk.K, tk.es + tk.col0 + p, tk.stride, s_w, s_rank, bm,
                                                  &next_set);
    }
}

// words of a warp's bitmap region: WPL*32 for the register procedure
inline int es_region_words(int G, int wpl) { return wpl > 0 ? wpl * 32 : (G + 31) >> 5; }

inline int es_wpl(int G, bool ranks16) {
    const int need = (((G + 31) >> 5) + 31) >> 5;
    if (!ranks16) return 0;
    for (int w : {4, 8, 12, 16, 20, 24, 32, 40, 48, 64})
        if (need <= w) return w;
    return 0;
}

template <class T, class RankT, int WARPS, int STAGE>
size_t es_smem_bytes(int G) {
    const int region = es_region_words(G, es_wpl(G, sizeof(RankT) == 2));
    const size_t s = (es_stage_bytes<T, RankT, STAGE>(G) + 15) & ~(size_t)15;
    return s + sizeof(uint32_t) * (size_t)region * WARPS;
}

template <class T, class RankT, int WARPS, int STAGE, int WPL>
cudaError_t launch_es_v(const RankT* ranks, const T* sorted_abs, int G, int P, const int64_t* off,
                        const int32_t* genes, const int32_t* order, const T* decay, int K, T* es, int64_t stride,
                        int64_t col0, int grid, cudaStream_t st, const int* K_dev) {
    const size_t smem = es_smem_bytes<T, RankT, WARPS, STAGE>(G);
    auto kern = es_kernel<T, RankT, WARPS, STAGE, WPL>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;  // resident CTAs per SM: the grid fills the device once
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    grid *= per_sm;
    kern<<<grid, WARPS * 32, smem, st>>>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0,
                                         K_dev);
    launches_add(1);
    return cudaGetLastError();
}

template <class T, class RankT, int WARPS, int STAGE>
cudaError_t launch_es_w(const RankT* ranks, const T* sorted_abs, int G, int P, const int64_t* off,
                        const int32_t* genes, const int32_t* order, const T* decay, int K, T* es, int64_t stride,
                        int64_t col0, int grid, cudaStream_t st, const int* K_dev) {
    // words per lane for the register-resident list procedure (u16 positions);
    // 32-bit ranks (G > 65,536) always take the general procedure
    if constexpr (sizeof(RankT) == 4) {
        if (STAGE >= 2) return cudaErrorInvalidValue;
        return launch_es_v<T, RankT, WARPS, STAGE, 0>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride,
                                                      col0, grid, st, K_dev);
    } else if constexpr (STAGE >= 2 || WARPS == 24) {  // partial staging / 24 warps: the large-G classes
        switch (es_wpl(G, true)) {
            case 24: return launch_es_v<T, RankT, WARPS, STAGE, 24>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 32: return launch_es_v<T, RankT, WARPS, STAGE, 32>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 40: return launch_es_v<T, RankT, WARPS, STAGE, 40>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 48: return launch_es_v<T, RankT, WARPS, STAGE, 48>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 64: return launch_es_v<T, RankT, WARPS, STAGE, 64>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            default: return cudaErrorInvalidValue;
        }
    } else {
        switch (es_wpl(G, true)) {
            case 4: return launch_es_v<T, RankT, WARPS, STAGE, 4>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 8: return launch_es_v<T, RankT, WARPS, STAGE, 8>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 12: return launch_es_v<T, RankT, WARPS, STAGE, 12>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 16: return launch_es_v<T, RankT, WARPS, STAGE, 16>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 20: return launch_es_v<T, RankT, WARPS, STAGE, 20>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 24: return launch_es_v<T, RankT, WARPS, STAGE, 24>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 32: return launch_es_v<T, RankT, WARPS, STAGE, 32>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
            case 40:  // the staging of ranks and weights never fits beside these regions
                if constexpr (STAGE == 0) return launch_es_v<T, RankT, WARPS, 0, 40>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
                return cudaErrorInvalidValue;
            case 48:
                if constexpr (STAGE == 0) return launch_es_v<T, RankT, WARPS, 0, 48>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
                return cudaErrorInvalidValue;
            case 64:
                if constexpr (STAGE == 0) return launch_es_v<T, RankT, WARPS, 0, 64>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, K_dev);
                return cudaErrorInvalidValue;
            default: break;
        }
        return launch_es_v<T, RankT, WARPS, STAGE, 0>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride,
                                                      col0, grid, st, K_dev);
    }
}

template <class T, class RankT>
cudaError_t launch_es_t(const RankT* ranks, const T* sorted_abs, int G, int P, const int64_t* off,
                        const int32_t* genes, const int32_t* order, const T* decay, int K, T* es, int64_t stride,
                        int64_t col0, EsTuning tune, cudaStream_t st, const int* K_dev) {
    int dev = 0, max_smem = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t cap = (size_t)max_smem - 64;  // static shared counter
    const int grid = sms;  // times the resident CTAs per SM; the last round's permutations are split by sets
    // candidates in the automatic order: 32 warps first (staging ranks and
    // weights, then weights only, 24 warps with weights only, 32 with ranks
    // only, 32 with none), then fewer warps -- warps count for more than
    // staging (measured on 24,000-40,000 genes); the partial stagings are for
    // the large-G classes (24-64 bitmap words per lane)
    struct Cand { int warps; int stage; size_t smem; };
    const Cand cands[] = {{32, 1, es_smem_bytes<T, RankT, 32, 1>(G)},
                          {32, 3, es_smem_bytes<T, RankT, 32, 3>(G)},
                          {24, 3, es_smem_bytes<T, RankT, 24, 3>(G)},
                          {32, 2, es_smem_bytes<T, RankT, 32, 2>(G)},
                          {32, 0, es_smem_bytes<T, RankT, 32, 0>(G)},
                          {24, 0, es_smem_bytes<T, RankT, 24, 0>(G)},
                          {16, 1, es_smem_bytes<T, RankT, 16, 1>(G)},
                          {24, 2, es_smem_bytes<T, RankT, 24, 2>(G)},
                          {16, 2, es_smem_bytes<T, RankT, 16, 2>(G)},
                          {8, 1, es_smem_bytes<T, RankT, 8, 1>(G)},
                          {16, 0, es_smem_bytes<T, RankT, 16, 0>(G)},
                          {8, 0, es_smem_bytes<T, RankT, 8, 0>(G)}};
    const int wpl = es_wpl(G, sizeof(RankT) == 2);
    for (const Cand& c : cands) {
        if (c.smem > cap) continue;
        if ((c.stage >= 2 || c.warps == 24) && wpl < 24) continue;
        if (c.stage == 1 && wpl >= 40) continue;
        if (tune.warps && tune.warps != c.warps) continue;
        if (tune.stage >= 0 && tune.stage != c.stage) continue;
#define GSEA_ES(W, S) \
    return launch_es_w<T, RankT, W, S>(ranks, sorted_abs, G, P, off, genes, order, decay, K, es, stride, col0, grid, st, \
                                       K_dev)
        if (c.warps == 32 && c.stage == 1) GSEA_ES(32, 1);
        if (c.warps == 16 && c.stage == 1) GSEA_ES(16, 1);
        if (c.warps == 8 && c.stage == 1) GSEA_ES(8, 1);
        if (c.warps == 32 && c.stage == 3) GSEA_ES(32, 3);
        if (c.warps == 24 && c.stage == 3) GSEA_ES(24, 3);
        if (c.warps == 32 && c.stage == 2) GSEA_ES(32, 2);
        if (c.warps == 24 && c.stage == 2) GSEA_ES(24, 2);
        if (c.warps == 24 && c.stage == 0) GSEA_ES(24, 0);
        if (c.warps == 16 && c.stage == 2) GSEA_ES(16, 2);
        if (c.warps == 32) GSEA_ES(32, 0);
        if (c.warps == 16) GSEA_ES(16, 0);
        GSEA_ES(8, 0);
#undef GSEA_ES
    }
    return cudaErrorInvalidValue;  // the requested configuration does not fit
}

template <class T, int WARPS, int STAGE, int WPL>
cudaError_t launch_es_batch_v(const EsTask<T>* tasks, const int64_t* item_end, int ntasks, int64_t nitems,
                              unsigned long long* counter, int Gmax, cudaStream_t st) {
    const size_t smem = es_smem_bytes<T, uint16_t, WARPS, STAGE>(Gmax);
    auto kern = es_batch_kernel<T, uint16_t, WARPS, STAGE, WPL>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 1, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    const int64_t want = (int64_t)sms * per_sm;
    const int grid = (int)(nitems < want ? nitems : want);
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    kern<<<grid, WARPS * 32, smem, st>>>(tasks, item_end, ntasks, nitems, counter, Gmax);
    launches_add(1);
    return cudaGetLastError();
}

template <class T, int WARPS, int STAGE>
cudaError_t launch_es_batch_w(const EsTask<T>* tasks, const int64_t* item_end, int ntasks, int64_t nitems,
                              unsigned long long* counter, int Gmax, int wpl, cudaStream_t st) {
    if constexpr (STAGE >= 2 || WARPS == 24) {
        switch (wpl) {
            case 24: return launch_es_batch_v<T, WARPS, STAGE, 24>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            case 32: return launch_es_batch_v<T, WARPS, STAGE, 32>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            case 40: return launch_es_batch_v<T, WARPS, STAGE, 40>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            case 48: return launch_es_batch_v<T, WARPS, STAGE, 48>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            case 64: return launch_es_batch_v<T, WARPS, STAGE, 64>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            default: return cudaErrorInvalidValue;
        }
    } else {
    switch (wpl) {
        case 4: return launch_es_batch_v<T, WARPS, STAGE, 4>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 8: return launch_es_batch_v<T, WARPS, STAGE, 8>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 12: return launch_es_batch_v<T, WARPS, STAGE, 12>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 16: return launch_es_batch_v<T, WARPS, STAGE, 16>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 20: return launch_es_batch_v<T, WARPS, STAGE, 20>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 24: return launch_es_batch_v<T, WARPS, STAGE, 24>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 32: return launch_es_batch_v<T, WARPS, STAGE, 32>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        case 40:
            if constexpr (STAGE == 0) return launch_es_batch_v<T, WARPS, 0, 40>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            return cudaErrorInvalidValue;
        case 48:
            if constexpr (STAGE == 0) return launch_es_batch_v<T, WARPS, 0, 48>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            return cudaErrorInvalidValue;
        case 64:
            if constexpr (STAGE == 0) return launch_es_batch_v<T, WARPS, 0, 64>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
            return cudaErrorInvalidValue;
        case 0: return launch_es_batch_v<T, WARPS, STAGE, 0>(tasks, item_end, ntasks, nitems, counter, Gmax, st);
        default: return cudaErrorInvalidValue;
    }
    }
}

}  // namespace

template <class T>
cudaError_t launch_es_batch(const EsTask<T>* tasks, const int64_t* item_end, int ntasks, int64_t nitems,
                            unsigned long long* counter, int Gmax, int wpl, EsTuning tune, cudaStream_t st) {
    if (nitems <= 0 || ntasks <= 0) return cudaSuccess;
    if (Gmax > 65536 || es_wpl(Gmax, true) != wpl) return cudaErrorInvalidValue;
    int dev = 0, max_smem = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t cap = (size_t)max_smem - 64;
    struct Cand { int warps; int stage; size_t smem; };
    const Cand cands[] = {{32, 1, es_smem_bytes<T, uint16_t, 32, 1>(Gmax)},
                          {32, 3, es_smem_bytes<T, uint16_t, 32, 3>(Gmax)},
                          {24, 3, es_smem_bytes<T, uint16_t, 24, 3>(Gmax)},
                          {32, 2, es_smem_bytes<T, uint16_t, 32, 2>(Gmax)},
                          {32, 0, es_smem_bytes<T, uint16_t, 32, 0>(Gmax)},
                          {24, 0, es_smem_bytes<T, uint16_t, 24, 0>(Gmax)},
                          {16, 1, es_smem_bytes<T, uint16_t, 16, 1>(Gmax)},
                          {24, 2, es_smem_bytes<T, uint16_t, 24, 2>(Gmax)},
                          {16, 2, es_smem_bytes<T, uint16_t, 16, 2>(Gmax)},
                          {8, 1, es_smem_bytes<T, uint16_t, 8, 1>(Gmax)},
                          {16, 0, es_smem_bytes<T, uint16_t, 16, 0>(Gmax)},
                          {8, 0, es_smem_bytes<T, uint16_t, 8, 0>(Gmax)}};
    for (const Cand& c : cands) {
        if (c.smem > cap) continue;
        if ((c.stage >= 2 || c.warps == 24) && wpl < 24) continue;
        if (c.stage == 1 && wpl >= 40) continue;
        if (tune.warps && tune.warps != c.warps) continue;
        if (tune.stage >= 0 && tune.stage != c.stage) continue;
#define GSEA_ESB(W, S) return launch_es_batch_w<T, W, S>(tasks, item_end, ntasks, nitems, counter, Gmax, wpl, st)
        if (c.warps == 32 && c.stage == 1) GSEA_ESB(32, 1);
        if (c.warps == 16 && c.stage == 1) GSEA_ESB(16, 1);
        if (c.warps == 8 && c.stage == 1) GSEA_ESB(8, 1);
        if (c.warps == 32 && c.stage == 3) GSEA_ESB(32, 3);
        if (c.warps == 24 && c.stage == 3) GSEA_ESB(24, 3);
        if (c.warps == 32 && c.stage == 2) GSEA_ESB(32, 2);
        if (c.warps == 24 && c.stage == 2) GSEA_ESB(24, 2);
        if (c.warps == 24 && c.stage == 0) GSEA_ESB(24, 0);
        if (c.warps == 16 && c.stage == 2) GSEA_ESB(16, 2);
        if (c.warps == 32) GSEA_ESB(32, 0);
        if (c.warps == 16) GSEA_ESB(16, 0);
        GSEA_ESB(8, 0);
#undef GSEA_ESB
    }
    return cudaErrorInvalidValue;
}

template <class T>
cudaError_t launch_es(const void* ranks, bool ranks16, const T* sorted_abs, int G, int num_perms,
                      const int64_t* set_offsets, const int32_t* set_genes, const int32_t* set_order,
                      const T* decay, int K, T* es, int64_t es_stride, int64_t perm_col0, cudaStream_t st,
                      EsTuning tune, const int* K_dev) {
    if (num_perms <= 0 || K <= 0) return cudaSuccess;
    if (ranks16)
        return launch_es_t<T, uint16_t>(static_cast<const uint16_t*>(ranks), sorted_abs, G, num_perms, set_offsets,
                                        set_genes, set_order, decay, K, es, es_stride, perm_col0, tune, st, K_dev);
    return launch_es_t<T, uint32_t>(static_cast<const uint32_t*>(ranks), sorted_abs, G, num_perms, set_offsets,
                                    set_genes, set_order, decay, K, es, es_stride, perm_col0, tune, st, K_dev);
}

// decay[n] = (T)(1.0 / (G - n)) for n < G, 0 for n = G: the miss step of a
// set with n hits, rounded from double as the reference does
// (enrichment_scores.cuh:178)
template <class T>
__global__ void decay_table_kernel(int G, T* decay) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n <= G) decay[n] = n < G ? (T)(1.0 / (double)(G - n)) : T(0);
}

template <class T>
cudaError_t launch_decay_table(int G, T* decay, cudaStream_t st) {
    decay_table_kernel<T><<<(G + 256) / 256, 256, 0, st>>>(G, decay);
    launches_add(1);
    return cudaGetLastError();
}


}  // namespace gsea
