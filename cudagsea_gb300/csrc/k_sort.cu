// k_sort.cu -- per-permutation stable ranking of genes by metric.
//
// Replaces pathway_sort_gpu (src/include/batched_sort.cuh:91-269), which runs
// CUB's DeviceSegmentedRadixSort in descending order on (metric, gene id)
// pairs, 128 segments per call.  Here one CTA owns one permutation's segment
// and runs an LSD radix sort with 8-bit digits on the IEEE radix key:
//
//   * stable, so tied metrics keep ascending gene order (CUB's semantics);
//   * -0.0 ranks below +0.0 and NaNs sit at the two ends, as with CUB;
//   * digit ranks inside a warp come from per-bit ballots (lanes with equal
//     digits) and one shared-memory atomicAdd per digit group on the warp's
//     counter; ranks across warps from a digit-major scan of the per-warp
//     counters.
//
// Variants:
//   sort_regs_kernel   the whole segment lives in registers (1024 threads x
//                      ITEMS keys); each pass exchanges keys and gene ids
//                      through one shared-memory buffer.  fp32, G <= 20,480.
//   sort_cluster_kernel the same over a cluster of two CTAs (SMs), the
//                      exchange through distributed shared memory: fp32,
//                      20,480 < G <= 40,960; fp64 (keys and gene ids
//                      exchanged separately), one CTA up to 10,240 genes,
//                      two up to 20,480.
//   sort_tiled_kernel  any key width and any G: the segment ping-pongs
//                      between two per-CTA global buffers; one read counts
//                      the digits of every pass, and each pass streams the
//                      segment in tiles of 4,096 items staged in shared
//                      memory by double-buffered bulk copies.
//
// Outputs per permutation: ranks[g] (position of gene g), sorted_abs[r]
// (|metric| of the gene at position r, the running-sum weight of
// enrichment_scores.cuh:146,183) and optionally order[r] (gene at position r).
#include <cooperative_groups.h>
#include <type_traits>

#include "bulk.cuh"
#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace gsea {
namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;

template <class U>
__device__ __forceinline__ uint32_t digit_of(U key, int shift) {
    return (uint32_t)(key >> shift) & 0xFFu;
}

// lanes holding the same 8-bit digit (BITS significant bits), from one
// ballot per bit: cheaper than the general match instruction
template <int BITS>
__device__ __forceinline__ uint32_t match_digit(uint32_t dig) {
    uint32_t peers = kFullMask;
#pragma unroll
    for (int b = 0; b < BITS; b++) {
        const bool set = (dig >> b) & 1u;
        const uint32_t vote = __ballot_sync(kFullMask, set);
        peers &= set ? vote : ~vote;
    }
    return peers;
}

// inverse of RadixKey<T>::from
template <class T>
__device__ __forceinline__ T value_of(typename RadixKey<T>::U key, bool descending);
template <>
__device__ __forceinline__ float value_of<float>(uint32_t key, bool descending) {
    uint32_t u = descending ? ~key : key;
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(u);
}
template <>
__device__ __forceinline__ double value_of<double>(unsigned long long key, bool descending) {
    unsigned long long u = descending ? ~key : key;
    u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)u);
}

template <class RankT, class T>
__device__ __forceinline__ void emit(int64_t base, int pos, uint32_t gene, T v, RankT* ranks,
                                     T* sorted_abs, uint32_t* order) {
    ranks[base + gene] = (RankT)pos;
    sorted_abs[base + pos] = cuabs(v);
    if (order) order[base + pos] = gene;
}

// Offsets of a tile's items (all 1,024 threads; four __syncthreads()).  In:
// cnt[w][d], the count of warp w's items with digit d (w < 32, d < 256); base[d],
// the running output offset of digit d.  Out: cnt[w][d] = the tile-local
// position of warp w's first item with digit d (digit-major: the digit's
// start in the tile plus the earlier warps' items), delta[d] = base[d] - the
// digit's start in the tile (a tile position + delta is the destination),
// base[d] advanced by the tile's count.  Thread (q, d) scans warps 8q..8q+7 of
// digit d; warps 0-7 scan the 256 digit totals.
__device__ __forceinline__ void tile_offsets(uint32_t (*cnt)[256], uint32_t (*qsum)[256], uint32_t* warp_sums,
                                             uint32_t* toff, uint32_t* delta, uint32_t* base) {
    static_assert(kWarps == 32, "four quarters of eight warps");
    const int d = threadIdx.x & 255, q = threadIdx.x >> 8, lane = threadIdx.x & 31;
    uint32_t c[8];
#pragma unroll
    for (int i = 0; i < 8; i++) c[i] = cnt[8 * q + i][d];
    uint32_t run = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t x = c[i];
        c[i] = run;
        run += x;
    }
    qsum[q][d] = run;
    __syncthreads();
    uint32_t off = 0;
    for (int j = 0; j < q; j++) off += qsum[j][d];
    if (q == 0) {  // warps 0-7: exclusive scan of the digit totals
        const uint32_t total = qsum[0][d] + qsum[1][d] + qsum[2][d] + qsum[3][d];
        uint32_t incl = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[d >> 5] = incl;
        toff[d] = incl - total;  // within its group of 32 digits; groups added below
        delta[d] = total;        // the digit total, until the groups are added
    }
    __syncthreads();
    if (q == 0) {
        uint32_t before = 0;
        for (int w = 0; w < (d >> 5); w++) before += warp_sums[w];
        const uint32_t start = toff[d] + before, total = delta[d];
        toff[d] = start;
        delta[d] = base[d] - start;
        base[d] += total;
    }
    __syncthreads();
    off += toff[d];
#pragma unroll
    for (int i = 0; i < 8; i++) cnt[8 * q + i][d] = c[i] + off;
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Digit counters of the register sort: 16 bits each (a warp counts at most
// 32*ITEMS <= 640 items of a digit, a scanned offset is below TILE <= 20,480),
// two digits to a 32-bit word so that a shifted atomicAdd updates one half
// without carry into the other.
__device__ __forceinline__ uint32_t cnt16_add(uint32_t* words, uint32_t dig, uint32_t n) {
    const uint32_t sh = (dig & 1u) << 4;
    return (atomicAdd(&words[dig >> 1], n << sh) >> sh) & 0xFFFFu;
}

// fp32 keys, the whole segment in registers (1024 threads x ITEMS keys).  A
// pass ranks every key inside its warp (per-bit ballots, one shared atomic
// per digit group), scans the per-warp digit counters digit-major, and moves
// each (key, gene id) pair as one 8-byte slot through the exchange buffer:
// one scatter, one gather, two barriers.
template <class T, class RankT, int ITEMS>
__device__ __forceinline__ void
sort_regs_body(int bx, int gx, const T* __restrict__ keys, int G, int num_perms, bool descending,
               RankT* __restrict__ ranks, T* __restrict__ sorted_abs, uint32_t* __restrict__ order) {
    using U = typename RadixKey<T>::U;
    static_assert(sizeof(U) == 4, "register sort: fp32 keys");
    constexpr int TILE = kThreads * ITEMS;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* exch = reinterpret_cast<unsigned long long*>(smem);      // [TILE] (key, gene id)
    uint16_t* dst16 = reinterpret_cast<uint16_t*>(smem + 8 * (size_t)TILE);      // [TILE]
    uint16_t(*cnt)[256] = reinterpret_cast<uint16_t(*)[256]>(smem + 10 * (size_t)TILE);
    uint32_t* tot = reinterpret_cast<uint32_t*>(cnt + kWarps);
    uint32_t* warp_sums = tot + 256;
    uint32_t* flag = warp_sums + 8;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const int my0 = warp * 32 * ITEMS + lane;  // slot of item i: my0 + 32*i
    uint32_t* wcnt = reinterpret_cast<uint32_t*>(cnt[warp]);  // this warp's 128 counter words
    if (threadIdx.x == 0) *flag = 0u;
    __syncthreads();

    for (int p = bx; p < num_perms; p += gx) {
        const T* kp = keys + (int64_t)p * G;
        U key[ITEMS];
        uint32_t val[ITEMS];
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
            const int pos = my0 + 32 * i;
            key[i] = pos < G ? RadixKey<T>::from(kp[pos], descending) : ~U(0);
            val[i] = (uint32_t)pos;
        }
        for (int shift = 0; shift < 8 * (int)sizeof(U); shift += 8) {
            for (int w = lane; w < 128; w += 32) wcnt[w] = 0u;
            __syncwarp();
            // rank within the warp: the lowest lane of each digit group adds
            // the group's size to the warp's digit counter; the atomics of
            // successive items retire in program order, so ranks follow the
            // logical item order (stable)
#pragma unroll
            for (int i = 0; i < ITEMS; i++) {
                const uint32_t dig = digit_of(key[i], shift);
                const uint32_t peers = match_digit<8>(dig);
                const int leader = __ffs(peers) - 1;
                uint32_t before = 0;
                if (lane == leader) before = cnt16_add(wcnt, dig, (uint32_t)__popc(peers));
                before = __shfl_sync(kFullMask, before, leader);
                dst16[my0 + 32 * i] = (uint16_t)(before + __popc(peers & lt));
            }
            __syncthreads();
            // digit-major exclusive scan of cnt[w][d] (destinations of this tile)
            uint32_t run = 0;
            if (threadIdx.x < 256) {
                for (int w = 0; w < kWarps; w++) {
                    const uint32_t c = cnt[w][threadIdx.x];
                    cnt[w][threadIdx.x] = (uint16_t)run;
                    run += c;
                }
                tot[threadIdx.x] = run;
                if (run == (uint32_t)TILE) *flag = 1u;
                uint32_t incl = run;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
                    if (lane >= o) incl += y;
                }
                if (lane == 31) warp_sums[threadIdx.x >> 5] = incl;
                run = incl - run;  // exclusive within this warp of digits
            }
            __syncthreads();
            const bool skip = *flag != 0u;
            if (threadIdx.x < 256 && !skip) {
                uint32_t before = 0;
                for (int w = 0; w < (threadIdx.x >> 5); w++) before += warp_sums[w];
                const uint32_t excl = before + run;
                for (int w = 0; w < kWarps; w++) cnt[w][threadIdx.x] = (uint16_t)(cnt[w][threadIdx.x] + excl);
            }
            __syncthreads();
            if (threadIdx.x == 0) *flag = 0u;
            if (skip) continue;  // every item has the same digit: order unchanged
#pragma unroll
            for (int i = 0; i < ITEMS; i++) {
                const uint32_t dig = digit_of(key[i], shift);
                const uint32_t d = cnt[warp][dig] + dst16[my0 + 32 * i];
                exch[d] = (unsigned long long)key[i] | ((unsigned long long)val[i] << 32);
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < ITEMS; i++) {
                const unsigned long long e = exch[my0 + 32 * i];
                key[i] = (U)(e & 0xFFFFFFFFull);
                val[i] = (uint32_t)(e >> 32);
            }
            __syncthreads();
        }
        // weights (and gene ids) at their positions: coalesced; ranks by gene:
        // gathered in shared memory first so the global write is coalesced
        // too (exch is free: every pass ended with a barrier)
        const int64_t base = (int64_t)p * G;
        RankT* s_rk = reinterpret_cast<RankT*>(exch);  // [G] (exch holds TILE >= G slots)
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
            const int pos = my0 + 32 * i;
            if (val[i] < (uint32_t)G) {
                s_rk[val[i]] = (RankT)pos;
                sorted_abs[base + pos] = cuabs(value_of<T>(key[i], descending));
                if (order) order[base + pos] = val[i];
            }
        }
        __syncthreads();
        for (int g = threadIdx.x; g < G; g += kThreads) ranks[base + g] = s_rk[g];
        __syncthreads();  // exch is reused by the next permutation
    }
}

template <class T, class RankT, int ITEMS>
__global__ void __launch_bounds__(kThreads, 1)
sort_regs_kernel(const T* __restrict__ keys, int G, int num_perms, bool descending,
                 RankT* __restrict__ ranks, T* __restrict__ sorted_abs, uint32_t* __restrict__ order) {
    sort_regs_body<T, RankT, ITEMS>(blockIdx.x, gridDim.x, keys, G, num_perms, descending, ranks, sorted_abs, order);
}

// every instance of a batch (same ITEMS class) at once: blockIdx.z = the
// instance, its gridDim.x CTAs share its permutations
template <class T, class RankT, int ITEMS>
__global__ void __launch_bounds__(kThreads, 1) sort_regs_multi(const SortTask* __restrict__ tasks) {
    const SortTask& t = tasks[blockIdx.z];
    sort_regs_body<T, RankT, ITEMS>(blockIdx.x, gridDim.x, static_cast<const T*>(t.keys), t.G, t.num_perms,
                                    t.descending != 0, static_cast<RankT*>(t.ranks), static_cast<T*>(t.sorted),
                                    t.order);
}

template <class T, int ITEMS>
size_t regs_smem_bytes() {
    return 10 * (size_t)kThreads * ITEMS + sizeof(uint16_t) * kWarps * 256 + sizeof(uint32_t) * (256 + 8 + 4);
}

// ---------------------------------------------------------------------------
// Cluster form (G <= CL x 1024 x ITEMS; fp32 beyond 20,480 genes, fp64 from
// the smallest G): one cluster of CL CTAs (1 or 2) per permutation, CTA r holding the items of positions
// [r*TILE, (r+1)*TILE) in registers as sort_regs_kernel does.  A pass ranks
// items inside each warp as there, then the CTAs' digit totals are read
// through distributed shared memory: an item's destination is
//   sum over digits < d of all CTAs' totals + the totals of d of the CTAs
//   before its own + the earlier warps of its CTA + its rank in its warp,
// stable because lower CTAs hold the earlier positions.  Each (key, gene id)
// pair -- one 8-byte slot at up to 16 items per thread, else keys then gene
// ids -- is stored into the exchange buffer of the CTA that owns its
// destination (local or remote shared-memory stores) and gathered back in
// position order.  Cluster barriers separate the phases; nothing spins.
//
template <class T, int ITEMS>
constexpr bool cluster_packed() { return sizeof(typename RadixKey<T>::U) == 4 && ITEMS <= 16; }

template <class T, class RankT, int ITEMS, int CL>
__device__ __forceinline__ void
sort_cluster_body(int bx, int gx, const T* __restrict__ keys, int G, int num_perms, bool descending,
                  RankT* __restrict__ ranks, T* __restrict__ sorted_abs, uint32_t* __restrict__ order) {
    using U = typename RadixKey<T>::U;
    constexpr bool PACK = cluster_packed<T, ITEMS>();
    using E = typename std::conditional<PACK, unsigned long long, U>::type;  // exchange slot
    constexpr int TILE = kThreads * ITEMS;
    extern __shared__ __align__(16) unsigned char smem[];
    E* exch = reinterpret_cast<E*>(smem);                                     // [TILE]
    uint16_t* dst16 = reinterpret_cast<uint16_t*>(smem + sizeof(E) * TILE);  // [TILE]
    uint32_t(*cnt)[256] = reinterpret_cast<uint32_t(*)[256]>(smem + (sizeof(E) + 2) * TILE);
    uint32_t* tot = reinterpret_cast<uint32_t*>(cnt + kWarps);  // this CTA's digit totals
    uint32_t* base = tot + 256;                                  // destination base per digit
    uint32_t* warp_sums = base + 256;                            // [8]

    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    // the exchange buffer holding positions [r*TILE, (r+1)*TILE): CTA r's
    auto buf = [&](uint32_t r) -> E* { return (int)r == rank ? exch : cluster.map_shared_rank(exch, (int)r); };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const int my0 = warp * 32 * ITEMS + lane;  // slot of item i: my0 + 32*i
    const int first = rank * TILE;              // global position of slot 0
    const int clusters = gx / CL;

    for (int p = bx / CL; p < num_perms; p += clusters) {
        const T* kp = keys + (int64_t)p * G;
        U key[ITEMS];
        uint32_t val[ITEMS];
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
            const int pos = first + my0 + 32 * i;
            key[i] = pos < G ? RadixKey<T>::from(kp[pos], descending) : ~U(0);
            val[i] = (uint32_t)pos;
        }
        for (int shift = 0; shift < 8 * (int)sizeof(U); shift += 8) {
            for (int d = lane; d < 256; d += 32) cnt[warp][d] = 0;
            __syncwarp();
#pragma unroll
            for (int i = 0; i < ITEMS; i++) {
                const uint32_t dig = digit_of(key[i], shift);
                const uint32_t peers = match_digit<8>(dig);
                const int leader = __ffs(peers) - 1;
                uint32_t before = 0;
                if (lane == leader) before = atomicAdd(&cnt[warp][dig], (uint32_t)__popc(peers));
                before = __shfl_sync(kFullMask, before, leader);
                dst16[my0 + 32 * i] = (uint16_t)(before + __popc(peers & lt));
            }
            __syncthreads();
            // exclusive over the warps, per digit; this CTA's totals
            if (threadIdx.x < 256) {
                uint32_t run = 0;
                for (int w = 0; w < kWarps; w++) {
                    const uint32_t c = cnt[w][threadIdx.x];
                    cnt[w][threadIdx.x] = run;
                    run += c;
                }
                tot[threadIdx.x] = run;
            }
            // both CTAs' totals visible; the peer finished last pass's gather
            cluster.sync();
            bool skip = false;
            if (threadIdx.x < 256) {
                const int d = threadIdx.x;
                uint32_t all = 0, lower = 0;  // every CTA's count of d; those of the CTAs before this one
#pragma unroll
                for (int r = 0; r < CL; r++) {
                    const uint32_t t = r == rank ? tot[d] : cluster.map_shared_rank(tot, r)[d];
                    all += t;
                    if (r < rank) lower += t;
                }
                uint32_t incl = all;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
                    if (lane >= o) incl += y;
                }
                if (lane == 31) warp_sums[d >> 5] = incl;
                base[d] = incl - all + lower;  // warp part; the earlier warps added below
                skip = all == (uint32_t)(CL * TILE);
            }
            // every key has the same digit (both CTAs see the same totals)
            const bool all_same = __syncthreads_or(skip) != 0;
            if (all_same) {
                cluster.sync();  // the peer has read this CTA's totals before they change
                continue;
            }
            if (threadIdx.x < 256) {
                uint32_t before = 0;
                for (int w = 0; w < (threadIdx.x >> 5); w++) before += warp_sums[w];
                const uint32_t b = base[threadIdx.x] + before;
                for (int w = 0; w < kWarps; w++) cnt[w][threadIdx.x] += b;
            }
            __syncthreads();
            if constexpr (PACK) {
                // key and gene id in one slot: one scatter, one gather
#pragma unroll
                for (int i = 0; i < ITEMS; i++) {
                    const uint32_t dig = digit_of(key[i], shift);
                    const uint32_t d = cnt[warp][dig] + dst16[my0 + 32 * i];  // global destination < CL*TILE
                    const E e = (E)key[i] | ((E)val[i] << 32);
                    buf(d / TILE)[d % TILE] = e;
                }
                cluster.sync();  // scattered (the peer read the totals before its scatter)
#pragma unroll
                for (int i = 0; i < ITEMS; i++) {
                    const E e = exch[my0 + 32 * i];
                    key[i] = (U)(e & 0xFFFFFFFFull);
                    val[i] = (uint32_t)(e >> 32);
                }
            } else {
#pragma unroll
                for (int i = 0; i < ITEMS; i++) {
                    const uint32_t dig = digit_of(key[i], shift);
                    const uint32_t d = cnt[warp][dig] + dst16[my0 + 32 * i];  // global destination < CL*TILE
                    dst16[my0 + 32 * i] = (uint16_t)d;
                    buf(d / TILE)[d % TILE] = key[i];
                }
                cluster.sync();
#pragma unroll
                for (int i = 0; i < ITEMS; i++) key[i] = exch[my0 + 32 * i];
                cluster.sync();  // both CTAs gathered their keys: the buffers take the gene ids
#pragma unroll
                for (int i = 0; i < ITEMS; i++) {
                    const uint32_t d = dst16[my0 + 32 * i];
                    reinterpret_cast<uint32_t*>(buf(d / TILE))[d % TILE] = val[i];
                }
                cluster.sync();
#pragma unroll
                for (int i = 0; i < ITEMS; i++) val[i] = reinterpret_cast<uint32_t*>(exch)[my0 + 32 * i];
            }
        }
        cluster.sync();  // both CTAs gathered: the buffers take the ranks
        // outputs: weights (and gene ids) at their positions, coalesced; the
        // rank of gene g staged in the shared memory of the CTA owning g
        const int64_t obase = (int64_t)p * G;
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
            const int pos = first + my0 + 32 * i;
            if (val[i] < (uint32_t)G) {
                const uint32_t v = val[i];
                reinterpret_cast<RankT*>(buf(v / TILE))[v % TILE] = (RankT)pos;
                sorted_abs[obase + pos] = cuabs(value_of<T>(key[i], descending));
                if (order) order[obase + pos] = v;
            }
        }
        cluster.sync();
        const RankT* s_rk = reinterpret_cast<const RankT*>(exch);
        const int g_end = min(G, first + TILE);
        for (int g = first + threadIdx.x; g < g_end; g += kThreads) ranks[obase + g] = s_rk[g - first];
        cluster.sync();  // the staging is reused by the next permutation
    }
}

template <class T, class RankT, int ITEMS, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(kThreads, 1)
sort_cluster_kernel(const T* __restrict__ keys, int G, int num_perms, bool descending,
                    RankT* __restrict__ ranks, T* __restrict__ sorted_abs, uint32_t* __restrict__ order) {
    sort_cluster_body<T, RankT, ITEMS, CL>(blockIdx.x, gridDim.x, keys, G, num_perms, descending, ranks, sorted_abs,
                                           order);
}

template <class T, class RankT, int ITEMS, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(kThreads, 1)
sort_cluster_multi(const SortTask* __restrict__ tasks) {
    const SortTask& t = tasks[blockIdx.z];
    sort_cluster_body<T, RankT, ITEMS, CL>(blockIdx.x, gridDim.x, static_cast<const T*>(t.keys), t.G, t.num_perms,
                                           t.descending != 0, static_cast<RankT*>(t.ranks), static_cast<T*>(t.sorted),
                                           t.order);
}

template <class T, int ITEMS>
size_t cluster_smem_bytes() {
    using U = typename RadixKey<T>::U;
    const size_t slot = cluster_packed<T, ITEMS>() ? 8 : sizeof(U);
    return (slot + 2) * (size_t)kThreads * ITEMS + sizeof(uint32_t) * (kWarps * 256 + 256 + 256 + 8);
}

// ---------------------------------------------------------------------------
// Tiled form (any key width, any G).  Each CTA owns two global ping-pong
// buffers of (radix key, gene id) with rows of Gp = G rounded up to a
// multiple of 4 items, so that every tile starts and ends on a 16-byte
// boundary.  Per permutation: one read of its metric values writes the radix
// keys into buffer A and counts the digits of every pass at once (one
// histogram per digit position); then every pass whose digit is not uniform
// streams buffer A in tiles of 4,096 items.  Each tile is staged in shared
// memory by bulk copies (keys, gene ids) into one of three stage buffers --
// the next two tiles' copies in flight while it is ranked -- ranked within
// its warps, put in digit order in the stage buffer it came from, and written
// to buffer B in runs of equal digits (consecutive threads, consecutive
// destinations).  The first pass that moves anything takes the gene ids as
// the identity and copies keys only.
constexpr int kTileItems = 4;
constexpr int kTile = kThreads * kTileItems;

__host__ __device__ __forceinline__ int tiled_row(int G) { return (G + 3) & ~3; }
template <class U>
__host__ __device__ __forceinline__ size_t tiled_cta_bytes(int G) {
    return (sizeof(U) + sizeof(uint32_t)) * 2 * (size_t)tiled_row(G);
}
// the stage buffers (keys, then gene ids): two tiles in flight while one is
// ranked
constexpr int kStages = 3;
template <class U>
constexpr size_t tiled_stage_bytes() { return kStages * (size_t)kTile * (sizeof(U) + sizeof(uint32_t)); }

// tile t of a (key, gene id) buffer into stage buffer b, completing on
// bar[b] (one thread); sizes rounded up to 16 bytes stay inside the
// tiled_row(G)-item rows.  With ident the gene ids are not copied.
template <class U>
__device__ __forceinline__ void tiled_issue(U* s_key, uint32_t* s_val, unsigned long long* bar, const U* kA,
                                            const uint32_t* vA, bool ident, int G, int t, int b) {
    const int t0 = t * kTile;
    const int n = min(kTile, G - t0);
    const uint32_t kbytes = (uint32_t)(((size_t)n * sizeof(U) + 15) & ~(size_t)15);
    const uint32_t vbytes = ident ? 0u : (uint32_t)(((size_t)n * 4 + 15) & ~(size_t)15);
    const uint32_t bb = smem_u32(&bar[b]);
    fence_proxy_async();
    mbar_expect_tx(bb, kbytes + vbytes);
    bulk_copy(smem_u32(s_key + (size_t)b * kTile), kA + t0, kbytes, bb);
    if (vbytes) bulk_copy(smem_u32(s_val + (size_t)b * kTile), vA + t0, vbytes, bb);
}

template <class T, class RankT>
__global__ void __launch_bounds__(kThreads, 1)
sort_tiled_kernel(const T* __restrict__ keys, int G, int num_perms, bool descending,
                  RankT* __restrict__ ranks, T* __restrict__ sorted_abs, uint32_t* __restrict__ order,
                  unsigned char* __restrict__ scratch, bool stage_ranks, int* __restrict__ error_flag) {
    using U = typename RadixKey<T>::U;
    constexpr int NPASS = (int)sizeof(U);
    // stage buffers [2][kTile] keys and [2][kTile] gene ids; after the
    // passes, the ranks by gene when stage_ranks
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    U* const s_key = reinterpret_cast<U*>(dyn_smem);
    uint32_t* const s_val = reinterpret_cast<uint32_t*>(dyn_smem + kStages * (size_t)kTile * sizeof(U));
    __shared__ uint32_t cnt[kWarps][256];
    __shared__ uint32_t qsum[4][256];
    __shared__ uint32_t hist[NPASS][256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t toff[256];
    __shared__ uint32_t delta[256];
    __shared__ uint32_t warp_sums[8];
    __shared__ int failed;
    __shared__ __align__(8) unsigned long long bar[kStages];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t lt = lanemask_lt();
    const int Gp = tiled_row(G);
    U* const k0 = reinterpret_cast<U*>(scratch + tiled_cta_bytes<U>(G) * blockIdx.x);
    uint32_t* const v0 = reinterpret_cast<uint32_t*>(k0 + 2 * (size_t)Gp);
    if (tid == 0) {
        for (int b = 0; b < kStages; b++) mbar_init(smem_u32(&bar[b]), 1);
        fence_mbar_init();
        failed = 0;
    }
    __syncthreads();
    uint32_t phases = 0u;  // bit b: parity of stage buffer b's barrier (the same in every thread)
    const int ntiles = (G + kTile - 1) / kTile;

    for (int p = blockIdx.x; p < num_perms; p += gridDim.x) {
        int a_off = 0;  // buffer A = rows at a_off, buffer B = rows at Gp - a_off
        bool ident = true;  // buffer A's gene ids are the identity (not yet written)
        const T* kp = keys + (int64_t)p * G;
        for (int i = tid; i < NPASS * 256; i += kThreads) (&hist[0][0])[i] = 0u;
        __syncthreads();
#pragma unroll 4
        for (int i = tid; i < G; i += kThreads) {
            const U k = RadixKey<T>::from(kp[i], descending);
            k0[i] = k;
#pragma unroll
            for (int s = 0; s < NPASS; s++) atomicAdd(&hist[s][digit_of(k, 8 * s)], 1u);
        }
        for (int s = 0; s < NPASS; s++) {
            // histograms complete / the previous pass's scatter done; a
            // uniform digit moves nothing
            if (__syncthreads_or(tid < 256 && hist[s][tid] == (uint32_t)G)) continue;
            const int shift = 8 * s;
            if (tid == 0) {  // the first two tiles
                tiled_issue<U>(s_key, s_val, bar, k0 + a_off, v0 + a_off, ident, G, 0, 0);
                if (ntiles > 1) tiled_issue<U>(s_key, s_val, bar, k0 + a_off, v0 + a_off, ident, G, 1, 1);
            }
            // exclusive scan of this position's digit counts into base
            {
                const uint32_t v = tid < 256 ? hist[s][tid] : 0u;
                uint32_t incl = v;
                if (tid < 256) {
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
                        if (lane >= o) incl += y;
                    }
                    if (lane == 31) warp_sums[warp] = incl;
                }
                __syncthreads();
                if (tid < 256) {
                    uint32_t before = 0;
                    for (int w = 0; w < warp; w++) before += warp_sums[w];
                    base[tid] = before + incl - v;
                }
            }
            for (int t = 0, buf = 0; t < ntiles; t++, buf = buf == kStages - 1 ? 0 : buf + 1) {
                const int t0 = t * kTile;
                const int n = min(kTile, G - t0);
                for (int d = lane; d < 256; d += 32) cnt[warp][d] = 0;
                if (!mbar_wait(smem_u32(&bar[buf]), (phases >> buf) & 1u)) failed = 1;
                phases ^= 1u << buf;
                __syncwarp();
                U* tk = s_key + (size_t)buf * kTile;
                uint32_t* tv = s_val + (size_t)buf * kTile;
                U k[kTileItems];
                uint32_t v[kTileItems], r[kTileItems], dg[kTileItems];
#pragma unroll
                for (int i = 0; i < kTileItems; i++) {
                    const int l = warp * 32 * kTileItems + 32 * i + lane;
                    const bool valid = l < n;
                    k[i] = valid ? tk[l] : U(0);
                    v[i] = valid ? (ident ? (uint32_t)(t0 + l) : tv[l]) : 0u;
                    dg[i] = valid ? digit_of(k[i], shift) : 256u;
                    const uint32_t peers = match_digit<9>(dg[i]);
                    const int leader = __ffs(peers) - 1;
                    uint32_t before = 0;
                    if (valid && lane == leader) before = atomicAdd(&cnt[warp][dg[i]], (uint32_t)__popc(peers));
                    before = __shfl_sync(kFullMask, before, leader);
                    r[i] = before + __popc(peers & lt);
                }
                __syncthreads();  // counters complete; both stage buffers read
                if (failed) {  // uniform: written before the barrier
                    if (tid == 0) {
                        // let the copies still in flight land before leaving
                        mbar_wait(smem_u32(&bar[buf]), ((phases >> buf) & 1u) ^ 1u);
                        const int nb = buf == kStages - 1 ? 0 : buf + 1;
                        if (t + 1 < ntiles) mbar_wait(smem_u32(&bar[nb]), (phases >> nb) & 1u);
                        if (error_flag) atomicExch(error_flag, 1);
                    }
                    return;
                }
                // tile t + 2's copies, into the buffer the previous tile used
                if (tid == 0 && t + 2 < ntiles)
                    tiled_issue<U>(s_key, s_val, bar, k0 + a_off, v0 + a_off, ident, G, t + 2,
                                   buf == 0 ? kStages - 1 : buf - 1);
                tile_offsets(cnt, qsum, warp_sums, toff, delta, base);
                // the tile in digit order, in the stage buffer it came from ...
#pragma unroll
                for (int i = 0; i < kTileItems; i++) {
                    if (dg[i] < 256u) {
                        const uint32_t lp = cnt[warp][dg[i]] + r[i];
                        tk[lp] = k[i];
                        tv[lp] = v[i];
                    }
                }
                __syncthreads();
                // ... then out in runs of equal digits: consecutive threads
                // write consecutive destinations within a run
                U* const kB = k0 + (Gp - a_off);
                uint32_t* const vB = v0 + (Gp - a_off);
#pragma unroll
                for (int i = 0; i < kTileItems; i++) {
                    const int lp = tid + i * kThreads;
                    if (lp < n) {
                        const U key = tk[lp];
                        const uint32_t dst = delta[digit_of(key, shift)] + (uint32_t)lp;
                        kB[dst] = key;
                        vB[dst] = tv[lp];
                    }
                }
            }
            a_off = Gp - a_off;
            ident = false;
        }
        __syncthreads();
        const int64_t b = (int64_t)p * G;
        const U* kA = k0 + a_off;
        const uint32_t* vA = v0 + a_off;
        if (stage_ranks) {
            // ranks by gene gathered in shared memory (over the stage
            // buffers, idle now), then written coalesced
            RankT* s_rk = reinterpret_cast<RankT*>(dyn_smem);
#pragma unroll 4
            for (int pos = tid; pos < G; pos += kThreads) {
                const uint32_t gene = ident ? (uint32_t)pos : vA[pos];
                s_rk[gene] = (RankT)pos;
                sorted_abs[b + pos] = cuabs(value_of<T>(kA[pos], descending));
                if (order) order[b + pos] = gene;
            }
            __syncthreads();
            for (int g = tid; g < G; g += kThreads) ranks[b + g] = s_rk[g];
        } else {
#pragma unroll 4
            for (int pos = tid; pos < G; pos += kThreads)
                emit<RankT, T>(b, pos, ident ? (uint32_t)pos : vA[pos], value_of<T>(kA[pos], descending), ranks,
                               sorted_abs, order);
        }
        __syncthreads();
    }
}

int g_num_sms = 0;
int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

template <class T, class RankT, int ITEMS>
cudaError_t launch_regs(const T* keys, int G, int P, bool desc, const SortBuffers& o, cudaStream_t st) {
    const size_t smem = regs_smem_bytes<T, ITEMS>();
    auto kern = sort_regs_kernel<T, RankT, ITEMS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = P < 4 * num_sms() ? P : 4 * num_sms();
    kern<<<grid, kThreads, smem, st>>>(keys, G, P, desc, static_cast<RankT*>(o.ranks),
                                       static_cast<T*>(o.sorted_abs), o.order);
    launches_add(1);
    return cudaGetLastError();
}

template <class T, class RankT, int ITEMS, int CL>
cudaError_t launch_cluster(const T* keys, int G, int P, bool desc, const SortBuffers& o, cudaStream_t st) {
    const size_t smem = cluster_smem_bytes<T, ITEMS>();
    auto kern = sort_cluster_kernel<T, RankT, ITEMS, CL>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 1;  // a one-CTA "cluster" may share its SM with another CTA
    if (CL == 1) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidValue;
    }
    const int groups = num_sms() * per_sm / CL > 0 ? num_sms() * per_sm / CL : 1;
    const int clusters = P < groups ? P : groups;
    kern<<<CL * clusters, kThreads, smem, st>>>(keys, G, P, desc, static_cast<RankT*>(o.ranks),
                                                static_cast<T*>(o.sorted_abs), o.order);
    launches_add(1);
    return cudaGetLastError();
}

// largest G of the register-resident forms (variant 1): fp32 keys and gene
// ids as 8-byte slots, 20 per thread over two CTAs; fp64 keys 10 per thread
// (16 spill registers at 1,024 threads)
template <class T>
constexpr int regs_max_genes() { return sizeof(T) == 4 ? 2 * kThreads * 20 : 2 * kThreads * 10; }

template <class T, class RankT>
cudaError_t launch_sort_t(const T* keys, int G, int P, bool desc, const SortBuffers& o, cudaStream_t st) {
    if (o.variant == 1 && G > regs_max_genes<T>()) return cudaErrorInvalidValue;
    if constexpr (sizeof(T) == 8) {
        // fp64: the cluster form holds the segment in registers (keys and
        // gene ids exchanged separately); one CTA up to 10,240 genes, a
        // two-CTA cluster beyond
        if (o.variant != 2) {
            if (G <= kThreads * 4) return launch_cluster<T, RankT, 4, 1>(keys, G, P, desc, o, st);
            if (G <= kThreads * 10) return launch_cluster<T, RankT, 10, 1>(keys, G, P, desc, o, st);
            if (G <= 2 * kThreads * 10) return launch_cluster<T, RankT, 10, 2>(keys, G, P, desc, o, st);
        }
    }
    if constexpr (sizeof(T) == 4) {
      if (o.variant != 2) {
        if (G <= kThreads * 4) return launch_regs<T, RankT, 4>(keys, G, P, desc, o, st);
        if (G <= kThreads * 8) return launch_regs<T, RankT, 8>(keys, G, P, desc, o, st);
        if (G <= kThreads * 12) return launch_regs<T, RankT, 12>(keys, G, P, desc, o, st);
        if (G <= kThreads * 16) return launch_regs<T, RankT, 16>(keys, G, P, desc, o, st);
        if (G <= kThreads * 20) return launch_regs<T, RankT, 20>(keys, G, P, desc, o, st);
        // two-CTA clusters: a four-CTA cluster ran ~2.4x slower per SM
        // (four-way barriers, scatters to three peers, GPC packing)
        if (G <= 2 * kThreads * 16) return launch_cluster<T, RankT, 16, 2>(keys, G, P, desc, o, st);
        if (G <= 2 * kThreads * 20) return launch_cluster<T, RankT, 20, 2>(keys, G, P, desc, o, st);
      }
    }
    using U = typename RadixKey<T>::U;
    const int grid = P < num_sms() ? P : num_sms();
    if (o.scratch_bytes < sort_scratch_bytes<T>(G, P)) return cudaErrorInvalidValue;
    // the bulk copies read the scratch rows from 16-byte boundaries
    if (reinterpret_cast<uintptr_t>(o.scratch) & 15u) return cudaErrorInvalidValue;
    // stage the ranks by gene in shared memory (over the stage buffers) when
    // they fit beside the kernel's static counters (~42 KB)
    const size_t rbytes = sizeof(RankT) * (size_t)G;
    const bool stage = rbytes <= 160 * 1024;
    const size_t dyn = stage && rbytes > tiled_stage_bytes<U>() ? rbytes : tiled_stage_bytes<U>();
    auto kern = sort_tiled_kernel<T, RankT>;
    // opt in every time: static + dynamic pass the 48 KB default
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    kern<<<grid, kThreads, dyn, st>>>(keys, G, P, desc, static_cast<RankT*>(o.ranks), static_cast<T*>(o.sorted_abs),
                                      o.order, static_cast<unsigned char*>(o.scratch), stage, o.error_flag);
    launches_add(1);
    return cudaGetLastError();
}

template <class T, class RankT, int ITEMS>
cudaError_t launch_regs_multi(const SortTask* d, int n, cudaStream_t st) {
    const size_t smem = regs_smem_bytes<T, ITEMS>();
    auto kern = sort_regs_multi<T, RankT, ITEMS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int per = (2 * num_sms() + n - 1) / n;  // CTAs per instance: about two waves over the SMs in all
    kern<<<dim3((unsigned)(per > 0 ? per : 1), 1, (unsigned)n), kThreads, smem, st>>>(d);
    launches_add(1);
    return cudaGetLastError();
}

template <class T, class RankT, int ITEMS, int CL>
cudaError_t launch_cluster_multi(const SortTask* d, int n, cudaStream_t st) {
    const size_t smem = cluster_smem_bytes<T, ITEMS>();
    auto kern = sort_cluster_multi<T, RankT, ITEMS, CL>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int per = (2 * num_sms() / CL + n - 1) / n;  // clusters per instance
    kern<<<dim3((unsigned)(CL * (per > 0 ? per : 1)), 1, (unsigned)n), kThreads, smem, st>>>(d);
    launches_add(1);
    return cudaGetLastError();
}

}  // namespace

int sort_multi_class(int G, bool fp64) {
    if (G <= 0 || G > 65536) return 0;
    if (!fp64) {
        for (int items : {4, 8, 12, 16, 20})
            if (G <= kThreads * items) return items;
        if (G <= 2 * kThreads * 16) return 116;
        if (G <= 2 * kThreads * 20) return 120;
        return 0;
    }
    if (G <= kThreads * 4) return 204;
    if (G <= kThreads * 10) return 210;
    if (G <= 2 * kThreads * 10) return 310;
    return 0;
}

cudaError_t launch_sort_multi(const SortTask* d_tasks, int n, int cls, bool fp64, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > 65535) return cudaErrorInvalidValue;
    using R = uint16_t;  // batch instances have at most 65,536 genes
    if (!fp64) {
        switch (cls) {
            case 4: return launch_regs_multi<float, R, 4>(d_tasks, n, st);
            case 8: return launch_regs_multi<float, R, 8>(d_tasks, n, st);
            case 12: return launch_regs_multi<float, R, 12>(d_tasks, n, st);
            case 16: return launch_regs_multi<float, R, 16>(d_tasks, n, st);
            case 20: return launch_regs_multi<float, R, 20>(d_tasks, n, st);
            case 116: return launch_cluster_multi<float, R, 16, 2>(d_tasks, n, st);
            case 120: return launch_cluster_multi<float, R, 20, 2>(d_tasks, n, st);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (cls) {
        case 204: return launch_cluster_multi<double, R, 4, 1>(d_tasks, n, st);
        case 210: return launch_cluster_multi<double, R, 10, 1>(d_tasks, n, st);
        case 310: return launch_cluster_multi<double, R, 10, 2>(d_tasks, n, st);
        default: return cudaErrorInvalidValue;
    }
}

template <class T>
size_t sort_scratch_bytes(int G, int num_perms) {
    using U = typename RadixKey<T>::U;
    // sized for the tiled variant, which any G may be tuned to
    const int grid = num_perms < num_sms() ? num_perms : num_sms();
    return tiled_cta_bytes<U>(G) * (size_t)(grid > 0 ? grid : 1);
}
template size_t sort_scratch_bytes<float>(int, int);
template size_t sort_scratch_bytes<double>(int, int);

template <class T>
cudaError_t launch_sort(const T* keys, int G, int num_perms, bool ascending, const SortBuffers& out,
                        cudaStream_t st) {
    if (num_perms <= 0) return cudaSuccess;
    if (out.ranks16) return launch_sort_t<T, uint16_t>(keys, G, num_perms, !ascending, out, st);
    return launch_sort_t<T, uint32_t>(keys, G, num_perms, !ascending, out, st);
}
template cudaError_t launch_sort<float>(const float*, int, int, bool, const SortBuffers&, cudaStream_t);
template cudaError_t launch_sort<double>(const double*, int, int, bool, const SortBuffers&, cudaStream_t);

}  // namespace gsea
