// k_chosen.cu -- class statistics on the tcgen05 tensor cores (chosen form).
//
// For every permutation p and gene g the reference sums class-A values and
// squares over the samples (src/include/functors.cuh:87-433).  With the
// permuted labels as a 0/1 matrix L[s][p] (class A = 1) these sums are the
// contractions
//     SA [g][p] = sum_s x'[s][g]   * L[s][p]
//     SA2[g][p] = sum_s x'[s][g]^2 * L[s][p]
// over centred values x' = x - mean_g (the gene mean over all samples, kept
// as FP32; x' exact as a float-float); class B follows from the per-gene
// totals (T1 - SA, T2 - SA2).
//
// Operands: x' and x'^2 are split into three BF16 parts each (hi + mid + lo
// carries ~24 significant bits) stacked along K, the labels are exact 0/1 in
// BF16 and repeated for each part, so one BF16 x BF16 -> FP32 GEMM of depth
// 3*S gives each sum.  A tile is 128 genes x TN permutations:
//   * two FP32 accumulators in tensor memory (SA in the first TN columns,
//     SA2 in the next TN), allocated with tcgen05.alloc;
//   * the operands are pre-arranged in the canonical no-swizzle K-major
//     layout (8x8 core matrices of 128 bytes), 32 K-elements per chunk, so a
//     chunk of A (8 KB), A2 (8 KB) and B (8 or 16 KB) is one contiguous 1-D
//     TMA bulk copy each (cp.async.bulk) completing on an mbarrier, a stage
//     refilled as soon as the MMAs of its chunk retired;
//   * one thread issues tcgen05.mma (M=128, N=TN, K=16) with shared-memory
//     descriptors and tcgen05.commit to the stage's mbarrier (the sums are
//     the same MMA chain per element for every form below);
//   * warps read the accumulators with tcgen05.ld (a warp reads its lane
//     quarter, 32 lanes x 16 columns at a time), finalise the metric and
//     store the keys.
// TN = 128, the default: class_stats_persistent, one CTA per SM walking the
// tiles, a copy thread, an MMA thread and sixteen epilogue warps, two
// accumulator pairs so that a tile's epilogue overlaps the next tile's MMAs
// (its own section below); TN = 256: class_stats_kernel, one tile per CTA,
// 6 stages, one thread for copies and MMAs, eight epilogue warps after the
// last commit.
// Every mbarrier wait is bounded (about one second of clock); on expiry the
// kernel records an error flag, waits a bounded time for its own copies and
// MMAs, frees its tensor memory and returns -- no wait can hang the GPU.
//
// Finalisation: means and the mean-square-minus-squared-mean variances are
// formed from the FP32 sums, the subtraction either in FP64
// (GSEA_FORM_CHOSEN_FP64) or as an error-free FP32 transformation
// (GSEA_FORM_CHOSEN, see variance()); the metric itself
// (difference, ratio, log2 ratio, signal-to-noise, T test, with the
// reference's fixlow floors) is then evaluated in FP32 on centred
// differences.  The result is the metric of the FP32 inputs to ~1e-6
// relative, not the reference's operation order: near-tied genes may swap.
#include <algorithm>
#include <cuda_bf16.h>

#include <cstdint>

#include "bulk.cuh"
#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace chosen {

constexpr int BM = 128;          // genes per CTA (TMEM lanes)
constexpr int BN = 256;          // permutations per CTA (the default tile; 128 is the other)
constexpr int BK = 32;           // K elements per chunk
constexpr int A_CHUNK = BM * BK * 2;   // 8 KB
constexpr int B_CHUNK = BN * BK * 2;   // 16 KB (a 128-permutation tile uses half)
// pipeline stages: 6 for the 256-permutation tile (192 KB, one CTA per SM);
// 4 for the 128-permutation tile (96 KB and 256 TMEM columns: two CTAs per
// SM, so one CTA's epilogue runs beside the other's loads and MMAs).  Small
// chunks keep several stages' copies in flight while one is multiplied.
template <int TN>
constexpr int stages() { return TN == 128 ? 4 : 6; }
template <int TN>
constexpr int stage_bytes() { return 2 * A_CHUNK + TN * BK * 2; }
constexpr int THREADS = 256;     // 8 warps: two per TMEM lane quarter in the epilogue

// byte offset of element (row, k) inside a chunk laid out as 8x8 core
// matrices: core (row/8, k/8) at ((row/8)*8 + k/8)*128, row-major inside
__host__ __device__ __forceinline__ uint32_t core_offset(int row, int k) {
    return (uint32_t)((((row >> 3) * (BK / 8) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

// shared-memory matrix descriptor, no swizzle, K-major
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    // base offset 0, lbo mode 0, layout type 0 (no swizzle)
    return d;
}

// instruction descriptor: kind::f16, BF16 x BF16 -> F32, K-major A and B
__host__ __device__ constexpr uint32_t make_idesc(int m, int n) {
    return (1u << 4)                       // D format F32
           | (1u << 7)                     // A format BF16
           | (1u << 10)                    // B format BF16
           | ((uint32_t)(n >> 3) << 17)    // N / 8
           | ((uint32_t)(m >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// metric from centred class statistics (see the file comment)
template <int COMB>
__device__ __forceinline__ float finalize(float mAc, float mBc, float mu, float vA, float vB, float nA, float nB) {
    const float diff = mAc - mBc;
    const float mA = mu + mAc, mB = mu + mBc;
    if (COMB == 0) return diff;
    if (COMB == 1) return mA / mB;
    if (COMB == 2) return logf(mA / mB) * 1.44269504089f;
    if (COMB == 3) {
        float sA = sqrtf(vA), sB = sqrtf(vB);
        const float lowA = 0.2f * fabsf(mA), lowB = 0.2f * fabsf(mB);
        sA = lowA < sA ? sA : lowA;
        sB = lowB < sB ? sB : lowB;
        return diff / (sA + sB);
    }
    float wA = vA, wB = vB;
    const float lowA = 0.04f * fabsf(mA), lowB = 0.04f * fabsf(mB);
    wA = lowA < wA ? wA : lowA;
    wB = lowB < wB ? wB : lowB;
    return diff / sqrtf(wA / nA + wB / nB);
}

__device__ __forceinline__ float canonical_nan_f(float v) { return v != v ? __uint_as_float(0x7fffffffu) : v; }

// variance = mean square - squared mean
//   FP64SUB:  the subtraction in FP64 (the squared mean is exact in FP64)
//   else:     error-free FP32 transformation -- p = m*m rounded, e = fma(m, m,
//             -p) its exact rounding error, v = (ms - p) - e -- which agrees
//             with the FP64 form to about one ulp at FP32 speed (GB300's FP64
//             rate is a small fraction of its FP32 rate)
template <bool FP64SUB>
__device__ __forceinline__ float variance(float ms, float m) {
    if (FP64SUB) return (float)fma(-(double)m, (double)m, (double)ms);
    const float p = m * m;
    const float e = fmaf(m, m, -p);
    return (ms - p) - e;
}

// Epilogue of one warp: TMEM lane quarter `quarter` (genes 32*quarter..+31 of
// gene tile gt), the 16-column blocks part, part + PARTS, ... of the two
// accumulators at `acc` (SA in columns [0, TN), SA2 in [TN, 2*TN)): class
// means, variances and the metric, keys[p][g] stored coalesced (a warp writes
// 32 consecutive genes of one permutation at a time).
template <int COMB, bool FP64SUB, int TN, int PARTS>
__device__ __forceinline__ void tile_epilogue(uint32_t acc, int quarter, int part, int lane, int gt, int pt, int G,
                                              int num_perms, const float* __restrict__ gene_mu,
                                              const double* __restrict__ gene_t1,
                                              const double* __restrict__ gene_t2, float nA, float nB,
                                              float* __restrict__ keys) {
    const int row = quarter * 32 + lane;   // TMEM lane = gene within the tile
    const int g = gt * BM + row;
    const bool gv = g < G;
    const float mu = gv ? gene_mu[g] : 0.f;
    const float t1 = gv ? (float)gene_t1[g] : 0.f, t2 = gv ? (float)gene_t2[g] : 0.f;
    const float inA = 1.f / nA, inB = 1.f / nB;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    for (int cb = part; cb < TN / 16; cb += PARTS) {
        uint32_t va[16], vq[16];
        tmem_ld16(acc + lane_base + cb * 16, va);
        tmem_ld16(acc + lane_base + TN + cb * 16, vq);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int p = pt * TN + cb * 16 + j;
            const float sA = __uint_as_float(va[j]), sA2 = __uint_as_float(vq[j]);
            // class means and mean squares (centred); B from the totals
            const float mAc = sA * inA;
            const float mBc = (t1 - sA) * inB;
            const float eA = sA2 * inA;
            const float eB = (t2 - sA2) * inB;
            const float vA = variance<FP64SUB>(eA, mAc);
            const float vB = variance<FP64SUB>(eB, mBc);
            const float key = finalize<COMB>(mAc, mBc, mu, vA, vB, nA, nB);
            if (gv && p < num_perms) keys[(size_t)p * G + g] = canonical_nan_f(key);
        }
    }
}

// one CTA = one tile of BM genes x TN permutations (gt, pt)
template <int COMB, bool FP64SUB, int TN>
__device__ __forceinline__ void
class_stats_tile(int gt, int pt, const unsigned char* __restrict__ A1, const unsigned char* __restrict__ A2,
                 const unsigned char* __restrict__ B, int chunks, int G, int num_perms,
                 const float* __restrict__ gene_mu, const double* __restrict__ gene_t1,
                 const double* __restrict__ gene_t2, float nA, float nB, float* __restrict__ keys,
                 int* __restrict__ error_flag) {
    constexpr int STAGES = stages<TN>();
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar_full[STAGES];
    __shared__ __align__(8) uint64_t bar_done[STAGES];
    __shared__ uint32_t tmem_slot;
    __shared__ int failed;
    constexpr int TB_CHUNK = TN * BK * 2;
    constexpr int TSTAGE = stage_bytes<TN>();
    constexpr int TCOLS = 2 * TN;  // two FP32 accumulators of TN columns
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "n"(TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(smem_u32(&bar_full[s]), 1);
            mbar_init(smem_u32(&bar_done[s]), 1);
        }
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;

    if (tid == 0) {
        const uint32_t idesc = make_idesc(BM, TN);
        uint32_t ph_full[STAGES] = {}, ph_done[STAGES] = {};
        bool ok = true;
        // stage s holds chunk c with c % STAGES == s
        auto load = [&](int c) {
            const int s = c % STAGES;
            unsigned char* st = smem + s * TSTAGE;
            const uint32_t bar = smem_u32(&bar_full[s]);
            mbar_expect_tx(bar, TSTAGE);
            bulk_copy(smem_u32(st), A1 + ((size_t)gt * chunks + c) * A_CHUNK, A_CHUNK, bar);
            bulk_copy(smem_u32(st + A_CHUNK), A2 + ((size_t)gt * chunks + c) * A_CHUNK, A_CHUNK, bar);
            bulk_copy(smem_u32(st + 2 * A_CHUNK), B + ((size_t)pt * chunks + c) * TB_CHUNK, TB_CHUNK, bar);
        };
        const int pre = chunks < STAGES ? chunks : STAGES;
        for (int c = 0; c < pre; c++) load(c);
        int committed = 0;  // chunks whose MMAs were committed
        int loaded = pre;   // chunks whose loads were issued
        for (int c = 0; c < chunks && ok; c++) {
            const int s = c % STAGES;
            ok = mbar_wait(smem_u32(&bar_full[s]), ph_full[s]);
            ph_full[s] ^= 1;
            if (!ok) break;
            fence_after();
            const uint32_t a1 = smem_u32(smem + s * TSTAGE), a2 = a1 + A_CHUNK, b = a1 + 2 * A_CHUNK;
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++) {
                // K = 16 spans two core matrices along K: LBO = 128 B apart,
                // row groups SBO = (BK/8)*128 B apart
                const uint32_t koff = kk * 256;
                const uint64_t da1 = make_desc(a1 + koff, 128, (BK / 8) * 128);
                const uint64_t da2 = make_desc(a2 + koff, 128, (BK / 8) * 128);
                const uint64_t db = make_desc(b + koff, 128, (BK / 8) * 128);
                const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
                mma_bf16(tmem, da1, db, idesc, acc);
                mma_bf16(tmem + TN, da2, db, idesc, acc);
            }
            mma_commit(smem_u32(&bar_done[s]));
            committed = c + 1;
            // refill the stage of the previous chunk once its MMAs have read it
            if (c >= 1 && loaded < chunks) {
                const int sp = (c - 1) % STAGES;
                ok = mbar_wait(smem_u32(&bar_done[sp]), ph_done[sp]);
                ph_done[sp] ^= 1;
                if (!ok) break;
                load(loaded++);
            }
        }
        // wait for every commit not yet waited for
        {
            int waited_upto = 0;  // chunks c < waited_upto had their done-barrier consumed
            // the refill waits consumed the done phases of chunks 0 .. loaded-STAGES-1
            waited_upto = loaded - pre;
            for (int c = waited_upto; c < committed; c++) {
                const int sd = c % STAGES;
                if (!mbar_wait(smem_u32(&bar_done[sd]), ph_done[sd])) ok = false;
                ph_done[sd] ^= 1;
            }
        }
        if (!ok) {
            failed = 1;
            atomicExch(error_flag, 1);
        }
        fence_before();
    }
    __syncthreads();
    fence_after();

    if (!failed)
        tile_epilogue<COMB, FP64SUB, TN, 2>(tmem, warp & 3, warp >> 2, lane, gt, pt, G, num_perms, gene_mu, gene_t1,
                                         gene_t2, nA, nB, keys);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TCOLS) : "memory");
    }
}

template <int COMB, bool FP64SUB, int TN>
__global__ void __launch_bounds__(THREADS, TN == 128 ? 2 : 1)
class_stats_kernel(const unsigned char* __restrict__ A1, const unsigned char* __restrict__ A2,
                   const unsigned char* __restrict__ B, int chunks, int G, int num_perms,
                   const float* __restrict__ gene_mu, const double* __restrict__ gene_t1,
                   const double* __restrict__ gene_t2, float nA, float nB, float* __restrict__ keys,
                   int* __restrict__ error_flag) {
    class_stats_tile<COMB, FP64SUB, TN>(blockIdx.x, blockIdx.y, A1, A2, B, chunks, G, num_perms, gene_mu, gene_t1,
                                        gene_t2, nA, nB, keys, error_flag);
}

// ---------------------------------------------------------------------------
// Persistent form of the 128-permutation tile (the default): one CTA per SM
// walks the tiles t = blockIdx.x, blockIdx.x + gridDim.x, ... (gene tile
// t / ptiles, permutation tile t % ptiles: neighbouring CTAs share operand
// tiles in L2) with three roles:
//   warp 0, one thread: the bulk copies of every chunk of every tile into a
//     ring of PSTAGES shared-memory stages, a stage refilled as soon as the
//     MMAs that read it retired (their commit arrives on the stage's `empty`);
//   warp 1, one thread: the MMAs of each tile into one of two accumulator
//     pairs in TMEM (2 x 2 x 128 columns = all 512), alternating, each
//     chunk's commit freeing its stage and the tile's last commit handing
//     the pair to the epilogue (`acc_full`);
//   warps 2-17: the epilogue of the tile whose pair is full (four warps per
//     TMEM lane quarter, each taking every fourth 16-column block) while the
//     MMAs of the next
//     tile run on the other pair; each warp hands the pair back with one
//     arrival on `acc_empty` once its TMEM loads completed.
// The same body serves a batch (class_stats_persistent_multi: the tiles of
// every instance, instance after instance).  The MMA chain per key is the
// same as the one-tile form's, so the keys are identical.  Every wait is bounded and also ends when another role has
// failed; the failing role records the error flag, the MMA thread then waits
// (bounded) for its MMAs and the copy thread for its copies before the CTA
// frees its tensor memory.
constexpr int PSTAGES = 8;              // 8 x 24 KB stages
constexpr int PEPI = 16;                // epilogue warps: four per TMEM lane quarter
constexpr int PTHREADS = 32 * (2 + PEPI);
constexpr int PTN = 128;

// one tile's operands and outputs
struct TileJob {
    const unsigned char* A1;
    const unsigned char* A2;
    const unsigned char* B;
    const float* mu;
    const double* t1;
    const double* t2;
    float* keys;
    float nA, nB;
    int chunks, G, num_perms, gt, pt;
};

// the tiles of one problem: tile t = gene tile t / ptiles, permutation tile t % ptiles
struct SoloTiles {
    const unsigned char* A1;
    const unsigned char* A2;
    const unsigned char* B;
    const float* mu;
    const double* t1;
    const double* t2;
    float* keys;
    int* error_flag;
    float nA, nB;
    int chunks, G, num_perms, total;
    __device__ __forceinline__ TileJob job(int t) {
        const int ptiles = (num_perms + PTN - 1) / PTN;
        const int gt = t / ptiles;
        return TileJob{A1, A2, B, mu, t1, t2, keys, nA, nB, chunks, G, num_perms, gt, t - gt * ptiles};
    }
    __device__ __forceinline__ int* flag() const { return error_flag; }
};

// the tiles of every instance of a batch, instance after instance; a role
// walks them in increasing order, so its cursor only moves forward
struct MultiTiles {
    const ChosenTask* tasks;
    int ntasks, total;
    int i = 0, base = 0;  // cursor: instance i's tiles start at tile `base`
    __device__ __forceinline__ TileJob job(int t) {
        int ptiles, n;
        for (;;) {
            const ChosenTask& k = tasks[i];
            ptiles = (k.num_perms + PTN - 1) / PTN;
            n = ((k.G + BM - 1) / BM) * ptiles;
            if (t < base + n || i + 1 >= ntasks) break;
            base += n;
            ++i;
        }
        const ChosenTask& k = tasks[i];
        const int lt = t - base, gt = lt / ptiles;
        return TileJob{k.A1, k.A2, k.Bm, k.mu, k.t1, k.t2, k.keys, k.nA, k.nB, k.chunks, k.G, k.num_perms, gt,
                       lt - gt * ptiles};
    }
    __device__ __forceinline__ int* flag() const { return tasks[0].error_flag; }
};

template <int COMB, bool FP64SUB, class Tiles>
__device__ __forceinline__ void persistent_body(Tiles src) {
    constexpr int TSTAGE = stage_bytes<PTN>();
    constexpr int TB_CHUNK = PTN * BK * 2;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[PSTAGES];
    __shared__ __align__(8) uint64_t empty[PSTAGES];
    __shared__ __align__(8) uint64_t acc_full[2];
    __shared__ __align__(8) uint64_t acc_empty[2];
    __shared__ __align__(8) uint64_t drain;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntiles = src.total;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        for (int s = 0; s < PSTAGES; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&acc_full[b]), 1);
            mbar_init(smem_u32(&acc_empty[b]), PEPI);
        }
        mbar_init(smem_u32(&drain), 1);
        failed = 0;
        fence_mbar_init();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // copies
            Tiles tiles = src;
            uint32_t n = 0;  // chunk loads issued: stage n % PSTAGES, its (n / PSTAGES)-th use
            for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
                const TileJob jb = tiles.job(t);
                for (int c = 0; c < jb.chunks; c++, n++) {
                    const int s = (int)(n % PSTAGES);
                    const uint32_t k = n / PSTAGES;
                    if (k > 0 && !mbar_wait_or_fail(smem_u32(&empty[s]), (k - 1) & 1u, &failed)) {
                        failed = 1;
                        break;
                    }
                    unsigned char* st = smem + (size_t)s * TSTAGE;
                    const uint32_t bar = smem_u32(&full[s]);
                    mbar_expect_tx(bar, TSTAGE);
                    bulk_copy(smem_u32(st), jb.A1 + ((size_t)jb.gt * jb.chunks + c) * A_CHUNK, A_CHUNK, bar);
                    bulk_copy(smem_u32(st + A_CHUNK), jb.A2 + ((size_t)jb.gt * jb.chunks + c) * A_CHUNK, A_CHUNK,
                              bar);
                    bulk_copy(smem_u32(st + 2 * A_CHUNK), jb.B + ((size_t)jb.pt * jb.chunks + c) * TB_CHUNK,
                              TB_CHUNK, bar);
                }
            }
            if (failed) {
                atomicExch(src.flag(), 1);
                // the last copies issued into each stage land before the CTA leaves
                for (uint32_t m = n > PSTAGES ? n - PSTAGES : 0; m < n; m++)
                    mbar_wait(smem_u32(&full[m % PSTAGES]), (m / PSTAGES) & 1u);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMAs
            Tiles tiles = src;
            const uint32_t idesc = make_idesc(BM, PTN);
            uint32_t n = 0;  // chunks consumed
            int j = 0;       // tiles of this CTA
            for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x, j++) {
                const int chunks = tiles.job(t).chunks;
                const int b = j & 1;
                const uint32_t kb = (uint32_t)j >> 1;
                if (kb > 0 && !mbar_wait_or_fail(smem_u32(&acc_empty[b]), (kb - 1) & 1u, &failed)) {
                    failed = 1;
                    break;
                }
                fence_after();
                const uint32_t d = tmem + (uint32_t)(b * 2 * PTN);
                bool ok = true;
                for (int c = 0; c < chunks; c++, n++) {
                    const int s = (int)(n % PSTAGES);
                    if (!mbar_wait_or_fail(smem_u32(&full[s]), (n / PSTAGES) & 1u, &failed)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t a1 = smem_u32(smem + (size_t)s * TSTAGE), a2 = a1 + A_CHUNK, bb = a1 + 2 * A_CHUNK;
#pragma unroll
                    for (int kk = 0; kk < BK / 16; kk++) {
                        const uint32_t koff = kk * 256;
                        const uint64_t da1 = make_desc(a1 + koff, 128, (BK / 8) * 128);
                        const uint64_t da2 = make_desc(a2 + koff, 128, (BK / 8) * 128);
                        const uint64_t db = make_desc(bb + koff, 128, (BK / 8) * 128);
                        const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
                        mma_bf16(d, da1, db, idesc, acc);
                        mma_bf16(d + PTN, da2, db, idesc, acc);
                    }
                    mma_commit(smem_u32(&empty[s]));
                }
                if (!ok) {
                    failed = 1;
                    break;
                }
                mma_commit(smem_u32(&acc_full[b]));
            }
            if (failed) atomicExch(src.flag(), 1);
            // every MMA issued has retired before TMEM is freed
            mma_commit(smem_u32(&drain));
            mbar_wait(smem_u32(&drain), 0);
        }
    } else {  // epilogue
        Tiles tiles = src;
        const int e = warp - 2;
        const int quarter = warp & 3;  // the TMEM lane quarter this warp may read
        const int part = e >> 2;
        int j = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, j++) {
            const int b = j & 1;
            const uint32_t kb = (uint32_t)j >> 1;
            int ok = 0;
            if (lane == 0) ok = mbar_wait_or_fail(smem_u32(&acc_full[b]), kb & 1u, &failed) ? 1 : 0;
            ok = __shfl_sync(kFullMask, ok, 0);
            if (!ok) {
                if (lane == 0) {
                    failed = 1;
                    atomicExch(src.flag(), 1);
                }
                break;
            }
            fence_after();
            const TileJob jb = tiles.job(t);
            tile_epilogue<COMB, FP64SUB, PTN, PEPI / 4>(tmem + (uint32_t)(b * 2 * PTN), quarter, part, lane, jb.gt,
                                                        jb.pt, jb.G, jb.num_perms, jb.mu, jb.t1, jb.t2, jb.nA, jb.nB,
                                                        jb.keys);
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&acc_empty[b]));
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
}

template <int COMB, bool FP64SUB>
__global__ void __launch_bounds__(PTHREADS, 1)
class_stats_persistent(const unsigned char* __restrict__ A1, const unsigned char* __restrict__ A2,
                       const unsigned char* __restrict__ B, int chunks, int G, int num_perms,
                       const float* __restrict__ gene_mu, const double* __restrict__ gene_t1,
                       const double* __restrict__ gene_t2, float nA, float nB, float* __restrict__ keys,
                       int* __restrict__ error_flag) {
    const int total = ((G + BM - 1) / BM) * ((num_perms + PTN - 1) / PTN);
    persistent_body<COMB, FP64SUB>(SoloTiles{A1, A2, B, gene_mu, gene_t1, gene_t2, keys, error_flag, nA, nB, chunks, G,
                                             num_perms, total});
}

// every instance of a batch (one metric family): the tiles of all
// instances, instance after instance, over one CTA per SM
template <int COMB, bool FP64SUB>
__global__ void __launch_bounds__(PTHREADS, 1)
class_stats_persistent_multi(const ChosenTask* __restrict__ tasks, int ntasks, int total) {
    MultiTiles src;
    src.tasks = tasks;
    src.ntasks = ntasks;
    src.total = total;
    persistent_body<COMB, FP64SUB>(src);
}

// ---------------------------------------------------------------------------
// operand preparation

// Float-float arithmetic (value = h + l, |l| <= ulp(h)/2) on the FP32 pipe:
// error-free two-sum and two-product (FMA), so sums of a few hundred terms
// and the operand splits keep ~44 bits -- more than the FP32 results need --
// without the FP64 pipe.
struct FF {
    float h, l;
};
__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_sq(FF a) {  // (h + l)^2, the l^2 term dropped
    const float p = __fmul_rn(a.h, a.h);
    const float e = __fmaf_rn(a.h, a.h, -p);
    return fast_two_sum(p, __fmaf_rn(__fadd_rn(a.h, a.h), a.l, e));
}
__device__ __forceinline__ double ff_value(FF a) { return (double)a.h + (double)a.l; }

// per gene: the mean over all samples (kept as FP32: mu_f) and the totals of
// x - mu_f and (x - mu_f)^2 -- centred at the same mu_f as the GEMM operands,
// so class B = totals - class A is exact up to the accumulation.  Sums in
// float-float; x - mu_f is exact as a float-float.  Block of 256 threads =
// 32 genes x 8 sample groups: a warp reads 32 consecutive genes of one sample
// (coalesced); the 8 partial sums of a gene are added in group order.
template <class T>
__global__ void __launch_bounds__(256) gene_moments_kernel(const T* __restrict__ X, int G, int S,
                                                           float* __restrict__ mu_f, double* __restrict__ t1,
                                                           double* __restrict__ t2) {
    __shared__ FF part[8][32], part2[8][32];
    __shared__ float s_mu[32];
    const int gi = threadIdx.x & 31, j = threadIdx.x >> 5;
    const int g = blockIdx.x * 32 + gi;
    const bool gv = g < G;
    FF s = {0.f, 0.f};
    if (gv)
        for (int i = j; i < S; i += 8) s = ff_add(s, FF{(float)X[(size_t)i * G + g], 0.f});
    part[j][gi] = s;
    __syncthreads();
    if (j == 0) {
        FF tot = {0.f, 0.f};
        for (int k = 0; k < 8; k++) tot = ff_add(tot, part[k][gi]);
        s_mu[gi] = (float)(ff_value(tot) / S);
    }
    __syncthreads();
    const float mu = s_mu[gi];
    FF a = {0.f, 0.f}, b = {0.f, 0.f};
    if (gv)
        for (int i = j; i < S; i += 8) {
            const FF d = two_sum((float)X[(size_t)i * G + g], -mu);
            a = ff_add(a, d);
            b = ff_add(b, ff_sq(d));
        }
    part[j][gi] = a;
    part2[j][gi] = b;
    __syncthreads();
    if (j == 0 && gv) {
        FF ta = {0.f, 0.f}, tb = {0.f, 0.f};
        for (int k = 0; k < 8; k++) {
            ta = ff_add(ta, part[k][gi]);
            tb = ff_add(tb, part2[k][gi]);
        }
        mu_f[g] = s_mu[gi];
        t1[g] = ff_value(ta);
        t2[g] = ff_value(tb);
    }
}

// v = hi + mid + lo, three BF16 values: hi = bf16(v.h); v.h - hi and
// r1 - mid are exact (Sterbenz), so the parts carry v to ~2^-25 relative
__device__ __forceinline__ void split3(FF v, __nv_bfloat16& hi, __nv_bfloat16& mid, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(v.h);
    const float r1 = __fadd_rn(__fsub_rn(v.h, __bfloat162float(hi)), v.l);
    mid = __float2bfloat16_rn(r1);
    lo = __float2bfloat16_rn(__fsub_rn(r1, __bfloat162float(mid)));
}

__device__ __forceinline__ uint4 pack8(const __nv_bfloat16 (&a)[8]) {
    auto w = [&](int i) {
        return (uint32_t)__bfloat16_as_ushort(a[i]) | ((uint32_t)__bfloat16_as_ushort(a[i + 1]) << 16);
    };
    return make_uint4(w(0), w(2), w(4), w(6));
}

// A1 (x') and A2 (x'^2) in chunked core-matrix layout; K index = part*S + s.
// One thread per (gene, 8 consecutive samples): the 8 values of a part are
// one 16-byte row segment of a core matrix when part*S + s0 is a multiple of
// 8 (always when S is), written with one vector store per operand and part;
// otherwise element by element.  The buffers are zeroed beforehand.
template <class T>
__global__ void split_operands_kernel(const T* __restrict__ X, int G, int S, int chunks,
                                      const float* __restrict__ mu_f, unsigned char* __restrict__ A1,
                                      unsigned char* __restrict__ A2) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int s0 = blockIdx.y * 8;
    if (g >= G) return;
    const float mu = mu_f[g];
    __nv_bfloat16 p[3][8], q[3][8];
    const int ns = S - s0 < 8 ? S - s0 : 8;
#pragma unroll
    for (int e = 0; e < 8; e++) {
        const FF d = e < ns ? two_sum((float)X[(size_t)(s0 + e) * G + g], -mu) : FF{0.f, 0.f};
        split3(d, p[0][e], p[1][e], p[2][e]);
        split3(ff_sq(d), q[0][e], q[1][e], q[2][e]);
    }
    const int gt = g / BM, row = g % BM;
    for (int part = 0; part < 3; part++) {
        const int k0 = part * S + s0;
        if ((k0 & 7) == 0 && ns == 8) {
            const int c = k0 / BK, kk = k0 % BK;
            const size_t off = ((size_t)gt * chunks + c) * A_CHUNK + core_offset(row, kk);
            *reinterpret_cast<uint4*>(A1 + off) = pack8(p[part]);  // off is 16-byte aligned (kk % 8 == 0)
            *reinterpret_cast<uint4*>(A2 + off) = pack8(q[part]);
        } else {
            for (int e = 0; e < ns; e++) {
                const int k = k0 + e;
                const int c = k / BK, kk = k % BK;
                const size_t off = ((size_t)gt * chunks + c) * A_CHUNK + core_offset(row, kk);
                *reinterpret_cast<__nv_bfloat16*>(A1 + off) = p[part][e];
                *reinterpret_cast<__nv_bfloat16*>(A2 + off) = q[part][e];
            }
        }
    }
}

// B: class-A indicator of every (permutation, sample), repeated for the three
// parts, in tiles of TN permutations; one thread per (permutation, sample);
// the buffer is zeroed before.
template <int TN>
__device__ __forceinline__ void label_operand_body(int bx, int s, const uint32_t* __restrict__ masks, int words,
                                                   int S, int num_perms, int chunks, unsigned char* __restrict__ Bm) {
    const int p = bx * blockDim.x + threadIdx.x;
    if (p >= num_perms || s >= S) return;
    const bool a = (masks[(size_t)p * words + (s >> 5)] >> (s & 31)) & 1u;
    const __nv_bfloat16 v = __float2bfloat16(a ? 1.f : 0.f);
    const int pt = p / TN, row = p % TN;
    for (int part = 0; part < 3; part++) {
        const int k = part * S + s;
        const int c = k / BK, kk = k % BK;
        *reinterpret_cast<__nv_bfloat16*>(Bm + ((size_t)pt * chunks + c) * (TN * BK * 2) + core_offset(row, kk)) = v;
    }
}

template <int TN>
__global__ void label_operand_kernel(const uint32_t* __restrict__ masks, int words, int S, int num_perms,
                                     int chunks, unsigned char* __restrict__ Bm) {
    label_operand_body<TN>(blockIdx.x, blockIdx.y, masks, words, S, num_perms, chunks, Bm);
}

template <int TN>
__global__ void label_operand_multi(const ChosenTask* __restrict__ tasks) {
    const ChosenTask& t = tasks[blockIdx.z];
    label_operand_body<TN>(blockIdx.x, blockIdx.y, t.masks, t.words, t.S, t.num_perms, t.chunks, t.Bm);
}

// the B operand of every instance cleared (16-byte stores; a buffer is a
// whole number of TN x BK x 2-byte chunks)
template <int TN>
__global__ void zero_b_multi(const ChosenTask* __restrict__ tasks) {
    const ChosenTask& t = tasks[blockIdx.z];
    const size_t n16 = (size_t)((t.num_perms + TN - 1) / TN) * t.chunks * (TN * BK * 2) / 16;
    uint4* b = reinterpret_cast<uint4*>(t.Bm);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_uint4(0u, 0u, 0u, 0u);
}

}  // namespace chosen

int chosen_chunks(int S) { return (3 * S + chosen::BK - 1) / chosen::BK; }
size_t chosen_a_bytes(int G, int S) {
    return (size_t)((G + chosen::BM - 1) / chosen::BM) * chosen_chunks(S) * chosen::A_CHUNK;
}
size_t chosen_b_bytes(int P, int S) {
    return (size_t)((P + chosen::BN - 1) / chosen::BN) * chosen_chunks(S) * chosen::B_CHUNK;
}

template <class T>
cudaError_t launch_chosen_prepare(const T* X, int G, int S, float* mu, double* t1, double* t2, unsigned char* A1,
                                  unsigned char* A2, cudaStream_t st) {
    const size_t ab = chosen_a_bytes(G, S);
    cudaError_t e = cudaMemsetAsync(A1, 0, ab, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A2, 0, ab, st);
    if (e != cudaSuccess) return e;
    chosen::gene_moments_kernel<T><<<(G + 31) / 32, 256, 0, st>>>(X, G, S, mu, t1, t2);
    chosen::split_operands_kernel<T><<<dim3((G + 127) / 128, (S + 7) / 8), 128, 0, st>>>(X, G, S, chosen_chunks(S), mu,
                                                                                     A1, A2);
    launches_add(2);
    return cudaGetLastError();
}
template cudaError_t launch_chosen_prepare<float>(const float*, int, int, float*, double*, double*, unsigned char*,
                                                  unsigned char*, cudaStream_t);

namespace {
int sm_count() {
    static int cached[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int& n = cached[dev & 63];
    if (n <= 0) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

using ClassStatsFn = void (*)(const unsigned char*, const unsigned char*, const unsigned char*, int, int, int,
                             const float*, const double*, const double*, float, float, float*, int*);
// the kernel of a tile width: persistent for 128 permutations, one tile per CTA otherwise
template <int C, int TN>
ClassStatsFn pick_class_stats(bool fp64_variance) {
    using namespace chosen;
    if constexpr (TN == PTN)
        return fp64_variance ? class_stats_persistent<C, true> : class_stats_persistent<C, false>;
    else
        return fp64_variance ? class_stats_kernel<C, true, TN> : class_stats_kernel<C, false, TN>;
}

template <int TN>
cudaError_t launch_chosen_tn(int comb, bool fp64_variance, const uint32_t* masks, int words, int G, int S,
                             int num_perms, int64_t nA, int64_t nB, const float* mu, const double* t1,
                             const double* t2, const unsigned char* A1, const unsigned char* A2, unsigned char* Bm,
                             float* keys, int* error_flag, cudaStream_t st) {
    using namespace chosen;
    const int chunks = chosen_chunks(S);
    const size_t bbytes = (size_t)((num_perms + TN - 1) / TN) * chunks * (TN * BK * 2);
    cudaError_t e = cudaMemsetAsync(Bm, 0, bbytes, st);
    if (e != cudaSuccess) return e;
    label_operand_kernel<TN><<<dim3((num_perms + 127) / 128, S), 128, 0, st>>>(masks, words, S, num_perms, chunks, Bm);
    dim3 grid((G + BM - 1) / BM, (num_perms + TN - 1) / TN);
    size_t smem = (size_t)stages<TN>() * stage_bytes<TN>();
    int threads = THREADS;
    if (TN == PTN) {  // persistent: one CTA per SM over all tiles
        const int tiles = (int)(grid.x * grid.y);
        const int sms = sm_count();
        grid = dim3((unsigned)(tiles < sms ? tiles : sms));
        smem = (size_t)PSTAGES * stage_bytes<PTN>();
        threads = PTHREADS;
    }
#define GSEA_CHOSEN(C)                                                                                         \
    {                                                                                                          \
        auto kern = pick_class_stats<C, TN>(fp64_variance);                                                   \
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                \
        if (e != cudaSuccess) return e;                                                                        \
        kern<<<grid, threads, smem, st>>>(A1, A2, Bm, chunks, G, num_perms, mu, t1, t2, (float)nA, (float)nB,  \
                                          keys, error_flag);                                                   \
    }
    switch (comb) {
        case 0: GSEA_CHOSEN(0) break;
        case 1: GSEA_CHOSEN(1) break;
        case 2: GSEA_CHOSEN(2) break;
        case 3: GSEA_CHOSEN(3) break;
        default: GSEA_CHOSEN(4) break;
    }
#undef GSEA_CHOSEN
    launches_add(2);
    return cudaGetLastError();
}
}  // namespace

int chosen_comb(int metric) {
    return metric == 0 || metric == 3 ? 0 : metric == 1 || metric == 4 ? 1 : metric == 2 || metric == 5 ? 2
         : (metric == 6 || metric == 8 || metric == 10 || metric == 12) ? 3 : 4;
}

cudaError_t launch_chosen_metric_multi(const ChosenTask* d_tasks, const ChosenTask* h_tasks, int n,
                                       bool fp64_variance, cudaStream_t st) {
    using namespace chosen;
    constexpr int TN = 128;
    if (n <= 0) return cudaSuccess;
    if (n > 65535) return cudaErrorInvalidValue;
    int gmax = 0, pmax = 0, smax = 0;
    for (int i = 0; i < n; i++) {
        const ChosenTask& t = h_tasks[i];
        if (t.comb != h_tasks[0].comb) return cudaErrorInvalidValue;  // one metric family per launch
        gmax = std::max(gmax, t.G);
        pmax = std::max(pmax, t.num_perms);
        smax = std::max(smax, t.S);
    }
    const unsigned z = (unsigned)n;
    zero_b_multi<TN><<<dim3(152, 1, z), 256, 0, st>>>(d_tasks);
    label_operand_multi<TN><<<dim3((unsigned)((pmax + 127) / 128), (unsigned)smax, z), 128, 0, st>>>(d_tasks);
    // the persistent kernel over the tiles of every instance
    int64_t total = 0;
    for (int i = 0; i < n; i++)
        total += (int64_t)((h_tasks[i].G + BM - 1) / BM) * ((h_tasks[i].num_perms + PTN - 1) / PTN);
    if (total > INT32_MAX) return cudaErrorInvalidValue;
    const int sms = sm_count();
    const dim3 grid((unsigned)(total < sms ? total : sms));
    const size_t smem = (size_t)PSTAGES * stage_bytes<PTN>();
    cudaError_t e = cudaSuccess;
#define GSEA_CHOSEN_MULTI(C)                                                                                    \
    {                                                                                                           \
        auto kern = fp64_variance ? class_stats_persistent_multi<C, true> : class_stats_persistent_multi<C, false>; \
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                 \
        if (e != cudaSuccess) return e;                                                                         \
        kern<<<grid, PTHREADS, smem, st>>>(d_tasks, n, (int)total);                                             \
    }
    switch (h_tasks[0].comb) {
        case 0: GSEA_CHOSEN_MULTI(0) break;
        case 1: GSEA_CHOSEN_MULTI(1) break;
        case 2: GSEA_CHOSEN_MULTI(2) break;
        case 3: GSEA_CHOSEN_MULTI(3) break;
        default: GSEA_CHOSEN_MULTI(4) break;
    }
#undef GSEA_CHOSEN_MULTI
    launches_add(3);
    return cudaGetLastError();
}

cudaError_t launch_chosen_metric(int metric, bool fp64_variance, const uint32_t* masks, int words, int G, int S,
                                 int num_perms, int64_t nA, int64_t nB, const float* mu, const double* t1,
                                 const double* t2, const unsigned char* A1, const unsigned char* A2,
                                 unsigned char* Bm, float* keys, int* error_flag, cudaStream_t st, int tile_n) {
    const int comb = chosen_comb(metric);
    // default (0): the 128-permutation tile, two CTAs per SM
    if (tile_n == 0 || tile_n == 128)
        return launch_chosen_tn<128>(comb, fp64_variance, masks, words, G, S, num_perms, nA, nB, mu, t1, t2, A1, A2,
                                     Bm, keys, error_flag, st);
    if (tile_n != 256) return cudaErrorInvalidValue;
    return launch_chosen_tn<256>(comb, fp64_variance, masks, words, G, S, num_perms, nA, nB, mu, t1, t2, A1, A2, Bm,
                                 keys, error_flag, st);
}

}  // namespace gsea
