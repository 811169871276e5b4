// k_metric.cuh -- plain-form class statistics and ranking metric.
//
// For every (permutation, gene) the kernel accumulates class-A / class-B
// statistics over the samples in index order and finalises one of the 14
// reference metrics, reproducing the reference arithmetic operation by
// operation (src/include/functors.cuh:10-433, dispatch
// src/include/correlate_genes.cuh:166-295):
//
//   accumulators  naive (87-124)   kahan (126-176)  onepass (178-229)
//                 twopass (232-295) overkill (297-375) knuth (377-433)
//   combiners     difference (10-15) quotient (17-22) log2 quotient (24-29)
//                 signal2noise, fixlow (31-54)  T test, fixlow (57-80)
//
// All statistics are biased (the reference never forwards `biased`, so the
// accumulators use their default biased=true).  Every product is rounded
// before it is added (Exact<T>), matching the reference's CPU arithmetic.
//
// Work decomposition (GB300): a thread owns one gene and PB permutations.
// Each expression value x[s][g] is loaded once per PB permutations (coalesced
// across the genes of a warp, patient-major table) and the class bit of each
// permutation is a warp-uniform bit of a shared-memory mask word, so the
// class selection never diverges.
#pragma once
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace gsea {

enum AccKind { ACC_NAIVE, ACC_KAHAN, ACC_ONEPASS, ACC_TWOPASS, ACC_KNUTH, ACC_OVERKILL };
enum CombKind { COMB_DIFF, COMB_RATIO, COMB_LOG2, COMB_S2N, COMB_TTEST };

template <class T, int COMB>
__device__ __forceinline__ T combine(T mA, T vA, T nA, T mB, T vB, T nB) {
    using E = Exact<T>;
    if (COMB == COMB_DIFF) return E::sub(mA, mB);
    if (COMB == COMB_RATIO) return E::div(mA, mB);
    if (COMB == COMB_LOG2) return E::log2q(E::div(mA, mB));
    if (COMB == COMB_S2N) {
        T sA = E::sqrt(vA), sB = E::sqrt(vB);
        const T lowA = E::low(0.2, cuabs(mA));
        const T lowB = E::low(0.2, cuabs(mB));
        sA = lowA < sA ? sA : lowA;
        sB = lowB < sB ? sB : lowB;
        return E::div(E::sub(mA, mB), E::add(sA, sB));
    }
    // COMB_TTEST
    T wA = vA, wB = vB;
    const T lowA = E::low(0.04, cuabs(mA));
    const T lowB = E::low(0.04, cuabs(mB));
    wA = lowA < wA ? wA : lowA;
    wB = lowB < wB ? wB : lowB;
    return E::div(E::sub(mA, mB), E::sqrt(E::add(E::div(wA, nA), E::div(wB, nB))));
}

// NaN keys (0/0 in the ratio metrics, log of a negative mean, ...) are
// written as the positive all-ones NaN, whatever payload the arithmetic gave:
// the radix order then ranks every NaN first (descending) in gene order, the
// order CUDA's canonical NaN gets from the reference's GPU sort, on any host.
__device__ __forceinline__ float canonical_nan(float v) { return v != v ? __uint_as_float(0x7fffffffu) : v; }
__device__ __forceinline__ double canonical_nan(double v) {
    return v != v ? __longlong_as_double(0x7fffffffffffffffll) : v;
}

// Exact, predicated form: every class update is a conditional operation, as
// in the reference, so it is bit-exact for any input including inf / NaN.
// Called by one thread per gene with the block's masks in shared memory.
template <int ACC, int COMB, class T, int PB>
__device__ __forceinline__ void metric_exact(const T* __restrict__ X, int G, int S, const uint32_t* sm_masks,
                                             int words, int num_perms, int p0, T nA, T nB, T* __restrict__ keys,
                                             int g) {
    using E = Exact<T>;
    const T* xg = X + g;

    T mA[PB], mB[PB], vA[PB], vB[PB], cA[PB], cB[PB];
    int iA[PB], iB[PB];
#pragma unroll
    for (int j = 0; j < PB; j++) {
        mA[j] = mB[j] = vA[j] = vB[j] = cA[j] = cB[j] = T(0);
        iA[j] = iB[j] = 0;
    }

    // ---------------- pass 1 ----------------
    for (int s0 = 0, w = 0; s0 < S; s0 += 32, w++) {
        uint32_t mw[PB];
#pragma unroll
        for (int j = 0; j < PB; j++) mw[j] = sm_masks[j * words + w];
        const int n = min(32, S - s0);
        for (int t = 0; t < n; t++) {
            const T x = __ldg(xg + (int64_t)(s0 + t) * G);
            T xx = T(0);
            if (ACC == ACC_ONEPASS) xx = E::mul(x, x);
#pragma unroll
            for (int j = 0; j < PB; j++) {
                const bool l = (mw[j] >> t) & 1u;  // class A <=> permuted label 0
                if (ACC == ACC_NAIVE) {
                    mA[j] = E::add(mA[j], E::mul(l ? T(1) : T(0), x));
                    mB[j] = E::add(mB[j], E::mul(l ? T(0) : T(1), x));
                } else if (ACC == ACC_KAHAN || ACC == ACC_OVERKILL) {
                    const T acc = l ? mA[j] : mB[j];
                    const T alpha = E::sub(x, l ? cA[j] : cB[j]);
                    const T beta = E::add(acc, alpha);
                    const T kk = E::sub(E::sub(beta, acc), alpha);
                    if (l) { cA[j] = kk; mA[j] = beta; } else { cB[j] = kk; mB[j] = beta; }
                } else if (ACC == ACC_ONEPASS) {
                    // one add into the selected accumulator (the same rounding
                    // as the reference's conditional add, one FP64 / FP32 op)
                    const T m = E::add(l ? mA[j] : mB[j], x);
                    const T v = E::add(l ? vA[j] : vB[j], xx);
                    mA[j] = l ? m : mA[j];
                    mB[j] = l ? mB[j] : m;
                    vA[j] = l ? v : vA[j];
                    vB[j] = l ? vB[j] : v;
                } else if (ACC == ACC_TWOPASS) {
                    const T m = E::add(l ? mA[j] : mB[j], x);
                    mA[j] = l ? m : mA[j];
                    mB[j] = l ? mB[j] : m;
                } else {  // ACC_KNUTH: the update of the selected class
                    const int it = (l ? iA[j] : iB[j]) + 1;
                    const T mo = l ? mA[j] : mB[j];
                    const T d = E::sub(x, mo);
                    const T mn = E::add(mo, E::div(d, (T)it));
                    const T vn = E::add(l ? vA[j] : vB[j], E::mul(d, E::sub(x, mn)));
                    iA[j] = l ? it : iA[j];
                    iB[j] = l ? iB[j] : it;
                    mA[j] = l ? mn : mA[j];
                    mB[j] = l ? mB[j] : mn;
                    vA[j] = l ? vn : vA[j];
                    vB[j] = l ? vB[j] : vn;
                }
            }
        }
    }

    if (ACC != ACC_KNUTH) {
#pragma unroll
        for (int j = 0; j < PB; j++) { mA[j] = E::div(mA[j], nA); mB[j] = E::div(mB[j], nB); }
    }
    if (ACC == ACC_ONEPASS) {
#pragma unroll
        for (int j = 0; j < PB; j++) {
            vA[j] = E::sub(E::div(vA[j], nA), E::mul(mA[j], mA[j]));
            vB[j] = E::sub(E::div(vB[j], nB), E::mul(mB[j], mB[j]));
        }
    }

    // ---------------- pass 2 (twopass, overkill) ----------------
    if (ACC == ACC_TWOPASS || ACC == ACC_OVERKILL) {
        // cA/cB hold the sums of deviations (overkill's aux) from here on
#pragma unroll
        for (int j = 0; j < PB; j++) cA[j] = cB[j] = T(0);
        for (int s0 = 0, w = 0; s0 < S; s0 += 32, w++) {
            uint32_t mw[PB];
#pragma unroll
            for (int j = 0; j < PB; j++) mw[j] = sm_masks[j * words + w];
            const int n = min(32, S - s0);
            for (int t = 0; t < n; t++) {
                const T x = __ldg(xg + (int64_t)(s0 + t) * G);
#pragma unroll
                for (int j = 0; j < PB; j++) {
                    const bool l = (mw[j] >> t) & 1u;
                    const T d = E::sub(x, l ? mA[j] : mB[j]);
                    const T dd = E::mul(d, d);
                    if (ACC == ACC_OVERKILL) {
                        const T c = E::add(l ? cA[j] : cB[j], d);
                        cA[j] = l ? c : cA[j];
                        cB[j] = l ? cB[j] : c;
                    }
                    const T v = E::add(l ? vA[j] : vB[j], dd);
                    vA[j] = l ? v : vA[j];
                    vB[j] = l ? vB[j] : v;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < PB; j++) {
            if (ACC == ACC_OVERKILL) {
                vA[j] = E::sub(vA[j], E::div(E::mul(cA[j], cA[j]), nA));
                vB[j] = E::sub(vB[j], E::div(E::mul(cB[j], cB[j]), nB));
            }
            vA[j] = E::div(vA[j], nA);
            vB[j] = E::div(vB[j], nB);
        }
    }
    if (ACC == ACC_KNUTH) {
#pragma unroll
        for (int j = 0; j < PB; j++) { vA[j] = E::div(vA[j], nA); vB[j] = E::div(vB[j], nB); }
    }

#pragma unroll
    for (int j = 0; j < PB; j++) {
        if (p0 + j < num_perms)
            keys[(int64_t)(p0 + j) * G + g] = canonical_nan(combine<T, COMB>(mA[j], vA[j], nA, mB[j], vB[j], nB));
    }
}

// one CTA of the exact form: genes bx*128.., permutations by*PB..
template <int ACC, int COMB, class T, int PB>
__device__ __forceinline__ void metric_exact_block(const T* __restrict__ X, int G, int S,
                                                   const uint32_t* __restrict__ masks, int words, int num_perms,
                                                   T nA, T nB, T* __restrict__ keys, int bx, int by) {
    extern __shared__ uint32_t sm_masks[];  // [PB][words]
    const int p0 = by * PB;
    for (int i = threadIdx.x; i < PB * words; i += blockDim.x) {
        const int j = i / words, w = i - j * words;
        sm_masks[i] = (p0 + j < num_perms) ? masks[(int64_t)(p0 + j) * words + w] : 0u;
    }
    __syncthreads();
    const int g = bx * blockDim.x + threadIdx.x;
    if (g >= G) return;
    metric_exact<ACC, COMB, T, PB>(X, G, S, sm_masks, words, num_perms, p0, nA, nB, keys, g);
}

template <int ACC, int COMB, class T, int PB>
__global__ void __launch_bounds__(128)
metric_kernel(const T* __restrict__ X, int G, int S, const uint32_t* __restrict__ masks, int words,
              int num_perms, T nA, T nB, T* __restrict__ keys) {
    metric_exact_block<ACC, COMB, T, PB>(X, G, S, masks, words, num_perms, nA, nB, keys, blockIdx.x, blockIdx.y);
}

// every instance of a batch group in one launch (blockIdx.z = instance; the
// grid covers the largest instance, CTAs beyond an instance's extent leave)
template <int ACC, int COMB, class T, int PB>
__global__ void __launch_bounds__(128) metric_multi(const MetricTask<T>* __restrict__ tasks) {
    const MetricTask<T> t = tasks[blockIdx.z];
    if ((int)blockIdx.x * 128 >= t.G || (int)blockIdx.y * PB >= t.num_perms) return;
    metric_exact_block<ACC, COMB, T, PB>(t.X, t.G, t.S, t.masks, t.words, t.num_perms, t.nA, t.nB, t.keys,
                                         blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------------------
// Packed fast form (fp32, naive / onepass / twopass accumulators).
//
// With a class weight l in {0, 1}, fma(l, v, acc) rounds exactly like the
// reference's conditional `acc + v` when v is finite (l = 1: one rounding of
// acc + v; l = 0: acc unchanged), and the naive accumulator's literal
// `acc + l*v` for any v.  Blackwell's paired-FP32 instructions (fma / add /
// mul .rn.f32x2) then update two permutations per instruction with no
// predication: pass 1 is one packed FMA per class and permutation pair, pass 2
// selects the class mean as lA*mA + lB*mB (exact: one product is zero) and
// adds the squared deviation with the class weights.  The expression table is
// checked once per upload (gsea::launch_finite_check): any value that is not
// finite or has |x| >= 2^60 (whose square could overflow) sends the kernel to
// the exact predicated form instead.
__device__ __forceinline__ unsigned long long f2_pack(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// one CTA of the packed form: genes bx*128.., permutations by*PB..
template <int ACC, int COMB, int PB>
__device__ __forceinline__ void metric_fast_block(const float* __restrict__ X, int G, int S,
                                                  const uint32_t* __restrict__ masks, int words, int num_perms,
                                                  float nA, float nB, float* __restrict__ keys,
                                                  const int* __restrict__ fast_ok, int bx, int by) {
    static_assert(PB % 2 == 0, "permutations are processed in pairs");
    constexpr int PAIRS = PB / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ulonglong2* lab = reinterpret_cast<ulonglong2*>(smem_raw);                       // [S][PAIRS]
    uint32_t* sm_masks = reinterpret_cast<uint32_t*>(lab + (size_t)S * PAIRS);        // [PB][words]
    const int p0 = by * PB;
    for (int i = threadIdx.x; i < PB * words; i += blockDim.x) {
        const int j = i / words, w = i - j * words;
        sm_masks[i] = (p0 + j < num_perms) ? masks[(int64_t)(p0 + j) * words + w] : 0u;
    }
    __syncthreads();
    const bool fast = ACC == ACC_NAIVE || *fast_ok != 0;
    if (fast) {
        for (int i = threadIdx.x; i < S * PAIRS; i += blockDim.x) {
            const int sidx = i / PAIRS, q = i - sidx * PAIRS;
            const int w = sidx >> 5, t = sidx & 31;
            const float a0 = (float)((sm_masks[(2 * q) * words + w] >> t) & 1u);
            const float a1 = (float)((sm_masks[(2 * q + 1) * words + w] >> t) & 1u);
            lab[i] = make_ulonglong2(f2_pack(a0, a1), f2_pack(1.f - a0, 1.f - a1));
        }
    }
    __syncthreads();
    const int g = bx * blockDim.x + threadIdx.x;
    if (g >= G) return;
    if (!fast) {
        metric_exact<ACC, COMB, float, PB>(X, G, S, sm_masks, words, num_perms, p0, nA, nB, keys, g);
        return;
    }
    const float* xg = X + g;
    unsigned long long mA[PAIRS], mB[PAIRS], vA[PAIRS], vB[PAIRS];
#pragma unroll
    for (int q = 0; q < PAIRS; q++) mA[q] = mB[q] = vA[q] = vB[q] = 0ull;
    // samples per unrolled step: eight loads of the table in flight (two
    // for onepass, whose extra accumulators leave no registers for more)
    constexpr int kUnroll = ACC == ACC_ONEPASS ? 2 : 8;
    // pass 1: class sums (and sums of squares for onepass)
#pragma unroll kUnroll
    for (int sidx = 0; sidx < S; sidx++) {
        const float x = __ldg(xg + (int64_t)sidx * G);
        const unsigned long long xx = f2_pack(x, x);
        unsigned long long sq = 0ull;
        if (ACC == ACC_ONEPASS) {
            const float x2 = __fmul_rn(x, x);
            sq = f2_pack(x2, x2);
        }
        const ulonglong2* ls = lab + (size_t)sidx * PAIRS;
#pragma unroll
        for (int q = 0; q < PAIRS; q++) {
            const ulonglong2 l = ls[q];
            mA[q] = f2_fma(l.x, xx, mA[q]);
            mB[q] = f2_fma(l.y, xx, mB[q]);
            if (ACC == ACC_ONEPASS) {
                vA[q] = f2_fma(l.x, sq, vA[q]);
                vB[q] = f2_fma(l.y, sq, vB[q]);
            }
        }
    }
    float fmA[PB], fmB[PB];
#pragma unroll
    for (int q = 0; q < PAIRS; q++) {
        f2_unpack(mA[q], fmA[2 * q], fmA[2 * q + 1]);
        f2_unpack(mB[q], fmB[2 * q], fmB[2 * q + 1]);
    }
#pragma unroll
    for (int j = 0; j < PB; j++) {
        fmA[j] = __fdiv_rn(fmA[j], nA);
        fmB[j] = __fdiv_rn(fmB[j], nB);
    }
    float fvA[PB], fvB[PB];
#pragma unroll
    for (int j = 0; j < PB; j++) fvA[j] = fvB[j] = 0.f;
    if (ACC == ACC_ONEPASS) {
#pragma unroll
        for (int q = 0; q < PAIRS; q++) {
            f2_unpack(vA[q], fvA[2 * q], fvA[2 * q + 1]);
            f2_unpack(vB[q], fvB[2 * q], fvB[2 * q + 1]);
        }
#pragma unroll
        for (int j = 0; j < PB; j++) {
            fvA[j] = __fsub_rn(__fdiv_rn(fvA[j], nA), __fmul_rn(fmA[j], fmA[j]));
            fvB[j] = __fsub_rn(__fdiv_rn(fvB[j], nB), __fmul_rn(fmB[j], fmB[j]));
        }
    }
    if (ACC == ACC_TWOPASS) {
        // pass 2: squared deviations from the own class mean
#pragma unroll
        for (int q = 0; q < PAIRS; q++) {
            mA[q] = f2_pack(fmA[2 * q], fmA[2 * q + 1]);
            mB[q] = f2_pack(fmB[2 * q], fmB[2 * q + 1]);
        }
#pragma unroll kUnroll
        for (int sidx = 0; sidx < S; sidx++) {
            const float x = __ldg(xg + (int64_t)sidx * G);
            const unsigned long long xx = f2_pack(x, x);
            const ulonglong2* ls = lab + (size_t)sidx * PAIRS;
#pragma unroll
            for (int q = 0; q < PAIRS; q++) {
                const ulonglong2 l = ls[q];
                const unsigned long long m = f2_fma(l.x, mA[q], f2_mul(l.y, mB[q]));  // own class mean
                const unsigned long long dv = f2_sub(xx, m);
                const unsigned long long dd = f2_mul(dv, dv);
                vA[q] = f2_fma(l.x, dd, vA[q]);
                vB[q] = f2_fma(l.y, dd, vB[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < PAIRS; q++) {
            f2_unpack(vA[q], fvA[2 * q], fvA[2 * q + 1]);
            f2_unpack(vB[q], fvB[2 * q], fvB[2 * q + 1]);
        }
#pragma unroll
        for (int j = 0; j < PB; j++) {
            fvA[j] = __fdiv_rn(fvA[j], nA);
            fvB[j] = __fdiv_rn(fvB[j], nB);
        }
    }
#pragma unroll
    for (int j = 0; j < PB; j++) {
        if (p0 + j < num_perms)
            keys[(int64_t)(p0 + j) * G + g] =
                canonical_nan(combine<float, COMB>(fmA[j], fvA[j], nA, fmB[j], fvB[j], nB));
    }
}

template <int ACC, int COMB, int PB>
__global__ void __launch_bounds__(128, 8)
metric_fast_kernel(const float* __restrict__ X, int G, int S, const uint32_t* __restrict__ masks, int words,
                   int num_perms, float nA, float nB, float* __restrict__ keys, const int* __restrict__ fast_ok) {
    metric_fast_block<ACC, COMB, PB>(X, G, S, masks, words, num_perms, nA, nB, keys, fast_ok, blockIdx.x,
                                     blockIdx.y);
}

template <int ACC, int COMB, int PB>
__global__ void __launch_bounds__(128, 8) metric_fast_multi(const MetricTask<float>* __restrict__ tasks) {
    const MetricTask<float> t = tasks[blockIdx.z];
    if ((int)blockIdx.x * 128 >= t.G || (int)blockIdx.y * PB >= t.num_perms) return;
    metric_fast_block<ACC, COMB, PB>(t.X, t.G, t.S, t.masks, t.words, t.num_perms, t.nA, t.nB, t.keys, t.fast_ok,
                                     blockIdx.x, blockIdx.y);
}

template <int ACC, int COMB, int PB>
cudaError_t launch_metric_fast_pb(const float* X, int G, int S, const uint32_t* masks, int words, int num_perms,
                                  int64_t nA, int64_t nB, float* keys, const int* fast_ok, cudaStream_t st) {
    const int threads = 128;
    dim3 grid((G + threads - 1) / threads, (num_perms + PB - 1) / PB);
    const size_t smem = sizeof(ulonglong2) * (size_t)S * (PB / 2) + sizeof(uint32_t) * PB * words;
    auto kern = metric_fast_kernel<ACC, COMB, PB>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, threads, smem, st>>>(X, G, S, masks, words, num_perms, (float)nA, (float)nB, keys, fast_ok);
    launches_add(1);
    return cudaGetLastError();
}

// pb: permutations per thread (4 or 8; 0 = 8), identical keys either way
template <int ACC, int COMB>
cudaError_t launch_metric_fast(const float* X, int G, int S, const uint32_t* masks, int words, int num_perms,
                               int64_t nA, int64_t nB, float* keys, const int* fast_ok, int pb, cudaStream_t st) {
    if (pb == 4)
        return launch_metric_fast_pb<ACC, COMB, 4>(X, G, S, masks, words, num_perms, nA, nB, keys, fast_ok, st);
    return launch_metric_fast_pb<ACC, COMB, 8>(X, G, S, masks, words, num_perms, nA, nB, keys, fast_ok, st);
}

template <int ACC, int COMB, class T>
cudaError_t launch_metric_t(const T* X, int G, int S, const uint32_t* masks, int words,
                            int num_perms, int64_t nA, int64_t nB, T* keys, cudaStream_t st) {
    constexpr int PB = 8;
    const int threads = 128;
    dim3 grid((G + threads - 1) / threads, (num_perms + PB - 1) / PB);
    const size_t smem = sizeof(uint32_t) * PB * words;
    metric_kernel<ACC, COMB, T, PB><<<grid, threads, smem, st>>>(X, G, S, masks, words, num_perms,
                                                                 (T)nA, (T)nB, keys);
    launches_add(1);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_metric_impl(int metric, const T* X, int G, int S, const uint32_t* masks,
                               int words, int num_perms, int64_t nA, int64_t nB, T* keys,
                               const int* fast_ok, cudaStream_t st, int pb) {
    if (pb != 0 && pb != 4 && pb != 8) return cudaErrorInvalidValue;
    if (num_perms <= 0) return cudaSuccess;
    if constexpr (std::is_same<T, float>::value) {
      if (fast_ok && (size_t)S * 4 * 16 + 32 * (size_t)words <= 100 * 1024) {
        const float* Xf = X;
        float* kf = keys;
        switch (metric) {
            case 0: return launch_metric_fast<ACC_NAIVE, COMB_DIFF>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            case 1: return launch_metric_fast<ACC_NAIVE, COMB_RATIO>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            case 2: return launch_metric_fast<ACC_NAIVE, COMB_LOG2>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            case 6: return launch_metric_fast<ACC_ONEPASS, COMB_S2N>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            case 7: return launch_metric_fast<ACC_ONEPASS, COMB_TTEST>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            case 8: return launch_metric_fast<ACC_TWOPASS, COMB_S2N>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            case 9: return launch_metric_fast<ACC_TWOPASS, COMB_TTEST>(Xf, G, S, masks, words, num_perms, nA, nB, kf, fast_ok, pb, st);
            default: break;
        }
      }
    }
#define GSEA_M(ID, A, C)                                                                        \
    case ID:                                                                                   \
        return launch_metric_t<A, C, T>(X, G, S, masks, words, num_perms, nA, nB, keys, st);
    switch (metric) {
        GSEA_M(0, ACC_NAIVE, COMB_DIFF)
        GSEA_M(1, ACC_NAIVE, COMB_RATIO)
        GSEA_M(2, ACC_NAIVE, COMB_LOG2)
        GSEA_M(3, ACC_KAHAN, COMB_DIFF)
        GSEA_M(4, ACC_KAHAN, COMB_RATIO)
        GSEA_M(5, ACC_KAHAN, COMB_LOG2)
        GSEA_M(6, ACC_ONEPASS, COMB_S2N)
        GSEA_M(7, ACC_ONEPASS, COMB_TTEST)
        GSEA_M(8, ACC_TWOPASS, COMB_S2N)
        GSEA_M(9, ACC_TWOPASS, COMB_TTEST)
        GSEA_M(10, ACC_KNUTH, COMB_S2N)
        GSEA_M(11, ACC_KNUTH, COMB_TTEST)
        GSEA_M(12, ACC_OVERKILL, COMB_S2N)
        GSEA_M(13, ACC_OVERKILL, COMB_TTEST)
        default:
            return cudaErrorInvalidValue;
    }
#undef GSEA_M
}

// Batched instances: the group key of an instance (instances with equal keys
// share one launch) -- the metric and the path launch_metric_impl takes for
// it (exact, or packed with 4 or 8 permutations per thread).
template <class T>
int metric_multi_key_impl(int metric, int S, int words, bool fast_ok, int pb) {
    bool fast = false;
    if constexpr (std::is_same<T, float>::value)
        fast = fast_ok && (size_t)S * 4 * 16 + 32 * (size_t)words <= 100 * 1024 &&
               (metric <= 2 || (metric >= 6 && metric <= 9));
    return metric * 4 + (fast ? (pb == 4 ? 1 : 2) : 0);
}

// grid over the largest instance of a group; PB permutations per thread,
// `lab` bytes of packed class weights per sample (0 for the exact form)
template <class T>
void multi_extent(const MetricTask<T>* h, int n, int PB, size_t lab, dim3& grid, size_t& smem) {
    unsigned gx = 1, gy = 1;
    smem = 0;
    for (int i = 0; i < n; i++) {
        gx = std::max(gx, (unsigned)((h[i].G + 127) / 128));
        gy = std::max(gy, (unsigned)((h[i].num_perms + PB - 1) / PB));
        smem = std::max(smem, lab * (size_t)h[i].S + sizeof(uint32_t) * PB * (size_t)h[i].words);
    }
    grid = dim3(gx, gy, (unsigned)n);
}

template <int ACC, int COMB, int PB>
cudaError_t launch_fast_multi_pb(const MetricTask<float>* d, const MetricTask<float>* h, int n, cudaStream_t st) {
    dim3 grid;
    size_t smem;
    multi_extent<float>(h, n, PB, sizeof(ulonglong2) * (PB / 2), grid, smem);
    auto kern = metric_fast_multi<ACC, COMB, PB>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, 128, smem, st>>>(d);
    launches_add(1);
    return cudaGetLastError();
}

template <int ACC, int COMB, class T>
cudaError_t launch_exact_multi(const MetricTask<T>* d, const MetricTask<T>* h, int n, cudaStream_t st) {
    constexpr int PB = 8;
    dim3 grid;
    size_t smem;
    multi_extent<T>(h, n, PB, 0, grid, smem);
    auto kern = metric_multi<ACC, COMB, T, PB>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, 128, smem, st>>>(d);
    launches_add(1);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_metric_multi_impl(int key, const MetricTask<T>* d, const MetricTask<T>* h, int n,
                                     cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > 65535) return cudaErrorInvalidValue;
    for (int i = 0; i < n; i++)
        if ((h[i].num_perms + 7) / 8 > 65535) return cudaErrorInvalidValue;
    const int metric = key / 4, path = key % 4;
    if constexpr (std::is_same<T, float>::value) {
        if (path != 0) {
#define GSEA_F(ID, A, C)                                                                   \
    case ID:                                                                              \
        return path == 1 ? launch_fast_multi_pb<A, C, 4>(d, h, n, st) : launch_fast_multi_pb<A, C, 8>(d, h, n, st);
            switch (metric) {
                GSEA_F(0, ACC_NAIVE, COMB_DIFF)
                GSEA_F(1, ACC_NAIVE, COMB_RATIO)
                GSEA_F(2, ACC_NAIVE, COMB_LOG2)
                GSEA_F(6, ACC_ONEPASS, COMB_S2N)
                GSEA_F(7, ACC_ONEPASS, COMB_TTEST)
                GSEA_F(8, ACC_TWOPASS, COMB_S2N)
                GSEA_F(9, ACC_TWOPASS, COMB_TTEST)
                default:
                    return cudaErrorInvalidValue;
            }
#undef GSEA_F
        }
    }
    if (path != 0) return cudaErrorInvalidValue;
#define GSEA_X(ID, A, C) \
    case ID:             \
        return launch_exact_multi<A, C, T>(d, h, n, st);
    switch (metric) {
        GSEA_X(0, ACC_NAIVE, COMB_DIFF)
        GSEA_X(1, ACC_NAIVE, COMB_RATIO)
        GSEA_X(2, ACC_NAIVE, COMB_LOG2)
        GSEA_X(3, ACC_KAHAN, COMB_DIFF)
        GSEA_X(4, ACC_KAHAN, COMB_RATIO)
        GSEA_X(5, ACC_KAHAN, COMB_LOG2)
        GSEA_X(6, ACC_ONEPASS, COMB_S2N)
        GSEA_X(7, ACC_ONEPASS, COMB_TTEST)
        GSEA_X(8, ACC_TWOPASS, COMB_S2N)
        GSEA_X(9, ACC_TWOPASS, COMB_TTEST)
        GSEA_X(10, ACC_KNUTH, COMB_S2N)
        GSEA_X(11, ACC_KNUTH, COMB_TTEST)
        GSEA_X(12, ACC_OVERKILL, COMB_S2N)
        GSEA_X(13, ACC_OVERKILL, COMB_TTEST)
        default:
            return cudaErrorInvalidValue;
    }
#undef GSEA_X
}

}  // namespace gsea
