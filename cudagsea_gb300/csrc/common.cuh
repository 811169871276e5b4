// common.cuh -- shared device helpers of libgsea103 (GB300 / sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gsea {

constexpr uint32_t kFullMask = 0xffffffffu;

// ---------------------------------------------------------------------------
// Exact IEEE operations.  The reference's metric arithmetic is reproduced
// bit for bit, so no product may be fused into an addition: the *_rn
// intrinsics are never contracted into FMA by the compiler.
template <class T> struct Exact;
template <> struct Exact<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
    // floor of a standard deviation / variance: (T)(c * |m|) evaluated in double
    // (functors.cuh:46-47, 72-73 multiply a double literal by a float)
    static __device__ __forceinline__ float low(double c, float m) {
        return __double2float_rn(__dmul_rn(c, (double)m));
    }
    // culog(q) * 1.44269504089 : float log, double product, rounded to float
    // (functors.cuh:24-29, math_helpers.cuh:5, 37-40)
    static __device__ __forceinline__ float log2q(float q) {
        return __double2float_rn(__dmul_rn((double)logf(q), 1.44269504089));
    }
};
template <> struct Exact<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
    static __device__ __forceinline__ double low(double c, double m) { return __dmul_rn(c, m); }
    static __device__ __forceinline__ double log2q(double q) { return __dmul_rn(log(q), 1.44269504089); }
};

// cuabs of math_helpers.cuh:10-13 (keeps -0.0 and NaN as they are)
template <class T> __device__ __forceinline__ T cuabs(T x) { return x < T(0) ? -x : x; }

// ---------------------------------------------------------------------------
// Radix order of IEEE keys: unsigned ascending order of radix_bits(x) equals
// ascending value order with -0 < +0 and NaNs at the two ends, which is the
// order CUB's radix sort gives the reference GPU path (batched_sort.cuh:144).
template <class T> struct RadixKey;
template <> struct RadixKey<float> {
    using U = uint32_t;
    static __device__ __forceinline__ U from(float f, bool descending) {
        U u = __float_as_uint(f);
        u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        return descending ? ~u : u;
    }
};
template <> struct RadixKey<double> {
    using U = unsigned long long;
    static __device__ __forceinline__ U from(double f, bool descending) {
        U u = (U)__double_as_longlong(f);
        u = (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
        return descending ? ~u : u;
    }
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace gsea
