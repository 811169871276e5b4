// k_permute.cu -- on-device label permutations.
//
// Permutation p (global index q = perm_offset + p) shuffles the label vector
// with a Fisher-Yates pass driven by a fast-KISS generator seeded with
// q + seed, exactly as correlate_gpu does on thread 0 of each block
// (src/include/correlate_genes.cuh:44-56; generator src/include/rngpu/rngpu.hpp:
// 27-38 hash, 145-178 KISS, 288-303 shuffle).  Permutation 0 is the identity.
// The generator is counter-based in q: any permutation range can be produced
// independently, which is what shards and perm batches rely on.
//
// Output: one bit per sample, bit set <=> class A (permuted label 0), the
// form the metric kernels consume.
#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace {

__device__ __forceinline__ uint32_t nv_hash(uint32_t x) {
    x = (x + 0x7ed55d16u) + (x << 12);
    x = (x ^ 0xc761c23cu) ^ (x >> 19);
    x = (x + 0x165667b1u) + (x << 5);
    x = (x + 0xd3a2646cu) ^ (x << 9);
    x = (x + 0xfd7046c5u) + (x << 3);
    x = (x ^ 0xb55a4f09u) ^ (x >> 16);
    return x;
}

struct Kiss {
    uint32_t x, y, z, w, c;
    __device__ __forceinline__ explicit Kiss(uint32_t seed) {
        w = seed ? seed : 0xFFFFFFFFu;
        x = y = z = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            x = nv_hash(w);
            y = nv_hash(x);
            z = nv_hash(y);
            w = nv_hash(z);
        }
        c = 0;
    }
    __device__ __forceinline__ uint32_t next() {
        y ^= y << 5;
        y ^= y >> 7;
        y ^= y << 22;
        const int32_t t = (int32_t)(z + w + c);
        z = w;
        c = t < 0;
        w = (uint32_t)t & 2147483647u;
        x += 1411392427u;
        return x + y + w;
    }
};

constexpr int kPermThreads = 32;

// one thread per permutation; the label vector of each thread lives in
// shared memory, interleaved by thread
__device__ __forceinline__ void permute_body(int64_t bx, const uint8_t* __restrict__ labels, int S, int64_t num_perms,
                                             int64_t perm_offset, uint32_t seed, uint32_t* __restrict__ masks,
                                             int words) {
    extern __shared__ uint8_t lab[];  // [S][kPermThreads]
    const int t = threadIdx.x;
    const int64_t p = bx * kPermThreads + t;
    for (int s = 0; s < S; s++) lab[s * kPermThreads + t] = labels[s];
    if (p >= num_perms) return;
    const uint64_t q = (uint64_t)(perm_offset + p);
    if (q != 0) {
        Kiss rng((uint32_t)(q + seed));
        for (int i = S - 1; i >= 1; i--) {
            // (double)u * (i+1) / 2^32 truncated: the product is exact in
            // double for i+1 < 2^21, so it equals the integer (u*(i+1)) >> 32
            const uint32_t u = rng.next();
            const int r = (int)(((uint64_t)u * (uint64_t)(i + 1)) >> 32);
            const uint8_t a = lab[i * kPermThreads + t];
            lab[i * kPermThreads + t] = lab[r * kPermThreads + t];
            lab[r * kPermThreads + t] = a;
        }
    }
    uint32_t* out = masks + p * words;
    for (int w = 0; w < words; w++) {
        uint32_t m = 0;
        const int s_end = min(S, (w + 1) * 32);
        for (int s = w * 32; s < s_end; s++)
            m |= (uint32_t)(lab[s * kPermThreads + t] == 0) << (s - w * 32);
        out[w] = m;
    }
}

__global__ void __launch_bounds__(kPermThreads)
permute_kernel(const uint8_t* __restrict__ labels, int S, int64_t num_perms, int64_t perm_offset,
               uint32_t seed, uint32_t* __restrict__ masks, int words) {
    permute_body(blockIdx.x, labels, S, num_perms, perm_offset, seed, masks, words);
}

// every instance of a batch at once: blockIdx.z = the instance
__global__ void __launch_bounds__(kPermThreads) permute_multi(const PermTask* __restrict__ tasks) {
    const PermTask t = tasks[blockIdx.z];
    if ((int64_t)blockIdx.x * kPermThreads >= t.num_perms) return;
    permute_body(blockIdx.x, t.labels, t.S, t.num_perms, t.perm_offset, t.seed, t.masks, t.words);
}

// fast_ok stays 1 unless some value is not finite or has |x| >= 2^60
template <class T>
__global__ void finite_check_kernel(const T* __restrict__ x, int64_t n, int* __restrict__ fast_ok) {
    bool ok = true;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T v = x[i];
        ok &= (v == v) && fabs(v) < T(1.152921504606846976e18);  // 2^60
    }
    if (!__all_sync(kFullMask, ok) && (threadIdx.x & 31) == 0) atomicExch(fast_ok, 0);
}

}  // namespace

template <class T>
cudaError_t launch_finite_check(const T* exprs, int64_t n, int* fast_ok, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(fast_ok, 1, sizeof(int), st);  // non-zero = packed form allowed
    if (e != cudaSuccess) return e;
    const int threads = 256;
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    finite_check_kernel<T><<<(unsigned)blocks, threads, 0, st>>>(exprs, n, fast_ok);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_finite_check<float>(const float*, int64_t, int*, cudaStream_t);
template cudaError_t launch_finite_check<double>(const double*, int64_t, int*, cudaStream_t);

cudaError_t launch_permute(const uint8_t* labels, int S, int64_t num_perms, int64_t perm_offset,
                           uint32_t seed, uint32_t* masks, int words, cudaStream_t st) {
    if (num_perms <= 0) return cudaSuccess;
    const size_t smem = (size_t)S * kPermThreads;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(permute_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int64_t blocks = (num_perms + kPermThreads - 1) / kPermThreads;
    permute_kernel<<<(unsigned)blocks, kPermThreads, smem, st>>>(labels, S, num_perms, perm_offset,
                                                               seed, masks, words);
    launches_add(1);
    return cudaGetLastError();
}

cudaError_t launch_permute_multi(const PermTask* d_tasks, const PermTask* h_tasks, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > 65535) return cudaErrorInvalidValue;
    int64_t pmax = 0;
    int smax = 0;
    for (int i = 0; i < n; i++) {
        pmax = pmax > h_tasks[i].num_perms ? pmax : h_tasks[i].num_perms;
        smax = smax > h_tasks[i].S ? smax : h_tasks[i].S;
    }
    const size_t smem = (size_t)smax * kPermThreads;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(permute_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t blocks = (pmax + kPermThreads - 1) / kPermThreads;
    permute_multi<<<dim3((unsigned)blocks, 1, (unsigned)n), kPermThreads, smem, st>>>(d_tasks);
    launches_add(1);
    return cudaGetLastError();
}

}  // namespace gsea
