// sets.cu -- gene-set membership built on the device: gene symbols hashed
// once into a device table, every set member looked up there, then per-set
// membership bitmasks compacted into the CSR the plans take.
//
// Replaces create_bitmaps (src/include/create_bitmaps.cuh:13-65), which fills
// a host unordered_set per 32/64-set batch for every permutation batch, with
// the same semantics: members whose symbol is not a gene of the expression
// table are dropped silently, duplicates collapse, and (as the CSR is sorted)
// each set's genes come out in ascending gene index.  A symbol repeated in the
// expression table maps to its first gene (the reference's map insertion,
// src/cudaGSEA_wrapper.cu:244-252).
//
// Kernels:
//   insert_kernel   thread per gene: FNV-1a 64 hash of the symbol, linear
//                   probing in a power-of-two table (>= 2x genes) with
//                   atomicCAS on the key and atomicMin on the gene index;
//   lookup_kernel   thread per member: probe, then compare the bytes with the
//                   stored gene's symbol (a 64-bit hash match of different
//                   strings sets an error flag instead of merging them);
//   mark_kernel     thread per member: atomicOr into the set's bitmask row
//                   (K rows of ceil(G/32) words);
//   count_kernel / emit_kernel  block per set: popcounts, block scan, and the
//                   member indices written in ascending order.
// Every probe loop is bounded by the table size.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "plan.h"

namespace {
using gsea::fail;

__host__ __device__ inline uint64_t fnv1a(const char* s, int64_t n) {
    uint64_t h = 1469598103934665603ull;
    for (int64_t i = 0; i < n; i++) {
        h ^= (unsigned char)s[i];
        h *= 1099511628211ull;
    }
    return h | 1ull;  // 0 marks an empty slot
}

__device__ inline bool same_bytes(const char* a, int64_t na, const char* b, int64_t nb) {
    if (na != nb) return false;
    for (int64_t i = 0; i < na; i++)
        if (a[i] != b[i]) return false;
    return true;
}

__global__ void insert_kernel(const char* __restrict__ blob, const int64_t* __restrict__ off, int64_t G,
                              unsigned long long* __restrict__ keys, int* __restrict__ vals, uint64_t mask) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const uint64_t h = fnv1a(blob + off[g], off[g + 1] - off[g]);
    uint64_t slot = h & mask;
    for (uint64_t probe = 0; probe <= mask; probe++) {
        const unsigned long long prev = atomicCAS(&keys[slot], 0ull, (unsigned long long)h);
        if (prev == 0ull || prev == h) {
            atomicMin(&vals[slot], (int)g);
            return;
        }
        slot = (slot + 1) & mask;
    }
}

__global__ void lookup_kernel(const char* __restrict__ gblob, const int64_t* __restrict__ goff,
                              const char* __restrict__ mblob, const int64_t* __restrict__ moff, int64_t M,
                              const unsigned long long* __restrict__ keys, const int* __restrict__ vals,
                              uint64_t mask, int* __restrict__ idx, int* __restrict__ collision) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const char* s = mblob + moff[m];
    const int64_t n = moff[m + 1] - moff[m];
    const uint64_t h = fnv1a(s, n);
    uint64_t slot = h & mask;
    int found = -1;
    for (uint64_t probe = 0; probe <= mask; probe++) {
        const unsigned long long k = keys[slot];
        if (k == 0ull) break;
        if (k == h) {
            const int g = vals[slot];
            if (same_bytes(gblob + goff[g], goff[g + 1] - goff[g], s, n)) found = g;
            else atomicExch(collision, 1);
            break;
        }
        slot = (slot + 1) & mask;
    }
    idx[m] = found;
}

// member m of set k (set_of[m] = k) marks bit idx[m] of row k
__global__ void mark_kernel(const int* __restrict__ idx, const int* __restrict__ set_of, int64_t M,
                            uint32_t* __restrict__ bits, int64_t words) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int g = idx[m];
    if (g < 0) return;
    atomicOr(&bits[(int64_t)set_of[m] * words + (g >> 5)], 1u << (g & 31));
}

__global__ void count_kernel(const uint32_t* __restrict__ bits, int64_t words, int64_t* __restrict__ counts) {
    __shared__ int64_t part[32];
    const int64_t k = blockIdx.x;
    int64_t c = 0;
    for (int64_t w = threadIdx.x; w < words; w += blockDim.x) c += __popc(bits[k * words + w]);
    for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += part[i];
        counts[k] = t;
    }
}

// block per set: chunks of blockDim words; per chunk a block scan of the
// words' popcounts places each thread's members after the preceding ones
__global__ void emit_kernel(const uint32_t* __restrict__ bits, int64_t words, const int64_t* __restrict__ offsets,
                            int32_t* __restrict__ genes) {
    __shared__ int warp_tot[32];
    __shared__ int64_t carry;
    const int64_t k = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = offsets[k];
    __syncthreads();
    for (int64_t w0 = 0; w0 < words; w0 += blockDim.x) {
        const int64_t w = w0 + threadIdx.x;
        const uint32_t word = w < words ? bits[k * words + w] : 0u;
        const int c = __popc(word);
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        int before = 0;
        for (int i = 0; i < warp; i++) before += warp_tot[i];
        int64_t pos = carry + before + incl - c;
        uint32_t x = word;
        while (x) {
            const int b = __ffs(x) - 1;
            x &= x - 1;
            genes[pos++] = (int32_t)((w << 5) + b);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int i = 0; i < nw; i++) t += warp_tot[i];
            carry += t;
        }
        __syncthreads();
    }
}

struct DevBuf {
    std::vector<void*> ptrs;
    ~DevBuf() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t bytes) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
        if (e == cudaSuccess) {
            ptrs.push_back(q);
            *p = static_cast<T*>(q);
        }
        return e;
    }
};

}  // namespace

extern "C" int gsea_map_sets(int64_t num_genes, const char* const* gene_symbols, int64_t num_sets,
                             const int64_t* set_symbol_offsets, const char* const* set_symbols,
                             int64_t* set_offsets_out, int32_t* set_genes_out, int64_t capacity, int64_t* nnz_out) {
    if (num_genes < 1 || num_genes > INT_MAX || num_sets < 0 || !gene_symbols || !set_offsets_out ||
        (num_sets > 0 && (!set_symbol_offsets || !set_symbols)))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    const int64_t G = num_genes, K = num_sets;
    const int64_t M = K ? set_symbol_offsets[K] : 0;
    if (K && set_symbol_offsets[0] != 0) return fail(GSEA_ERR_INVALID_INPUT, "set_symbol_offsets[0] must be 0");
    for (int64_t k = 0; k < K; k++)
        if (set_symbol_offsets[k + 1] < set_symbol_offsets[k])
            return fail(GSEA_ERR_INVALID_INPUT, "set_symbol_offsets must be non-decreasing");
    // byte blobs of the symbols
    std::vector<int64_t> goff((size_t)G + 1, 0), moff((size_t)M + 1, 0);
    std::vector<int> set_of((size_t)M);
    for (int64_t g = 0; g < G; g++) {
        if (!gene_symbols[g]) return fail(GSEA_ERR_INVALID_ARGUMENT, "null gene symbol");
        goff[g + 1] = goff[g] + (int64_t)std::strlen(gene_symbols[g]);
    }
    for (int64_t k = 0; k < K; k++)
        for (int64_t m = set_symbol_offsets[k]; m < set_symbol_offsets[k + 1]; m++) {
            if (!set_symbols[m]) return fail(GSEA_ERR_INVALID_ARGUMENT, "null set symbol");
            moff[m + 1] = moff[m] + (int64_t)std::strlen(set_symbols[m]);
            set_of[m] = (int)k;
        }
    std::vector<char> gblob((size_t)goff[G]), mblob((size_t)moff[M]);
    for (int64_t g = 0; g < G; g++) std::memcpy(gblob.data() + goff[g], gene_symbols[g], goff[g + 1] - goff[g]);
    for (int64_t m = 0; m < M; m++) std::memcpy(mblob.data() + moff[m], set_symbols[m], moff[m + 1] - moff[m]);

    uint64_t cap = 1;
    while (cap < 2 * (uint64_t)G) cap <<= 1;
    const int64_t words = (G + 31) / 32;
    DevBuf db;
    char *d_gblob, *d_mblob;
    int64_t *d_goff, *d_moff, *d_counts, *d_offsets;
    unsigned long long* d_keys;
    int *d_vals, *d_idx, *d_setof, *d_coll;
    uint32_t* d_bits;
    int32_t* d_genes;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = db.alloc(&d_gblob, gblob.size());
    if (e == cudaSuccess) e = db.alloc(&d_mblob, mblob.size());
    if (e == cudaSuccess) e = db.alloc(&d_goff, sizeof(int64_t) * goff.size());
    if (e == cudaSuccess) e = db.alloc(&d_moff, sizeof(int64_t) * moff.size());
    if (e == cudaSuccess) e = db.alloc(&d_keys, sizeof(unsigned long long) * cap);
    if (e == cudaSuccess) e = db.alloc(&d_vals, sizeof(int) * cap);
    if (e == cudaSuccess) e = db.alloc(&d_idx, sizeof(int) * (size_t)M);
    if (e == cudaSuccess) e = db.alloc(&d_setof, sizeof(int) * (size_t)M);
    if (e == cudaSuccess) e = db.alloc(&d_coll, sizeof(int));
    if (e == cudaSuccess) e = db.alloc(&d_bits, sizeof(uint32_t) * (size_t)K * words);
    if (e == cudaSuccess) e = db.alloc(&d_counts, sizeof(int64_t) * (size_t)(K + 1));
    if (e == cudaSuccess) e = db.alloc(&d_offsets, sizeof(int64_t) * (size_t)(K + 1));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gsea::cuda_fail(e, "set mapping buffers");
    }
    GSEA_CUDA(cudaMemcpy(d_gblob, gblob.data(), gblob.size(), cudaMemcpyHostToDevice), "copy symbols");
    GSEA_CUDA(cudaMemcpy(d_mblob, mblob.data(), mblob.size(), cudaMemcpyHostToDevice), "copy symbols");
    GSEA_CUDA(cudaMemcpy(d_goff, goff.data(), sizeof(int64_t) * goff.size(), cudaMemcpyHostToDevice), "copy offsets");
    GSEA_CUDA(cudaMemcpy(d_moff, moff.data(), sizeof(int64_t) * moff.size(), cudaMemcpyHostToDevice), "copy offsets");
    if (M) GSEA_CUDA(cudaMemcpy(d_setof, set_of.data(), sizeof(int) * (size_t)M, cudaMemcpyHostToDevice), "copy sets");
    GSEA_CUDA(cudaMemset(d_keys, 0, sizeof(unsigned long long) * cap), "clear table");
    GSEA_CUDA(cudaMemset(d_vals, 0x7f, sizeof(int) * cap), "clear table");
    GSEA_CUDA(cudaMemset(d_coll, 0, sizeof(int)), "clear flag");
    GSEA_CUDA(cudaMemset(d_bits, 0, sizeof(uint32_t) * (size_t)K * words), "clear bitmasks");
    insert_kernel<<<(unsigned)((G + 255) / 256), 256>>>(d_gblob, d_goff, G, d_keys, d_vals, cap - 1);
    if (M) {
        lookup_kernel<<<(unsigned)((M + 255) / 256), 256>>>(d_gblob, d_goff, d_mblob, d_moff, M, d_keys, d_vals,
                                                           cap - 1, d_idx, d_coll);
        mark_kernel<<<(unsigned)((M + 255) / 256), 256>>>(d_idx, d_setof, M, d_bits, words);
    }
    if (K) count_kernel<<<(unsigned)K, 256>>>(d_bits, words, d_counts);
    GSEA_CUDA(cudaGetLastError(), "set mapping kernels");
    int coll = 0;
    GSEA_CUDA(cudaMemcpy(&coll, d_coll, sizeof(int), cudaMemcpyDeviceToHost), "read flag");
    if (coll) return fail(GSEA_ERR_INVALID_INPUT, "two different symbols share a 64-bit hash");
    std::vector<int64_t> counts((size_t)K);
    if (K) GSEA_CUDA(cudaMemcpy(counts.data(), d_counts, sizeof(int64_t) * K, cudaMemcpyDeviceToHost), "read counts");
    set_offsets_out[0] = 0;
    for (int64_t k = 0; k < K; k++) set_offsets_out[k + 1] = set_offsets_out[k] + counts[k];
    const int64_t nnz = set_offsets_out[K];
    if (nnz_out) *nnz_out = nnz;
    if (!set_genes_out) return GSEA_OK;
    if (capacity < nnz) return fail(GSEA_ERR_INVALID_ARGUMENT, "set_genes_out is smaller than the mapped members");
    if (nnz) {
        GSEA_CUDA(db.alloc(&d_genes, sizeof(int32_t) * (size_t)nnz), "mapped members");
        GSEA_CUDA(cudaMemcpy(d_offsets, set_offsets_out, sizeof(int64_t) * (K + 1), cudaMemcpyHostToDevice),
                  "copy offsets");
        emit_kernel<<<(unsigned)K, 256>>>(d_bits, words, d_offsets, d_genes);
        GSEA_CUDA(cudaGetLastError(), "emit kernel");
        GSEA_CUDA(cudaMemcpy(set_genes_out, d_genes, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost), "copy members");
    }
    return GSEA_OK;
}
