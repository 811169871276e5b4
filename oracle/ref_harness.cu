// Test-infrastructure harness around the REFERENCE's own CPU implementation.
//
// This file is compiled only by oracle/build_ref.sh, against the untouched
// cudaGSEA sources (staged as symlinks so that CUDA 13's CCCL CUB replaces the
// vendored CUB 1.5).  It is never linked into the product library.  It exposes
// the reference's CPU pipeline stages behind extern "C" entry points so that
// tests/golden/make_golden.py can generate golden vectors with ctypes:
//
//   ref_correlate_*   -> correllate_genes_cpu   (src/include/correlate_genes.cuh:302-462)
//   ref_sort_*        -> pathway_sort_cpu       (src/include/batched_sort.cuh:271-326)
//   ref_scores_*      -> create_bitmaps + compute_scores_cpu
//                        (src/include/create_bitmaps.cuh:13-65,
//                         src/include/enrichment_scores.cuh:259-336)
//   ref_pipeline_*    -> the loop of compute_gsea_cpu (src/include/cugsea.cuh:273-453)
//                        without file parsing, followed by final_statistics
//                        (src/include/statistics.cuh:46-117)
//
// The reference CPU path reads the expression table gene-major
// (table[gene*S + sample], correlate_genes.cuh:111-112 with transposed=false).

#include <cstdint>
#include <cstring>
#include <numeric>
#include <climits>
#include <functional>
#include <algorithm>
#include <string>
#include <vector>
#include <cuda_runtime.h>

// The CPU stages call CUERR after each dispatch; with no GPU in the build
// container cudaGetLastError() would report a driver error and exit.
#define cudaGetLastError() cudaSuccess
#define CUDA_GSEA_OPENMP_ENABLED

#include "include/configuration.cuh"
#undef CUDA_GSEA_PRINT_INFO
#undef CUDA_GSEA_PRINT_WARNINGS
#include "include/bitmap_types.cuh"
#include "include/create_bitmaps.cuh"
#include "include/correlate_genes.cuh"
#include "include/batched_sort.cuh"
#include "include/enrichment_scores.cuh"
#include "include/statistics.cuh"

namespace {

std::vector<std::string> gene_symbols(size_t G) {
    std::vector<std::string> s(G);
    for (size_t g = 0; g < G; g++) s[g] = "g" + std::to_string(g);
    return s;
}

std::vector<std::vector<std::string>> set_symbols(const int64_t* off, const int32_t* genes,
                                                  size_t K) {
    std::vector<std::vector<std::string>> sets(K);
    for (size_t k = 0; k < K; k++)
        for (int64_t i = off[k]; i < off[k + 1]; i++)
            sets[k].push_back("g" + std::to_string(genes[i]));
    return sets;
}

template <class T>
int correlate(const char* metric, const T* exprs_gm, const uint8_t* labels, size_t G,
              size_t S, size_t P, size_t shift, T* out) {
    size_t nA = 0, nB = 0;
    for (size_t i = 0; i < S; i++) { nA += labels[i] == 0; nB += labels[i] == 1; }
    std::vector<T> table(exprs_gm, exprs_gm + G * S);
    std::vector<unsigned char> lab(labels, labels + S);
    correllate_genes_cpu(table.data(), lab.data(), out, G, nA, nB, P, std::string(metric),
                         shift);
    return 0;
}

template <class T>
int sort_desc(T* keys, size_t G, size_t P, uint32_t* idx_out, int ascending) {
    std::vector<unsigned int> oindx(G);
    std::iota(oindx.begin(), oindx.end(), 0);
    if (ascending)
        pathway_sort_cpu<T, unsigned int, size_t, true>(keys, oindx.data(), idx_out, G, P);
    else
        pathway_sort_cpu<T, unsigned int, size_t, false>(keys, oindx.data(), idx_out, G, P);
    return 0;
}

template <class T, class bitmap_t>
int scores(const T* sorted_keys, const uint32_t* sorted_idx, size_t G, size_t P,
           const int64_t* off, const int32_t* genes, size_t K, T* es_out /* K x P */) {
    auto gsymb = gene_symbols(G);
    auto pathw = set_symbols(off, genes, K);
    const size_t batch = 8 * sizeof(bitmap_t);
    std::vector<T> keys(sorted_keys, sorted_keys + G * P);
    std::vector<unsigned int> idx(sorted_idx, sorted_idx + G * P);
    std::vector<bitmap_t> opath;
    for (size_t lo = 0; lo < K; lo += batch) {
        size_t width = std::min(batch, K - lo);
        create_bitmaps(gsymb, pathw, opath, lo, width);
        std::vector<T> local(width * P, 0);
        compute_scores_cpu(keys.data(), idx.data(), opath.data(), local.data(), G, P, width);
        for (size_t a = 0; a < width; a++)
            for (size_t p = 0; p < P; p++) es_out[(lo + a) * P + p] = local[a * P + p];
    }
    return 0;
}

template <class T, class bitmap_t>
int pipeline(const char* metric, const T* exprs_gm, const uint8_t* labels, size_t G, size_t S,
             const int64_t* off, const int32_t* genes, size_t K, size_t P, int ascending,
             T* es_out, T* stats_out) {
    // one permutation batch holding all permutations (the reference's scheduler
    // only splits batches for memory, which does not change any value)
    std::vector<T> correl(G * P);
    correlate<T>(metric, exprs_gm, labels, G, S, P, 0, correl.data());
    std::vector<uint32_t> idx(G * P);
    sort_desc<T>(correl.data(), G, P, idx.data(), ascending);
    scores<T, bitmap_t>(correl.data(), idx.data(), G, P, off, genes, K, es_out);
    std::vector<T> global(es_out, es_out + K * P);
    auto res = final_statistics(global, K, P);
    std::copy(res.begin(), res.end(), stats_out);
    return 0;
}

}  // namespace

extern "C" {

int ref_correlate_f32(const char* m, const float* x, const uint8_t* l, size_t G, size_t S,
                      size_t P, size_t shift, float* out) {
    return correlate<float>(m, x, l, G, S, P, shift, out);
}
int ref_correlate_f64(const char* m, const double* x, const uint8_t* l, size_t G, size_t S,
                      size_t P, size_t shift, double* out) {
    return correlate<double>(m, x, l, G, S, P, shift, out);
}
int ref_sort_f32(float* keys, size_t G, size_t P, uint32_t* idx, int asc) {
    return sort_desc<float>(keys, G, P, idx, asc);
}
int ref_sort_f64(double* keys, size_t G, size_t P, uint32_t* idx, int asc) {
    return sort_desc<double>(keys, G, P, idx, asc);
}
int ref_scores_f32(const float* k, const uint32_t* i, size_t G, size_t P, const int64_t* off,
                   const int32_t* genes, size_t K, float* es) {
    return scores<float, bitmap32_t>(k, i, G, P, off, genes, K, es);
}
int ref_scores_f64(const double* k, const uint32_t* i, size_t G, size_t P, const int64_t* off,
                   const int32_t* genes, size_t K, double* es) {
    return scores<double, bitmap64_t>(k, i, G, P, off, genes, K, es);
}
int ref_final_statistics_f32(const float* es, size_t K, size_t P, float* out) {
    std::vector<float> v(es, es + K * P);
    auto r = final_statistics(v, K, P);
    std::copy(r.begin(), r.end(), out);
    return 0;
}
int ref_final_statistics_f64(const double* es, size_t K, size_t P, double* out) {
    std::vector<double> v(es, es + K * P);
    auto r = final_statistics(v, K, P);
    std::copy(r.begin(), r.end(), out);
    return 0;
}
int ref_pipeline_f32(const char* m, const float* x, const uint8_t* l, size_t G, size_t S,
                     const int64_t* off, const int32_t* genes, size_t K, size_t P, int asc,
                     float* es, float* stats) {
    return pipeline<float, bitmap32_t>(m, x, l, G, S, off, genes, K, P, asc, es, stats);
}
int ref_pipeline_f64(const char* m, const double* x, const uint8_t* l, size_t G, size_t S,
                     const int64_t* off, const int32_t* genes, size_t K, size_t P, int asc,
                     double* es, double* stats) {
    return pipeline<double, bitmap64_t>(m, x, l, G, S, off, genes, K, P, asc, es, stats);
}

}  // extern "C"
