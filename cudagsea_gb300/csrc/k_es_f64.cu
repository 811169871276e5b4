// k_es_f64.cu -- the fp64 instantiations of the enrichment kernels (k_es.cuh).
#include "k_es.cuh"

namespace gsea {

template cudaError_t launch_es<double>(const void*, bool, const double*, int, int, const int64_t*, const int32_t*,
                                       const int32_t*, const double*, int, double*, int64_t, int64_t, cudaStream_t,
                                       EsTuning, const int*);
template cudaError_t launch_es_batch<double>(const EsTask<double>*, const int64_t*, int, int64_t,
                                             unsigned long long*, int, int, EsTuning, cudaStream_t);
template cudaError_t launch_decay_table<double>(int, double*, cudaStream_t);

}  // namespace gsea
