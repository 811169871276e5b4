// k_es_f32.cu -- the fp32 instantiations of the enrichment kernels (k_es.cuh).
#include "k_es.cuh"

namespace gsea {

int es_size_class(int G) { return es_wpl(G, G <= 65536); }

template cudaError_t launch_es<float>(const void*, bool, const float*, int, int, const int64_t*, const int32_t*,
                                      const int32_t*, const float*, int, float*, int64_t, int64_t, cudaStream_t,
                                      EsTuning, const int*);
template cudaError_t launch_es_batch<float>(const EsTask<float>*, const int64_t*, int, int64_t, unsigned long long*,
                                            int, int, EsTuning, cudaStream_t);
template cudaError_t launch_decay_table<float>(int, float*, cudaStream_t);

}  // namespace gsea
