// k_metric_f32.cu -- float instantiation of the plain-form metric kernels.
#include "k_metric.cuh"
namespace gsea {
template <>
cudaError_t launch_metric<float>(int metric, const float* X, int G, int S, const uint32_t* masks,
                                 int words, int num_perms, int64_t nA, int64_t nB, float* keys,
                                 const int* fast_ok, cudaStream_t st, int pb) {
    return launch_metric_impl<float>(metric, X, G, S, masks, words, num_perms, nA, nB, keys, fast_ok, st, pb);
}
template <>
int metric_multi_key<float>(int metric, int S, int words, bool fast_ok, int pb) {
    return metric_multi_key_impl<float>(metric, S, words, fast_ok, pb);
}
template <>
cudaError_t launch_metric_multi<float>(int key, const MetricTask<float>* d, const MetricTask<float>* h, int n,
                                   cudaStream_t st) {
    return launch_metric_multi_impl<float>(key, d, h, n, st);
}
}  // namespace gsea
