// k_metric_f64.cu -- double instantiation of the plain-form metric kernels.
#include "k_metric.cuh"
namespace gsea {
template <>
cudaError_t launch_metric<double>(int metric, const double* X, int G, int S, const uint32_t* masks,
                                  int words, int num_perms, int64_t nA, int64_t nB, double* keys,
                                  const int* fast_ok, cudaStream_t st, int pb) {
    return launch_metric_impl<double>(metric, X, G, S, masks, words, num_perms, nA, nB, keys, fast_ok, st, pb);
}
template <>
int metric_multi_key<double>(int metric, int S, int words, bool fast_ok, int pb) {
    return metric_multi_key_impl<double>(metric, S, words, fast_ok, pb);
}
template <>
cudaError_t launch_metric_multi<double>(int key, const MetricTask<double>* d, const MetricTask<double>* h, int n,
                                   cudaStream_t st) {
    return launch_metric_multi_impl<double>(key, d, h, n, st);
}
}  // namespace gsea
