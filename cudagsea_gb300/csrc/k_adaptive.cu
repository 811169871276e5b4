// k_adaptive.cu -- device helpers of the learned permutation allocator: metric
// moments, per-set null statistics, training samples, features and the
// exceedance counts of the sequential stopping rule.  No counterpart in the
// reference.
#include <math_constants.h>

#include "common.cuh"
#include "kernels.h"

namespace gsea {
namespace {

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < nw; w++) r += sh[w];
    return r;
}

// moments[0..4] = mean, sd, skewness of the finite keys; mean and sd of |key|
template <class T>
__global__ void __launch_bounds__(1024) moments_kernel(const T* __restrict__ keys, int G, double* __restrict__ out) {
    __shared__ double sh[32];
    double n = 0, s1 = 0, a1 = 0;
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
        const double v = (double)keys[g];
        if (isfinite(v)) {
            n += 1.0;
            s1 += v;
            a1 += fabs(v);
        }
    }
    n = block_sum(n, sh);
    s1 = block_sum(s1, sh);
    a1 = block_sum(a1, sh);
    const double mean = n > 0 ? s1 / n : 0.0, amean = n > 0 ? a1 / n : 0.0;
    double c2 = 0, c3 = 0, d2 = 0;
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
        const double v = (double)keys[g];
        if (isfinite(v)) {
            const double c = v - mean, d = fabs(v) - amean;
            c2 += c * c;
            c3 += c * c * c;
            d2 += d * d;
        }
    }
    c2 = block_sum(c2, sh);
    c3 = block_sum(c3, sh);
    d2 = block_sum(d2, sh);
    if (threadIdx.x == 0) {
        const double var = n > 0 ? c2 / n : 0.0, sd = sqrt(var);
        out[0] = mean;
        out[1] = sd;
        out[2] = sd > 0 ? (c3 / n) / (var * sd) : 0.0;
        out[3] = amean;
        out[4] = n > 0 ? sqrt(d2 / n) : 0.0;
    }
}

// mean |ES| of every set over columns [0, P)
template <class T>
__global__ void set_means_kernel(const T* __restrict__ es, int64_t ld, int64_t P, double* __restrict__ means) {
    __shared__ double sh[32];
    const int64_t k = blockIdx.x;
    double a = 0.0;
    for (int64_t p = threadIdx.x; p < P; p += blockDim.x) a += fabs((double)es[k * ld + p]);
    a = block_sum(a, sh);
    if (threadIdx.x == 0) means[k] = a / (double)P;
}

// x = [log n_k, r, mu/sd, skewness, cv of |metric|] with r a score in units
// of the set's null mean |ES|
__device__ __forceinline__ void features(float* x, double nk, double r, const double* mom) {
    const double n = nk > 1.0 ? nk : 1.0;
    x[0] = (float)log(n);
    x[1] = (float)r;
    x[2] = (float)(mom[1] > 0 ? mom[0] / mom[1] : 0.0);
    x[3] = (float)mom[2];
    x[4] = (float)(mom[3] > 0 ? mom[4] / mom[3] : 0.0);
}

// stratified query multiplier j of set k: 0.25 * 36^((j + h) / queries),
// h in [0, 1) from a hash of (k, j), so the multipliers cover [0.25, 9)
__device__ __forceinline__ double query_factor(int64_t k, int j, int queries) {
    uint64_t h = (uint64_t)k * 0x9E3779B97F4A7C15ull + (uint64_t)j * 0xC2B2AE3D27D4EB4Full + 0x165667B19E3779F9ull;
    h ^= h >> 33;
    h *= 0xFF51AFD7ED558CCDull;
    h ^= h >> 33;
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
    return 0.25 * exp(log(36.0) * ((double)j + u) / (double)queries);
}

constexpr int kMaxQueries = 24;

// Block per set with slot[k] != -1: queries u_j = m_k f_j (f_j from
// query_factor) and the observed |ES_k|; targets = fraction of the P columns
// with |ES| >= u, log m_k.  slot[k] >= 0: sample rows slot[k] .. of (x, t);
// slot[k] <= -2: rows -(slot[k] + 2) .. of (xv, tv).
template <class T>
__global__ void __launch_bounds__(256) model_samples_kernel(const T* __restrict__ es, int64_t ld, int64_t P,
                                                            const int64_t* __restrict__ off,
                                                            const double* __restrict__ mom,
                                                            const double* __restrict__ means, int queries,
                                                            const int64_t* __restrict__ slot, float* __restrict__ x,
                                                            float* __restrict__ t, float* __restrict__ xv,
                                                            float* __restrict__ tv) {
    __shared__ unsigned cnt[kMaxQueries + 1];
    __shared__ double u[kMaxQueries + 1];
    const int64_t k = blockIdx.x;
    const int64_t sl = slot[k];
    if (sl == -1) return;
    const double m = means[k];
    const T* row = es + k * ld;
    if (threadIdx.x < queries) u[threadIdx.x] = m * query_factor(k, threadIdx.x, queries);
    if (threadIdx.x == 0) u[queries] = fabs((double)row[0]);
    if (threadIdx.x <= kMaxQueries) cnt[threadIdx.x] = 0;
    __syncthreads();
    unsigned c[kMaxQueries + 1];
#pragma unroll
    for (int j = 0; j <= kMaxQueries; j++) c[j] = 0;
    for (int64_t p = threadIdx.x; p < P; p += blockDim.x) {
        const double v = fabs((double)row[p]);
#pragma unroll
        for (int j = 0; j <= kMaxQueries; j++)
            if (j <= queries) c[j] += v >= u[j];
    }
#pragma unroll
    for (int j = 0; j <= kMaxQueries; j++) {
        if (j > queries) break;
        unsigned v = c[j];
        for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&cnt[j], v);
    }
    __syncthreads();
    if (threadIdx.x <= queries) {
        const int j = threadIdx.x;
        const int64_t row_out = (sl >= 0 ? sl : -(sl + 2)) + j;
        float* xo = (sl >= 0 ? x : xv) + row_out * 5;
        float* to = (sl >= 0 ? t : tv) + row_out * 2;
        features(xo, (double)(off[k + 1] - off[k]), u[j] / m, mom);
        to[0] = (float)((double)cnt[j] / (double)P);
        to[1] = (float)log(m);
    }
}

// features of every set at its observed score, in units of the mean |ES| of
// its first n scores (sumabs[k] / n)
template <class T>
__global__ void model_features_kernel(const T* __restrict__ es, int64_t ld, const int64_t* __restrict__ off, int K,
                                      const double* __restrict__ mom, const double* __restrict__ sumabs, int64_t n,
                                      float* __restrict__ x) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const double m = sumabs[k] / (double)n;
    features(x + (int64_t)k * 5, (double)(off[k + 1] - off[k]), fabs((double)es[(int64_t)k * ld]) / m, mom);
}

// warp per listed set: exceed[k] += #{p in [lo, hi): |S_kp| >= |S_k0|},
// sumabs[k] += sum |S_kp|, sumabs[K + k] += sum S_kp^2
template <class T>
__global__ void exceed_kernel(const T* __restrict__ es, int64_t ld, const int32_t* __restrict__ list, int n_list,
                              int K, int64_t lo, int64_t hi, unsigned long long* __restrict__ exceed,
                              double* __restrict__ sumabs, const int* __restrict__ n_dev) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (n_dev) n_list = min(n_list, *n_dev);
    if (warp >= n_list) return;
    const int64_t k = list ? list[warp] : warp;
    const T* row = es + k * ld;
    const T a0 = fabs(row[0]);
    unsigned long long c = 0;
    double s = 0.0, s2 = 0.0;
    for (int64_t p = lo + lane; p < hi; p += 32) {
        const T a = fabs(row[p]);
        c += a >= a0;
        s += (double)a;
        s2 += (double)a * (double)a;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        c += __shfl_xor_sync(kFullMask, c, o);
        s += __shfl_xor_sync(kFullMask, s, o);
        s2 += __shfl_xor_sync(kFullMask, s2, o);
    }
    if (lane == 0) {
        exceed[k] += c;
        sumabs[k] += s;
        sumabs[K + k] += s2;
    }
}

// ---- the adaptive test's decisions on the device -------------------------

__device__ __forceinline__ double block_max(double v, double* sh) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v = fmax(v, __shfl_xor_sync(kFullMask, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = sh[0];
    for (int w = 1; w < nw; w++) r = fmax(r, sh[w]);
    return r;
}

// one block of 1,024 threads
template <class T>
__global__ void __launch_bounds__(1024)
adaptive_prepare_kernel(int K, const T* __restrict__ stats, const float* __restrict__ pred,
                        const double* __restrict__ sumabs, AdaptiveRule rule, double* __restrict__ err,
                        AdaptiveCtl* __restrict__ ctl) {
    __shared__ double sh[32];
    double pstar = 0.0, plo = CUDART_INF, valid = 0.0, ok = 0.0;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const double q = (double)stats[4 * (size_t)K + k], np = (double)stats[2 * (size_t)K + k];
        if (q < rule.q_call && np > pstar) pstar = np;
        if (!(q < rule.q_call) && np < plo) plo = np;  // the pilot's non-calls
        if (pred) {
            const double mt = (double)pred[2 * (size_t)k + 1], mh = sumabs[k] / (double)rule.P0;
            double e = CUDART_NAN;
            if (isfinite(mt) && mt > 0.0 && isfinite(mh) && mh > 0.0) {
                e = fabs(log(mt / mh));
                valid += 1.0;
                ok += e <= rule.tol ? 1.0 : 0.0;
            }
            err[k] = e;
        }
    }
    pstar = block_max(pstar, sh);
    plo = -block_max(-plo, sh);
    valid = block_sum(valid, sh);
    ok = block_sum(ok, sh);
    if (threadIdx.x == 0) {
        ctl->stop_p = fmin(1.0, fmax(rule.p_floor, rule.margin * pstar));
        ctl->p_sig = rule.sig_margin > 0.0 ? plo / rule.sig_margin : 0.0;
        // the median error is within tolerance iff at least n/2 + 1 of the n errors are
        const unsigned long long nv = (unsigned long long)valid, nk = (unsigned long long)ok;
        ctl->model_used = (pred && nv > 0 && nk >= nv / 2 + 1) ? 1 : 0;
        ctl->valid = nv;
        ctl->within_tol = nk;
    }
}

// the model's prior of set k: probability pm and pseudo-count w (w = 0: none),
// rounded through float as the host rule receives them
__device__ __forceinline__ void model_prior(const float* pred, int64_t k, const AdaptiveRule& rule, double& pm,
                                            double& w) {
    const double v = fmin(fmax((double)pred[2 * k], 1e-6), 1.0 - 1e-6);
    const float pf = (float)v;
    const float wf = (float)fmin(1.0 / (rule.s2 * v * (1.0 - v)), rule.cap);
    pm = fmin(fmax((double)pf, 1e-6), 1.0 - 1e-6);
    w = (isfinite(pf) && isfinite(wf) && wf > 0.f) ? (double)wf : 0.0;
}

__device__ __forceinline__ bool prior_agrees_dev(double pm, double w, double n, double c, double z) {
    const double sd_pp = sqrt(pm * (1.0 - pm) * (w + n) / (n * (w + 1.0)));
    return fabs(c / n - pm) <= z * sd_pp;
}

__global__ void adaptive_decide_kernel(int K, const int32_t* __restrict__ list, const int* __restrict__ n_dev,
                                       const int64_t* __restrict__ counts, const unsigned long long* __restrict__ exceed,
                                       const float* __restrict__ pred, const float* __restrict__ qlow,
                                       const float* __restrict__ qhigh, int bound_on, int pilot, AdaptiveRule rule,
                                       uint8_t* __restrict__ stop, AdaptiveCtl* __restrict__ ctl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_list = list ? min(K, *n_dev) : K;
    if (i >= n_list) return;
    const int64_t k = list ? list[i] : i;
    const double n = (double)counts[k], c = (double)exceed[k];
    uint8_t s = 0;
    if (n > 0 && c >= 0 && c <= n) {
        double a = 0.5 + c, b = 0.5 + (n - c);
        if (pred && ctl->model_used) {
            double pm, w;
            model_prior(pred, k, rule, pm, w);
            if (w > 0.0) {
                const bool agree = prior_agrees_dev(pm, w, n, c, rule.z);
                if (agree) {
                    a += pm * w;
                    b += (1.0 - pm) * w;
                }
                if (pilot) {
                    atomicAdd(&ctl->prior_sets, 1ull);
                    if (agree) atomicAdd(&ctl->prior_agreed, 1ull);
                }
            }
        }
        const double t = a + b, mean = a / t, sd = sqrt(a * b / (t * t * (t + 1.0)));
        s = mean - rule.z * sd >= ctl->stop_p ? 1 : 0;
        // clearly significant: p confidently below every pilot non-call's
        // p (by sig_margin) and the q upper bound below the call level (by
        // sig_margin)
        if (!s && bound_on && qhigh && rule.sig_margin > 0.0 && counts[k] < rule.P &&
            mean + rule.z * sd <= ctl->p_sig && (double)qhigh[k] <= rule.q_call / rule.sig_margin) {
            s = 1;
            atomicAdd(&ctl->stopped_sig, 1ull);
        }
    }
    if (bound_on && !s && rule.q_stop > 0.0 && counts[k] < rule.P && (double)qlow[k] >= rule.q_stop) {
        s = 1;
        atomicAdd(&ctl->stopped_q, 1ull);
    }
    if (pilot && s) atomicAdd(&ctl->stopped_pilot, 1ull);
    stop[k] = s;
}

// one block of 1,024 threads: a block-wide scan per chunk of the set order
__global__ void __launch_bounds__(1024)
adaptive_compact_kernel(int K, const int32_t* __restrict__ order, const uint8_t* __restrict__ stop,
                        int32_t* __restrict__ active, AdaptiveCtl* __restrict__ ctl) {
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < K; base += 1024) {
        const int i = base + threadIdx.x;
        const int k = i < K ? order[i] : 0;
        const int f = (i < K && !stop[k]) ? 1 : 0;
        const unsigned bal = __ballot_sync(kFullMask, f);
        const int in_warp = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        int before = carry;
        for (int w = 0; w < warp; w++) before += warp_tot[w];
        if (f) active[before + in_warp] = k;
        int total = 0;
        for (int w = 0; w < 32; w++) total += warp_tot[w];
        __syncthreads();  // warp_tot is rewritten by the next chunk
        carry += total;
    }
    if (threadIdx.x == 0) ctl->n_active = carry;
}

__global__ void adaptive_counts_kernel(int K, const int32_t* __restrict__ active, AdaptiveCtl* __restrict__ ctl,
                                       int64_t next, int64_t* __restrict__ counts) {
    const int n = min(K, ctl->n_active);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) counts[active[i]] = next;
    if (i == 0 && n > 0) ctl->rounds += 1;
}

__global__ void adaptive_reset_kernel(int K, int64_t v, int64_t* __restrict__ counts, AdaptiveCtl* __restrict__ ctl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < K) counts[i] = v;
    if (i == 0) {
        AdaptiveCtl z{};
        z.rounds = 1;
        z.n_active = K;
        *ctl = z;
    }
}

}  // namespace

template <class T>
cudaError_t launch_adaptive_prepare(int K, const T* stats, const float* pred, const double* sumabs,
                                    const AdaptiveRule& rule, double* err, AdaptiveCtl* ctl, cudaStream_t st) {
    adaptive_prepare_kernel<T><<<1, 1024, 0, st>>>(K, stats, pred, sumabs, rule, err, ctl);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_adaptive_prepare<float>(int, const float*, const float*, const double*,
                                                    const AdaptiveRule&, double*, AdaptiveCtl*, cudaStream_t);
template cudaError_t launch_adaptive_prepare<double>(int, const double*, const float*, const double*,
                                                     const AdaptiveRule&, double*, AdaptiveCtl*, cudaStream_t);

cudaError_t launch_adaptive_decide(int K, const int32_t* list, const int* n_dev, const int64_t* counts,
                                   const unsigned long long* exceed, const float* pred, const float* qlow,
                                   const float* qhigh, bool bound_on, bool pilot, const AdaptiveRule& rule,
                                   uint8_t* stop, AdaptiveCtl* ctl, cudaStream_t st) {
    if (K <= 0) return cudaSuccess;
    adaptive_decide_kernel<<<(K + 255) / 256, 256, 0, st>>>(K, list, n_dev, counts, exceed, pred, qlow, qhigh,
                                                            bound_on ? 1 : 0, pilot ? 1 : 0, rule, stop, ctl);
    launches_add(1);
    return cudaGetLastError();
}

cudaError_t launch_adaptive_compact(int K, const int32_t* order, const uint8_t* stop, int32_t* active,
                                    AdaptiveCtl* ctl, cudaStream_t st) {
    adaptive_compact_kernel<<<1, 1024, 0, st>>>(K, order, stop, active, ctl);
    launches_add(1);
    return cudaGetLastError();
}

cudaError_t launch_adaptive_counts(int K, const int32_t* active, AdaptiveCtl* ctl, int64_t next,
                                   int64_t* counts, cudaStream_t st) {
    if (K <= 0) return cudaSuccess;
    adaptive_counts_kernel<<<(K + 255) / 256, 256, 0, st>>>(K, active, ctl, next, counts);
    launches_add(1);
    return cudaGetLastError();
}

cudaError_t launch_adaptive_reset(int K, int64_t v, int64_t* counts, AdaptiveCtl* ctl, cudaStream_t st) {
    adaptive_reset_kernel<<<(K + 255) / 256, 256, 0, st>>>(K, v, counts, ctl);
    launches_add(1);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_moments(const T* keys, int G, double* moments, cudaStream_t st) {
    moments_kernel<T><<<1, 1024, 0, st>>>(keys, G, moments);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_moments<float>(const float*, int, double*, cudaStream_t);
template cudaError_t launch_moments<double>(const double*, int, double*, cudaStream_t);

template <class T>
cudaError_t launch_set_means(const T* es, int64_t ld, int64_t P, int K, double* means, cudaStream_t st) {
    if (K <= 0) return cudaSuccess;
    set_means_kernel<T><<<K, 256, 0, st>>>(es, ld, P, means);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_set_means<float>(const float*, int64_t, int64_t, int, double*, cudaStream_t);
template cudaError_t launch_set_means<double>(const double*, int64_t, int64_t, int, double*, cudaStream_t);

int model_max_queries() { return kMaxQueries; }

template <class T>
cudaError_t launch_model_samples(const T* es, int64_t ld, int64_t P, const int64_t* off, int K, const double* mom,
                                 const double* means, int queries, const int64_t* slot, float* x, float* t,
                                 float* xv, float* tv, cudaStream_t st) {
    if (K <= 0) return cudaSuccess;
    if (queries < 1 || queries > kMaxQueries) return cudaErrorInvalidValue;
    model_samples_kernel<T><<<K, 256, 0, st>>>(es, ld, P, off, mom, means, queries, slot, x, t, xv, tv);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_model_samples<float>(const float*, int64_t, int64_t, const int64_t*, int, const double*,
                                                 const double*, int, const int64_t*, float*, float*, float*, float*,
                                                 cudaStream_t);
template cudaError_t launch_model_samples<double>(const double*, int64_t, int64_t, const int64_t*, int, const double*,
                                                  const double*, int, const int64_t*, float*, float*, float*, float*,
                                                  cudaStream_t);

template <class T>
cudaError_t launch_model_features(const T* es, int64_t ld, const int64_t* off, int K, const double* mom,
                                  const double* sumabs, int64_t n, float* x, cudaStream_t st) {
    if (K <= 0) return cudaSuccess;
    model_features_kernel<T><<<(K + 255) / 256, 256, 0, st>>>(es, ld, off, K, mom, sumabs, n, x);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_model_features<float>(const float*, int64_t, const int64_t*, int, const double*,
                                                  const double*, int64_t, float*, cudaStream_t);
template cudaError_t launch_model_features<double>(const double*, int64_t, const int64_t*, int, const double*,
                                                   const double*, int64_t, float*, cudaStream_t);

template <class T>
cudaError_t launch_exceed(const T* es, int64_t ld, int K, const int32_t* list, int n_list, int64_t lo, int64_t hi,
                          unsigned long long* exceed, double* sumabs, cudaStream_t st, const int* n_dev) {
    if (n_list <= 0 || hi <= lo) return cudaSuccess;
    exceed_kernel<T><<<(n_list + 7) / 8, 256, 0, st>>>(es, ld, list, n_list, K, lo, hi, exceed, sumabs, n_dev);
    launches_add(1);
    return cudaGetLastError();
}
template cudaError_t launch_exceed<float>(const float*, int64_t, int, const int32_t*, int, int64_t, int64_t,
                                          unsigned long long*, double*, cudaStream_t, const int*);
template cudaError_t launch_exceed<double>(const double*, int64_t, int, const int32_t*, int, int64_t, int64_t,
                                           unsigned long long*, double*, cudaStream_t, const int*);

}  // namespace gsea
