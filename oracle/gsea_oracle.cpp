// gsea_oracle.cpp -- CPU restatement of cudaGSEA's permutation pipeline.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is compared
// against; it is imported by tests/, by __graft_entry__.smoke() and by the
// cpu_baseline / reference leg of bench.py, and by nothing else.  The product
// library (cudagsea_gb300/csrc) never links or calls it.
//
// Each stage restates the reference algorithm (paths relative to the
// cudaGSEA project, src/ = cudaGSEA/src/):
//   nvidia_hash                     src/include/rngpu/rngpu.hpp:27-38
//   fast KISS init / step           src/include/rngpu/rngpu.hpp:145-178
//   Fisher-Yates on labels          src/include/rngpu/rngpu.hpp:288-303,
//                                   caller src/include/correlate_genes.cuh:94-103
//   6 accumulators, 5 combiners     src/include/functors.cuh:10-433
//   metric dispatch (14 names)      src/include/correlate_genes.cuh:166-295
//   per-permutation sort            src/include/batched_sort.cuh:91-269 (GPU
//                                   semantics: stable LSD radix order, see below)
//   running-sum ES (Kahan)          src/include/enrichment_scores.cuh:259-336
//   final statistics                src/include/statistics.cuh:46-117
//   FDR (absent in the reference, which returns NaN at statistics.cuh:112-114)
//
// Sort order: the reference GPU path sorts with CUB's stable segmented radix
// sort on the IEEE bit pattern (batched_sort.cuh:144-186), so ties keep gene
// order and -0.0 ranks below +0.0; the reference CPU path uses std::sort
// (batched_sort.cuh:317), which leaves ties in unspecified order.  This oracle
// adopts the GPU semantics; comparisons against the reference CPU build treat
// tie groups as unordered.
//
// Compile with -ffp-contract=off: every product is rounded before it is added,
// as in the reference's x86-64 CPU build.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace {

// ---------------------------------------------------------------- RNG
inline uint32_t nv_hash(uint32_t x) {
    x = (x + 0x7ed55d16u) + (x << 12);
    x = (x ^ 0xc761c23cu) ^ (x >> 19);
    x = (x + 0x165667b1u) + (x << 5);
    x = (x + 0xd3a2646cu) ^ (x << 9);
    x = (x + 0xfd7046c5u) + (x << 3);
    x = (x ^ 0xb55a4f09u) ^ (x >> 16);
    return x;
}

struct Kiss { uint32_t x, y, z, w, c; };

inline Kiss kiss_seed(uint32_t seed) {
    Kiss s;
    s.w = seed ? seed : 0xFFFFFFFFu;
    s.x = s.y = s.z = 0;
    for (int it = 0; it < 8; it++) {
        s.x = nv_hash(s.w);
        s.y = nv_hash(s.x);
        s.z = nv_hash(s.y);
        s.w = nv_hash(s.z);
    }
    s.c = 0;
    return s;
}

inline uint32_t kiss_next(Kiss& s) {
    s.y ^= s.y << 5;
    s.y ^= s.y >> 7;
    s.y ^= s.y << 22;
    int32_t t = (int32_t)(s.z + s.w + s.c);
    s.z = s.w;
    s.c = t < 0;
    s.w = (uint32_t)t & 2147483647u;
    s.x += 1411392427u;
    return s.x + s.y + s.w;
}

// labels of permutation `gperm` (global index); permutation 0 is the identity
void permuted_labels(const uint8_t* labels, size_t S, size_t gperm, uint32_t seed, uint8_t* out) {
    std::memcpy(out, labels, S);
    if (gperm == 0 || S < 2) return;
    Kiss st = kiss_seed((uint32_t)(gperm + seed));
    for (size_t i = S - 1; i >= 1; i--) {
        size_t r = (size_t)((double)kiss_next(st) * (double)(i + 1) / 4294967296.0);
        uint8_t t = out[i];
        out[i] = out[r];
        out[r] = t;
    }
}

// ---------------------------------------------------------------- metrics
enum Acc { NAIVE, KAHAN, ONEPASS, TWOPASS, KNUTH, OVERKILL };
enum Comb { DIFF, RATIO, LOG2, S2N, TTEST };

struct MetricSpec { Acc acc; Comb comb; };
const MetricSpec kMetrics[14] = {
    {NAIVE, DIFF},   {NAIVE, RATIO},   {NAIVE, LOG2},                       // naive_*
    {KAHAN, DIFF},   {KAHAN, RATIO},   {KAHAN, LOG2},                       // stable_*_of_classes
    {ONEPASS, S2N},  {ONEPASS, TTEST},                                      // onepass_*
    {TWOPASS, S2N},  {TWOPASS, TTEST},                                      // twopass_*
    {KNUTH, S2N},    {KNUTH, TTEST},                                        // stable_s2n / t
    {OVERKILL, S2N}, {OVERKILL, TTEST}};                                    // overkill_*

template <class T> inline T cuabs(T x) { return x < 0 ? -x : x; }
inline float c_sqrt(float x) { return sqrtf(x); }
inline double c_sqrt(double x) { return sqrt(x); }
inline float c_log(float x) { return logf(x); }
inline double c_log(double x) { return log(x); }

template <class T>
T combine(Comb c, T mA, T vA, size_t nA, T mB, T vB, size_t nB) {
    switch (c) {
        case DIFF: return mA - mB;
        case RATIO: return mA / mB;
        case LOG2: return (T)(c_log(mA / mB) * 1.44269504089);  // double literal product
        case S2N: {
            T sA = c_sqrt(vA), sB = c_sqrt(vB);
            T lowA = 0.2 * cuabs(mA);  // product in double, rounded to T
            T lowB = 0.2 * cuabs(mB);
            sA = lowA < sA ? sA : lowA;
            sB = lowB < sB ? sB : lowB;
            return (mA - mB) / (sA + sB);
        }
        case TTEST: {
            T wA = vA, wB = vB;
            T lowA = 0.04 * cuabs(mA);
            T lowB = 0.04 * cuabs(mB);
            wA = lowA < wA ? wA : lowA;
            wB = lowB < wB ? wB : lowB;
            return (mA - mB) / c_sqrt(wA / (T)nA + wB / (T)nB);
        }
    }
    return 0;
}

// x(s) = table[s*G + g]; lab[s] = permuted label (class A <=> label 0)
template <class T>
T metric_one(const MetricSpec& ms, const T* table, size_t G, size_t g, const uint8_t* lab, size_t S,
             size_t nA, size_t nB) {
    T mA = 0, mB = 0, vA = 0, vB = 0;
    switch (ms.acc) {
        case NAIVE: {  // functors.cuh:87-124
            for (size_t s = 0; s < S; s++) {
                const uint8_t l = !lab[s];
                const T x = table[s * G + g];
                mA += (T)l * x;
                mB += (T)(!l) * x;
            }
            mA /= (T)nA; mB /= (T)nB;
            return combine<T>(ms.comb, mA, 0, nA, mB, 0, nB);
        }
        case KAHAN: case OVERKILL: {  // functors.cuh:126-176, 297-375
            T kA = 0, kB = 0;
            for (size_t s = 0; s < S; s++) {
                const bool l = !lab[s];
                const T x = table[s * G + g];
                const T acc = l ? mA : mB;
                const T alpha = x - (l ? kA : kB);
                const T beta = acc + alpha;
                const T kk = (beta - acc) - alpha;
                if (l) { kA = kk; mA = beta; } else { kB = kk; mB = beta; }
            }
            mA /= (T)nA; mB /= (T)nB;
            if (ms.acc == KAHAN) return combine<T>(ms.comb, mA, 0, nA, mB, 0, nB);
            T aA = 0, aB = 0;
            for (size_t s = 0; s < S; s++) {
                const bool l = !lab[s];
                const T x = table[s * G + g];
                if (l) { const T d = x - mA; aA = aA + d; vA = vA + d * d; }
                else   { const T d = x - mB; aB = aB + d; vB = vB + d * d; }
            }
            vA = vA - aA * aA / (T)nA;
            vB = vB - aB * aB / (T)nB;
            vA = vA / (T)nA; vB = vB / (T)nB;
            return combine<T>(ms.comb, mA, vA, nA, mB, vB, nB);
        }
        case ONEPASS: {  // functors.cuh:178-229 (biased)
            for (size_t s = 0; s < S; s++) {
                const bool l = !lab[s];
                const T x = table[s * G + g];
                if (l) { mA = mA + x; vA = vA + x * x; }
                else   { mB = mB + x; vB = vB + x * x; }
            }
            mA /= (T)nA; mB /= (T)nB;
            vA = vA / (T)nA - mA * mA;
            vB = vB / (T)nB - mB * mB;
            return combine<T>(ms.comb, mA, vA, nA, mB, vB, nB);
        }
        case TWOPASS: {  // functors.cuh:232-295 (biased)
            for (size_t s = 0; s < S; s++) {
                const bool l = !lab[s];
                const T x = table[s * G + g];
                if (l) mA = mA + x; else mB = mB + x;
            }
            mA /= (T)nA; mB /= (T)nB;
            for (size_t s = 0; s < S; s++) {
                const bool l = !lab[s];
                const T x = table[s * G + g];
                if (l) vA = vA + (x - mA) * (x - mA);
                else   vB = vB + (x - mB) * (x - mB);
            }
            vA = vA / (T)nA; vB = vB / (T)nB;
            return combine<T>(ms.comb, mA, vA, nA, mB, vB, nB);
        }
        case KNUTH: {  // functors.cuh:377-433 (biased)
            size_t iA = 0, iB = 0;
            for (size_t s = 0; s < S; s++) {
                const bool l = !lab[s];
                const T x = table[s * G + g];
                if (l) {
                    iA++;
                    const T d = x - mA;
                    mA = mA + d / (T)iA;
                    vA = vA + d * (x - mA);
                } else {
                    iB++;
                    const T d = x - mB;
                    mB = mB + d / (T)iB;
                    vB = vB + d * (x - mB);
                }
            }
            vA = vA / (T)nA; vB = vB / (T)nB;
            return combine<T>(ms.comb, mA, vA, nA, mB, vB, nB);
        }
    }
    return 0;
}

// NaN keys are written as the positive all-ones NaN: the platform's default
// NaN differs (x86 produces a negative one, Arm and CUDA positive ones), and
// its sign decides where NaNs rank.  Canonical NaNs rank first when
// descending, in gene order, as CUDA's canonical NaN does in the reference's
// GPU sort.
inline float canonical_nan(float v) {
    if (v == v) return v;
    uint32_t u = 0x7fffffffu; float f; std::memcpy(&f, &u, 4); return f;
}
inline double canonical_nan(double v) {
    if (v == v) return v;
    uint64_t u = 0x7fffffffffffffffull; double f; std::memcpy(&f, &u, 8); return f;
}

template <class T>
int metric_all(int metric, const T* table, const uint8_t* labels, size_t G, size_t S, size_t P,
               size_t shift, uint32_t seed, T* keys) {
    if (metric < 0 || metric >= 14) return 2;
    size_t nA = 0, nB = 0;
    for (size_t s = 0; s < S; s++) { nA += labels[s] == 0; nB += labels[s] == 1; }
    const MetricSpec ms = kMetrics[metric];
#pragma omp parallel for schedule(dynamic)
    for (long long p = 0; p < (long long)P; p++) {
        std::vector<uint8_t> lab(S);
        permuted_labels(labels, S, (size_t)p + shift, seed, lab.data());
        for (size_t g = 0; g < G; g++)
            keys[(size_t)p * G + g] = canonical_nan(metric_one<T>(ms, table, G, g, lab.data(), S, nA, nB));
    }
    return 0;
}

// ---------------------------------------------------------------- sort
// radix order of an IEEE value: ascending unsigned order == ascending value
// order with -0 < +0 and NaNs (by sign) at the two ends.
inline uint32_t radix_key(float f) {
    uint32_t u; std::memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
inline uint64_t radix_key(double f) {
    uint64_t u; std::memcpy(&u, &f, 8);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

template <class T>
void sort_all(const T* keys, size_t G, size_t P, int ascending, T* sorted_keys, uint32_t* idx) {
#pragma omp parallel for schedule(dynamic)
    for (long long p = 0; p < (long long)P; p++) {
        const T* k = keys + (size_t)p * G;
        std::vector<uint32_t> ord(G);
        std::iota(ord.begin(), ord.end(), 0u);
        if (ascending)
            std::stable_sort(ord.begin(), ord.end(),
                             [&](uint32_t a, uint32_t b) { return radix_key(k[a]) < radix_key(k[b]); });
        else
            std::stable_sort(ord.begin(), ord.end(),
                             [&](uint32_t a, uint32_t b) { return radix_key(k[a]) > radix_key(k[b]); });
        for (size_t i = 0; i < G; i++) {
            sorted_keys[(size_t)p * G + i] = k[ord[i]];
            idx[(size_t)p * G + i] = ord[i];
        }
    }
}

// ---------------------------------------------------------------- ES
// Dense two-pass Kahan running sum of enrichment_scores.cuh:267-336.  Set
// membership is a per-gene flag (duplicates collapse, as with the bitmaps of
// create_bitmaps.cuh:13-65).
template <class T>
void es_all(const T* sorted_keys, const uint32_t* idx, size_t G, size_t P, const int64_t* off,
            const int32_t* genes, size_t K, T* es) {
#pragma omp parallel for schedule(dynamic)
    for (long long k = 0; k < (long long)K; k++) {
        std::vector<uint8_t> member(G, 0);
        for (int64_t i = off[k]; i < off[k + 1]; i++)
            if (genes[i] >= 0 && (size_t)genes[i] < G) member[genes[i]] = 1;
        for (size_t p = 0; p < P; p++) {
            const T* key = sorted_keys + p * G;
            const uint32_t* ix = idx + p * G;
            T Bsf = 0, Res = 0, Kah = 0, N_R = 0;
            size_t N_H = 0;
            for (size_t r = 0; r < G; r++) {
                const T sigma = member[ix[r]] ? (T)1 : (T)0;
                const T input = cuabs(key[r]);
                const T alpha = sigma ? input - Kah : 0;
                const T futre = sigma ? alpha + N_R : N_R;
                Kah = sigma ? (futre - N_R) - alpha : Kah;
                N_R = sigma ? futre : N_R;
                N_H = (size_t)((T)N_H + sigma);
            }
            Kah = 0;
            const T decay = (T)(-1.0 / (double)(G - N_H));
            for (size_t r = 0; r < G; r++) {
                const bool hit = member[ix[r]] != 0;
                const T input = hit ? cuabs(key[r]) / N_R : decay;
                const T alpha = input - Kah;
                const T futre = alpha + Res;
                Kah = (futre - Res) - alpha;
                Res = futre;
                Bsf = cuabs(Res) > cuabs(Bsf) ? Res : Bsf;
            }
            es[(size_t)k * P + p] = Bsf;
        }
    }
}

// ---------------------------------------------------------------- statistics
// statistics.cuh:46-117 in the precision T, followed by the FDR q-value.
//
// FDR (no counterpart in the reference): for a set with NES* > 0,
//   q = [#{null NES >= NES*} / #{null NES >= 0}] / [#{obs NES >= NES*} / #{obs NES >= 0}]
// and symmetrically (<=, <= 0) for NES* <= 0, capped at 1.  "null NES" are the
// normalised scores of permutations 1..P-1 of every set (normalised with the
// same per-set factor P / sum|ES| as NES), "obs NES" the K observed NES.
template <class T>
void stats_all(const T* es_in, size_t K, size_t P, T* out) {
    std::vector<T> S(es_in, es_in + K * P);
    for (size_t k = 0; k < K; k++) out[k] = S[k * P];
    for (size_t k = 0; k < K; k++) {
        T sum = 0;
        for (size_t p = 0; p < P; p++) sum += std::abs(S[k * P + p]);
        T factor = (T)P / sum;
        out[K + k] = out[k] * factor;
        out[3 * K + k] = factor;
    }
    for (size_t k = 0; k < K; k++) {
        const T v = out[k];
        size_t c = 0;
        for (size_t p = 0; p < P; p++) c += std::abs(S[k * P + p]) >= std::abs(v);
        T pv = (T)c;
        out[2 * K + k] = pv / (T)P;
    }
    const T inf = std::numeric_limits<T>::infinity();
    std::vector<T> mx(P, -inf), mn(P, inf);
    for (size_t k = 0; k < K; k++) {
        const T f = out[3 * K + k];
        for (size_t p = 0; p < P; p++) {
            const T v = S[k * P + p] * f;
            S[k * P + p] = v;
            mx[p] = mx[p] < v ? v : mx[p];
            mn[p] = mn[p] > v ? v : mn[p];
        }
    }
    for (size_t k = 0; k < K; k++) {
        const T score = out[K + k];
        size_t c = 0;
        if (score > 0) { for (size_t p = 0; p < P; p++) c += mx[p] >= score; }
        else           { for (size_t p = 0; p < P; p++) c += mn[p] <= score; }
        T pv = (T)c;
        out[3 * K + k] = pv / (T)P;
    }
    // FDR
    std::vector<T> null_pos, null_neg, obs_pos, obs_neg;
    for (size_t k = 0; k < K; k++) {
        for (size_t p = 1; p < P; p++) {
            const T v = S[k * P + p];
            if (v >= 0) null_pos.push_back(v);
            if (v <= 0) null_neg.push_back(v);
        }
        const T o = out[K + k];
        if (o >= 0) obs_pos.push_back(o);
        if (o <= 0) obs_neg.push_back(o);
    }
    std::sort(null_pos.begin(), null_pos.end());
    std::sort(null_neg.begin(), null_neg.end());
    std::sort(obs_pos.begin(), obs_pos.end());
    std::sort(obs_neg.begin(), obs_neg.end());
    for (size_t k = 0; k < K; k++) {
        const T o = out[K + k];
        double q;
        if (!(o == o)) { out[4 * K + k] = o; continue; }
        if (o > 0) {
            const double nn = (double)(null_pos.end() - std::lower_bound(null_pos.begin(), null_pos.end(), o));
            const double no = (double)(obs_pos.end() - std::lower_bound(obs_pos.begin(), obs_pos.end(), o));
            const double fn = null_pos.empty() ? 0.0 : nn / (double)null_pos.size();
            const double fo = no / (double)obs_pos.size();
            q = fn / fo;
        } else {
            const double nn = (double)(std::upper_bound(null_neg.begin(), null_neg.end(), o) - null_neg.begin());
            const double no = (double)(std::upper_bound(obs_neg.begin(), obs_neg.end(), o) - obs_neg.begin());
            const double fn = null_neg.empty() ? 0.0 : nn / (double)null_neg.size();
            const double fo = no / (double)obs_neg.size();
            q = fn / fo;
        }
        out[4 * K + k] = (T)(q < 1.0 ? q : 1.0);
    }
}

template <class T>
int gsea_all(int metric, const T* table, const uint8_t* labels, size_t G, size_t S,
             const int64_t* off, const int32_t* genes, size_t K, size_t P, int ascending,
             uint32_t seed, T* es, T* stats) {
    std::vector<T> keys(G * P), sk(G * P);
    std::vector<uint32_t> idx(G * P);
    int rc = metric_all<T>(metric, table, labels, G, S, P, 0, seed, keys.data());
    if (rc) return rc;
    sort_all<T>(keys.data(), G, P, ascending, sk.data(), idx.data());
    es_all<T>(sk.data(), idx.data(), G, P, off, genes, K, es);
    stats_all<T>(es, K, P, stats);
    return 0;
}

}  // namespace

extern "C" {

void orc_perm_labels(const uint8_t* labels, size_t S, size_t P, size_t shift, uint32_t seed,
                     uint8_t* out) {
    for (size_t p = 0; p < P; p++) permuted_labels(labels, S, p + shift, seed, out + p * S);
}
uint32_t orc_kiss_stream(uint32_t seed, size_t n, uint32_t* out) {
    Kiss s = kiss_seed(seed);
    for (size_t i = 0; i < n; i++) out[i] = kiss_next(s);
    return n ? out[n - 1] : 0;
}
int orc_metric_f32(int m, const float* x, const uint8_t* l, size_t G, size_t S, size_t P,
                   size_t shift, uint32_t seed, float* keys) {
    return metric_all<float>(m, x, l, G, S, P, shift, seed, keys);
}
int orc_metric_f64(int m, const double* x, const uint8_t* l, size_t G, size_t S, size_t P,
                   size_t shift, uint32_t seed, double* keys) {
    return metric_all<double>(m, x, l, G, S, P, shift, seed, keys);
}
void orc_sort_f32(const float* k, size_t G, size_t P, int asc, float* sk, uint32_t* idx) {
    sort_all<float>(k, G, P, asc, sk, idx);
}
void orc_sort_f64(const double* k, size_t G, size_t P, int asc, double* sk, uint32_t* idx) {
    sort_all<double>(k, G, P, asc, sk, idx);
}
void orc_es_f32(const float* sk, const uint32_t* idx, size_t G, size_t P, const int64_t* off,
                const int32_t* genes, size_t K, float* es) {
    es_all<float>(sk, idx, G, P, off, genes, K, es);
}
void orc_es_f64(const double* sk, const uint32_t* idx, size_t G, size_t P, const int64_t* off,
                const int32_t* genes, size_t K, double* es) {
    es_all<double>(sk, idx, G, P, off, genes, K, es);
}
void orc_stats_f32(const float* es, size_t K, size_t P, float* out) { stats_all<float>(es, K, P, out); }
void orc_stats_f64(const double* es, size_t K, size_t P, double* out) { stats_all<double>(es, K, P, out); }
int orc_gsea_f32(int m, const float* x, const uint8_t* l, size_t G, size_t S, const int64_t* off,
                 const int32_t* genes, size_t K, size_t P, int asc, uint32_t seed, float* es,
                 float* stats) {
    return gsea_all<float>(m, x, l, G, S, off, genes, K, P, asc, seed, es, stats);
}
int orc_gsea_f64(int m, const double* x, const uint8_t* l, size_t G, size_t S,
                 const int64_t* off, const int32_t* genes, size_t K, size_t P, int asc,
                 uint32_t seed, double* es, double* stats) {
    return gsea_all<double>(m, x, l, G, S, off, genes, K, P, asc, seed, es, stats);
}

}  // extern "C"
