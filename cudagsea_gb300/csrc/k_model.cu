// k_model.cu -- the learned permutation allocator's network: a 5 -> 64 -> 64 -> 2
// multilayer perceptron (tanh hidden layers) with BF16 parameters and FP32
// arithmetic, trained on the GPU by the kernels below.  No counterpart in the
// reference.
//
// Parameters live twice on the device: FP32 master copies (updated by Adam)
// and the BF16-rounded copies every forward / backward pass computes with.
// Gradients are taken with respect to the BF16 copies and applied to the FP32
// masters.
//
// Per sample (x: 5 raw features, normalised in the kernel):
//   h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), z = W3 h2 + b3
//   loss = 0.5 w (z0 - logit(tc))^2              (tail, in logit space)
//        + 0.5 (z1 - (t1 - y_mean) / y_std)^2    (log null mean)
//   tc = clamp(t0, 1e-4, 1 - 1e-4), w = min(1, 400 tc (1 - tc)): every tail
//   probability in [~0.0025, ~0.9975] weighs the same in logit units, so the
//   range the stopping rule reads (p ~ 0.005 .. 0.5) is fitted as closely as
//   the bulk; w tapers the extremes whose logits the targets barely resolve.
//   dL/dz0 = w (z0 - logit(tc)),  dL/dz1 = z1 - u1
//
// Training kernel: a CTA takes a tile of 128 samples, one thread per sample,
// keeps h1, h2, dz2, dz1 of the tile in shared memory (rows padded to 65
// words so a warp's row accesses fall in distinct banks) and folds the tile's
// weight gradients cooperatively into one partial vector; a second kernel
// sums the partials in a fixed order (deterministic), a third applies Adam.
// One training step = these three launches, captured in a CUDA graph.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <random>
#include <vector>

#include "kernels.h"
#include "plan.h"

namespace gsea {
namespace model {

constexpr int IN = GSEA_MODEL_INPUTS, H = GSEA_MODEL_HIDDEN, OUT = GSEA_MODEL_OUTPUTS;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + OUT * H, NPARAM = OFF_B3 + OUT;
static_assert(NPARAM == GSEA_MODEL_PARAMS, "parameter layout");
constexpr int NPART = NPARAM + 1;  // partial gradient + loss sum
constexpr int TILE = 128;          // samples per training CTA (one thread each)
constexpr int HP = H + 1;          // padded row of the per-sample activations

struct Norm {
    float x_mean[IN], x_scale[IN];
    float y_mean, y_std;
};

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }

__device__ __forceinline__ void load_params(const __nv_bfloat16* __restrict__ wq, float* w) {
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = __bfloat162float(wq[i]);
}

// standardised inputs, clamped to +-kInputClamp training standard deviations
// (a feature that did not vary in training has scale 0 and drops out)
constexpr float kInputClamp = 8.f;
__device__ __forceinline__ void normalise(const float* __restrict__ x, const Norm& nm, float* xin) {
#pragma unroll
    for (int d = 0; d < IN; d++)
        xin[d] = fminf(fmaxf((x[d] - nm.x_mean[d]) * nm.x_scale[d], -kInputClamp), kInputClamp);
}

// forward pass of one sample; h1 kept in registers, h2 handed to `sink(j, h2_j)`
template <class Sink>
__device__ __forceinline__ void forward_one(const float* w, const float* xin, float* h1, float& z0, float& z1,
                                            Sink sink) {
#pragma unroll
    for (int i = 0; i < H; i++) {
        float a = w[OFF_B1 + i];
#pragma unroll
        for (int d = 0; d < IN; d++) a = fmaf(w[OFF_W1 + i * IN + d], xin[d], a);
        h1[i] = tanhf(a);
    }
    z0 = w[OFF_B3];
    z1 = w[OFF_B3 + 1];
#pragma unroll 1
    for (int j = 0; j < H; j++) {
        float a = w[OFF_B2 + j];
#pragma unroll
        for (int i = 0; i < H; i++) a = fmaf(w[OFF_W2 + j * H + i], h1[i], a);
        const float h2 = tanhf(a);
        sink(j, h2);
        z0 = fmaf(w[OFF_W3 + j], h2, z0);
        z1 = fmaf(w[OFF_W3 + H + j], h2, z1);
    }
}

__global__ void __launch_bounds__(128) model_predict_kernel(const __nv_bfloat16* __restrict__ wq, Norm nm,
                                                            const float* __restrict__ x, int64_t n,
                                                            float* __restrict__ y) {
    __shared__ float w[NPARAM];
    load_params(wq, w);
    __syncthreads();
    // one sample per thread (a loop over samples would let the compiler hoist
    // the shared-memory parameters into registers)
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float xin[IN], h1[H], z0, z1;
    normalise(x + s * IN, nm, xin);
    forward_one(w, xin, h1, z0, z1, [](int, float) {});
    y[s * 2] = sigmoidf_(z0);
    y[s * 2 + 1] = expf(fmaf(z1, nm.y_std, nm.y_mean));
}

// sample index of slot i of step `step` of a random minibatch over n samples
__device__ __forceinline__ int64_t batch_index(uint64_t step, int64_t i, int64_t n) {
    uint64_t h = step * 0x9E3779B97F4A7C15ull + (uint64_t)i * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    h *= 0x94D049BB133111EBull;
    h ^= h >> 32;
    return (int64_t)(h % (uint64_t)n);
}

// One tile of `rows` samples: forward, loss, backward; partial[blockIdx.x]
// gets the tile's gradient sums and loss sum.  Samples: tile rows
// [blockIdx.x * TILE, ...) of the data (step == null) or a random minibatch
// of `rows_total` draws from the n samples (step = device step counter).
__global__ void __launch_bounds__(TILE) model_grad_kernel(const __nv_bfloat16* __restrict__ wq, Norm nm,
                                                          const float* __restrict__ x, const float* __restrict__ t,
                                                          int64_t n, int64_t rows_total,
                                                          const unsigned long long* __restrict__ step,
                                                          float* __restrict__ partial) {
    extern __shared__ float smem[];
    float* w = smem;                       // NPARAM
    float* H1 = w + NPARAM;                // TILE * HP
    float* H2 = H1 + TILE * HP;            // TILE * HP
    float* DZ2 = H2 + TILE * HP;           // TILE * HP
    float* DZ1 = DZ2 + TILE * HP;          // TILE * HP
    float* X = DZ1 + TILE * HP;            // TILE * IN (normalised)
    float* DY = X + TILE * IN;             // TILE * 2
    float* LOSS = DY + TILE * 2;           // TILE
    const int tid = threadIdx.x;
    load_params(wq, w);
    const int64_t r0 = (int64_t)blockIdx.x * TILE;
    const int rows = (int)(rows_total - r0 < TILE ? rows_total - r0 : TILE);
    __syncthreads();
    if (tid < rows) {
        const int64_t s = step ? batch_index(*step, r0 + tid, n) : r0 + tid;
        float xin[IN], h1[H], z0, z1;
        normalise(x + s * IN, nm, xin);
#pragma unroll
        for (int d = 0; d < IN; d++) X[tid * IN + d] = xin[d];
        float* h2row = H2 + tid * HP;
        forward_one(w, xin, h1, z0, z1, [h2row](int j, float v) { h2row[j] = v; });
#pragma unroll
        for (int i = 0; i < H; i++) H1[tid * HP + i] = h1[i];
        const float tc = fminf(fmaxf(t[s * 2], 1e-4f), 1.f - 1e-4f), u1 = (t[s * 2 + 1] - nm.y_mean) / nm.y_std;
        const float lt = logf(tc / (1.f - tc)), w0 = fminf(1.f, 400.f * tc * (1.f - tc));
        const float dy0 = w0 * (z0 - lt), dy1 = z1 - u1;
        DY[tid * 2] = dy0;
        DY[tid * 2 + 1] = dy1;
        LOSS[tid] = 0.5f * (dy0 * (z0 - lt) + dy1 * dy1);
        // dz2_j = (W3[0][j] dy0 + W3[1][j] dy1) (1 - h2_j^2); dh1 = W2^T dz2
        float dh1[H];
#pragma unroll
        for (int i = 0; i < H; i++) dh1[i] = 0.f;
        for (int j = 0; j < H; j++) {
            const float h2 = h2row[j];
            const float dz = fmaf(w[OFF_W3 + j], dy0, w[OFF_W3 + H + j] * dy1) * (1.f - h2 * h2);
            DZ2[tid * HP + j] = dz;
#pragma unroll
            for (int i = 0; i < H; i++) dh1[i] = fmaf(w[OFF_W2 + j * H + i], dz, dh1[i]);
        }
#pragma unroll
        for (int i = 0; i < H; i++) DZ1[tid * HP + i] = dh1[i] * (1.f - h1[i] * h1[i]);
    }
    __syncthreads();
    float* out = partial + (int64_t)blockIdx.x * NPART;
    // dW2[j][i0 .. i0+32) for j = tid % 64, i0 = 32 * (tid / 64)
    {
        const int j = tid & (H - 1), i0 = (tid >> 6) * 32;
        float acc[32];
#pragma unroll
        for (int ii = 0; ii < 32; ii++) acc[ii] = 0.f;
        for (int s = 0; s < rows; s++) {
            const float a = DZ2[s * HP + j];
#pragma unroll
            for (int ii = 0; ii < 32; ii++) acc[ii] = fmaf(a, H1[s * HP + i0 + ii], acc[ii]);
        }
#pragma unroll
        for (int ii = 0; ii < 32; ii++) out[OFF_W2 + j * H + i0 + ii] = acc[ii];
    }
    // dW3[o][j] for o = tid / 64, j = tid % 64
    {
        const int o = tid >> 6, j = tid & (H - 1);
        float acc = 0.f;
        for (int s = 0; s < rows; s++) acc = fmaf(DY[s * 2 + o], H2[s * HP + j], acc);
        out[OFF_W3 + o * H + j] = acc;
    }
    // dW1[i][d]
    for (int o = tid; o < H * IN; o += TILE) {
        const int i = o / IN, d = o % IN;
        float acc = 0.f;
        for (int s = 0; s < rows; s++) acc = fmaf(DZ1[s * HP + i], X[s * IN + d], acc);
        out[OFF_W1 + o] = acc;
    }
    if (tid < H) {
        float a1 = 0.f, a2 = 0.f;
        for (int s = 0; s < rows; s++) {
            a1 += DZ1[s * HP + tid];
            a2 += DZ2[s * HP + tid];
        }
        out[OFF_B1 + tid] = a1;
        out[OFF_B2 + tid] = a2;
    } else if (tid < H + OUT) {
        const int o = tid - H;
        float a = 0.f;
        for (int s = 0; s < rows; s++) a += DY[s * 2 + o];
        out[OFF_B3 + o] = a;
    } else if (tid == H + OUT) {
        float a = 0.f;
        for (int s = 0; s < rows; s++) a += LOSS[s];
        out[NPARAM] = a;
    }
}

constexpr size_t grad_smem_bytes() {
    return sizeof(float) * ((size_t)NPARAM + 4 * (size_t)TILE * HP + (size_t)TILE * IN + 2 * TILE + TILE);
}

// grad[i] = sum over tiles (in tile order) / rows; loss likewise.  When
// loss_curve is given, the loss also goes to loss_curve[*step].
__global__ void model_reduce_kernel(const float* __restrict__ partial, int tiles, int64_t rows,
                                    float* __restrict__ grad, float* __restrict__ loss,
                                    const unsigned long long* __restrict__ step, float* __restrict__ loss_curve) {
    const float inv = 1.f / (float)rows;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPART; i += gridDim.x * blockDim.x) {
        float a = 0.f;
        for (int c = 0; c < tiles; c++) a += partial[(int64_t)c * NPART + i];
        if (i < NPARAM) {
            grad[i] = a * inv;
        } else {
            if (loss) *loss = a * inv;
            if (loss_curve && step) loss_curve[*step] = a * inv;
        }
    }
}

// Adam with a cosine-decayed rate; one block, so the step counter can be
// advanced after every thread has read it
__global__ void __launch_bounds__(1024) model_adam_kernel(float* __restrict__ master, __nv_bfloat16* __restrict__ wq,
                                                          float* __restrict__ m1, float* __restrict__ m2,
                                                          const float* __restrict__ grad,
                                                          unsigned long long* __restrict__ step, float lr,
                                                          int total_steps) {
    const unsigned long long s = *step;
    const float tt = (float)(s + 1);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - powf(b1, tt), c2 = 1.f - powf(b2, tt);
    const float frac = total_steps > 0 ? fminf((float)s / (float)total_steps, 1.f) : 0.f;
    const float rate = lr * 0.5f * (1.f + cospif(frac));
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) {
        const float g = grad[i];
        const float a = b1 * m1[i] + (1.f - b1) * g;
        const float b = b2 * m2[i] + (1.f - b2) * g * g;
        m1[i] = a;
        m2[i] = b;
        const float v = master[i] - rate * (a / c1) / (sqrtf(b / c2) + eps);
        master[i] = v;
        wq[i] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    if (threadIdx.x == 0) *step = s + 1;
}

__global__ void model_quantise_kernel(const float* __restrict__ master, __nv_bfloat16* __restrict__ wq) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x)
        wq[i] = __float2bfloat16_rn(master[i]);
}

}  // namespace model
}  // namespace gsea

struct gsea_model_s {
    int device = 0;
    float* master = nullptr;
    __nv_bfloat16* wq = nullptr;
    float* m1 = nullptr;
    float* m2 = nullptr;
    float* grad = nullptr;
    float* loss = nullptr;
    unsigned long long* step = nullptr;
    float norms[GSEA_MODEL_NORMS];
};

namespace {
using namespace gsea::model;
using gsea::fail;

Norm norm_of(const gsea_model_s* m) {
    Norm n;
    for (int d = 0; d < IN; d++) {
        n.x_mean[d] = m->norms[d];
        n.x_scale[d] = m->norms[IN + d];
    }
    n.y_mean = m->norms[2 * IN];
    n.y_std = m->norms[2 * IN + 1];
    return n;
}

void free_model(gsea_model_s* m) {
    void* b[] = {m->master, m->wq, m->m1, m->m2, m->grad, m->loss, m->step};
    for (void* p : b)
        if (p) cudaFree(p);
}

int use(const gsea_model_s* m) {
    GSEA_CUDA(cudaSetDevice(m->device), "cudaSetDevice");
    return GSEA_OK;
}

int grad_pass(gsea_model_s* m, const float* x, const float* t, int64_t n, int64_t rows, bool random,
              float* partial, float* grad, float* loss, float* loss_curve, int total_steps, float lr, bool adam,
              cudaStream_t st) {
    const int tiles = (int)((rows + TILE - 1) / TILE);
    const Norm nm = norm_of(m);
    model_grad_kernel<<<tiles, TILE, grad_smem_bytes(), st>>>(m->wq, nm, x, t, n, rows, random ? m->step : nullptr,
                                                              partial);
    model_reduce_kernel<<<(NPART + 255) / 256, 256, 0, st>>>(partial, tiles, rows, grad, loss,
                                                             random ? m->step : nullptr, loss_curve);
    if (adam) model_adam_kernel<<<1, 1024, 0, st>>>(m->master, m->wq, m->m1, m->m2, grad, m->step, lr, total_steps);
    GSEA_CUDA(cudaGetLastError(), "model kernels");
    return GSEA_OK;
}

// the training kernel's shared-memory opt-in, on the current device
int set_grad_smem() {
    GSEA_CUDA(cudaFuncSetAttribute(model_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)grad_smem_bytes()),
              "cudaFuncSetAttribute");
    return GSEA_OK;
}

}  // namespace

extern "C" {

int gsea_model_create(uint32_t seed, int device, gsea_model* out) {
    if (!out) return fail(GSEA_ERR_INVALID_ARGUMENT, "null model pointer");
    *out = nullptr;
    if (device >= 0) GSEA_CUDA(cudaSetDevice(device), "cudaSetDevice");
    gsea_model_s* m = new (std::nothrow) gsea_model_s();
    if (!m) return fail(GSEA_ERR_OUT_OF_MEMORY, "host allocation");
    cudaError_t e = cudaGetDevice(&m->device);
    void** bufs[] = {(void**)&m->master, (void**)&m->wq, (void**)&m->m1, (void**)&m->m2, (void**)&m->grad};
    for (void** b : bufs)
        if (e == cudaSuccess) e = cudaMalloc(b, sizeof(float) * NPARAM);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->step, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        cudaGetLastError();
        free_model(m);
        delete m;
        return gsea::cuda_fail(e, "model buffers");
    }
    // Glorot-uniform weights, zero biases, from a seeded host generator
    std::vector<float> p(NPARAM, 0.f);
    std::mt19937 gen(seed);
    auto fill = [&](int off, int fan_out, int fan_in) {
        const float a = std::sqrt(6.f / (float)(fan_in + fan_out));
        std::uniform_real_distribution<float> u(-a, a);
        for (int i = 0; i < fan_out * fan_in; i++) p[off + i] = u(gen);
    };
    fill(OFF_W1, H, IN);
    fill(OFF_W2, H, H);
    fill(OFF_W3, OUT, H);
    for (int i = 0; i < GSEA_MODEL_NORMS; i++) m->norms[i] = 0.f;
    for (int d = 0; d < IN; d++) m->norms[IN + d] = 1.f;
    m->norms[2 * IN + 1] = 1.f;  // y_std
    m->norms[2 * IN + 2] = 1.f;  // sigma_tail
    m->norms[2 * IN + 3] = 1.f;  // sigma_mean
    *out = m;
    int rc = gsea_model_set(m, p.data(), nullptr);
    if (rc) {
        gsea_model_destroy(m);
        *out = nullptr;
    }
    return rc;
}

int gsea_model_destroy(gsea_model m) {
    if (!m) return GSEA_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    free_model(m);
    delete m;
    return GSEA_OK;
}

int gsea_model_get(gsea_model m, float* params, float* norms) {
    if (!m) return fail(GSEA_ERR_INVALID_ARGUMENT, "null model");
    int rc = use(m);
    if (rc) return rc;
    if (params) GSEA_CUDA(cudaMemcpy(params, m->master, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost), "copy params");
    if (norms)
        for (int i = 0; i < GSEA_MODEL_NORMS; i++) norms[i] = m->norms[i];
    return GSEA_OK;
}

int gsea_model_set(gsea_model m, const float* params, const float* norms) {
    if (!m) return fail(GSEA_ERR_INVALID_ARGUMENT, "null model");
    int rc = use(m);
    if (rc) return rc;
    if (norms) {
        for (int i = 0; i < GSEA_MODEL_NORMS; i++) m->norms[i] = norms[i];
        if (!(m->norms[2 * IN + 1] > 0.f)) return fail(GSEA_ERR_INVALID_ARGUMENT, "y_std must be positive");
    }
    if (params) {
        GSEA_CUDA(cudaMemcpy(m->master, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice), "copy params");
        GSEA_CUDA(cudaMemset(m->m1, 0, sizeof(float) * NPARAM), "clear moments");
        GSEA_CUDA(cudaMemset(m->m2, 0, sizeof(float) * NPARAM), "clear moments");
        GSEA_CUDA(cudaMemset(m->step, 0, sizeof(unsigned long long)), "clear step");
        model_quantise_kernel<<<(NPARAM + 255) / 256, 256>>>(m->master, m->wq);
        GSEA_CUDA(cudaGetLastError(), "quantise kernel");
        GSEA_CUDA(cudaDeviceSynchronize(), "device sync");
    }
    return GSEA_OK;
}

int gsea_model_predict(gsea_model m, const float* x, int64_t n, float* y, void* stream) {
    if (!m || (n > 0 && (!x || !y)) || n < 0) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    if (n == 0) return GSEA_OK;
    int rc = use(m);
    if (rc) return rc;
    if (n > (int64_t)1 << 36) return fail(GSEA_ERR_INVALID_ARGUMENT, "too many samples");
    const unsigned blocks = (unsigned)((n + 127) / 128);
    model_predict_kernel<<<blocks, 128, 0, static_cast<cudaStream_t>(stream)>>>(m->wq, norm_of(m), x, n, y);
    GSEA_CUDA(cudaGetLastError(), "model predict kernel");
    gsea::launches_add(1);
    return GSEA_OK;
}

int gsea_model_loss_grad(gsea_model m, const float* x, const float* t, int64_t n, float* grad, float* loss,
                         void* stream) {
    if (!m || !x || !t || !grad || n < 1) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    int rc = use(m);
    if (rc || (rc = set_grad_smem())) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int tiles = (int)((n + TILE - 1) / TILE);
    void* partial = nullptr;
    GSEA_CUDA(cudaMalloc(&partial, sizeof(float) * NPART * (size_t)tiles), "partial gradients");
    rc = grad_pass(m, x, t, n, n, false, static_cast<float*>(partial), grad, loss, nullptr, 0, 0.f, false, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(partial);
    if (rc) return rc;
    GSEA_CUDA(e, "stream sync");
    return GSEA_OK;
}

int gsea_model_train(gsea_model m, const float* x, const float* t, int64_t n, int steps, int batch, float lr,
                     float* loss_curve) {
    if (!m || !x || !t || n < 2 || steps < 1 || batch < 1 || !(lr > 0.f))
        return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    int rc = use(m);
    if (rc || (rc = set_grad_smem())) return rc;
    // normalisers from the samples (host pass over a copy)
    std::vector<float> hx((size_t)n * IN), ht((size_t)n * 2);
    GSEA_CUDA(cudaMemcpy(hx.data(), x, sizeof(float) * hx.size(), cudaMemcpyDeviceToHost), "copy samples");
    GSEA_CUDA(cudaMemcpy(ht.data(), t, sizeof(float) * ht.size(), cudaMemcpyDeviceToHost), "copy targets");
    // two passes (mean, then squared deviations): a feature that is constant
    // over the samples -- a property of the calibration data set, e.g. the
    // metric's moments -- gets an exact zero spread and scale 0, so the
    // network ignores it instead of amplifying rounding noise
    for (int d = 0; d <= IN; d++) {
        auto val = [&](int64_t i) { return d < IN ? (double)hx[(size_t)i * IN + d] : (double)ht[(size_t)i * 2 + 1]; };
        double s = 0;
        for (int64_t i = 0; i < n; i++) s += val(i);
        const double mean = s / n;
        double ss = 0;
        for (int64_t i = 0; i < n; i++) ss += (val(i) - mean) * (val(i) - mean);
        const double sd = std::sqrt(ss / n);
        const bool varies = sd > 1e-5 * std::max(1.0, std::fabs(mean));
        if (d < IN) {
            m->norms[d] = (float)mean;
            m->norms[IN + d] = varies ? (float)(1.0 / sd) : 0.f;
        } else {
            m->norms[2 * IN] = (float)mean;
            m->norms[2 * IN + 1] = varies ? (float)sd : 1.f;
        }
    }
    m->norms[2 * IN + 4] = 0.f;
    GSEA_CUDA(cudaMemset(m->step, 0, sizeof(unsigned long long)), "clear step");
    GSEA_CUDA(cudaMemset(m->m1, 0, sizeof(float) * NPARAM), "clear moments");
    GSEA_CUDA(cudaMemset(m->m2, 0, sizeof(float) * NPARAM), "clear moments");
    const int tiles = (batch + TILE - 1) / TILE;
    float* partial = nullptr;
    float* curve = nullptr;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaMalloc((void**)&partial, sizeof(float) * NPART * (size_t)tiles);
    if (e == cudaSuccess) e = cudaMalloc((void**)&curve, sizeof(float) * (size_t)steps);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    // one graph holds `chunk` steps; it is launched until `steps` are done
    const int chunk = std::min(steps, 50);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int i = 0; i < chunk && rc == GSEA_OK; i++)
            rc = grad_pass(m, x, t, n, batch, true, partial, m->grad, m->loss, curve, steps, lr, true, st);
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (e == cudaSuccess) e = ce;
    }
    if (e == cudaSuccess && rc == GSEA_OK) e = cudaGraphInstantiate(&exec, graph, 0);
    int done = 0;
    while (e == cudaSuccess && rc == GSEA_OK && done + chunk <= steps) {
        e = cudaGraphLaunch(exec, st);
        done += chunk;
    }
    for (; e == cudaSuccess && rc == GSEA_OK && done < steps; done++)
        rc = grad_pass(m, x, t, n, batch, true, partial, m->grad, m->loss, curve, steps, lr, true, st);
    if (e == cudaSuccess && rc == GSEA_OK) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && rc == GSEA_OK && loss_curve)
        e = cudaMemcpy(loss_curve, curve, sizeof(float) * (size_t)steps, cudaMemcpyDeviceToHost);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (st) cudaStreamDestroy(st);
    if (partial) cudaFree(partial);
    if (curve) cudaFree(curve);
    if (rc) return rc;
    GSEA_CUDA(e, "model training");
    m->norms[2 * IN + 4] = 1.f;
    gsea::launches_add(3 * (int64_t)steps);
    return GSEA_OK;
}

int gsea_model_calibrate(gsea_model m, const float* x, const float* t, int64_t n) {
    if (!m || !x || !t || n < 1) return fail(GSEA_ERR_INVALID_ARGUMENT, "invalid arguments");
    int rc = use(m);
    if (rc) return rc;
    float* y = nullptr;
    GSEA_CUDA(cudaMalloc((void**)&y, sizeof(float) * 2 * (size_t)n), "predictions");
    rc = gsea_model_predict(m, x, n, y, nullptr);
    std::vector<float> hy((size_t)n * 2), ht((size_t)n * 2);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(hy.data(), y, sizeof(float) * hy.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ht.data(), t, sizeof(float) * ht.size(), cudaMemcpyDeviceToHost);
    cudaFree(y);
    if (rc) return rc;
    GSEA_CUDA(e, "calibration copies");
    // robust spread (1.4826 * median absolute deviation) of the logit error of
    // the tail (targets strictly inside (0, 1)) and of the log error of the mean
    std::vector<double> et, em;
    for (int64_t i = 0; i < n; i++) {
        const double pt = ht[(size_t)i * 2], pp = std::min(std::max((double)hy[(size_t)i * 2], 1e-7), 1 - 1e-7);
        if (pt > 0.0 && pt < 1.0) et.push_back(std::log(pp / (1 - pp)) - std::log(pt / (1 - pt)));
        em.push_back(std::log(std::max((double)hy[(size_t)i * 2 + 1], 1e-30)) - ht[(size_t)i * 2 + 1]);
    }
    auto mad = [](std::vector<double>& v) {
        if (v.empty()) return 1.0;
        for (double& a : v) a = std::fabs(a);
        std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
        return 1.4826 * v[v.size() / 2];
    };
    m->norms[2 * IN + 2] = (float)std::max(mad(et), 1e-3);
    m->norms[2 * IN + 3] = (float)std::max(mad(em), 1e-4);
    return GSEA_OK;
}

}  // extern "C"
