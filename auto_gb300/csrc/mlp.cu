// The learned screen proposer: a 16 -> 256 -> 256 -> 3 MLP in BF16 with FP32 accumulation,
// trained by hand-written forward and backward kernels.
//
// It predicts, from a world's kernel and growth parameters, P(survives), P(moves), P(explodes);
// the batched simulator generates the labels and remains the judge of every proposed world.  The
// reference has no learned component; its world screen samples parameters uniformly
// (scripts/life_screen.py:143-179), which is the baseline this proposer is compared with.
//
// Parameters: FP32 master weights updated by Adam; BF16 copies feed every GEMM; activations are
// stored in BF16 for the backward pass; every GEMM accumulates in FP32.
//   layer 1: W1 [256 x 16],  b1 [256]      h1 = relu(x W1^T + b1)
//   layer 2: W2 [256 x 256], b2 [256]      h2 = relu(h1 W2^T + b2)
//   layer 3: W3 [3 x 256],   b3 [3]        z  = h2 W3^T + b3,  p = sigmoid(z)
//   loss: mean over the batch and the 3 labels of softplus(z) - y z  (binary cross-entropy)
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace lenia {
namespace mlp {

constexpr int IN = 16, HID = 256, OUT = 3;
constexpr int P_W1 = 0, P_B1 = P_W1 + HID * IN, P_W2 = P_B1 + HID, P_B2 = P_W2 + HID * HID, P_W3 = P_B2 + HID,
              P_B3 = P_W3 + OUT * HID, NPARAM = P_B3 + OUT;

using bf16 = __nv_bfloat16;

// C[M x N] = A[M x K] * B^T (B is [N x K]) with bf16 operands and FP32 accumulation, when
// TRANS_B is false; C = A * B (B is [K x N]) when TRANS_B is true.  TRANS_A reads A as [K x M].
// Epilogue: + bias[n], relu, and output in f32 and/or bf16.  64 x 64 tiles, 256 threads, 4 x 4
// outputs per thread, K in steps of 16 through shared memory.
template <bool TRANS_A, bool TRANS_B>
__global__ void __launch_bounds__(256) gemm_bf16(const bf16* __restrict__ A, const bf16* __restrict__ B, int M, int N,
                                                 int K, const float* __restrict__ bias, int relu, float* __restrict__ Cf,
                                                 bf16* __restrict__ Cb, const bf16* __restrict__ mask) {
    __shared__ float As[16][64 + 1];
    __shared__ float Bs[16][64 + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int i = threadIdx.x; i < 16 * 64; i += 256) {
            const int kk = i / 64, mm = i % 64;
            const int m = m0 + mm, k = k0 + kk;
            float a = 0.f;
            if (m < M && k < K) a = __bfloat162float(TRANS_A ? A[(size_t)k * M + m] : A[(size_t)m * K + k]);
            As[kk][mm] = a;
            const int n = n0 + mm;
            float b = 0.f;
            if (n < N && k < K) b = __bfloat162float(TRANS_B ? B[(size_t)k * N + n] : B[(size_t)n * K + k]);
            Bs[kk][mm] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j] + (bias ? bias[n] : 0.f);
            if (relu) v = fmaxf(v, 0.f);
            if (mask && __bfloat162float(mask[(size_t)m * N + n]) <= 0.f) v = 0.f;
            if (Cf) Cf[(size_t)m * N + n] = v;
            if (Cb) Cb[(size_t)m * N + n] = __float2bfloat16_rn(v);
        }
}

__global__ void to_bf16(const float* __restrict__ x, bf16* __restrict__ y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// BCE with logits: dz = (sigmoid(z) - y) / (B * OUT); per-row losses for the host to average.
__global__ void bce_loss(const float* __restrict__ z, const float* __restrict__ y, int B, float* __restrict__ dz,
                         bf16* __restrict__ dzb, float* __restrict__ loss_rows) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float l = 0.f;
    for (int j = 0; j < OUT; j++) {
        const float zz = z[b * OUT + j], yy = y[b * OUT + j];
        const float p = 1.f / (1.f + expf(-zz));
        l += fmaxf(zz, 0.f) - zz * yy + log1pf(expf(-fabsf(zz)));
        const float g = (p - yy) / (float)(B * OUT);
        dz[b * OUT + j] = g;
        dzb[b * OUT + j] = __float2bfloat16_rn(g);
    }
    loss_rows[b] = l / OUT;
}

// Column sums of g [B x N] (bias gradients), FP32.
__global__ void col_sum(const float* __restrict__ g, int B, int N, float* __restrict__ out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int b = 0; b < B; b++) s += g[(size_t)b * N + n];
    out[n] = s;
}

__global__ void sigmoid_k(const float* __restrict__ z, float* __restrict__ p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = 1.f / (1.f + expf(-z[i]));
}

// Adam on the FP32 master weights, refreshing their BF16 copies.
__global__ void adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                     bf16* __restrict__ wb, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
}

}  // namespace mlp
}  // namespace lenia

using namespace lenia;
using namespace lenia::mlp;

struct LeniaMlp {
    int max_batch = 0;
    int t = 0;
    cudaStream_t stream = nullptr;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, grads, Adam moments
    bf16* wb = nullptr;                                             // BF16 copy of the parameters
    float *x = nullptr, *y = nullptr, *z = nullptr, *dz = nullptr, *dh = nullptr, *loss = nullptr, *p = nullptr;
    bf16 *xb = nullptr, *h1 = nullptr, *h2 = nullptr, *dzb = nullptr, *dh2b = nullptr, *dh1b = nullptr;
    std::vector<void*> allocs;
};

namespace {

template <typename T>
bool mal(LeniaMlp* n, T** p, size_t count) {
    void* v = nullptr;
    if (cudaMalloc(&v, count * sizeof(T)) != cudaSuccess) return false;
    n->allocs.push_back(v);
    *p = (T*)v;
    return true;
}

int err(const char* msg) {
    set_thread_error(msg);
    return LENIA_ECUDA;
}

dim3 grid_for(int M, int N) { return dim3((N + 63) / 64, (M + 63) / 64); }

// forward pass of `B` rows already in n->x; logits into n->z
void forward(LeniaMlp* n, int B) {
    cudaStream_t s = n->stream;
    to_bf16<<<(B * IN + 255) / 256, 256, 0, s>>>(n->x, n->xb, B * IN);
    gemm_bf16<false, false><<<grid_for(B, HID), 256, 0, s>>>(n->xb, n->wb + P_W1, B, HID, IN, n->w + P_B1, 1, nullptr,
                                                              n->h1, nullptr);
    gemm_bf16<false, false><<<grid_for(B, HID), 256, 0, s>>>(n->h1, n->wb + P_W2, B, HID, HID, n->w + P_B2, 1, nullptr,
                                                              n->h2, nullptr);
    gemm_bf16<false, false><<<grid_for(B, OUT), 256, 0, s>>>(n->h2, n->wb + P_W3, B, OUT, HID, n->w + P_B3, 0, n->z,
                                                              nullptr, nullptr);
}

// gradients of the mean BCE into n->g; per-row losses into n->loss
void backward(LeniaMlp* n, int B) {
    cudaStream_t s = n->stream;
    bce_loss<<<(B + 127) / 128, 128, 0, s>>>(n->z, n->y, B, n->dz, n->dzb, n->loss);
    // layer 3: dW3 = dz^T h2 [3 x 256], db3 = sum dz, dh2 = (dz W3) * (h2 > 0)
    gemm_bf16<true, true><<<grid_for(OUT, HID), 256, 0, s>>>(n->dzb, n->h2, OUT, HID, B, nullptr, 0, n->g + P_W3,
                                                             nullptr, nullptr);
    col_sum<<<1, 32, 0, s>>>(n->dz, B, OUT, n->g + P_B3);
    gemm_bf16<false, true><<<grid_for(B, HID), 256, 0, s>>>(n->dzb, n->wb + P_W3, B, HID, OUT, nullptr, 0, n->dh,
                                                            n->dh2b, n->h2);
    // layer 2: dW2 = dh2^T h1, db2 = sum dh2, dh1 = (dh2 W2) * (h1 > 0)
    gemm_bf16<true, true><<<grid_for(HID, HID), 256, 0, s>>>(n->dh2b, n->h1, HID, HID, B, nullptr, 0, n->g + P_W2,
                                                             nullptr, nullptr);
    col_sum<<<(HID + 127) / 128, 128, 0, s>>>(n->dh, B, HID, n->g + P_B2);
    gemm_bf16<false, true><<<grid_for(B, HID), 256, 0, s>>>(n->dh2b, n->wb + P_W2, B, HID, HID, nullptr, 0, n->dh,
                                                            n->dh1b, n->h1);
    // layer 1: dW1 = dh1^T x, db1 = sum dh1
    gemm_bf16<true, true><<<grid_for(HID, IN), 256, 0, s>>>(n->dh1b, n->xb, HID, IN, B, nullptr, 0, n->g + P_W1,
                                                            nullptr, nullptr);
    col_sum<<<(HID + 127) / 128, 128, 0, s>>>(n->dh, B, HID, n->g + P_B1);
}

int upload_batch(LeniaMlp* n, const float* x, const float* y, uint32_t B) {
    if (cudaMemcpyAsync(n->x, x, (size_t)B * IN * 4, cudaMemcpyHostToDevice, n->stream) != cudaSuccess) return -1;
    if (y && cudaMemcpyAsync(n->y, y, (size_t)B * OUT * 4, cudaMemcpyHostToDevice, n->stream) != cudaSuccess) return -1;
    return 0;
}

float mean_loss(LeniaMlp* n, uint32_t B) {
    std::vector<float> l(B);
    cudaMemcpyAsync(l.data(), n->loss, B * 4, cudaMemcpyDeviceToHost, n->stream);
    cudaStreamSynchronize(n->stream);
    double s = 0;
    for (float v : l) s += v;
    return (float)(s / B);
}

}  // namespace

extern "C" {

LENIA_API int lenia_mlp_create(uint32_t seed, uint32_t max_batch, LeniaMlp** out) {
    if (!out || max_batch < 1 || max_batch > (1u << 22)) {
        set_thread_error("mlp: need an output pointer and 1 <= max_batch <= 4M");
        return LENIA_EINVAL;
    }
    *out = nullptr;
    LeniaMlp* n = new LeniaMlp();
    n->max_batch = (int)max_batch;
    const size_t B = max_batch;
    bool ok = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) == cudaSuccess && mal(n, &n->w, NPARAM) &&
              mal(n, &n->g, NPARAM) && mal(n, &n->m, NPARAM) && mal(n, &n->v, NPARAM) && mal(n, &n->wb, NPARAM) &&
              mal(n, &n->x, B * IN) && mal(n, &n->y, B * OUT) && mal(n, &n->z, B * OUT) && mal(n, &n->dz, B * OUT) &&
              mal(n, &n->dh, B * HID) && mal(n, &n->loss, B) && mal(n, &n->p, B * OUT) && mal(n, &n->xb, B * IN) &&
              mal(n, &n->h1, B * HID) && mal(n, &n->h2, B * HID) && mal(n, &n->dzb, B * OUT) &&
              mal(n, &n->dh2b, B * HID) && mal(n, &n->dh1b, B * HID);
    if (!ok) {
        lenia_mlp_destroy(n);
        set_thread_error("mlp: device allocation failed");
        return LENIA_ENOMEM;
    }
    // He-uniform initialisation from the PCG hash, biases zero
    std::vector<float> w(NPARAM, 0.f);
    auto pcg = [](uint32_t v) {
        uint32_t s = v * 747796405u + 2891336453u;
        uint32_t x = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
        return (x >> 22u) ^ x;
    };
    auto init = [&](int off, int count, int fan_in) {
        const float a = std::sqrt(6.0f / fan_in);
        for (int i = 0; i < count; i++) {
            const uint32_t r = pcg(pcg(pcg((uint32_t)(off + i)) ^ seed) ^ 0x9E3779B9u);
            w[off + i] = a * (2.0f * ((float)r * (1.0f / 4294967296.0f)) - 1.0f);
        }
    };
    init(P_W1, HID * IN, IN);
    init(P_W2, HID * HID, HID);
    init(P_W3, OUT * HID, HID);
    int rc = lenia_mlp_set_params(n, w.data(), w.size());
    if (rc) {
        lenia_mlp_destroy(n);
        return rc;
    }
    cudaMemsetAsync(n->m, 0, NPARAM * 4, n->stream);
    cudaMemsetAsync(n->v, 0, NPARAM * 4, n->stream);
    if (cudaStreamSynchronize(n->stream) != cudaSuccess) {
        lenia_mlp_destroy(n);
        return err("mlp: initialisation failed");
    }
    *out = n;
    return 0;
}

LENIA_API int lenia_mlp_destroy(LeniaMlp* n) {
    if (!n) return 0;
    if (n->stream) cudaStreamSynchronize(n->stream);
    for (void* p : n->allocs) cudaFree(p);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return 0;
}

LENIA_API int lenia_mlp_param_count(uint32_t* count) {
    if (!count) return LENIA_EINVAL;
    *count = NPARAM;
    return 0;
}

LENIA_API int lenia_mlp_set_params(LeniaMlp* n, const float* host, size_t count) {
    if (!n || !host || count != (size_t)NPARAM) {
        set_thread_error("mlp: parameter vector has the wrong length");
        return LENIA_EINVAL;
    }
    if (cudaMemcpyAsync(n->w, host, NPARAM * 4, cudaMemcpyHostToDevice, n->stream) != cudaSuccess)
        return err("mlp: upload failed");
    to_bf16<<<(NPARAM + 255) / 256, 256, 0, n->stream>>>(n->w, n->wb, NPARAM);
    n->t = 0;
    return cudaStreamSynchronize(n->stream) == cudaSuccess ? 0 : err("mlp: set_params failed");
}

LENIA_API int lenia_mlp_get_params(LeniaMlp* n, float* host, size_t count) {
    if (!n || !host || count != (size_t)NPARAM) {
        set_thread_error("mlp: parameter vector has the wrong length");
        return LENIA_EINVAL;
    }
    if (cudaMemcpyAsync(host, n->w, NPARAM * 4, cudaMemcpyDeviceToHost, n->stream) != cudaSuccess ||
        cudaStreamSynchronize(n->stream) != cudaSuccess)
        return err("mlp: download failed");
    return 0;
}

LENIA_API int lenia_mlp_gradients(LeniaMlp* n, const float* x, const float* y, uint32_t batch, float* grads,
                                  float* loss) {
    if (!n || !x || !y || !grads || batch < 1 || (int)batch > n->max_batch) {
        set_thread_error("mlp: bad batch");
        return LENIA_EINVAL;
    }
    if (upload_batch(n, x, y, batch)) return err("mlp: upload failed");
    forward(n, (int)batch);
    backward(n, (int)batch);
    if (cudaGetLastError() != cudaSuccess) return err("mlp: launch failed");
    cudaMemcpyAsync(grads, n->g, NPARAM * 4, cudaMemcpyDeviceToHost, n->stream);
    const float l = mean_loss(n, batch);
    if (loss) *loss = l;
    return cudaGetLastError() == cudaSuccess ? 0 : err("mlp: gradients failed");
}

LENIA_API int lenia_mlp_train_step(LeniaMlp* n, const float* x, const float* y, uint32_t batch, float lr, float* loss) {
    if (!n || !x || !y || batch < 1 || (int)batch > n->max_batch || !(lr > 0.f)) {
        set_thread_error("mlp: bad batch or learning rate");
        return LENIA_EINVAL;
    }
    if (upload_batch(n, x, y, batch)) return err("mlp: upload failed");
    forward(n, (int)batch);
    backward(n, (int)batch);
    n->t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->t), c2 = 1.f - std::pow(b2, (float)n->t);
    adam<<<(NPARAM + 255) / 256, 256, 0, n->stream>>>(n->w, n->g, n->m, n->v, n->wb, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
    if (cudaGetLastError() != cudaSuccess) return err("mlp: launch failed");
    const float l = mean_loss(n, batch);
    if (loss) *loss = l;
    return 0;
}

LENIA_API int lenia_mlp_predict(LeniaMlp* n, const float* x, uint32_t count, float* probs) {
    if (!n || !x || !probs) {
        set_thread_error("mlp: NULL argument");
        return LENIA_EINVAL;
    }
    for (uint32_t off = 0; off < count; off += (uint32_t)n->max_batch) {
        const uint32_t B = count - off < (uint32_t)n->max_batch ? count - off : (uint32_t)n->max_batch;
        if (upload_batch(n, x + (size_t)off * IN, nullptr, B)) return err("mlp: upload failed");
        forward(n, (int)B);
        sigmoid_k<<<(B * OUT + 255) / 256, 256, 0, n->stream>>>(n->z, n->p, (int)(B * OUT));
        cudaMemcpyAsync(probs + (size_t)off * OUT, n->p, (size_t)B * OUT * 4, cudaMemcpyDeviceToHost, n->stream);
    }
    if (cudaStreamSynchronize(n->stream) != cudaSuccess) return err("mlp: predict failed");
    return 0;
}

}  // extern "C"
