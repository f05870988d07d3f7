// The learned screen proposer: a 16 -> 256 -> 256 -> 3 MLP in BF16 with FP32 accumulation,
// trained by hand-written forward and backward kernels.
//
// It predicts, from a world's kernel and growth parameters, P(survives), P(moves), P(explodes);
// the batched simulator generates the labels and remains the judge of every proposed world.  The
// reference has no learned component; its world screen samples parameters uniformly
// (scripts/life_screen.py:143-179), which is the baseline this proposer is compared with.
//
// Parameters: FP32 master weights updated by Adam; BF16 copies feed every GEMM; activations are
// stored in BF16 for the backward pass; every GEMM accumulates in FP32.  The GEMMs of the two
// 256-wide layers -- forward h1 and h2, backward dh1 and the weight gradients dW1 and dW2 -- run on
// the 5th-generation tensor cores (gemm_tc: tcgen05 MMAs, TMEM accumulators); the 3-wide output
// layer's (z, dW3, dh2) on the CUDA cores.
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
#include "tc_ptx.cuh"

namespace lenia {
namespace mlp {

constexpr int IN = 16, HID = 256, OUT = 3;
constexpr int P_W1 = 0, P_B1 = P_W1 + HID * IN, P_W2 = P_B1 + HID, P_B2 = P_W2 + HID * HID, P_W3 = P_B2 + HID,
              P_B3 = P_W3 + OUT * HID, NPARAM = P_B3 + OUT;

using bf16 = __nv_bfloat16;

// C[M x N] = A[M x K] * B^T (B is [N x K]) with bf16 operands and FP32 accumulation, when
// TRANS_B is false; C = A * B (B is [K x N]) when TRANS_B is true.  TRANS_A reads A as [K x M].
// Epilogue: + bias[n], relu, and output in f32 and/or bf16 (and bf16 transposed, CbT[n * ldt + m]).
// 64 x 64 tiles, 256 threads, 4 x 4 outputs per thread, K in steps of 16 through shared memory: the
// CUDA-core GEMM of the 3-wide output layer, where an MMA tile would be almost all padding.
template <bool TRANS_A, bool TRANS_B>
__global__ void __launch_bounds__(256) gemm_bf16(const bf16* __restrict__ A, const bf16* __restrict__ B, int M, int N,
                                                 int K, const float* __restrict__ bias, int relu, float* __restrict__ Cf,
                                                 bf16* __restrict__ Cb, const bf16* __restrict__ mask,
                                                 bf16* __restrict__ CbT = nullptr, int ldt = 0) {
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
            if (CbT) CbT[(size_t)n * ldt + m] = __float2bfloat16_rn(v);
        }
}

// ------------------------------------------------------------------ tensor-core GEMM (tcgen05)
// C[M x N] = A[M x K] * B[N x K]^T with A and B bf16, K-major (rows lda / ldb elements apart), and
// FP32 accumulation in TMEM: the GEMMs of the 256-wide layers.  A CTA of 128 threads owns 128 rows
// of C and all N columns (N a multiple of 16, at most 256) and loops over K in chunks of 64:
// every thread stages 16-byte pieces of both operands into shared memory with cp.async, in the
// canonical K-major layout without swizzle (8-row x 16-byte core matrices, K-adjacent ones 128 bytes
// apart, 8-row groups 1024 bytes apart), double-buffered, and one elected thread issues the
// M = 128, N, K = 16 MMAs of a chunk and commits them to that buffer's mbarrier.  Elements past M or
// K are zero-filled.  With ksplit > 1, CTA column kz of the grid takes every ksplit-th chunk and adds
// its partial sums into Cf (zeroed by the caller) with atomics; the bias, ReLU, mask and bf16 outputs
// need ksplit = 1.  Epilogue per row (a thread per TMEM lane): + bias[n], ReLU, zero where mask <= 0,
// then FP32 (Cf), bf16 (Cb) and transposed bf16 (CbT[n * ldt + m]) outputs, each optional.  Every
// barrier wait is bounded; a CTA that gives up waits (bounded) for its own MMAs, raises *err, frees
// its TMEM and writes nothing.
constexpr int TCK = 64;  // K elements per staged chunk: 128 bytes of bf16 per operand row
template <int N>
struct TcGemm {
    static constexpr int ABYTES = 128 * TCK * 2, BBYTES = N * TCK * 2, STAGE = ABYTES + BBYTES;
    static constexpr int SMEM = 2 * STAGE + 64;
    static constexpr uint32_t TCOLS = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "MMA N");
};

__device__ __forceinline__ void cp_async16_zfill(void* dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}

template <int N>
__global__ void __launch_bounds__(128, 1)
    gemm_tc(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B, int ldb, int M, int K, int ksplit,
            const float* __restrict__ bias, int relu, const bf16* __restrict__ mask, float* __restrict__ Cf,
            bf16* __restrict__ Cb, bf16* __restrict__ CbT, int ldt, int* __restrict__ err) {
    using P = TcGemm<N>;
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 2 * P::STAGE);  // MMA done, per buffer
    uint32_t* slot = reinterpret_cast<uint32_t*>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * 128, kz = blockIdx.y;
    const int nchunks_all = (K + TCK - 1) / TCK;
    const int nchunks = nchunks_all > kz ? (nchunks_all - kz + ksplit - 1) / ksplit : 0;  // this CTA's chunks
    if (tid == 0) {
        tc::mbar_init(bars, 1);
        tc::mbar_init(bars + 1, 1);
        tc::fence_barrier_init();
    }
    if (warp == 0) tc::tmem_alloc(slot, P::TCOLS);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *slot;

    // stage chunk `ci` (the ci-th of this CTA) into buffer b
    auto load = [&](int ci, int b) {
        uint8_t* sa = smem + b * P::STAGE;
        uint8_t* sb = sa + P::ABYTES;
        const int k0 = (kz + ci * ksplit) * TCK;
        constexpr int PIECES = (128 + N) * (TCK / 8);
        for (int idx = tid; idx < PIECES; idx += 128) {
            const int row = idx / (TCK / 8), kg = idx % (TCK / 8), k = k0 + 8 * kg;
            const bool is_a = row < 128;
            const int r = is_a ? row : row - 128;
            const int grow = is_a ? m0 + r : r;
            const bool valid = (!is_a || grow < M) && k < K;
            uint8_t* dst = (is_a ? sa : sb) + tc::kmajor_offset(r, 8 * kg, TCK, 2);
            if (valid && k + 8 <= K) {
                cp_async16_zfill(dst, (is_a ? A + (size_t)grow * lda : B + (size_t)grow * ldb) + k, 16);
            } else if (valid) {
                // the last piece of a row whose K is not a multiple of 8: element by element
                const uint16_t* src = reinterpret_cast<const uint16_t*>((is_a ? A + (size_t)grow * lda : B + (size_t)grow * ldb) + k);
                uint16_t h[8];
                for (int i = 0; i < 8; i++) h[i] = k + i < K ? src[i] : (uint16_t)0;
                *reinterpret_cast<uint4*>(dst) = make_uint4(h[0] | (uint32_t)h[1] << 16, h[2] | (uint32_t)h[3] << 16,
                                                            h[4] | (uint32_t)h[5] << 16, h[6] | (uint32_t)h[7] << 16);
            } else {
                *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    constexpr uint32_t IDESC = tc::instr_desc(1, 128, N);
    constexpr uint32_t SBO = TCK * 2 * 8;
    bool ok = true;
    int issued = 0;  // chunks whose MMAs were issued
    if (nchunks > 0) load(0, 0);
    for (int ci = 0; ci < nchunks && ok; ci++) {
        if (ci + 1 < nchunks) {
            // the buffer of chunk ci + 1 was read by the MMAs of chunk ci - 1
            if (ci >= 1 && __syncthreads_or(!tc::mbar_wait(bars + ((ci + 1) & 1), ((ci - 1) >> 1) & 1))) {
                ok = false;
                break;
            }
            load(ci + 1, (ci + 1) & 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_u32(smem + (ci & 1) * P::STAGE), sb = sa + P::ABYTES;
            const int k0 = (kz + ci * ksplit) * TCK;
            const int ksteps = (min(TCK, K - k0) + 15) / 16;
            for (int s = 0; s < ksteps; s++)
                tc::mma<false>(tmem, tc::smem_desc(sa + 256u * s, 128, SBO), tc::smem_desc(sb + 256u * s, 128, SBO),
                               IDESC, (ci > 0 || s > 0) ? 1u : 0u);
            tc::mma_commit(bars + (ci & 1));
        }
        issued = ci + 1;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    // the last issued chunk's commit covers every earlier MMA
    if (ok && issued > 0 && __syncthreads_or(!tc::mbar_wait(bars + ((issued - 1) & 1), ((issued - 1) >> 1) & 1)))
        ok = false;
    tc::tc_fence_after();
    if (ok && issued > 0) {
        const int row = m0 + tid;
        for (int n0 = 0; n0 < N; n0 += 32) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0, v);
            if (row >= M) continue;
            const int nn = N - n0 < 32 ? N - n0 : 32;
            for (int i = 0; i < nn; i++) {
                const int n = n0 + i;
                float x = v[i];
                if (ksplit > 1) {
                    atomicAdd(Cf + (size_t)row * N + n, x);
                    continue;
                }
                if (bias) x += bias[n];
                if (relu) x = fmaxf(x, 0.f);
                if (mask && __bfloat162float(mask[(size_t)row * N + n]) <= 0.f) x = 0.f;
                if (Cf) Cf[(size_t)row * N + n] = x;
                const bf16 xb = __float2bfloat16_rn(x);
                if (Cb) Cb[(size_t)row * N + n] = xb;
                if (CbT) CbT[(size_t)n * ldt + row] = xb;
            }
        }
    }
    if (!ok && tid == 0) {
        if (issued > 0) tc::mbar_wait(bars + ((issued - 1) & 1), ((issued - 1) >> 1) & 1);  // drain, bounded
        atomicExch(err, 1);
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, P::TCOLS);
    }
}

__global__ void to_bf16(const float* __restrict__ x, bf16* __restrict__ y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// The batch's inputs (B x IN, f32) as bf16, row-major and transposed (IN x ldt).
__global__ void inputs_bf16(const float* __restrict__ x, bf16* __restrict__ xb, bf16* __restrict__ xt, int B, int ldt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * IN) return;
    const bf16 v = __float2bfloat16_rn(x[i]);
    xb[i] = v;
    xt[(size_t)(i % IN) * ldt + i / IN] = v;
}

// W2 (FP32 master, [out][in]) as bf16 transposed, [in][out]: the B operand of dh1 = dh2 W2.
__global__ void w2_transposed(const float* __restrict__ w2, bf16* __restrict__ w2t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= HID * HID) return;
    const int o = i / HID, in = i % HID;
    w2t[(size_t)in * HID + o] = __float2bfloat16_rn(w2[i]);
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
    // transposed copies (feature-major, batch contiguous, ldt apart): the K-major operands of the
    // weight-gradient GEMMs, whose K is the batch; and W2 transposed for dh1 = dh2 W2
    int ldt = 0;
    bf16 *xt = nullptr, *h1t = nullptr, *dh2t = nullptr, *dh1t = nullptr, *w2t = nullptr;
    int* err = nullptr;  // set by a tensor-core GEMM that gave up waiting on a barrier
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

// One tensor-core GEMM launch (see gemm_tc): C [M x N] = A [M x K] B[N x K]^T.
template <int N>
void tc_gemm(LeniaMlp* n, const bf16* A, int lda, const bf16* B, int ldb, int M, int K, int ksplit, const float* bias,
             int relu, const bf16* mask, float* Cf, bf16* Cb, bf16* CbT) {
    static int configured = 0;
    if (!configured) {
        cudaFuncSetAttribute(gemm_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcGemm<N>::SMEM);
        configured = 1;
    }
    const dim3 grid((M + 127) / 128, ksplit);
    gemm_tc<N><<<grid, 128, TcGemm<N>::SMEM, n->stream>>>(A, lda, B, ldb, M, K, ksplit, bias, relu, mask, Cf, Cb, CbT,
                                                          n->ldt, n->err);
}

// K-splits of a weight-gradient GEMM whose K is the batch: enough CTAs to spread the batch over SMs
int ksplit_for(int B) {
    const int chunks = (B + TCK - 1) / TCK;
    return chunks < 32 ? chunks : 32;
}

// forward pass of `B` rows already in n->x; logits into n->z.  The 16 -> 256 and 256 -> 256 layers
// run on the tensor cores; the 256 -> 3 layer on the CUDA cores.
void forward(LeniaMlp* n, int B) {
    cudaStream_t s = n->stream;
    inputs_bf16<<<(B * IN + 255) / 256, 256, 0, s>>>(n->x, n->xb, n->xt, B, n->ldt);
    tc_gemm<HID>(n, n->xb, IN, n->wb + P_W1, IN, B, IN, 1, n->w + P_B1, 1, nullptr, nullptr, n->h1, n->h1t);
    tc_gemm<HID>(n, n->h1, HID, n->wb + P_W2, HID, B, HID, 1, n->w + P_B2, 1, nullptr, nullptr, n->h2, nullptr);
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
                                                            n->dh2b, n->h2, n->dh2t, n->ldt);
    // layer 2 (tensor cores): dW2 = dh2^T h1 (K = the batch, split over CTAs), db2 = sum dh2,
    // dh1 = (dh2 W2) * (h1 > 0)
    cudaMemsetAsync(n->g + P_W2, 0, (size_t)HID * HID * sizeof(float), s);
    tc_gemm<HID>(n, n->dh2t, n->ldt, n->h1t, n->ldt, HID, B, ksplit_for(B), nullptr, 0, nullptr, n->g + P_W2, nullptr,
                 nullptr);
    col_sum<<<(HID + 127) / 128, 128, 0, s>>>(n->dh, B, HID, n->g + P_B2);
    tc_gemm<HID>(n, n->dh2b, HID, n->w2t, HID, B, HID, 1, nullptr, 0, n->h1, n->dh, n->dh1b, n->dh1t);
    // layer 1 (tensor cores): dW1 = dh1^T x, db1 = sum dh1
    cudaMemsetAsync(n->g + P_W1, 0, (size_t)HID * IN * sizeof(float), s);
    tc_gemm<IN>(n, n->dh1t, n->ldt, n->xt, n->ldt, HID, B, ksplit_for(B), nullptr, 0, nullptr, n->g + P_W1, nullptr,
                nullptr);
    col_sum<<<(HID + 127) / 128, 128, 0, s>>>(n->dh, B, HID, n->g + P_B1);
}

int check_err(LeniaMlp* n) {
    int h = 0;
    if (cudaMemcpy(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return err("mlp: error flag read failed");
    if (h) {
        cudaMemset(n->err, 0, sizeof(int));
        return err("mlp: a tensor-core GEMM gave up waiting on a barrier; results are invalid");
    }
    return 0;
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
    n->ldt = (int)((B + 15) / 16 * 16);
    const size_t T = (size_t)n->ldt;
    ok = ok && mal(n, &n->xt, T * IN) && mal(n, &n->h1t, T * HID) && mal(n, &n->dh2t, T * HID) &&
         mal(n, &n->dh1t, T * HID) && mal(n, &n->w2t, (size_t)HID * HID) && mal(n, &n->err, 1);
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
    cudaMemsetAsync(n->err, 0, sizeof(int), n->stream);
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
    w2_transposed<<<(HID * HID + 255) / 256, 256, 0, n->stream>>>(n->w + P_W2, n->w2t);
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
    if (cudaGetLastError() != cudaSuccess) return err("mlp: gradients failed");
    return check_err(n);
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
    w2_transposed<<<(HID * HID + 255) / 256, 256, 0, n->stream>>>(n->w + P_W2, n->w2t);
    if (cudaGetLastError() != cudaSuccess) return err("mlp: launch failed");
    const float l = mean_loss(n, batch);
    if (loss) *loss = l;
    return check_err(n);
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
    return check_err(n);
}

}  // extern "C"
