// Tensor-core column pass for columns of 4096 points: two pipelines per SM.
//
// Same mathematics as step_tc.cu (a 4096-point column is 64 x 64; four DFT-as-GEMM stages with a
// twiddle between the two of each direction; the inverse through conj(DFT(conj z))), with the
// MMA orientation chosen per stage so that every hand-over from TMEM to the next shared-memory
// operand stays within the thread's own TMEM lane:
//
//   GEMM A   D[(k2,re/im)][(c,y1)] = F64 x X^T          data X: rows (c,y1), K (re/im, y2)
//   GEMM B   D[(c,k2)][(k1,re/im)] = X_B x F64^T        X_B: rows (c,k2), K (re/im, y1)
//   GEMM C   D[(y1,re/im)][(c,k2)] = F64 x X_C^T        X_C: rows (c,k2), K (re/im, k1)
//   GEMM D   D[(c,y1)][(y2,re/im)] = X_D x F64^T        X_D: rows (c,y1), K (re/im, k2)
//
// After A and C a thread's lane is (index, re or im): it takes the other component from the
// neighbouring lane with one shuffle for the complex twiddle.  One 64-point DFT matrix (bf16 hi and
// lo, or tf32) serves all four GEMMs.  Two 128-thread warpgroups run independent pipelines over
// different tile groups and share the matrix; each owns half of TMEM and its operand buffer, so one
// warpgroup's MMAs overlap the other's conversions.  Tile data is read straight from global memory
// (the next tile is prefetched into L2 by the bulk-copy engine); kernel-spectrum rows arrive by bulk
// copy.  Every barrier wait is bounded.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "engine.cuh"
#include "fft_core.cuh"
#include "step_tc.cuh"
#include "tc_ptx.cuh"

namespace lenia {
using namespace tc;

namespace {

template <bool X3>
struct Tc64 {
    static constexpr int H = 4096;
    static constexpr int E = X3 ? 2 : 4, NOP = X3 ? 2 : 1;
    static constexpr int OPND = 128 * 128 * E;         // one 128 x 128 operand copy
    static constexpr int FB = OPND;                    // the DFT matrix copy
    static constexpr int HQ = (H / 2 + 1 + 3) / 4 * 4; // kernel-spectrum row stride (floats)
    static constexpr int KH = TC * HQ * 4;             // two kernel-spectrum rows
    static constexpr int OFF_OP = FB * NOP;
    static constexpr int OFF_KH = OFF_OP + 2 * OPND * NOP;
    static constexpr int OFF_BAR = OFF_KH + 2 * KH;
    static constexpr int SMEM = OFF_BAR + 128;
    static_assert(SMEM <= 232448, "shared memory");
};

// BF16x3 split of two values at once (see step_tc.cu): the same bits as the per-value split.
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const float2 r = lfft::f2sub(make_float2(a, b), hf);
    const __nv_bfloat162 l = __floats2bfloat162_rn(r.x, r.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

template <bool X3>
__device__ __forceinline__ void store16(uint8_t* op, int r, int k0, const float* v) {
    // 16 bytes of K starting at k0 (8 bf16 hi and lo, or 4 tf32), row r of a 128 x 128 operand
    constexpr int OP = Tc64<X3>::OPND;
    if (X3) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int i = 0; i < 4; i++) split_bf16x2(v[2 * i], v[2 * i + 1], hi[i], lo[i]);
        const uint32_t off = kmajor_offset(r, k0, 128, 2);
        *reinterpret_cast<uint4*>(op + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(op + OP + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    } else {
        *reinterpret_cast<uint4*>(op + kmajor_offset(r, k0, 128, 4)) =
            make_uint4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
    }
}

// 32 consecutive K values of row r (k0 multiple of 32)
template <bool X3>
__device__ __forceinline__ void store32(uint8_t* op, int r, int k0, const float* v) {
    constexpr int CH = X3 ? 8 : 4;
#pragma unroll
    for (int i = 0; i < 32; i += CH) store16<X3>(op, r, k0 + i, v + i);
}

// D (128 x 128, f32 in TMEM) = A (128 x 128) * B^T (128 x 128), both K-major in shared memory.
template <bool X3>
__device__ __forceinline__ void gemm128(uint32_t d, uint32_t a, uint32_t b) {
    constexpr int E = X3 ? 2 : 4, OP = Tc64<X3>::OPND;
    constexpr uint32_t sbo = 128 * E * 8;
    constexpr uint32_t idesc = instr_desc(X3 ? 1 : 2, 128, 128);
#pragma unroll 1
    for (int s = 0; s < 128 * E / 32; s++) {
        const uint64_t ad = smem_desc(a + 256u * s, 128, sbo), bd = smem_desc(b + 256u * s, 128, sbo);
        mma<!X3>(d, ad, bd, idesc, s > 0 ? 1u : 0u);
        if (X3) {
            mma<false>(d, ad, smem_desc(b + OP + 256u * s, 128, sbo), idesc, 1u);
            mma<false>(d, smem_desc(a + OP + 256u * s, 128, sbo), bd, idesc, 1u);
        }
    }
}

}  // namespace

template <bool X3>
__global__ void __launch_bounds__(256, 1)
    col_pass_tc64(const DevWorld* __restrict__ worlds, const ColItem* __restrict__ groups, int ngroups,
                  const uint8_t* __restrict__ fmat, const float2* __restrict__ tw, int* ctl) {
    using S = Tc64<X3>;
    extern __shared__ __align__(128) uint8_t smem[];
    const int tid = threadIdx.x, wg = tid >> 7, t = tid & 127, warp = tid >> 5;
    uint8_t* f = smem;
    uint8_t* op = smem + S::OFF_OP + wg * S::OPND * S::NOP;
    float* kh = reinterpret_cast<float*>(smem + S::OFF_KH + wg * S::KH);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S::OFF_BAR);
    uint64_t* bar_f = bars;               // DFT matrix arrived
    uint64_t* bar_mma = bars + 1 + wg;    // this warpgroup's MMAs done
    uint64_t* bar_kh = bars + 3 + wg;     // this warpgroup's kernel-spectrum rows arrived
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 5);
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;

    if (tid == 0) {
        for (int i = 0; i < 5; i++) mbar_init(bars + i, 1);
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tslot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t t_x = *tslot + (uint32_t)(wg * 256);  // GEMMs A, C, D
    const uint32_t t_b = t_x + 128;                      // GEMM B, kept across the channel's kernels
    if (tid == 0) {
        mbar_arrive_expect_tx(bar_f, S::FB * S::NOP);
        bulk_g2s(f, fmat, S::FB * S::NOP, bar_f);
    }
    // Both hand-overs that need a twiddle (A -> B and C -> D) use exp(-2 pi i f j / 4096) with
    // f = t >> 1 fixed per thread and j in [0, 64) the column index: with j = 8a + b it is
    // P8[a] * P1[b], two exactly rounded table values and one product.
    // A thread whose lane holds the real part keeps both tables conjugated: the product is then
    // conj(w), and the hand-over's output is v * w.x + p * w.y on either lane (v its own
    // component, p the neighbour's), with no per-element select.
    float2 P8[8], P1[8];
    {
        const int fidx = t >> 1;
        const float sgn = (t & 1) ? 1.0f : -1.0f;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            P1[i] = tw[((fidx * i) & 4095) * (lfft::TWN / 4096)];
            P8[i] = tw[((fidx * 8 * i) & 4095) * (lfft::TWN / 4096)];
            P1[i].y *= sgn;
            P8[i].y *= sgn;
        }
    }
    // Every wait is bounded and each warpgroup decides to give up as a whole (named_sync_or), so
    // that no thread is left at a barrier the others skipped.  A warpgroup that gives up leaves its
    // group loop and, before TMEM is freed, waits (bounded again) for what it still has in flight:
    // the DFT-matrix load, its kernel-spectrum load, its issued MMAs and its output stores.
    const int bar_id = 1 + wg;
    auto wg_sync = [&]() { named_sync(bar_id, 128); };
    auto wg_any = [&](bool p) { return named_sync_or(bar_id, 128, p); };
    const bool f_failed = wg_any(!mbar_wait_n(bar_f, 0, f_wait_polls(ctl)));
    bool abort = f_failed, kh_pending = false, mma_pending = false;
    uint32_t ph_mma = 0, ph_kh = 0;
    const uint32_t fa = smem_u32(f), oa = smem_u32(op);
    // one GEMM from an elected thread; false (on the whole warpgroup) if its wait gave up
    auto gemm_wait = [&](uint32_t d, uint32_t a, uint32_t b) {
        tc_fence_before();
        fence_async_smem();
        wg_sync();
        if (t == 0) {
            tc_fence_after();
            gemm128<X3>(d, a, b);
            mma_commit(bar_mma);
        }
        if (wg_any(!mbar_wait(bar_mma, ph_mma))) {
            mma_pending = true;
            return false;
        }
        ph_mma ^= 1;
        tc_fence_after();
        return true;
    };

    const int stride = 2 * gridDim.x;
    for (int g = 2 * blockIdx.x + wg; g < ngroups && !abort; g += stride) {
        const ColItem it = groups[g];
        const DevWorld& wd = worlds[it.world];
        const int W = wd.W, K = wd.K;
        const size_t cplane = (size_t)(W / 2) * S::H;
        const float2* src = wd.spec + it.chan * cplane + (size_t)it.tile * S::H * TC;
        if (t == 0 && g + stride < ngroups) {
            const ColItem nx = groups[g + stride];
            const DevWorld& nw = worlds[nx.world];
            bulk_prefetch_l2(nw.spec + nx.chan * (size_t)(nw.W / 2) * S::H + (size_t)nx.tile * S::H * TC,
                             S::H * TC * 8);
        }
        // kernel-spectrum rows of the first kernel that reads this channel, in flight during the transforms
        int kfirst = 0;
        while (kfirst < K && wd.kern[kfirst].src != it.chan) kfirst++;
        if (kfirst < K) {
            if (t == 0) {
                mbar_arrive_expect_tx(bar_kh, S::KH);
                bulk_g2s(kh, wd.khat + ((size_t)kfirst * (W / 2 + 1) + (size_t)it.tile * TC) * S::HQ, S::KH, bar_kh);
            }
            kh_pending = true;
        }
        // ---- stage 0: X rows (c, y1) = t, K (re/im, y2), straight from global memory
        {
            const int c = t >> 6, y1 = t & 63;
            const float2* col = src + c;
#pragma unroll 1
            for (int y2 = 0; y2 < 64; y2 += 16) {
                float re[16], im[16];
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    const float2 v = col[(size_t)(y1 + 64 * (y2 + u)) * TC];
                    re[u] = v.x;
                    im[u] = v.y;
                }
                constexpr int CH = X3 ? 8 : 4;
#pragma unroll
                for (int u = 0; u < 16; u += CH) {
                    store16<X3>(op, t, y2 + u, re + u);
                    store16<X3>(op, t, 64 + y2 + u, im + u);
                }
            }
        }
        if (!gemm_wait(t_x, fa, oa)) {  // GEMM A: D[(k2, ro)][(c, y1)]
            abort = true;
            break;
        }
        // ---- A -> B: lane (k2, ro); twiddle exp(-2 pi i y1 k2 / 4096); X_B row (c, k2), K (ro, y1)
        {
            const int k2 = t >> 1, ro = t & 1;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float v[32], o[32];
                tmem_ld32(t_x + lane_off + 32 * q, v);
                const int c = q >> 1, ybase = 32 * (q & 1);
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const float p = __shfl_xor_sync(0xffffffffu, v[j], 1);
                    const float2 w = lfft::cmul(P8[(ybase + j) >> 3], P1[(ybase + j) & 7]);
                    o[j] = fmaf(p, w.y, v[j] * w.x);
                }
                store32<X3>(op, c * 64 + k2, ro * 64 + ybase, o);
            }
        }
        if (!gemm_wait(t_b, oa, fa)) {  // GEMM B: D[(c, k2)][(k1, ro)]
            abort = true;
            break;
        }
        for (int k = 0; k < K && !abort; k++) {
            if (wd.kern[k].src != it.chan) continue;
            if (k != kfirst) {
                if (t == 0) {
                    mbar_arrive_expect_tx(bar_kh, S::KH);
                    bulk_g2s(kh, wd.khat + ((size_t)k * (W / 2 + 1) + (size_t)it.tile * TC) * S::HQ, S::KH, bar_kh);
                }
                kh_pending = true;
            }
            if (wg_any(!mbar_wait(bar_kh, ph_kh))) {
                abort = true;
                break;
            }
            kh_pending = false;
            ph_kh ^= 1;
            // ---- B -> C: lane (c, k2); x khat, conjugate; X_C row (c, k2) = t, K (ro, k1)
            {
                const int c = t >> 6, k2 = t & 63;
                const float* khrow = kh + c * S::HQ;
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    float v[32], re[16], im[16];
                    tmem_ld32(t_b + lane_off + 32 * q, v);
#pragma unroll
                    for (int u = 0; u < 16; u++) {
                        const int ky = k2 + 64 * (16 * q + u);
                        const float s = khrow[ky <= 2048 ? ky : 4096 - ky];
                        re[u] = v[2 * u] * s;
                        im[u] = -v[2 * u + 1] * s;
                    }
                    constexpr int CH = X3 ? 8 : 4;
#pragma unroll
                    for (int u = 0; u < 16; u += CH) {
                        store16<X3>(op, t, 16 * q + u, re + u);
                        store16<X3>(op, t, 64 + 16 * q + u, im + u);
                    }
                }
            }
            if (!gemm_wait(t_x, fa, oa)) {  // GEMM C: D[(y1, ro)][(c, k2)]
                abort = true;
                break;
            }
            // ---- C -> D: lane (y1, ro); twiddle exp(-2 pi i k2 y1 / 4096); X_D row (c, y1), K (ro, k2)
            {
                const int y1 = t >> 1, ro = t & 1;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    float v[32], o[32];
                    tmem_ld32(t_x + lane_off + 32 * q, v);
                    const int c = q >> 1, kbase = 32 * (q & 1);
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const float p = __shfl_xor_sync(0xffffffffu, v[j], 1);
                        const float2 w = lfft::cmul(P8[(kbase + j) >> 3], P1[(kbase + j) & 7]);
                        o[j] = fmaf(p, w.y, v[j] * w.x);
                    }
                    store32<X3>(op, c * 64 + y1, ro * 64 + kbase, o);
                }
            }
            if (!gemm_wait(t_x, oa, fa)) {  // GEMM D: D[(c, y1)][(y2, ro)]
                abort = true;
                break;
            }
            // ---- output: lane (c, y1); conjugate; y = y1 + 64 y2 into the free operand buffer, then one
            // bulk copy to the convolved-spectrum tile
            {
                const int c = t >> 6, y1 = t & 63;
                float2* out = reinterpret_cast<float2*>(op) + c;
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    float v[32];
                    tmem_ld32(t_x + lane_off + 32 * q, v);
#pragma unroll
                    for (int u = 0; u < 16; u++) out[(y1 + 64 * (16 * q + u)) * TC] = make_float2(v[2 * u], -v[2 * u + 1]);
                }
            }
            fence_async_smem();
            wg_sync();
            if (t == 0) {
                bulk_s2g(wd.conv + (size_t)k * cplane + (size_t)it.tile * S::H * TC, op, S::H * TC * 8);
                bulk_commit();
                bulk_wait_read0();  // the operand buffer is rebuilt next
            }
            tc_fence_before();
            wg_sync();
        }
    }
    if (t == 0) {
        if (abort) {
            if (f_failed) mbar_wait(bar_f, 0);
            if (kh_pending) mbar_wait(bar_kh, ph_kh);
            if (mma_pending) mbar_wait(bar_mma, ph_mma);
            atomicExch(ctl + CTL_ERR, 1);
        }
        bulk_wait0();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(*tslot, 512);
    }
}

bool launch_col_tc64(bool x3, const void* fmat, const DevWorld* worlds, const ColItem* groups, int ngroups,
                     const float2* tw, int* err, cudaStream_t s, int reserve_sms) {
    static int attr[2] = {0, 0};
    const int smem = x3 ? Tc64<true>::SMEM : Tc64<false>::SMEM;
    if (!attr[x3]) {
        cudaError_t e = x3 ? cudaFuncSetAttribute(col_pass_tc64<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
                           : cudaFuncSetAttribute(col_pass_tc64<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return false;
        attr[x3] = 1;
    }
    if (ngroups <= 0) return true;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = (ngroups + 1) / 2;
    if (grid > sms - reserve_sms) grid = sms - reserve_sms;
    if (grid < 1) grid = 1;
    if (x3) col_pass_tc64<true><<<grid, 256, smem, s>>>(worlds, groups, ngroups, (const uint8_t*)fmat, tw, err);
    else col_pass_tc64<false><<<grid, 256, smem, s>>>(worlds, groups, ngroups, (const uint8_t*)fmat, tw, err);
    return true;
}

}  // namespace lenia
