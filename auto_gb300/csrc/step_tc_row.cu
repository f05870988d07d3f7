// Row pass as DFT-as-GEMM on the 5th-generation tensor cores (tcgen05), for the one-channel,
// one-kernel Lenia step on LENIA_PATH_TF32 and LENIA_PATH_BF16X3.
//
// The row pass takes each row's convolved half-spectrum back to U with an inverse real DFT along
// x, applies the Gaussian growth, the dt update and the clamp (spectral.rs:337-345), writes the
// state, and takes the new row forward again to its half-spectrum.  Here a row of length
// W = W1*W2 (x = n1 + W1*n2, k = k2 + W2*k1) goes through four real GEMMs against small DFT
// matrices, with the twiddles exp(-+2 pi i k2 n1 / W) applied in the hand-overs between them and
// the growth epilogue fused into the middle one:
//
//   GEMM P  rows (r, k2)  x  K (re/im, k1)  ->  N (re/im, n1)    inverse DFT over k1
//   GEMM Q  rows (r, n1)  x  K (re/im, k2)  ->  N (n2)           inverse DFT over k2, real part
//            U[r][n1 + W1*n2]  ->  growth, dt, clamp against the state  ->  new state
//   GEMM R  rows (r, n1)  x  K (n2)         ->  N (re/im, k2)    forward DFT over n2, real input
//   GEMM S  rows (r, k2)  x  K (re/im, n1)  ->  N (re/im, k1)    forward DFT over n1
//
// Every GEMM uses a forward DFT matrix, rows (re/im out, k) and K (re/im in, y); the inverses go
// through IDFT(z) = conj(DFT(conj z)), with the conjugations folded into the hand-overs.  Real input
// (GEMM R) multiplies by the matrix's first half of K; real output (GEMM Q) keeps its first half of
// the rows.  So a row is transformed as a real sequence, with no packing of two rows into one
// complex sequence and no Hermitian regroup.  The full spectrum of the inverse's input is formed
// from the half-spectrum in the first hand-over (k > W/2 from conj X[W - k]), and the forward
// output keeps k <= W/2, with the real DC and Nyquist values packed into slot 0 as the rest of
// the engine stores them.
//
// A group is RG rows of one world (M = RG*W1 and RG*W2 rows, blocks of 128).  Its half-spectrum rows
// come in by 16-byte asynchronous copies into shared memory (prefetched one group ahead), its state
// rows by bulk copies, and the new state leaves by bulk copies straight from the buffer the growth
// updated.  Waits are bounded and given up for the whole CTA at once, as in the column pass.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "cache_hints.cuh"
#include "step_fp32.cuh"
#include "step_tc.cuh"
#include "tc_opnd.cuh"
#include "tc_ptx.cuh"

namespace lenia {
using namespace tc;

constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int W1_, int W2_, int RG_, bool X3_, int LBO_>
struct TcRowShape {
    static constexpr int W1 = W1_, W2 = W2_, W = W1 * W2, RG = RG_, LBO = LBO_;
    static constexpr bool X3 = X3_;
    static constexpr int E = X3 ? 2 : 4;    // operand element bytes
    static constexpr int NOP = X3 ? 2 : 1;  // hi/lo copies
    static constexpr int MP = RG * W2, MQ = RG * W1;  // rows (r, k2) and (r, n1)
    static constexpr int KP = 2 * W1, KQ = 2 * W2, KR = W2, KS = 2 * W1;
    static constexpr int NP = 2 * W1, NQ = W2, NR = 2 * W2, NS = 2 * W1;
    static constexpr int OPND = cmax(cmax(kmajor_bytes(MP, KP, E, LBO), kmajor_bytes(MQ, KQ, E, LBO)),
                                     cmax(kmajor_bytes(MQ, KR, E, LBO), kmajor_bytes(MP, KS, E, LBO)));
    static constexpr bool SAME = W1 == W2;
    static constexpr int F1 = kmajor_bytes(2 * W1, 2 * W1, E, LBO), F2 = kmajor_bytes(2 * W2, 2 * W2, E, LBO);
    static constexpr int OFF_F1 = OPND * NOP;
    static constexpr int OFF_F2 = OFF_F1 + F1 * NOP;
    static constexpr int XR = W / 2 + 2;         // half-spectrum row stride in shared memory (float2)
    static constexpr int XSB = RG * XR * 8;      // one buffer of the group's half-spectrum rows
    static constexpr int OFF_XS = OFF_F2 + (SAME ? 0 : F2 * NOP);
    static constexpr int STR = W + 16;           // state row stride (floats): rows 64 bytes apart mod 128
    static constexpr int OFF_ST = OFF_XS + 2 * XSB;
    static constexpr int OFF_BAR = OFF_ST + RG * STR * 4;
    static constexpr int SMEM = OFF_BAR + 64;
    static constexpr int REGION = cmax(cmax((MP / 128) * NP, (MQ / 128) * NQ), cmax((MQ / 128) * NR, (MP / 128) * NS));
    static constexpr int TCOLS = REGION <= 32 ? 32 : REGION <= 64 ? 64 : REGION <= 128 ? 128 : REGION <= 256 ? 256 : 512;
    static_assert(MP % 128 == 0 && MQ % 128 == 0, "row blocks of 128");
    static_assert(W1 % 16 == 0 && W2 % 16 == 0, "hand-overs in runs of 16 columns; N >= 16");
    static_assert(REGION <= 512, "TMEM");
    static_assert((W * 4) % 16 == 0 && (STR * 4) % 16 == 0 && (XR * 8) % 16 == 0, "16-byte rows");
    static_assert(MQ * KQ * 2 <= OPND && MP * KS * 2 <= OPND, "MN-major operands fit the operand area");
    static_assert(SMEM <= 232448, "shared memory of one CTA");
};

// One group: RG rows of one world, from the FP32 row pass's item list (group_at).
template <class S>
__global__ void __launch_bounds__(128, 1)
    row_pass_tc(const DevWorld* __restrict__ worlds, const RowItem* __restrict__ items, int item_stride, int ngroups,
                const uint8_t* __restrict__ fmats, const float2* __restrict__ tw, int* ctl) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint8_t* op = smem;
    uint8_t* f1 = smem + S::OFF_F1;
    uint8_t* f2 = S::SAME ? f1 : smem + S::OFF_F2;
    float2* xsb = reinterpret_cast<float2*>(smem + S::OFF_XS);
    float* st = reinterpret_cast<float*>(smem + S::OFF_ST);
    uint64_t* bar_st = reinterpret_cast<uint64_t*>(smem + S::OFF_BAR);
    uint64_t* bar_mma = bar_st + 1;
    uint64_t* bar_f = bar_st + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_st + 4);
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr int FMT = S::X3 ? 1 : 2;
    // BF16x3: the transposing hand-overs (P -> Q, R -> S) store MN-major A operands, 16 bytes a store
    // (TF32 keeps every operand K-major)
    constexpr uint32_t ID_P = instr_desc(FMT, 128, S::NP), ID_Q = instr_desc(FMT, 128, S::NQ, S::X3);
    constexpr uint32_t ID_R = instr_desc(FMT, 128, S::NR), ID_S = instr_desc(FMT, 128, S::NS, S::X3);
    constexpr int CH = S::X3 ? 8 : 4;  // values per 16-byte operand chunk

    if (tid == 0) {
        mbar_init(bar_st, 1);
        mbar_init(bar_mma, 1);
        mbar_init(bar_f, 1);
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, S::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tx = *tmem_slot;
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;

    // Twiddles of the two hand-overs from per-thread tables.  A thread's rows are b*128 + tid, and
    // 128 is a multiple of W1 and W2, so its k2 (rows (r, k2)) and its n1 (rows (r, n1)) are the same in
    // every row block: exp(-2 pi i k2 n1 / W) with n1 = 16 q + u (P -> Q) is A_q[q] * A_u[u], and with
    // k2 = 16 q + u (R -> S) it is C_q[q] * C_u[u].
    constexpr int QA = S::W1 / 16, QC = S::W2 / 16;
    float2 Aq[QA], Au[16], Cq[QC], Cu[16];
    {
        const int k2 = tid % S::W2, n1 = tid % S::W1;
#pragma unroll
        for (int q = 0; q < QA; q++) Aq[q] = twid<S::W>(tw, k2, 16 * q);
#pragma unroll
        for (int q = 0; q < QC; q++) Cq[q] = twid<S::W>(tw, n1, 16 * q);
#pragma unroll
        for (int u = 0; u < 16; u++) {
            Au[u] = twid<S::W>(tw, k2, u);
            Cu[u] = twid<S::W>(tw, n1, u);
        }
    }

    // Group g's world and first row, from the row items.  item_stride > 0:
    // a group spans item_stride items; < 0: an item holds -item_stride groups.
    auto group_at = [&](int g) {
        if (item_stride > 0) return items[(size_t)g * item_stride];
        const int sub = -item_stride;
        RowItem it = items[g / sub];
        it.row0 += (g % sub) * S::RG;
        return it;
    };
    // The group's half-spectrum rows, 16 bytes (one tile's two columns of one row) per copy.
    auto fetch_rows = [&](int g, float2* dst) {
        const RowItem it = group_at(g);
        const DevWorld& wd = worlds[it.world];
        const float2* src = wd.conv + (size_t)it.row0 * TC;
        const int H = wd.H;
        for (int i = tid; i < S::W / 4 * S::RG; i += 128) {
            const int r = i % S::RG, t = i / S::RG;
            cp_async16(dst + r * S::XR + 2 * t, src + ((size_t)t * H + r) * TC);
        }
    };
    // The group's state rows by bulk copies (one thread).
    auto fetch_state = [&](int g) {
        const RowItem it = group_at(g);
        const float* src = worlds[it.world].state + (size_t)it.row0 * S::W;
        mbar_arrive_expect_tx(bar_st, S::RG * S::W * 4);
        for (int r = 0; r < S::RG; r++) bulk_g2s(st + r * S::STR, src + (size_t)r * S::W, S::W * 4, bar_st);
    };

    if (tid == 0) {
        const uint32_t fbytes = (S::F1 + (S::SAME ? 0 : S::F2)) * S::NOP;
        mbar_arrive_expect_tx(bar_f, fbytes);
        bulk_g2s(f1, fmats, fbytes, bar_f);
        if (blockIdx.x < ngroups) fetch_state(blockIdx.x);
    }
    if (blockIdx.x < ngroups) fetch_rows(blockIdx.x, xsb);
    // asynchronous work in flight that an early exit has to wait for (uniform across the CTA)
    bool st_pending = blockIdx.x < ngroups, mma_pending = false;
    const bool f_failed = __syncthreads_or(!mbar_wait_n(bar_f, 0, f_wait_polls(ctl)));
    bool abort = f_failed;
    uint32_t ph_st = 0, ph_mma = 0;
    // issue one GEMM from an elected thread and wait for it; false (on every thread) if the wait gave up
    auto gemm = [&](int M, int K, uint32_t f_addr, uint32_t f_lo, int fK, int N, uint32_t idesc, bool amn = false) {
        if (tid == 0) {
            tc_fence_after();
            if (S::X3 && amn)
                issue_gemm_amn<S::LBO>(tx, smem_u32(op), S::OPND, M, K, f_addr, f_lo, fK, N, idesc);
            else
                issue_gemm_k<S::X3, S::LBO>(tx, smem_u32(op), S::OPND, M, K, K, f_addr, f_lo, fK, N, idesc);
            mma_commit(bar_mma);
        }
        if (__syncthreads_or(!mbar_wait(bar_mma, ph_mma))) {
            mma_pending = true;
            return false;
        }
        ph_mma ^= 1;
        tc_fence_after();
        return true;
    };

    int buf = 0;
    for (int g = blockIdx.x; g < ngroups && !abort; g += gridDim.x, buf ^= 1) {
        const RowItem it = group_at(g);
        const DevWorld& wd = worlds[it.world];
        const int H = wd.H;
        float2* xs = xsb + buf * (S::XSB / 8);
        cp_async_wait_all();  // this group's half-spectrum rows
        __syncthreads();
        // the next group's rows into the other buffer (its previous group's output has gone out)
        if (g + (int)gridDim.x < ngroups) fetch_rows(g + gridDim.x, xsb + (buf ^ 1) * (S::XSB / 8));

        // ---- stage 0: full spectrum Z[k2 + W2 k1] (k > W/2 from conj X[W - k]; DC and Nyquist from
        //      slot 0), conjugated for the inverse: A_P rows (r, k2), K (re/im, k1)
        for (int b = 0; b < S::MP / 128; b++) {
            const int rm = b * 128 + tid, r = rm / S::W2, k2 = rm % S::W2;
            const float2* xr = xs + r * S::XR;
#pragma unroll 2
            for (int k10 = 0; k10 < S::W1; k10 += CH) {
                float re[CH], im[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int k = k2 + S::W2 * (k10 + u);
                    float2 z;
                    if (k < S::W / 2) {
                        z = xr[k];
                        if (k == 0) z.y = 0.0f;
                    } else if (k == S::W / 2) {
                        z = make_float2(xr[0].y, 0.0f);
                    } else {
                        const float2 v = xr[S::W - k];
                        z = make_float2(v.x, -v.y);
                    }
                    re[u] = z.x;
                    im[u] = -z.y;
                }
                store_chunk<S::X3, S::LBO>(op, S::OPND, rm, k10, S::KP, re);
                store_chunk<S::X3, S::LBO>(op, S::OPND, rm, S::W1 + k10, S::KP, im);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (!gemm(S::MP, S::KP, smem_u32(f1), S::F1, 2 * S::W1, S::NP, ID_P)) {
            abort = true;
            break;
        }

        // ---- P -> Q: conj(Y') = P * exp(-2 pi i k2 n1 / W) (P holds conj of the inverse over k1);
        //      A_Q rows (r, n1), K (re/im, k2)
        for (int b = 0; b < S::MP / 128; b++) {
            const int rm = b * 128 + tid, r = rm / S::W2, k2 = rm % S::W2;
#pragma unroll
            for (int q = 0; q < QA; q++) {
                float re[16], im[16];
                const uint32_t t0 = tx + lane_off + (uint32_t)(b * S::NP + 16 * q);
                tmem_ld16x2(t0, t0 + S::W1, re, im);
                if constexpr (S::X3) {
                    float vr[16], vi[16];
#pragma unroll
                    for (int u = 0; u < 16; u++) {
                        const float2 w = lfft::cmul(Aq[q], Au[u]);
                        vr[u] = re[u] * w.x - im[u] * w.y;
                        vi[u] = re[u] * w.y + im[u] * w.x;
                    }
                    const int m0 = r * S::W1 + 16 * q;
                    store_mn_chunk(op, S::OPND, m0, k2, S::MQ, vr);
                    store_mn_chunk(op, S::OPND, m0 + 8, k2, S::MQ, vr + 8);
                    store_mn_chunk(op, S::OPND, m0, S::W2 + k2, S::MQ, vi);
                    store_mn_chunk(op, S::OPND, m0 + 8, S::W2 + k2, S::MQ, vi + 8);
                } else {
#pragma unroll
                    for (int u = 0; u < 16; u++) {
                        const float2 w = lfft::cmul(Aq[q], Au[u]);
                        const int rr = r * S::W1 + 16 * q + u;
                        store_elem<S::X3, S::LBO>(op, S::OPND, rr, k2, S::KQ, re[u] * w.x - im[u] * w.y);
                        store_elem<S::X3, S::LBO>(op, S::OPND, rr, S::W2 + k2, S::KQ, re[u] * w.y + im[u] * w.x);
                    }
                }
            }
        }
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (!gemm(S::MQ, S::KQ, smem_u32(f2), S::F2, 2 * S::W2, S::NQ, ID_Q, true)) {
            abort = true;
            break;
        }

        // ---- growth: U at x = n1 + W1 n2; new state into the state buffer and into A_R rows (r, n1),
        //      K (n2), real
        if (__syncthreads_or(!mbar_wait(bar_st, ph_st))) {
            abort = true;
            break;
        }
        st_pending = false;
        ph_st ^= 1;
        {
            const DevKernel kp = wd.kern[0];
            const float dtw = wd.dt * kp.weight;
            const Growth growth(kp.mu, kp.sigma);
            for (int b = 0; b < S::MQ / 128; b++) {
                const int rm = b * 128 + tid, r = rm / S::W1, n1 = rm % S::W1;
                float* sr = st + r * S::STR + n1;
#pragma unroll
                for (int q = 0; q < S::W2 / 16; q++) {
                    float u[16], v[16];
                    tmem_ld16(tx + lane_off + (uint32_t)(b * S::NQ + 16 * q), u);
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        float* p = sr + S::W1 * (16 * q + j);
                        v[j] = __saturatef(fmaf(dtw, growth(u[j]), *p));
                        *p = v[j];
                    }
#pragma unroll
                    for (int c = 0; c < 16; c += CH) store_chunk<S::X3, S::LBO>(op, S::OPND, rm, 16 * q + c, S::KR, v + c);
                }
            }
        }
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            float* dst = wd.state + (size_t)it.row0 * S::W;
            for (int r = 0; r < S::RG; r++) bulk_s2g(dst + (size_t)r * S::W, st + r * S::STR, S::W * 4);
            bulk_commit();
        }
        if (!gemm(S::MQ, S::KR, smem_u32(f2), S::F2, 2 * S::W2, S::NR, ID_R)) {
            abort = true;
            break;
        }

        // ---- R -> S: V * exp(-2 pi i k2 n1 / W); A_S rows (r, k2), K (re/im, n1)
        for (int b = 0; b < S::MQ / 128; b++) {
            const int rm = b * 128 + tid, r = rm / S::W1, n1 = rm % S::W1;
#pragma unroll
            for (int q = 0; q < QC; q++) {
                float re[16], im[16];
                const uint32_t t0 = tx + lane_off + (uint32_t)(b * S::NR + 16 * q);
                tmem_ld16x2(t0, t0 + S::W2, re, im);
                if constexpr (S::X3) {
                    float vr[16], vi[16];
#pragma unroll
                    for (int u = 0; u < 16; u++) {
                        const float2 w = lfft::cmul(Cq[q], Cu[u]);
                        vr[u] = re[u] * w.x - im[u] * w.y;
                        vi[u] = re[u] * w.y + im[u] * w.x;
                    }
                    const int m0 = r * S::W2 + 16 * q;
                    store_mn_chunk(op, S::OPND, m0, n1, S::MP, vr);
                    store_mn_chunk(op, S::OPND, m0 + 8, n1, S::MP, vr + 8);
                    store_mn_chunk(op, S::OPND, m0, S::W1 + n1, S::MP, vi);
                    store_mn_chunk(op, S::OPND, m0 + 8, S::W1 + n1, S::MP, vi + 8);
                } else {
#pragma unroll
                    for (int u = 0; u < 16; u++) {
                        const float2 w = lfft::cmul(Cq[q], Cu[u]);
                        const int rr = r * S::W2 + 16 * q + u;
                        store_elem<S::X3, S::LBO>(op, S::OPND, rr, n1, S::KS, re[u] * w.x - im[u] * w.y);
                        store_elem<S::X3, S::LBO>(op, S::OPND, rr, S::W1 + n1, S::KS, re[u] * w.y + im[u] * w.x);
                    }
                }
            }
        }
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (!gemm(S::MP, S::KS, smem_u32(f1), S::F1, 2 * S::W1, S::NS, ID_S, true)) {
            abort = true;
            break;
        }

        // ---- output: X[k2 + W2 k1] for k <= W/2 into this group's spectrum buffer (natural order),
        //      DC and Nyquist (both real) packed into slot 0
        for (int b = 0; b < S::MP / 128; b++) {
            const int rm = b * 128 + tid, r = rm / S::W2, k2 = rm % S::W2;
            float2* xo = xs + r * S::XR;
            constexpr int HALF = S::W1 / 2;
            float dc = 0.0f, nyq = 0.0f;
#pragma unroll
            for (int q = 0; q < (HALF + 15) / 16; q++) {
                float re[16], im[16];
                const uint32_t t0 = tx + lane_off + (uint32_t)(b * S::NS + 16 * q);
                tmem_ld16x2(t0, t0 + S::W1, re, im);
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    const int k1 = 16 * q + u;
                    if (k1 < HALF) {
                        const int k = k2 + S::W2 * k1;
                        if (k == 0)
                            dc = re[u];
                        else
                            xo[k] = make_float2(re[u], im[u]);
                    }
                    if (HALF % 16 != 0 && k1 == HALF) nyq = re[u];
                }
            }
            if (HALF % 16 == 0) nyq = tmem_ld1(tx + lane_off + (uint32_t)(b * S::NS + HALF));
            if (k2 == 0) xo[0] = make_float2(dc, nyq);
        }
        tc_fence_before();
        __syncthreads();
        {
            // 16 bytes per (tile, row): consecutive threads on consecutive rows of one tile
            float2* dst = wd.spec + (size_t)it.row0 * TC;
            const uint64_t keep = hint::policy_keep();
            for (int i = tid; i < S::W / 4 * S::RG; i += 128) {
                const int r = i % S::RG, t = i / S::RG;
                hint::st4(reinterpret_cast<float4*>(dst + ((size_t)t * H + r) * TC),
                          *reinterpret_cast<const float4*>(xs + r * S::XR + 2 * t), keep);
            }
        }
        // the next group's state rows, once this group's state store has read the buffer
        if (g + (int)gridDim.x < ngroups) {
            if (tid == 0) {
                bulk_wait_read0();
                fetch_state(g + gridDim.x);
            }
            st_pending = true;
        }
    }
    // Exit: wait (bounded) for this CTA's own asynchronous work before its shared memory and TMEM
    // are released, then report.
    if (tid == 0) {
        if (abort) {
            if (f_failed) mbar_wait(bar_f, 0);
            if (st_pending) mbar_wait(bar_st, ph_st);
            if (mma_pending) mbar_wait(bar_mma, ph_mma);
            atomicExch(ctl + CTL_ERR, 1);
        }
        bulk_wait0();
    }
    cp_async_wait_all();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tx, S::TCOLS);
    }
}

// ------------------------------------------------------------------ host side

namespace {

// Forward DFT matrix of length n as the B operand: rows (re/im out, k), K (re/im in, y), entries
// of exp(-2 pi i y k / n) rounded from FP64, in the K-major layout, as bf16 hi then lo, or tf32.
void build_row_dft(int n, bool x3, std::vector<uint8_t>& out, int lbo) {
    const int N = 2 * n, K = 2 * n, E = x3 ? 2 : 4;
    const size_t bytes = (size_t)kmajor_bytes(N, K, E, lbo);
    const size_t base = out.size();
    out.resize(base + bytes * (x3 ? 2 : 1), 0);
    for (int row = 0; row < N; row++)
        for (int kk = 0; kk < K; kk++) {
            const int ro = row / n, k = row % n, ri = kk / n, y = kk % n;
            const double th = 2.0 * M_PI * (double)((long)y * k % n) / n, c = std::cos(th), s = std::sin(th);
            const double v = ro == 0 ? (ri == 0 ? c : s) : (ri == 0 ? -s : c);
            const uint32_t off = kmajor_offset(row, kk, K, E, lbo);
            if (x3) {
                const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
                const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
                *reinterpret_cast<__nv_bfloat16*>(&out[base + off]) = hi;
                *reinterpret_cast<__nv_bfloat16*>(&out[base + bytes + off]) = lo;
            } else {
                float f = (float)v;
                uint32_t u;
                memcpy(&u, &f, 4);
                u = (u + 0x1000u) & 0xFFFFE000u;  // nearest tf32, ties away from zero
                memcpy(&out[base + off], &u, 4);
            }
        }
}

// Row length, its factors W1 x W2 (W1 <= W2 keeps the GEMM work down: it is RG W (8 W1 + 4 W2)
// multiply-adds a group), rows per group, and the operand layout's LBO.
struct RowShapeInfo {
    int W, W1, W2, RG, LBO;
};
constexpr RowShapeInfo ROW_SHAPES[] = {{1024, 32, 32, 4, 144}, {512, 16, 32, 8, 144}, {256, 16, 16, 8, 144}};

const RowShapeInfo* row_shape_for(int W) {
    for (const auto& s : ROW_SHAPES)
        if (s.W == W) return &s;
    return nullptr;
}

template <class S>
bool launch_row_shape(const void* fm, const DevWorld* worlds, const RowItem* items, int item_stride, int ngroups,
                      const float2* tw, int* err, cudaStream_t st) {
    static int attr = 0;
    if (!attr) {
        if (cudaFuncSetAttribute(row_pass_tc<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM) != cudaSuccess ||
            cudaFuncSetAttribute(row_pass_tc<S>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return false;
        attr = 1;
    }
    if (ngroups <= 0) return true;
    // CTAs per SM from the SM's shared memory, registers and TMEM (persistent grid over the groups)
    static int per_sm = 0, sms = 0;
    if (!per_sm) {
        int dev = 0, smem_sm = 0, regs_sm = 0, reserved = 0;
        cudaFuncAttributes fa;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, row_pass_tc<S>) != cudaSuccess)
            return false;
        int n = smem_sm / (S::SMEM + reserved);
        const int by_regs = regs_sm / (128 * (fa.numRegs > 0 ? fa.numRegs : 255));
        if (by_regs < n) n = by_regs;
        if (n * S::TCOLS > 512) n = 512 / S::TCOLS;
        if (n > 16) n = 16;
        per_sm = n < 1 ? 1 : n;
    }
    int grid = sms * per_sm;
    if (grid > ngroups) grid = ngroups;
    row_pass_tc<S><<<grid, 128, S::SMEM, st>>>(worlds, items, item_stride, ngroups, (const uint8_t*)fm, tw, err);
    return true;
}

}  // namespace

bool tc_row_supports(int W) { return row_shape_for(W) != nullptr; }
int tc_row_group_rows(int W) {
    const RowShapeInfo* s = row_shape_for(W);
    return s ? s->RG : 0;
}

int tc_row_prepare(TcPlan& plan, int path, int W, std::string* err) {
    const RowShapeInfo* s = row_shape_for(W);
    if (!s) return 0;  // served by the FP32 row pass
    for (int i = 0; i < plan.nrsizes; i++)
        if (plan.rsizes[i] == W) return 0;
    if (plan.nrsizes >= 16) {
        if (err) *err = "too many tensor-core row sizes";
        return LENIA_EINVAL;
    }
    const bool x3 = path == LENIA_PATH_BF16X3;
    std::vector<uint8_t> host;
    build_row_dft(s->W1, x3, host, s->LBO);                  // F_W1 (hi, lo)
    if (s->W1 != s->W2) build_row_dft(s->W2, x3, host, s->LBO);  // F_W2 (hi, lo)
    void* d = nullptr;
    if (cudaMalloc(&d, host.size()) != cudaSuccess ||
        cudaMemcpy(d, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        if (d) cudaFree(d);
        if (err) *err = "row DFT matrix upload failed";
        return LENIA_ECUDA;
    }
    plan.rmats[plan.nrsizes] = d;
    plan.rsizes[plan.nrsizes] = W;
    plan.nrsizes++;
    return 0;
}

bool launch_row_tc(const TcPlan& plan, int path, int W, const DevWorld* worlds, const RowItem* items, int item_stride,
                   int ngroups, const float2* tw, cudaStream_t s) {
    const void* fm = nullptr;
    for (int i = 0; i < plan.nrsizes; i++)
        if (plan.rsizes[i] == W) fm = plan.rmats[i];
    if (!fm) return false;
    const bool x3 = path == LENIA_PATH_BF16X3;
    int* e = (int*)plan.d_err;
    switch (W) {
    case 1024:
        return x3 ? launch_row_shape<TcRowShape<32, 32, 4, true, 144>>(fm, worlds, items, item_stride, ngroups, tw, e, s)
                  : launch_row_shape<TcRowShape<32, 32, 4, false, 144>>(fm, worlds, items, item_stride, ngroups, tw, e, s);
    case 512:
        return x3 ? launch_row_shape<TcRowShape<16, 32, 8, true, 144>>(fm, worlds, items, item_stride, ngroups, tw, e, s)
                  : launch_row_shape<TcRowShape<16, 32, 8, false, 144>>(fm, worlds, items, item_stride, ngroups, tw, e, s);
    case 256:
        return x3 ? launch_row_shape<TcRowShape<16, 16, 8, true, 144>>(fm, worlds, items, item_stride, ngroups, tw, e, s)
                  : launch_row_shape<TcRowShape<16, 16, 8, false, 144>>(fm, worlds, items, item_stride, ngroups, tw, e, s);
    }
    return false;
}

void tc_row_release(TcPlan& plan) {
    for (int i = 0; i < plan.nrsizes; i++) cudaFree(plan.rmats[i]);
    plan.nrsizes = 0;
}

}  // namespace lenia
