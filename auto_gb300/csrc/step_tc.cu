// Column pass as DFT-as-GEMM on the 5th-generation tensor cores (tcgen05): LENIA_PATH_TF32 and
// LENIA_PATH_BF16X3.
//
// The column pass transforms every spectrum column along y, multiplies by the kernel spectrum
// and transforms back (the FP32 path does this with shared-memory butterflies).  Here a column
// of length H = H1*H2 (y = y1 + H1*y2) is transformed by the four-step method as two real GEMMs
// against small DFT matrices, with the twiddle exp(-2 pi i y1 k2 / H) applied between them:
//
//   GEMM A  rows (c, y1)  x  K (re/im, y2)  ->  N (k2, re/im)      DFT over y2, length H2
//   GEMM B  rows (c, k2)  x  K (re/im, y1)  ->  N (k1, re/im)      DFT over y1, length H1
//            spectrum X[c][k2 + H2*k1]  *  khat  (real), conjugated
//   GEMM C  rows (c, k2)  x  K (re/im, k1)  ->  N (y1, re/im)      DFT over k1
//   GEMM D  rows (c, y1)  x  K (re/im, k2)  ->  N (y2, re/im)      DFT over k2, then conjugated
//
// The inverse uses the forward matrices through IDFT(z) = conj(DFT(conj z)).  The data is the A
// operand (M = 128-row blocks of the CT columns a CTA owns), the DFT matrix is the B operand, both
// in shared memory in the canonical K-major layout, with FP32 accumulators in TMEM.  BF16X3 splits
// both operands into bf16 hi + lo and accumulates hi*hi + hi*lo + lo*hi; TF32 rounds both to tf32.
// Tiles arrive and leave by bulk (TMA) copies; one elected thread issues every MMA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "fft_core.cuh"
#include "step_tc.cuh"
#include "tc_opnd.cuh"
#include "tc_ptx.cuh"

namespace lenia {
using namespace tc;

template <int H1_, int H2_, int CT_, bool X3_, int LBO_, int WG_, int MINB_, bool STAGED_ = true>
struct TcShape {
    static constexpr int H1 = H1_, H2 = H2_, CT = CT_, H = H1 * H2;
    static constexpr bool X3 = X3_;
    static constexpr int WG = WG_, NT = 128 * WG_;    // warpgroups sharing each hand-over
    static constexpr int MINB = MINB_;                // CTAs per SM the register budget is set for
    // STAGED: the next tile group arrives by a bulk copy into a staging buffer while this one computes;
    // else stage 0 reads it from global memory (prefetched into L2 a group ahead) and the CTA needs
    // 32 KB less shared memory, so more CTAs fit an SM
    static constexpr bool STAGED = STAGED_;
    static constexpr int E = X3 ? 2 : 4;              // operand element bytes
    static constexpr int NOP = X3 ? 2 : 1;            // hi/lo copies
    static constexpr int MA = CT * H1, KA = 2 * H2, NA = 2 * H2;
    static constexpr int MB = CT * H2, KB = 2 * H1, NB = 2 * H1;
    static constexpr int LBO = LBO_;                  // K-major layout, packed (128) or padded (144): kmajor_offset
    static constexpr int OPND = kmajor_bytes(MA, KA, E, LBO);  // one operand copy (== MB x KB)
    static constexpr int FA = kmajor_bytes(NA, KA, E, LBO), FB = kmajor_bytes(NB, KB, E, LBO);
    static constexpr bool SAME = H1 == H2;
    static constexpr int STG = CT * H * 8;            // fp32 complex tile group
    static constexpr int OFF_F2 = OPND * NOP;
    static constexpr int OFF_F1 = OFF_F2 + FA * NOP;
    static constexpr int OFF_STG = OFF_F1 + (SAME ? 0 : FB * NOP);
    static constexpr int HQ = (H / 2 + 1 + 3) / 4 * 4;  // kernel-spectrum row stride (floats)
    static constexpr int OFF_KH = OFF_STG + (STAGED ? STG : 0);  // the group's CT kernel-spectrum rows
    static constexpr int KHB = CT * HQ * 4;
    static constexpr int OFF_BAR = OFF_KH + KHB;
    static constexpr int SMEM = OFF_BAR + 64;
    static constexpr int COLS_A = (MA / 128) * NA, COLS_B = (MB / 128) * NB;
    static constexpr int REGION = COLS_A > COLS_B ? COLS_A : COLS_B;
    static constexpr int TCOLS = 2 * REGION <= 32 ? 32 : (2 * REGION <= 64 ? 64 : (2 * REGION <= 128 ? 128 : (2 * REGION <= 256 ? 256 : 512)));
    static_assert(kmajor_bytes(MB, KB, E, LBO) == OPND, "both GEMM shapes fill one operand area");
    static_assert(OPND * NOP >= STG, "the output staging reuses the operand area");
    static_assert(MA % 128 == 0 && MB % 128 == 0, "row blocks of 128");
    static_assert(H1 % 8 == 0 && H2 % 8 == 0 && (H2 / WG) % 8 == 0, "hand-over units of 8 values");
    static_assert(2 * REGION <= 512, "TMEM");
    static_assert(SMEM <= 232448, "shared memory of one CTA");
};

// t[h] for a run-time h, by selects over the unrolled table (an indexed load would put the table in
// local memory)
template <int N>
__device__ __forceinline__ float2 pick(const float2 (&t)[N], int h) {
    float2 r = t[0];
#pragma unroll
    for (int i = 1; i < N; i++)
        if (h == i) r = t[i];
    return r;
}

// A group is (world, channel, first tile); it covers CT columns = CT / TC consecutive tiles.
//
// NT = 128 WG threads: thread t serves GEMM row lt = t mod 128 of every 128-row block (the TMEM lane its
// warp reads), and the WG warpgroups split each hand-over into units of 16 TMEM columns (8 complex
// values: one 16-byte operand chunk of real and one of imaginary parts), so that more warps hide the
// latency of the TMEM loads and shared-memory stores between the GEMMs.
//
// Every barrier wait is bounded, and the decision to give up is made for the whole CTA at once
// (__syncthreads_or), so that no thread is left at a barrier the others skipped.  A CTA that gives
// up leaves the group loop, waits (bounded again) for whatever it still has in flight -- the
// DFT-matrix load, a tile-group load, issued MMAs, its output stores -- then sets the error flag
// (ctl[CTL_ERR]), frees its TMEM and returns.
template <class S>
__global__ void __launch_bounds__(S::NT, S::MINB)
    col_pass_tc(const DevWorld* __restrict__ worlds, const ColItem* __restrict__ groups, int ngroups,
                const uint8_t* __restrict__ fmats, const float2* __restrict__ tw, int* ctl) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint8_t* op = smem;
    uint8_t* f2 = smem + S::OFF_F2;
    uint8_t* f1 = S::SAME ? f2 : smem + S::OFF_F1;
    float2* stg = reinterpret_cast<float2*>(smem + S::OFF_STG);
    uint64_t* bar_ld = reinterpret_cast<uint64_t*>(smem + S::OFF_BAR);
    uint64_t* bar_mma = bar_ld + 1;
    uint64_t* bar_f = bar_ld + 2;
    uint64_t* bar_kh = bar_ld + 3;  // the group's kernel-spectrum rows arrived
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_ld + 4);
    float* khs = reinterpret_cast<float*>(smem + S::OFF_KH);
    const int tid = threadIdx.x, warp = tid >> 5, lt = tid & 127, wg = tid >> 7;
    constexpr uint32_t IDESC_A = instr_desc(S::X3 ? 1 : 2, 128, S::NA);
    constexpr uint32_t IDESC_B = instr_desc(S::X3 ? 1 : 2, 128, S::NB);
    // BF16x3: the transposing hand-overs (A -> B, C -> D) store MN-major A operands, 16 bytes a store
    // (TF32 keeps every operand K-major)
    constexpr uint32_t IDESC_AM = instr_desc(S::X3 ? 1 : 2, 128, S::NA, S::X3);
    constexpr uint32_t IDESC_BM = instr_desc(S::X3 ? 1 : 2, 128, S::NB, S::X3);
    constexpr int CH = S::X3 ? 8 : 4;  // values per 16-byte K-major operand chunk

    if (tid == 0) {
        mbar_init(bar_ld, 1);
        mbar_init(bar_mma, 1);
        mbar_init(bar_f, 1);
        mbar_init(bar_kh, 1);
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, S::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tmem_slot;
    const uint32_t t_b = tbase;                 // D of GEMM B (kept while every kernel of the channel runs)
    const uint32_t t_x = tbase + S::REGION;     // D of GEMMs A, C, D
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;

    // The twiddles of the two hand-overs from per-thread tables.  A thread's rows are b*128 + lt, and
    // 128 is a multiple of H1 and of H2, so its y1 (A -> B) and its k2 (C -> D) are the same in every
    // row block: exp(-2 pi i y1 k2 / H) with k2 = 8 h + j is A8[h] * A1[j], and with y1 = 8 h + j it is
    // C8[h] * C1[j] -- two exactly rounded table values and one product.
    float2 A8[S::H2 / 8], A1[8], C8[S::H1 / 8], C1[8];
    {
        const int y1 = lt % S::H1, k2 = lt % S::H2;
#pragma unroll
        for (int h = 0; h < S::H2 / 8; h++) A8[h] = twid<S::H>(tw, y1, 8 * h);
#pragma unroll
        for (int h = 0; h < S::H1 / 8; h++) C8[h] = twid<S::H>(tw, k2, 8 * h);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            A1[j] = twid<S::H>(tw, y1, j);
            C1[j] = twid<S::H>(tw, k2, j);
        }
    }

    // DFT matrices (hi, lo) once per CTA; first tile group
    if (tid == 0) {
        const uint32_t fbytes = (S::FA + (S::SAME ? 0 : S::FB)) * S::NOP;
        mbar_arrive_expect_tx(bar_f, fbytes);
        bulk_g2s(f2, fmats, fbytes, bar_f);
    }
    // the CT columns of group g: CT / TC consecutive tiles, contiguous
    auto group_src = [&](int g) {
        const ColItem it = groups[g];
        const DevWorld& wd = worlds[it.world];
        return wd.spec + (size_t)it.chan * (wd.W / 2) * S::H + (size_t)it.tile * S::H * TC;
    };
    auto load_group = [&](int g) {
        if constexpr (S::STAGED) {
            mbar_arrive_expect_tx(bar_ld, S::STG);
            bulk_g2s(stg, group_src(g), S::STG, bar_ld);
        } else {
            bulk_prefetch_l2(group_src(g), S::STG);
        }
    };
    // the group's CT kernel-spectrum rows of kernel k (kx0 .. kx0 + CT - 1, HQ floats each, contiguous)
    // by one bulk copy into shared memory, instead of a global load per element of the hand-over
    auto load_khat = [&](const DevWorld& wd, int k, int kx0) {
        mbar_arrive_expect_tx(bar_kh, S::KHB);
        bulk_g2s(khs, wd.khat + ((size_t)k * (wd.W / 2 + 1) + kx0) * wd.HQ, S::KHB, bar_kh);
    };
    if (tid == 0 && blockIdx.x < ngroups) load_group(blockIdx.x);
    // asynchronous work in flight that an early exit has to wait for (uniform across the CTA)
    bool ld_pending = S::STAGED && blockIdx.x < ngroups, mma_pending = false, kh_pending = false;
    uint32_t ph_kh = 0;
    const bool f_failed = __syncthreads_or(!mbar_wait_n(bar_f, 0, f_wait_polls(ctl)));
    bool abort = f_failed;
    uint32_t ph_ld = 0, ph_mma = 0;
    // issue one GEMM from an elected thread and wait for it; false (on every thread) if the wait gave up
    auto gemm = [&](uint32_t d, uint32_t a_off, int M, int K, uint32_t f_addr, uint32_t f_lo, int N, uint32_t idesc,
                    bool amn = false) {
        if (tid == 0) {
            tc_fence_after();
            if (S::X3 && amn)
                issue_gemm_amn<S::LBO>(d, smem_u32(op), a_off, M, K, f_addr, f_lo, K, N, idesc);
            else
                issue_gemm<S::X3, S::LBO>(d, smem_u32(op), a_off, M, K, f_addr, f_lo, N, idesc);
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
    // Units [0, U) of a hand-over, this warpgroup's share (u = wg, wg + WG, ...), two at a time: both
    // units' TMEM columns are loaded before one wait (tmem_ld16x2), so the two loads' latencies overlap.
    // col(u) is a unit's first TMEM column, fn(u, v) its work on the 16 values v.
    auto units2 = [&](int U, auto col, auto fn) {
        int u = wg;
        for (; u + S::WG < U; u += 2 * S::WG) {
            float va[16], vb[16];
            tmem_ld16x2(col(u), col(u + S::WG), va, vb);
            fn(u, va);
            fn(u + S::WG, vb);
        }
        if (u < U) {
            float v[16];
            tmem_ld16(col(u), v);
            fn(u, v);
        }
    };
    // A transposing hand-over unit: 8 complex values (interleaved re, im) v_j times w(j) = W8 * W1[j],
    // into an A operand at rows m0..m0+7 (MN-major, BF16x3) or rows m0 + j (K-major), columns k (real
    // part) and k + KH (imaginary part).
    auto store_t8 = [&](const float* v, float2 w8, const float2* w1, int m0, int k, int KH, int M, int K) {
        float vr[8], vi[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float2 w = lfft::cmul(w8, w1[j]);
            vr[j] = v[2 * j] * w.x - v[2 * j + 1] * w.y;
            vi[j] = v[2 * j] * w.y + v[2 * j + 1] * w.x;
        }
        if constexpr (S::X3) {
            store_mn_chunk(op, S::OPND, m0, k, M, vr);
            store_mn_chunk(op, S::OPND, m0, k + KH, M, vi);
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                store_elem<false, S::LBO>(op, S::OPND, m0 + j, k, K, vr[j]);
                store_elem<false, S::LBO>(op, S::OPND, m0 + j, k + KH, K, vi[j]);
            }
        }
    };

    for (int g = blockIdx.x; g < ngroups && !abort; g += gridDim.x) {
        const ColItem it = groups[g];
        const DevWorld& wd = worlds[it.world];
        const int W = wd.W, K = wd.K;
        const int kx0 = it.tile * TC;
        if (tid == 0) bulk_wait_read0();  // the previous group's output has left the operand area
        if constexpr (S::STAGED) {
            if (__syncthreads_or(!mbar_wait(bar_ld, ph_ld))) {
                abort = true;
                break;
            }
            ld_pending = false;
            ph_ld ^= 1;
        } else {
            __syncthreads();
            // the next group's columns into L2 while this one computes
            if (tid == 0 && g + (int)gridDim.x < ngroups) load_group(g + gridDim.x);
        }
        // the kernel-spectrum rows of the first kernel that reads this channel, fetched now so that
        // they have arrived when the hand-over after GEMM B needs them
        int kfirst = 0;
        while (kfirst < K && wd.kern[kfirst].src != it.chan) kfirst++;
        if (kfirst < K) {
            if (tid == 0) load_khat(wd, kfirst, kx0);
            kh_pending = true;
        }

        // ---- stage 0: tile group (fp32, [tile][y][c][re,im]) -> A_A rows (c, y1), K (re/im, y2); the
        //      warpgroups split y2
        for (int b = 0; b < S::MA / 128; b++) {
            const int r = b * 128 + lt, c = r / S::H1, y1 = r % S::H1;
            const float2* col = (S::STAGED ? stg : group_src(g)) + (size_t)(c / TC) * S::H * TC + (c % TC);
#pragma unroll 2
            for (int y2 = wg * (S::H2 / S::WG); y2 < (wg + 1) * (S::H2 / S::WG); y2 += CH) {
                float re[CH], im[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const float2 v = col[(size_t)(y1 + S::H1 * (y2 + u)) * TC];
                    re[u] = v.x;
                    im[u] = v.y;
                }
                store_chunk<S::X3, S::LBO>(op, S::OPND, r, y2, S::KA, re);
                store_chunk<S::X3, S::LBO>(op, S::OPND, r, S::H2 + y2, S::KA, im);
            }
        }
        fence_async_smem();
        __syncthreads();
        // the staging buffer is free: fetch the next group while this one computes
        if (S::STAGED && g + (int)gridDim.x < ngroups) {
            if (tid == 0) load_group(g + gridDim.x);
            ld_pending = true;
        }

        // ---- GEMM A
        if (!gemm(t_x, S::OPND, S::MA, S::KA, smem_u32(f2), S::FA, S::NA, IDESC_A)) {
            abort = true;
            break;
        }

        // ---- A -> B: twiddle exp(-2 pi i y1 k2 / H), rows (c, k2), K (re/im, y1); units (block, 8 k2)
        units2((S::MA / 128) * (S::NA / 16),
               [&](int un) { return t_x + lane_off + (uint32_t)((un / (S::NA / 16)) * S::NA + 16 * (un % (S::NA / 16))); },
               [&](int un, const float* v) {
                   const int b = un / (S::NA / 16), h = un % (S::NA / 16);
                   const int r = b * 128 + lt, c = r / S::H1, y1 = r % S::H1;
                   store_t8(v, pick(A8, h), A1, c * S::H2 + 8 * h, y1, S::H1, S::MB, S::KB);
               });
        tc_fence_before();
        fence_async_smem();
        __syncthreads();

        // ---- GEMM B -> spectrum of the channel along y, kept in TMEM region t_b
        if (!gemm(t_b, S::OPND, S::MB, S::KB, smem_u32(f1), S::FB, S::NB, IDESC_BM, true)) {
            abort = true;
            break;
        }

        for (int k = kfirst; k < K && !abort; k++) {
            if (wd.kern[k].src != it.chan) continue;
            if (__syncthreads_or(!mbar_wait(bar_kh, ph_kh))) {
                abort = true;
                break;
            }
            kh_pending = false;
            ph_kh ^= 1;
            // ---- B -> C: x khat (real, even), conjugate; rows (c, k2), K (re/im, k1); units (block, 8 k1)
            units2((S::MB / 128) * (S::NB / 16),
                   [&](int un) { return t_b + lane_off + (uint32_t)((un / (S::NB / 16)) * S::NB + 16 * (un % (S::NB / 16))); },
                   [&](int un, const float* v) {
                const int b = un / (S::NB / 16), h = un % (S::NB / 16);
                const int r = b * 128 + lt, c = r / S::H2, k2 = r % S::H2;
                const float* khrow = khs + c * S::HQ;
                float re[8], im[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int ky = k2 + S::H2 * (8 * h + j);
                    const float sc = khrow[ky <= S::H / 2 ? ky : S::H - ky];
                    re[j] = v[2 * j] * sc;
                    im[j] = -v[2 * j + 1] * sc;
                }
#pragma unroll
                for (int j = 0; j < 8; j += CH) {
                    store_chunk<S::X3, S::LBO>(op, S::OPND, r, 8 * h + j, S::KB, re + j);
                    store_chunk<S::X3, S::LBO>(op, S::OPND, r, S::H1 + 8 * h + j, S::KB, im + j);
                }
            });
            tc_fence_before();
            fence_async_smem();
            __syncthreads();
            // the next kernel's rows (if another kernel reads this channel) while this one finishes
            {
                int kn = k + 1;
                while (kn < K && wd.kern[kn].src != it.chan) kn++;
                if (kn < K) {
                    if (tid == 0) load_khat(wd, kn, kx0);
                    kh_pending = true;
                }
            }
            // ---- GEMM C
            if (!gemm(t_x, S::OPND, S::MB, S::KB, smem_u32(f1), S::FB, S::NB, IDESC_B)) {
                abort = true;
                break;
            }
            // ---- C -> D: twiddle exp(-2 pi i k2 y1 / H); rows (c, y1), K (re/im, k2); units (block, 8 y1)
            units2((S::MB / 128) * (S::NB / 16),
                   [&](int un) { return t_x + lane_off + (uint32_t)((un / (S::NB / 16)) * S::NB + 16 * (un % (S::NB / 16))); },
                   [&](int un, const float* v) {
                       const int b = un / (S::NB / 16), h = un % (S::NB / 16);
                       const int r = b * 128 + lt, c = r / S::H2, k2 = r % S::H2;
                       store_t8(v, pick(C8, h), C1, c * S::H1 + 8 * h, k2, S::H2, S::MA, S::KA);
                   });
            tc_fence_before();
            fence_async_smem();
            __syncthreads();
            // ---- GEMM D
            if (!gemm(t_x, S::OPND, S::MA, S::KA, smem_u32(f2), S::FA, S::NA, IDESC_AM, true)) {
                abort = true;
                break;
            }
            // ---- output: conjugate, natural order y = y1 + H1*y2, into the operand area; units (block, 8 y2)
            float2* out = reinterpret_cast<float2*>(op);
            units2((S::MA / 128) * (S::NA / 16),
                   [&](int un) { return t_x + lane_off + (uint32_t)((un / (S::NA / 16)) * S::NA + 16 * (un % (S::NA / 16))); },
                   [&](int un, const float* v) {
                       const int b = un / (S::NA / 16), h = un % (S::NA / 16);
                       const int r = b * 128 + lt, c = r / S::H1, y1 = r % S::H1;
                       float2* col = out + (size_t)(c / TC) * S::H * TC + (c % TC);
#pragma unroll
                       for (int j = 0; j < 8; j++)
                           col[(size_t)(y1 + S::H1 * (8 * h + j)) * TC] = make_float2(v[2 * j], -v[2 * j + 1]);
                   });
            tc_fence_before();
            fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                float2* dst = wd.conv + (size_t)k * (W / 2) * S::H + (size_t)it.tile * S::H * TC;
                bulk_s2g(dst, out, S::STG);
                bulk_commit();
                bulk_wait_read0();  // the next kernel (if any) rebuilds the operand area
            }
            __syncthreads();
        }
    }
    // Early exit: wait (bounded) for this CTA's own asynchronous work before its shared memory and
    // TMEM are released, then report.
    if (tid == 0) {
        if (abort) {
            if (f_failed) mbar_wait(bar_f, 0);
            if (ld_pending) mbar_wait(bar_ld, ph_ld);
            if (mma_pending) mbar_wait(bar_mma, ph_mma);
            if (kh_pending) mbar_wait(bar_kh, ph_kh);
            atomicExch(ctl + CTL_ERR, 1);
        }
        bulk_wait0();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tbase, S::TCOLS);
    }
}

// ------------------------------------------------------------------ host side

namespace {

// DFT matrix of length n as the B operand: rows (k, re/im out), K (re/im in, y), exp(-2 pi i y k / n),
// in the K-major layout, as bf16 hi then lo, or tf32 -- rounded from FP64.
void build_dft_operand(int n, bool x3, std::vector<uint8_t>& out, int lbo) {
    const int N = 2 * n, K = 2 * n, E = x3 ? 2 : 4;
    const size_t bytes = (size_t)kmajor_bytes(N, K, E, lbo);
    const size_t base = out.size();
    out.resize(base + bytes * (x3 ? 2 : 1), 0);
    for (int row = 0; row < N; row++)
        for (int kk = 0; kk < K; kk++) {
            const int k = row / 2, ro = row % 2, ri = kk / n, y = kk % n;
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
                // round to nearest tf32 (10 mantissa bits), ties away from zero
                u = (u + 0x1000u) & 0xFFFFE000u;
                memcpy(&out[base + off], &u, 4);
            }
        }
}

// Column length, its factors H1 x H2, columns per group, and the operand layouts' LBO per path: BF16x3
// packed (128: its transposing hand-overs store MN-major operands, the others whole 16-byte rows),
// TF32 padded (144: its transposing hand-overs store 4-byte values into K-major operands, and 16 bytes
// between K-adjacent core matrices spread a warp's stores over the banks) where that fits.
struct ShapeInfo {
    int H, H1, H2, CT, LBO_X3, LBO_TF32;
};
constexpr ShapeInfo SHAPES[] = {{4096, 64, 64, 2, 128, 128}, {2048, 64, 32, 4, 128, 128},
                                {1024, 32, 32, 4, 128, 144}, {512, 32, 16, 8, 128, 144},
                                {256, 16, 16, 8, 128, 144}};

const ShapeInfo* shape_for(int H) {
    for (const auto& s : SHAPES)
        if (s.H == H) return &s;
    return nullptr;
}

template <class S>
bool launch_shape(const void* fm, const DevWorld* worlds, const ColItem* groups, int ngroups, const float2* tw,
                  int* err, cudaStream_t st, int reserve_sms) {
    static int attr = 0;
    if (!attr) {
        // the whole shared-memory carveout: two CTAs of these shapes fit an SM, and with the default
        // carveout the occupancy query answered one (measured at 1024: 4 warps per SM)
        if (cudaFuncSetAttribute(col_pass_tc<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM) != cudaSuccess ||
            cudaFuncSetAttribute(col_pass_tc<S>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return false;
        attr = 1;
    }
    if (ngroups <= 0) return true;
    // CTAs per SM from the SM's shared memory and registers (the occupancy query answered one where
    // two fit, and so left half the SMs' slots empty), and TMEM: co-resident CTAs share 512 columns.
    // The grid is persistent over the groups, so a CTA that does not find room simply starts later.
    static int per_sm = 0, sms = 0;
    if (!per_sm) {
        int dev = 0, smem_sm = 0, regs_sm = 0, reserved = 0;
        cudaFuncAttributes fa;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, col_pass_tc<S>) != cudaSuccess)
            return false;
        int n = smem_sm / (S::SMEM + reserved);
        const int by_regs = regs_sm / (S::NT * (fa.numRegs > 0 ? fa.numRegs : 255));
        if (by_regs < n) n = by_regs;
        if (n * S::TCOLS > 512) n = 512 / S::TCOLS;
        per_sm = n < 1 ? 1 : n;
    }
    int grid = (sms - reserve_sms) * per_sm;
    if (grid > ngroups) grid = ngroups;
    if (grid < 1) grid = 1;
    col_pass_tc<S><<<grid, S::NT, S::SMEM, st>>>(worlds, groups, ngroups, (const uint8_t*)fm, tw, err);
    return true;
}

}  // namespace

int tc_columns_per_group(int H) {
    const ShapeInfo* s = shape_for(H);
    return s ? s->CT : 0;
}

int tc_setup(TcPlan& plan, int path, std::string* err) {
    (void)err;
    plan.path = path;
    plan.ready = 1;
    if (!plan.d_err) {
        if (cudaMalloc(&plan.d_err, CTL_WORDS * sizeof(int)) != cudaSuccess) {
            if (err) *err = "tensor-core control words allocation failed";
            return LENIA_ENOMEM;
        }
        if (cudaMemset(plan.d_err, 0, CTL_WORDS * sizeof(int)) != cudaSuccess) {
            if (err) *err = "tensor-core control words initialisation failed";
            return LENIA_ECUDA;
        }
    }
    return 0;
}

int tc_prepare_size(TcPlan& plan, int path, int H, std::string* err) {
    const ShapeInfo* s = shape_for(H);
    if (!s) return 0;  // served by the FP32 column pass
    for (int i = 0; i < plan.nsizes; i++)
        if (plan.sizes[i] == H) return 0;
    if (plan.nsizes >= 16) {
        if (err) *err = "too many tensor-core sizes";
        return LENIA_EINVAL;
    }
    const bool x3 = path == LENIA_PATH_BF16X3;
    std::vector<uint8_t> host;
    const int lbo = x3 ? s->LBO_X3 : s->LBO_TF32;
    build_dft_operand(s->H2, x3, host, lbo);                  // F_H2 (hi, lo)
    if (s->H1 != s->H2) build_dft_operand(s->H1, x3, host, lbo);  // F_H1 (hi, lo)
    void* d = nullptr;
    if (cudaMalloc(&d, host.size()) != cudaSuccess ||
        cudaMemcpy(d, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        if (d) cudaFree(d);
        if (err) *err = "DFT matrix upload failed";
        return LENIA_ECUDA;
    }
    plan.mats[plan.nsizes] = d;
    plan.sizes[plan.nsizes] = H;
    plan.nsizes++;
    return 0;
}

bool tc_supports(int H) { return shape_for(H) != nullptr; }

bool launch_col_tc(const TcPlan& plan, int path, int H, int variant, const DevWorld* worlds, const ColItem* groups,
                   int ngroups, const float2* tw, cudaStream_t s, int reserve_sms) {
    const void* fm = nullptr;
    for (int i = 0; i < plan.nsizes; i++)
        if (plan.sizes[i] == H) fm = plan.mats[i];
    if (!fm) return false;
    const bool x3 = path == LENIA_PATH_BF16X3;
    int* e = (int*)plan.d_err;
    switch (H) {
    case 4096: return launch_col_tc64(x3, fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
    case 2048: return x3 ? launch_shape<TcShape<64, 32, 4, true, 128, 2, 1>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms)
                         : launch_shape<TcShape<64, 32, 4, false, 128, 2, 1>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
    case 1024:
        if (x3)
            return variant == 1 ? launch_shape<TcShape<32, 32, 4, true, 128, 1, 4, false>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms)
                                : launch_shape<TcShape<32, 32, 4, true, 128, 1, 2>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
        return launch_shape<TcShape<32, 32, 4, false, 144, 1, 1>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
    case 512:
        if (x3)
            return variant == 1 ? launch_shape<TcShape<32, 16, 8, true, 128, 1, 3, false>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms)
                                : launch_shape<TcShape<32, 16, 8, true, 128, 1, 2>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
        return launch_shape<TcShape<32, 16, 8, false, 144, 1, 1>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
    case 256:
        if (x3)
            return variant == 1 ? launch_shape<TcShape<16, 16, 8, true, 128, 1, 4, false>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms)
                                : launch_shape<TcShape<16, 16, 8, true, 128, 1, 2>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
        return launch_shape<TcShape<16, 16, 8, false, 144, 1, 1>>(fm, worlds, groups, ngroups, tw, e, s, reserve_sms);
    }
    return false;
}

int tc_check_error(TcPlan& plan, std::string* err) {
    if (!plan.d_err) return 0;
    int h = 0;
    if (cudaMemcpy(&h, (int*)plan.d_err + CTL_ERR, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return LENIA_ECUDA;
    if (h) {
        cudaMemset((int*)plan.d_err + CTL_ERR, 0, sizeof(int));
        if (err) *err = "a tensor-core column pass gave up waiting on a barrier; results of that step are invalid";
        return LENIA_ECUDA;
    }
    return 0;
}

int tc_set_wait_limit(TcPlan& plan, int limit_plus_one, std::string* err) {
    if (!plan.d_err) {
        if (err) *err = "the context has no tensor-core pass";
        return LENIA_ESTATE;
    }
    if (cudaMemcpy((int*)plan.d_err + CTL_F_POLLS, &limit_plus_one, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
        if (err) *err = "tensor-core control word update failed";
        return LENIA_ECUDA;
    }
    return 0;
}

void tc_release(TcPlan& plan) {
    for (int i = 0; i < plan.nsizes; i++) cudaFree(plan.mats[i]);
    plan.nsizes = 0;
    tc_row_release(plan);
    if (plan.d_err) cudaFree(plan.d_err);
    plan.d_err = nullptr;
    plan.ready = 0;
}

}  // namespace lenia

// ------------------------------------------------------------------ GEMM self-test
namespace lenia {

// amn: A in the MN-major layout (mnmajor_offset, BF16x3 only), as the transposing hand-overs store it;
// else K-major.  The A area is followed by `pad` zeroed bytes, so that a misread descriptor stays in
// the CTA's shared memory.
template <bool X3, bool AMN>
__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                                             int n, int k, int pad, float* d, int* err) {
    extern __shared__ __align__(128) uint8_t smem[];
    constexpr int E = X3 ? 2 : 4, NOP = X3 ? 2 : 1;
    const int abytes = 128 * k * E, bbytes = n * k * E;
    uint8_t* sb = smem;
    uint8_t* sa = smem + bbytes * NOP;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sa + abytes * NOP + pad);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid * 16; i < abytes * NOP; i += 128 * 16) *reinterpret_cast<uint4*>(sa + i) = *reinterpret_cast<const uint4*>(a + i);
    for (int i = tid * 16; i < pad; i += 128 * 16) *reinterpret_cast<uint4*>(sa + abytes * NOP + i) = make_uint4(0, 0, 0, 0);
    for (int i = tid * 16; i < bbytes * NOP; i += 128 * 16) *reinterpret_cast<uint4*>(sb + i) = *reinterpret_cast<const uint4*>(b + i);
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(slot, 256);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t t = *slot;
    if (tid == 0) {
        if (AMN)
            issue_gemm_amn<128>(t, smem_u32(sa), abytes, 128, k, smem_u32(sb), bbytes, k, n, instr_desc(1, 128, n, true));
        else
            issue_gemm<X3>(t, smem_u32(sa), abytes, 128, k, smem_u32(sb), bbytes, n, instr_desc(X3 ? 1 : 2, 128, n));
        mma_commit(bar);
    }
    const bool ok = !__syncthreads_or(!mbar_wait(bar, 0));
    tc_fence_after();
    if (!ok && tid == 0) {
        mbar_wait(bar, 0);  // the MMAs still in flight write TMEM: wait for them (bounded) before freeing it
        atomicExch(err, 1);
    }
    for (int q = 0; q < n / 32 && ok; q++) {
        float v[32];
        tmem_ld32(t + ((uint32_t)(warp * 32) << 16) + 32 * q, v);
        for (int j = 0; j < 32; j++) d[(size_t)tid * n + 32 * q + j] = v[j];
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(t, 256);
    }
}

namespace {
void pack_operand(const float* m, int rows, int k, bool x3, bool mn, std::vector<uint8_t>& out) {
    const int E = x3 ? 2 : 4;
    const size_t bytes = (size_t)rows * k * E;
    out.assign(bytes * (x3 ? 2 : 1), 0);
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < k; c++) {
            const float v = m[(size_t)r * k + c];
            const uint32_t off = mn ? mnmajor_offset(r, c, rows) : kmajor_offset(r, c, k, E);
            if (x3) {
                const __nv_bfloat16 hi = __float2bfloat16_rn(v);
                const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
                *reinterpret_cast<__nv_bfloat16*>(&out[off]) = hi;
                *reinterpret_cast<__nv_bfloat16*>(&out[bytes + off]) = lo;
            } else {
                uint32_t u;
                memcpy(&u, &v, 4);
                u = (u + 0x1000u) & 0xFFFFE000u;
                memcpy(&out[off], &u, 4);
            }
        }
}
}  // namespace

int tc_selftest(int path, int n, int k, const float* a, const float* b, float* d, std::string* err) {
    const bool amn = (path & LENIA_SELFTEST_A_MN) != 0;
    path &= ~LENIA_SELFTEST_A_MN;
    const bool x3 = path == LENIA_PATH_BF16X3;
    if ((path != LENIA_PATH_TF32 && !x3) || n < 32 || n > 256 || n % 32 || k < 16 || k > 256 || k % 16 ||
        (amn && (!x3 || k > 64))) {
        if (err) *err = "selftest: path must be TF32 or BF16X3, n in 32..256 (multiple of 32), k in 16..256 (multiple "
                        "of 16); an MN-major A needs BF16X3 and k <= 64";
        return LENIA_EINVAL;
    }
    std::vector<uint8_t> ha, hb;
    pack_operand(a, 128, k, x3, amn, ha);
    pack_operand(b, n, k, x3, false, hb);
    uint8_t *da = nullptr, *db = nullptr;
    float* dd = nullptr;
    int* de = nullptr;
    int rc = 0;
    const int pad = amn ? 64 * 1024 : 0;
    const size_t smem = ha.size() + hb.size() + pad + 64;
    if (cudaMalloc(&da, ha.size()) || cudaMalloc(&db, hb.size()) || cudaMalloc(&dd, (size_t)128 * n * 4) ||
        cudaMalloc(&de, 4)) {
        rc = LENIA_ENOMEM;
    } else {
        cudaMemcpy(da, ha.data(), ha.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(db, hb.data(), hb.size(), cudaMemcpyHostToDevice);
        cudaMemset(de, 0, 4);
        cudaMemset(dd, 0, (size_t)128 * n * 4);
        cudaError_t e;
        if (amn) {
            cudaFuncSetAttribute(tc_selftest_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            tc_selftest_kernel<true, true><<<1, 128, smem>>>(da, db, n, k, pad, dd, de);
        } else if (x3) {
            cudaFuncSetAttribute(tc_selftest_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            tc_selftest_kernel<true, false><<<1, 128, smem>>>(da, db, n, k, pad, dd, de);
        } else {
            cudaFuncSetAttribute(tc_selftest_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            tc_selftest_kernel<false, false><<<1, 128, smem>>>(da, db, n, k, pad, dd, de);
        }
        e = cudaDeviceSynchronize();
        int h = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&h, de, 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(d, dd, (size_t)128 * n * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            rc = LENIA_ECUDA;
            if (err) *err = std::string("selftest: ") + cudaGetErrorString(e);
        } else if (h) {
            rc = LENIA_ECUDA;
            if (err) *err = "selftest: MMA completion wait timed out";
        }
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(de);
    return rc;
}

}  // namespace lenia
