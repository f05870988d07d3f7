// Fused FP32 Lenia step on the CUDA cores: two launches per step.
//
// The reference's step is 4*log2(n)+5 full-grid dispatches (spectral.rs:199-264): load, log2 W
// x-stages, log2 H y-stages, spectrum copy, and per kernel multiply, inverse y, inverse x,
// convolved, then update.  Here the same mathematics is regrouped so that each grid sweep
// does as much as it can in shared memory:
//
//   column pass (per world, channel, tile of TC = 2 spectrum columns, kernel k reading it):
//       forward FFT along y  ->  x khat_k (real, even; includes 1/(W*H))  ->  inverse FFT along y
//   row pass (per world, block of 4 rows; Lenia: and target channel):
//       inverse real FFT along x of U_k  ->  growth, dt, clamp (spectral.rs:337-345)  ->
//       write state  ->  forward real FFT along x of the new rows  ->  write spectrum
//
// so one step reads and writes the half-spectrum twice and the state once.  Two real rows
// share one complex FFT (z = a + i b), and the real DC and Nyquist columns share spectrum
// column 0, so the half-spectrum takes exactly W*H*4 bytes per channel.
//
// The column pass is built twice: scalar (col_pass: a thread runs a butterfly of one column) and
// paired (col_pass_pair: a thread runs the same butterfly of both columns of the tile as f32x2
// pairs, half the threads and instructions); launch variant 2 selects the paired build.
#pragma once
#include <cuda_runtime.h>

#include "cache_hints.cuh"
#include "engine.cuh"
#include "fft_core.cuh"
#include "tc_ptx.cuh"

namespace lenia {
using namespace lfft;

// 16-byte asynchronous global -> shared copy: nothing is held in registers while it is in flight.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// f(Int<I>()) for I = 0..N-1, so that I (decltype(i)::value) can be a template argument.
template <int I>
struct Int {
    static constexpr int value = I;
    __host__ __device__ constexpr operator int() const { return I; }
};
template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
    if constexpr (I < N) {
        f(Int<I>());
        static_for<I + 1, N>(f);
    }
}

// Stages [I, I1) of the transform of S sequences of length N in shared memory (stride
// seq_stride(N)), in place, by NT threads; stw holds the per-stage twiddle tables
// (fill_stage_twiddles).  Starts after the caller's barrier; ends with a barrier.
// MR: the plan's radix cap (make_plan); 16 for every pass but the scalar column pass.
template <int N, int S, int NT, bool INV, int I, int I1, int MR = 16, class T, class W>
__device__ __forceinline__ void fft_stages(T* buf, const W* stw) {
    static_assert(MR == 32 || MR == max_radix<T>(), "radix-32 plans are built for scalar elements only");
    if constexpr (I < I1) {
        constexpr int R = plan_radix(N, I, MR);
        constexpr int L = plan_L(N, I, MR);
        constexpr int NB = N / R;
        constexpr int TOT = NB * S;
        constexpr int PER = (TOT + NT - 1) / NT;
        constexpr int SEQ = seq_stride(N);
        T v[PER][R];
#pragma unroll
        for (int p = 0; p < PER; p++) {
            const int b = threadIdx.x + p * NT;
            if ((TOT % NT) == 0 || b < TOT) {
                const int s = b / NB, j = b - s * NB;
                stage_load<N, R, L, INV>(buf + s * SEQ, j, v[p], stw + stage_tw_offset(N, I, MR));
            }
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < PER; p++) {
            const int b = threadIdx.x + p * NT;
            if ((TOT % NT) == 0 || b < TOT) {
                const int s = b / NB, j = b - s * NB;
                stage_store<N, R, L>(buf + s * SEQ, j, v[p]);
            }
        }
        __syncthreads();
        fft_stages<N, S, NT, INV, I + 1, I1, MR>(buf, stw);
    }
}

template <int N, int S, int NT, bool INV, int MR = 16, class T, class W>
__device__ __forceinline__ void fft_seqs(T* buf, const W* stw) {
    fft_stages<N, S, NT, INV, 0, plan_len(N, MR), MR>(buf, stw);
}

// Two transforms back to back (A, then B) with work on the values in between.  When the plan's
// first and last radix are equal, the last stage of A leaves butterfly j holding the elements
// j + m*N/R (m < R) in natural order -- exactly the inputs of butterfly j of B's first stage.  So
// `mid(s, j, v)` runs on those registers (sequence s, elements j + m*N/R) and B's first stage
// follows without a round trip through shared memory: two barriers and one shared-memory
// read/write sweep fewer than A, mid-pass, B.  `pre(s, j)` runs just before the last stage of A.
template <int N, int MR = 16>
FFT_CHD constexpr bool fusable() {
    return plan_len(N, MR) >= 2 && plan_radix(N, 0, MR) == plan_radix(N, plan_len(N, MR) - 1, MR);
}

struct NoPre {
    __device__ void operator()(int, int) const {}
};

template <int N, int S, int NT, bool INV_A, bool INV_B, int MR = 16, class T, class W, class Mid, class Pre = NoPre>
__device__ __forceinline__ void fft_fused(T* buf, const W* stw, Mid mid, Pre pre = Pre()) {
    constexpr int LAST = plan_len(N, MR) - 1;
    constexpr int R = plan_radix(N, LAST, MR), L = plan_L(N, LAST, MR), NB = N / R;
    static_assert(L == NB && plan_radix(N, 0, MR) == R, "fusable plans only");
    constexpr int TOT = NB * S, PER = (TOT + NT - 1) / NT, SEQ = seq_stride(N);
    fft_stages<N, S, NT, INV_A, 0, LAST, MR>(buf, stw);
    T v[PER][R];
#pragma unroll
    for (int p = 0; p < PER; p++) {
        const int b = threadIdx.x + p * NT;
        if ((TOT % NT) == 0 || b < TOT) {
            const int s = b / NB, j = b - s * NB;
            pre(s, j);  // global loads that mid needs, issued before the last stage of A
            stage_load<N, R, L, INV_A>(buf + s * SEQ, j, v[p], stw + stage_tw_offset(N, LAST, MR));
            mid(s, j, v[p]);
            Dft<R, INV_B>::run(v[p]);  // B's first stage: L = 1, no twiddle
        }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PER; p++) {
        const int b = threadIdx.x + p * NT;
        if ((TOT % NT) == 0 || b < TOT) stage_store<N, R, 1>(buf + (b / NB) * SEQ, b % NB, v[p]);
    }
    __syncthreads();
    fft_stages<N, S, NT, INV_B, 1, plan_len(N, MR), MR>(buf, stw);
}

// Shared memory of a pass: the sequences, then (float2-aligned) the stage twiddle tables.
template <int N, int MR = 16>
constexpr size_t stage_table_bytes() { return (size_t)(tw_table_size(N, MR) + 1) * sizeof(float2); }

// The scalar column pass's radix cap: radix-32 plans where they save a stage (1024 = 32.32 against
// 16.4.16: one shared-memory round trip fewer per transform; 3072, 8192), the radix-16 plan elsewhere.
// The column item holds its 32 elements a thread in registers between stages; the row pass, which also
// holds the state values of its rows there, keeps radix 16.
constexpr int CMR = 32;

// Column pass, fused form: after the stage tables (16-byte aligned), the tile's TC khat columns.
template <int H>
FFT_CHD constexpr int khat_cols_stride() { return (H / 2 + 1 + 3) / 4 * 4; }
template <int H>
constexpr size_t col_khat_bytes() { return fusable<H, CMR>() ? (size_t)TC * khat_cols_stride<H>() * sizeof(float) : 0; }
template <int H, int MR = CMR>
__device__ __forceinline__ float* col_khat_smem(float2* stw) {
    constexpr int TWS = tw_table_size(H, MR);
    return reinterpret_cast<float*>(((uintptr_t)(stw + TWS) + 15) & ~(uintptr_t)15);
}

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// Gaussian growth mapped to [-1, 1] (spectral.rs:341-344): 2 exp(-d^2/2) - 1, d = (u - mu)/sigma.
// Evaluated as 2 * 2^(-e^2) - 1 with e = u*k - mu*k, k = sqrt(log2(e)/2)/sigma: one FMA, one
// multiply, the hardware base-2 exponential (ex2.approx.ftz: a value below 2^-126 flushes to 0,
// which changes nothing because 2*2^(-e^2) - 1 then rounds to -1 either way) and one FMA.  Within
// 4e-7 of the direct form at the reference's parameters.
struct Growth {
    float k, mk;
    __device__ __forceinline__ Growth(float mu, float sigma) {
        k = 0.84932180028801904f / sigma;
        mk = mu * k;
    }
    __device__ __forceinline__ float operator()(float u) const {
        const float e = fmaf(u, k, -mk);
        float p;
        asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(p) : "f"(-e * e));
        return fmaf(2.0f, p, -1.0f);
    }
};

// 1 / (1 + e^(x k)) for a compile-time k, with the hardware base-2 exponential and reciprocal (one
// multiply, ex2, add, rcp).  A large x overflows e^(x k) to +inf, whose reciprocal is the 0 the
// logistic tends to; a value below 2^-126 flushes to 0 and the result rounds to 1 either way.
__device__ __forceinline__ float logistic_neg(float x, float k_log2e) {
    float e, r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x * k_log2e));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
    return r;
}

// SmoothLife update (spectral.rs:396-407): three logistic steps of width 4/AM and 4/AN.
__device__ __forceinline__ float smoothlife_update(float s, float c0, float c1) {
    const float B1 = 0.278f, B2 = 0.365f, D1 = 0.267f, D2 = 0.445f, DT = 0.1f;
    const float KM = 39.257007915345945f, KN = 206.09929155556621f;  // (4 / AM) log2(e), (4 / AN) log2(e)
    const float m = logistic_neg(0.5f - c0, KM);
    const float lo = B1 * (1.0f - m) + D1 * m, hi = B2 * (1.0f - m) + D2 * m;
    const float target = logistic_neg(lo - c1, KN) * (1.0f - logistic_neg(hi - c1, KN));
    return clamp01(s + DT * (2.0f * target - 1.0f));
}

// MNCA update (spectral.rs:461-472).
__device__ __forceinline__ float mnca_update(float s, float c0, float c1) {
    float o = s;
    if (c0 >= 0.210f && c0 <= 0.220f) o = 1.0f;
    if (c0 >= 0.350f && c0 <= 0.500f) o = 0.0f;
    if (c0 >= 0.750f && c0 <= 0.850f) o = 0.0f;
    if (c0 >= 0.120f && c0 <= 0.150f) o = 0.0f;
    if (c1 >= 0.100f && c1 <= 0.280f) o = 0.0f;
    if (c1 >= 0.430f && c1 <= 0.550f) o = 1.0f;
    return o;
}

// ---------------------------------------------------------------------------- row pass
//
// One CTA per item of 2S rows (S packed sequences, row pairs).  The single-kernel step uses S = 4 up to
// 1024 wide: an item then reads and writes each tile's spectrum as 128 contiguous bytes (8 rows x 16
// B) instead of 64, and on the 384-world batched workload the row pass went from 189 to 166 us a
// generation for the 1024 x 1024 class (512: 41 -> 34 us), the step from 1.75e11 to 1.87e11 cell-updates/s.
// Wider rows keep S = 2: measured at 4096 x 4096, S = 4 (1024 threads, one CTA per SM) was 10% slower
// (row pass 76 against 68 us) and S = 1 (256 threads, three or four CTAs per SM) 5-30% slower than
// S = 2 (512 threads, two CTAs per SM).  The general step keeps a plane of W x 2S floats besides
// the sequences; from W = 2048 up it uses S = 1 (at S = 2 a 4096-wide item needed 138 KB of shared
// memory, one CTA per SM; MNCA at 4096 x 4096 measured 7% faster at S = 1), up to 1024 wide S = 4 (the
// 3-channel 1024 x 1024 world: 5.97e10 -> 6.33e10 channel-cell updates/s from S = 2, and 5% slower at
// S = 1 than at S = 2), in between S = 2.
// Threads of a row item of S sequences of length N: one first-stage butterfly per thread; for sides
// 3 * 2^k at least one per four radix-3 butterflies as well.  768 = 16.3.16 with 192 threads for four
// sequences ran its radix-3 stage in six rounds, the last a third full, and needed 128 registers a
// thread; with 256 it fits 64, and the batched workload's 768 x 768 row pass went from 104 to 89 us a
// generation (the step from 1.87e11 to 1.93e11 cell-updates/s).
FFT_CHD constexpr int seq_threads(int N, int S) {
    return N % 3 == 0 && S * N / 12 > S * N / plan_radix(N, 0) ? S * N / 12 : S * N / plan_radix(N, 0);
}
FFT_CHD constexpr int row_seqs(int W, bool gen) { return gen ? (W >= 2048 ? 1 : (W <= 1024 ? 4 : 2)) : (W <= 1024 ? 4 : 2); }
template <int W, bool GEN>
constexpr int row_nt() {
    constexpr int n = seq_threads(W, row_seqs(W, GEN));
    return n < 64 ? 64 : (n > 1024 ? 1024 : n);
}
// variant 0: at most 1024 threads' worth of registers per SM (64 a thread at 512 threads);
// variant 1: at most 128 a thread
template <int W, int V, bool GEN>
constexpr int row_minb() {
    constexpr int t = V == 0 ? 1024 : 512;
    return t / row_nt<W, GEN>() < 1 ? 1 : t / row_nt<W, GEN>();
}
// Shared memory after the sequences and stage tables: the accumulation planes ([planes][2S][W]) of
// the general path.
template <int W>
__device__ __forceinline__ float* row_extra_smem(float2* stw) {
    constexpr int TWS = tw_table_size(W);
    return reinterpret_cast<float*>(((uintptr_t)(stw + TWS) + 15) & ~(uintptr_t)15);
}

// Half-spectra of rows r0..r0+2S-1 (tile layout) -> S packed complex sequences
// Z_p = A + iB with A = row r0+2p, B = row r0+2p+1, using Hermitian symmetry for k > W/2.
// One element per lane and column, consecutive lanes on consecutive columns: the shared-memory
// writes of a warp are contiguous (a tile per lane, with both its columns, would write at
// stride 2 and conflict; measured 4% slower at 4096 x 4096).
template <int W, int S, int NT, bool CG = false>
__device__ __forceinline__ void load_rows_spectrum(float2* Z, const float2* __restrict__ sp, int H, int r0) {
    constexpr int SEQ = seq_stride(W);
    constexpr int E = W / 2 * S, IT = (E + NT - 1) / NT;
    float2 A[IT], B[IT];
#pragma unroll
    for (int i = 0; i < IT; i++) {
        const int e = threadIdx.x + i * NT;
        if (IT * NT == E || e < E) {
            const int t = e / (S * TC), p = (e / TC) % S, c = e % TC;
            const float2* src = sp + ((size_t)t * H + r0 + 2 * p) * TC + c;
            const uint64_t keep = hint::policy_keep();
            A[i] = hint::ld2c<CG>(src, keep);
            B[i] = hint::ld2c<CG>(src + TC, keep);
        }
    }
    // When every iteration moves kx by the same multiple of 16 (D), the padded positions of kx and
    // W - kx move by D + D/16: two base pointers and compile-time offsets.
    constexpr int D = NT / S;
    constexpr bool STEP = NT % (S * TC) == 0 && D % 16 == 0;
    const int kx0 = TC * (threadIdx.x / (S * TC)) + threadIdx.x % TC, p0 = (threadIdx.x / TC) % S;
    float2* za = Z + p0 * SEQ + pad(kx0);
    float2* zb = Z + p0 * SEQ + pad(W - kx0);
#pragma unroll
    for (int i = 0; i < IT; i++) {
        const int e = threadIdx.x + i * NT;
        if (IT * NT == E || e < E) {
            const int t = e / (S * TC), p = (e / TC) % S, c = e % TC, kx = TC * t + c;
            float2* z = Z + p * SEQ;
            if (kx == 0) {
                z[pad(0)] = make_float2(A[i].x, B[i].x);
                z[pad(W / 2)] = make_float2(A[i].y, B[i].y);
            } else if constexpr (STEP) {
                za[i * (D + D / 16)] = make_float2(A[i].x - B[i].y, A[i].y + B[i].x);
                zb[-i * (D + D / 16)] = make_float2(A[i].x + B[i].y, B[i].x - A[i].y);
            } else {
                z[pad(kx)] = make_float2(A[i].x - B[i].y, A[i].y + B[i].x);
                z[pad(W - kx)] = make_float2(A[i].x + B[i].y, B[i].x - A[i].y);
            }
        }
    }
}

// S packed complex spectra Z_p = FFT(a + ib) -> half-spectra of rows r0+2p (A) and r0+2p+1 (B).
template <int W, int S, int NT>
__device__ __forceinline__ void store_rows_spectrum(const float2* Z, float2* __restrict__ sp, int H, int r0) {
    constexpr int SEQ = seq_stride(W);
    constexpr int E = W / 2 * S;
    // as in load_rows_spectrum: the padded positions of kx and W - kx move by a constant
    constexpr int D = NT / S;
    constexpr bool STEP = NT % (S * TC) == 0 && D % 16 == 0;
    const int kx0 = TC * (threadIdx.x / (S * TC)) + threadIdx.x % TC, p0 = (threadIdx.x / TC) % S;
    const float2* za = Z + p0 * SEQ + pad(kx0);
    const float2* zb = Z + p0 * SEQ + pad(W - kx0);
    for (int e = threadIdx.x; e < E; e += NT, za += STEP ? D + D / 16 : 0, zb -= STEP ? D + D / 16 : 0) {
        const int t = e / (S * TC), p = (e / TC) % S, c = e % TC, kx = TC * t + c;
        const float2* z = Z + p * SEQ;
        float2 A, B;
        if (kx == 0) {
            const float2 z0 = z[pad(0)], zn = z[pad(W / 2)];
            A = make_float2(z0.x, zn.x);
            B = make_float2(z0.y, zn.y);
        } else {
            const float2 a = STEP ? *za : z[pad(kx)], b = STEP ? *zb : z[pad(W - kx)];
            A = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
            B = make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x));
        }
        float2* dst = sp + ((size_t)t * H + r0 + 2 * p) * TC + c;
        const uint64_t keep = hint::policy_keep();
        hint::st2(dst, A, keep);
        hint::st2(dst + TC, B, keep);
    }
}

// Row-pass modes that run outside the step (after state writes, and for U-field reads).  Not
// inlined, so that their registers do not add to the step path's.
template <int W, int NT, int S>
__device__ __noinline__ void row_item_forward(float2* Z, const float2* stw, const DevWorld& wd, int r0, int d0, int d1) {
    constexpr int SEQ = seq_stride(W);
    const int H = wd.H;
    const size_t plane = (size_t)W * H, cplane = (size_t)(W / 2) * H;
    for (int d = d0; d < d1; d++) {
        const float* st = wd.state + d * plane + (size_t)r0 * W;
        constexpr int IT = (S * W + NT - 1) / NT;
        float a[IT], b[IT];
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const int e = threadIdx.x + i * NT, p = e / W, x = e - p * W;
            if (IT * NT == S * W || e < S * W) {
                a[i] = st[(2 * p) * W + x];
                b[i] = st[(2 * p + 1) * W + x];
            }
        }
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const int e = threadIdx.x + i * NT, p = e / W, x = e - p * W;
            if (IT * NT == S * W || e < S * W) Z[p * SEQ + pad(x)] = make_float2(a[i], b[i]);
        }
        __syncthreads();
        fft_seqs<W, S, NT, false>(Z, stw);
        store_rows_spectrum<W, S, NT>(Z, wd.spec + d * cplane, H, r0);
        __syncthreads();
    }
}

template <int W, int NT, int S>
__device__ __noinline__ void row_item_u(float2* Z, const float2* stw, const DevWorld& wd, int r0, int d0, bool per_chan) {
    constexpr int SEQ = seq_stride(W);
    const int H = wd.H, K = wd.K;
    const size_t plane = (size_t)W * H, cplane = (size_t)(W / 2) * H;
    for (int k = 0; k < K; k++) {
        if (per_chan && wd.kern[k].dst != d0) continue;
        load_rows_spectrum<W, S, NT>(Z, wd.conv + k * cplane, H, r0);
        __syncthreads();
        fft_seqs<W, S, NT, true>(Z, stw);
        float* u = wd.u_out + k * plane + (size_t)r0 * W;
        for (int e = threadIdx.x; e < S * W; e += NT) {
            const int p = e / W, x = e - p * W;
            const float2 z = Z[p * SEQ + pad(x)];
            u[(2 * p) * W + x] = z.x;
            u[(2 * p + 1) * W + x] = z.y;
        }
        __syncthreads();
    }
}

// The one-channel, one-kernel Lenia row step of rows r0..r0+3 of world wd: inverse row FFT of U, growth,
// dt update and clamp against the state, forward row FFT of the new rows.  Z: the two packed
// sequences, stw: the stage tables.  CG: spectrum and state loads bypass L1 (the persistent step,
// where another CTA of the same launch wrote them).
template <int W, int NT, bool CG>
__device__ __forceinline__ void row_item_simple(const DevWorld& wd, int r0, float2* Z, const float2* stw) {
    constexpr int S = row_seqs(W, false), ROWS = 2 * S;
    const int H = wd.H;
    const DevKernel kp = wd.kern[0];
    const float dtw = wd.dt * kp.weight;
    const Growth growth(kp.mu, kp.sigma);
    float* st = wd.state + (size_t)r0 * W;
    const uint64_t stream = hint::policy_stream();
    // The growth update runs in registers between the inverse and the forward row FFT (every
    // built width has a plan with equal first and last radix).  The item's state rows are
    // pulled into L2 when the CTA starts, and each thread's 2 x R state values are loaded into
    // registers just before the last inverse stage.
    static_assert(fusable<W>(), "row widths need a plan with equal first and last radix");
    constexpr int R = plan_radix(W, 0), NB = W / R;
    static_assert(S * NB <= NT, "one butterfly per thread in the fused stage");
    if (threadIdx.x == 0) tc::bulk_prefetch_l2(st, ROWS * W * (uint32_t)sizeof(float));
    load_rows_spectrum<W, S, NT, CG>(Z, wd.conv, H, r0);
    __syncthreads();
    float sa[R], sb[R];
    fft_fused<W, S, NT, true, false>(
        Z, stw,
        [&](int s, int j, float2* v) {
            float* ga = st + (2 * s) * W + j;
            static_for<0, R>([&](auto m) {
                const float n0 = __saturatef(fmaf(dtw, growth(v[m].x), sa[m]));
                const float n1 = __saturatef(fmaf(dtw, growth(v[m].y), sb[m]));
                hint::st1_at<decltype(m)::value * NB * 4>(ga, n0, stream);
                hint::st1_at<(W + decltype(m)::value * NB) * 4>(ga, n1, stream);
                v[m] = make_float2(n0, n1);
            });
        },
        [&](int s, int j) {
            const float* ga = st + (2 * s) * W + j;
            static_for<0, R>([&](auto m) {
                sa[m] = hint::ld1_atc<decltype(m)::value * NB * 4, CG>(ga, stream);
                sb[m] = hint::ld1_atc<(W + decltype(m)::value * NB) * 4, CG>(ga, stream);
            });
        });
    store_rows_spectrum<W, S, NT>(Z, wd.spec, H, r0);
}

// GEN: the instantiation for size classes with worlds that need the general step (several
// channels or kernels, SmoothLife, MNCA).  Without it the kernel carries only the one-channel,
// one-kernel Lenia step (and the forward and U modes), so the general path's register pressure
// does not set the budget of the common path.
template <int W, int NT, int MINB, bool GEN>
__global__ void __launch_bounds__(NT, MINB) row_pass(const DevWorld* __restrict__ worlds, const RowItem* __restrict__ items,
                                                int mode, int general, const float2* __restrict__ tw) {
    constexpr int S = row_seqs(W, GEN), ROWS = 2 * S;
    extern __shared__ float4 smem_raw[];
    constexpr int SEQ = seq_stride(W);
    float2* Z = reinterpret_cast<float2*>(smem_raw);
    float2* stw = Z + S * SEQ;
    float* extra = row_extra_smem<W>(stw);
    fill_stage_twiddles<W>(stw, tw, threadIdx.x, NT);
    const RowItem it = items[blockIdx.x];
    const DevWorld& wd = worlds[it.world];
    const int H = wd.H, C = wd.C, K = wd.K, r0 = it.row0;
    const size_t plane = (size_t)W * H, cplane = (size_t)(W / 2) * H;
    // Lenia items cover one target channel; SmoothLife and MNCA items every channel
    const bool per_chan = wd.rule == LENIA_RULE_LENIA;
    const int d0 = per_chan ? it.chan : 0, d1 = per_chan ? it.chan + 1 : C;

    if (mode == MODE_FORWARD) {
        row_item_forward<W, NT, S>(Z, stw, wd, r0, d0, d1);
        return;
    }
    if (mode == MODE_U) {
        row_item_u<W, NT, S>(Z, stw, wd, r0, d0, per_chan);
        return;
    }

    if constexpr (!GEN) {
        row_item_simple<W, NT, false>(wd, r0, Z, stw);
        return;
    }

    // General: several channels and/or kernels, or SmoothLife / MNCA (one channel, two kernels); also
    // any one-kernel world that shares a size class with such worlds.
    // Every kernel of the item but the last leaves its result in one shared-memory plane, straight
    // from the registers of its last inverse stage: Lenia adds its weighted growth, SmoothLife and
    // MNCA keep the first kernel's U.  The last kernel runs chained (fft_fused): its last inverse
    // stage, the rule's update with the plane and the state, and the first forward stage stay in
    // registers.  A thread owns the same cells (sequence s, x = j + m*N/R) in all of these stages,
    // so the plane needs no barrier of its own.
    const int rule = wd.rule;
    constexpr int R = plan_radix(W, 0), NB = W / R, LAST = plan_len(W) - 1;
    static_assert(fusable<W>(), "row widths need a plan with equal first and last radix");
    static_assert(S * NB <= NT, "one butterfly per thread in the chained stages");
    float* acc = extra;  // [ROWS][W]
    int nk = 0, klast = -1;
    for (int k = 0; k < K; k++)
        if (!per_chan || wd.kern[k].dst == d0) nk++, klast = k;
    float* st = wd.state + d0 * plane + (size_t)r0 * W;
    if (nk == 0) {
        // no kernel targets this channel: the update is the clamp alone
        for (int e = threadIdx.x; e < ROWS * W; e += NT) st[e] = clamp01(st[e]);
        __syncthreads();
        row_item_forward<W, NT, S>(Z, stw, wd, r0, d0, d0 + 1);
        return;
    }
    if (threadIdx.x == 0) tc::bulk_prefetch_l2(st, ROWS * W * (uint32_t)sizeof(float));
    bool first = true;
    for (int k = 0; k < klast; k++) {
        const DevKernel kp = wd.kern[k];
        if (per_chan && kp.dst != d0) continue;
        const Growth growth(kp.mu, kp.sigma);
        load_rows_spectrum<W, S, NT>(Z, wd.conv + k * cplane, H, r0);
        __syncthreads();
        fft_stages<W, S, NT, true, 0, LAST>(Z, stw);
        if ((int)threadIdx.x < S * NB) {
            const int s = threadIdx.x / NB, j = threadIdx.x - s * NB;
            float2 v[R];
            stage_load<W, R, NB, true>(Z + s * SEQ, j, v, stw + stage_tw_offset(W, LAST));
            float* a = acc + (2 * s) * W + j;
#pragma unroll
            for (int m = 0; m < R; m++) {
                if (rule == LENIA_RULE_LENIA) {
                    const float g0 = kp.weight * growth(v[m].x), g1 = kp.weight * growth(v[m].y);
                    a[m * NB] = first ? g0 : a[m * NB] + g0;
                    a[W + m * NB] = first ? g1 : a[W + m * NB] + g1;
                } else {
                    a[m * NB] = v[m].x;
                    a[W + m * NB] = v[m].y;
                }
            }
        }
        first = false;
        __syncthreads();  // Z is rewritten by the next kernel
    }
    const DevKernel kp = wd.kern[klast];
    const Growth growth(kp.mu, kp.sigma);
    const float dt = wd.dt;
    const bool have_acc = nk > 1;
    const uint64_t stream = hint::policy_stream();
    load_rows_spectrum<W, S, NT>(Z, wd.conv + klast * cplane, H, r0);
    __syncthreads();
    float sa[R], sb[R];
    fft_fused<W, S, NT, true, false>(
        Z, stw,
        [&](int s, int j, float2* v) {
            float* ga = st + (2 * s) * W + j;
            const float* a = acc + (2 * s) * W + j;
#pragma unroll
            for (int m = 0; m < R; m++) {
                float n0, n1;
                if (rule == LENIA_RULE_LENIA) {
                    float t0 = kp.weight * growth(v[m].x), t1 = kp.weight * growth(v[m].y);
                    if (have_acc) t0 = a[m * NB] + t0, t1 = a[W + m * NB] + t1;
                    n0 = clamp01(sa[m] + dt * t0);
                    n1 = clamp01(sb[m] + dt * t1);
                } else if (rule == LENIA_RULE_SMOOTHLIFE) {
                    n0 = smoothlife_update(sa[m], a[m * NB], v[m].x);
                    n1 = smoothlife_update(sb[m], a[W + m * NB], v[m].y);
                } else {
                    n0 = mnca_update(sa[m], a[m * NB], v[m].x);
                    n1 = mnca_update(sb[m], a[W + m * NB], v[m].y);
                }
                hint::st1(ga + m * NB, n0, stream);
                hint::st1(ga + W + m * NB, n1, stream);
                v[m] = make_float2(n0, n1);
            }
        },
        [&](int s, int j) {
            const float* ga = st + (2 * s) * W + j;
#pragma unroll
            for (int m = 0; m < R; m++) {
                sa[m] = hint::ld1(ga + m * NB, stream);
                sb[m] = hint::ld1(ga + W + m * NB, stream);
            }
        });
    store_rows_spectrum<W, S, NT>(Z, wd.spec + d0 * cplane, H, r0);
}

// ---------------------------------------------------------------------------- column pass

// X (TC sequences of length H, forward spectrum of tile `t`) times khat -> T.  Column 0 of
// tile 0 packs the DC column (real part) and the Nyquist column (imaginary part): both are
// real sequences, so with Z = FFT_y(packed), Z' = Z*(K0+KN)/2 + conj(Z[-ky])*(K0-KN)/2.
template <int H, int NT>
__device__ __forceinline__ void multiply_khat(const float2* X, float2* T, const float* __restrict__ kh, int HQ,
                                              int W, int t) {
    constexpr int SEQ = seq_stride(H);
    for (int e = threadIdx.x; e < TC * H; e += NT) {
        const int col = e / H, ky = e - col * H;
        if (t == 0 && col == 0) continue;
        const int kx = TC * t + col;
        const float kv = kh[(size_t)kx * HQ + (ky <= H / 2 ? ky : H - ky)];
        T[col * SEQ + pad(ky)] = cscale(X[col * SEQ + pad(ky)], kv);
    }
    if (t == 0) {
        for (int ky = threadIdx.x; ky <= H / 2; ky += NT) {
            const float K0 = kh[ky], KN = kh[(size_t)(W / 2) * HQ + ky];
            const float a = 0.5f * (K0 + KN), b = 0.5f * (K0 - KN);
            const int km = (H - ky) % H;
            const float2 z = X[pad(ky)], zm = X[pad(km)];
            T[pad(ky)] = make_float2(z.x * a + zm.x * b, z.y * a - zm.y * b);
            if (km != ky) T[pad(km)] = make_float2(zm.x * a + z.x * b, zm.y * a - z.y * b);
        }
    }
}

// One tile (H rows x TC columns, contiguous) <-> TC sequences in shared memory.
template <int H, int NT, bool CG = false>
__device__ __forceinline__ void load_tile(float2* X, const float2* __restrict__ src) {
    static_assert(TC == 2, "tile loads move one float4 (two columns) per row");
    constexpr int SEQ = seq_stride(H);
    constexpr int IT = (H + NT - 1) / NT;
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float4 v[IT];
#pragma unroll
    for (int i = 0; i < IT; i++) {
        const int y = threadIdx.x + i * NT;
        if (IT * NT == H || y < H) v[i] = hint::ld4c<CG>(s4 + y, hint::policy_keep());
    }
    // pad(tid + i NT) = pad(tid) + i (NT + NT / 16) when NT is a multiple of 16
    float2* x0 = X + pad(threadIdx.x);
#pragma unroll
    for (int i = 0; i < IT; i++) {
        const int y = threadIdx.x + i * NT;
        if (IT * NT == H || y < H) {
            float2* x = NT % 16 == 0 ? x0 + i * (NT + NT / 16) : X + pad(y);
            x[0] = make_float2(v[i].x, v[i].y);
            x[SEQ] = make_float2(v[i].z, v[i].w);
        }
    }
}

template <int H, int NT>
__device__ __forceinline__ void store_tile(const float2* X, float2* __restrict__ dst) {
    constexpr int SEQ = seq_stride(H);
    float4* d4 = reinterpret_cast<float4*>(dst);
    const float2* x = X + pad(threadIdx.x);
    for (int y = threadIdx.x; y < H; y += NT, x += NT + NT / 16) {
        if (NT % 16 != 0) x = X + pad(y);
        const float2 a = x[0], b = x[SEQ];
        hint::st4(d4 + y, make_float4(a.x, a.y, b.x, b.y), hint::policy_keep());
    }
}

// Unchained column item: tile 0 (its column 0 packs the DC and Nyquist columns, paired ky with
// H - ky in the khat multiply) or a khat array that is not 16-byte aligned.  Not inlined: one item
// in W/4 takes this path, and as a separate function its registers do not add to the chained path's.
template <int H, int NT, bool CG = false, int MR = CMR>
__device__ __noinline__ void col_item_unchained(float2* X, const float2* stw, const float2* src, float2* dst,
                                                const float* kh, int HQ, int W, int t) {
    load_tile<H, NT, CG>(X, src);
    __syncthreads();
    fft_seqs<H, TC, NT, false, MR>(X, stw);
    multiply_khat<H, NT>(X, X, kh, HQ, W, t);
    __syncthreads();
    fft_seqs<H, TC, NT, true, MR>(X, stw);
    store_tile<H, NT>(X, dst);
}

// One column item: tile `tile` (TC spectrum columns) of channel `chan`, convolved with kernel
// `kernel` (which reads that channel).  A channel read by several kernels has one item per kernel, each
// repeating the channel's forward column transform: that keeps every item on the chained path and
// multiplies the items, which the multichannel world needs more than it needs the saved transforms.
// CG: the tile loads bypass L1 (the persistent step, where another CTA of the same launch wrote them).
template <int H, int NT, bool CG, int MR = CMR>
__device__ __forceinline__ void col_item(const DevWorld& wd, const ColItem it, float2* X, float2* stw) {
    const int W = wd.W, c = it.chan, t = it.tile, k = it.kernel, HQ = wd.HQ;
    const size_t cplane = (size_t)(W / 2) * H;
    const float2* src = wd.spec + c * cplane + (size_t)t * H * TC;
    // Tiles without the packed DC/Nyquist column: the khat multiply runs in registers between the
    // forward and the inverse column FFT, and the tile's two khat columns (contiguous, HQ floats
    // each) are copied to shared memory while the tile loads.
    constexpr int HQC = khat_cols_stride<H>();
    const float* kh = wd.khat + ((size_t)k * (W / 2 + 1) + (size_t)TC * t) * HQC;
    if (fusable<H, MR>() && t != 0 && wd.HQ == HQC && ((uintptr_t)kh & 15) == 0) {
        float* ksm = col_khat_smem<H, MR>(stw);
        for (int e = threadIdx.x; e < TC * HQC / 4; e += NT) cp_async16(ksm + 4 * e, kh + 4 * e);
        load_tile<H, NT, CG>(X, src);
        cp_async_wait_all();
        __syncthreads();
        fft_fused<H, TC, NT, false, true, MR>(X, stw, [&](int s, int j, float2* v) {
            constexpr int R = plan_radix(H, 0, MR), NB = H / R;
            const float* kc = ksm + s * HQC;
#pragma unroll
            for (int m = 0; m < R; m++) {
                const int ky = j + m * NB;
                v[m] = cscale(v[m], kc[ky <= H / 2 ? ky : H - ky]);
            }
        });
        store_tile<H, NT>(X, wd.conv + k * cplane + (size_t)t * H * TC);
        return;
    }
    col_item_unchained<H, NT, CG, MR>(X, stw, src, wd.conv + k * cplane + (size_t)t * H * TC,
                                  wd.khat + (size_t)k * (W / 2 + 1) * HQ, HQ, W, t);
}

// MR: the radix cap of the build's plans (CMR; 16 for the radix-16 build of sizes whose CMR plan has
// radix 32, launch variant 3)
template <int H, int NT, int MINB, int MR = CMR>
__global__ void __launch_bounds__(NT, MINB) col_pass(const DevWorld* __restrict__ worlds, const ColItem* __restrict__ items,
                                                const float2* __restrict__ tw) {
    extern __shared__ float4 smem_raw[];
    constexpr int SEQ = seq_stride(H);
    float2* X = reinterpret_cast<float2*>(smem_raw);
    float2* stw = X + TC * SEQ;
    fill_stage_twiddles<H, float2, 0, MR>(stw, tw, threadIdx.x, NT);
    const ColItem it = items[blockIdx.x];
    col_item<H, NT, false, MR>(worlds[it.world], it, X, stw);
}

// ------------------------------------------------------------------ paired column pass
// The tile's two spectrum columns as one sequence of cpair elements (re = (c0.re, c1.re),
// im = (c0.im, c1.im)): one thread runs butterfly j of both columns with f32x2 arithmetic and
// 16-byte shared-memory accesses, so the item needs half the threads and about half the
// instructions of the scalar build.  Shared memory: the sequence, the tw2 stage tables, the khat
// columns.
constexpr int PMR = max_radix<cpair>();  // largest radix of the paired builds' plans
template <int H>
__device__ __forceinline__ float* col_khat_smem_pair(tw2* stw) {
    constexpr int TWS = tw_table_size(H, PMR);
    return reinterpret_cast<float*>(stw + TWS + 1);
}

template <int H, int NT>
__device__ __forceinline__ void load_tile_pair(cpair* X, const float2* __restrict__ src) {
    constexpr int IT = (H + NT - 1) / NT;
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float4 v[IT];
#pragma unroll
    for (int i = 0; i < IT; i++) {
        const int y = threadIdx.x + i * NT;
        if (IT * NT == H || y < H) v[i] = hint::ld4(s4 + y, hint::policy_keep());
    }
    cpair* x0 = X + pad(threadIdx.x);
#pragma unroll
    for (int i = 0; i < IT; i++) {
        const int y = threadIdx.x + i * NT;
        if (IT * NT == H || y < H)
            (NT % 16 == 0 ? x0[i * (NT + NT / 16)] : X[pad(y)]) =
                cpair{make_float2(v[i].x, v[i].z), make_float2(v[i].y, v[i].w)};
    }
}

template <int H, int NT>
__device__ __forceinline__ void store_tile_pair(const cpair* X, float2* __restrict__ dst) {
    float4* d4 = reinterpret_cast<float4*>(dst);
    const cpair* x = X + pad(threadIdx.x);
    for (int y = threadIdx.x; y < H; y += NT, x += NT + NT / 16) {
        const cpair a = NT % 16 == 0 ? *x : X[pad(y)];
        hint::st4(d4 + y, make_float4(a.re.x, a.im.x, a.re.y, a.im.y), hint::policy_keep());
    }
}

// The khat multiply of an unchained item (see multiply_khat): column 1 (lane y) by its khat
// column; in tile 0, column 0 (lane x) packs the DC and Nyquist columns and pairs ky with H - ky.
template <int H, int NT>
__device__ __forceinline__ void multiply_khat_pair(cpair* X, const float* __restrict__ kh, int HQ, int W, int t) {
    const float* k0 = kh + (size_t)(TC * t) * HQ;
    const float* k1 = k0 + HQ;
    if (t != 0) {
        for (int ky = threadIdx.x; ky < H; ky += NT) {
            const int kk = ky <= H / 2 ? ky : H - ky;
            X[pad(ky)] = cscale2(X[pad(ky)], make_float2(k0[kk], k1[kk]));
        }
        return;
    }
    for (int ky = threadIdx.x; ky <= H / 2; ky += NT) {
        const float K0 = kh[ky], KN = kh[(size_t)(W / 2) * HQ + ky], kv = k1[ky];
        const float a = 0.5f * (K0 + KN), b = 0.5f * (K0 - KN);
        const int km = (H - ky) % H;
        const cpair z = X[pad(ky)], zm = X[pad(km)];
        X[pad(ky)] = cpair{make_float2(z.re.x * a + zm.re.x * b, z.re.y * kv),
                           make_float2(z.im.x * a - zm.im.x * b, z.im.y * kv)};
        if (km != ky)
            X[pad(km)] = cpair{make_float2(zm.re.x * a + z.re.x * b, zm.re.y * kv),
                               make_float2(zm.im.x * a - z.im.x * b, zm.im.y * kv)};
    }
}

template <int H, int NT>
__device__ __noinline__ void col_item_unchained_pair(cpair* X, const tw2* stw, const float2* src, float2* dst,
                                                     const float* kh, int HQ, int W, int t) {
    load_tile_pair<H, NT>(X, src);
    __syncthreads();
    fft_seqs<H, 1, NT, false>(X, stw);
    multiply_khat_pair<H, NT>(X, kh, HQ, W, t);
    __syncthreads();
    fft_seqs<H, 1, NT, true>(X, stw);
    store_tile_pair<H, NT>(X, dst);
}

template <int H, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) col_pass_pair(const DevWorld* __restrict__ worlds,
                                                     const ColItem* __restrict__ items, const float2* __restrict__ tw) {
    extern __shared__ float4 smem_raw[];
    cpair* X = reinterpret_cast<cpair*>(smem_raw);
    tw2* stw = reinterpret_cast<tw2*>(X + seq_stride(H));
    fill_stage_twiddles<H>(stw, tw, threadIdx.x, NT);
    const ColItem it = items[blockIdx.x];
    const DevWorld& wd = worlds[it.world];
    const int W = wd.W, c = it.chan, t = it.tile, k = it.kernel, HQ = wd.HQ;
    const size_t cplane = (size_t)(W / 2) * H;
    const float2* src = wd.spec + c * cplane + (size_t)t * H * TC;
    float2* dst = wd.conv + k * cplane + (size_t)t * H * TC;
    constexpr int HQC = khat_cols_stride<H>();
    const float* kh = wd.khat + ((size_t)k * (W / 2 + 1) + (size_t)TC * t) * HQC;
    if (fusable<H, PMR>() && t != 0 && wd.HQ == HQC && ((uintptr_t)kh & 15) == 0) {
        float* ksm = col_khat_smem_pair<H>(stw);
        for (int e = threadIdx.x; e < TC * HQC / 4; e += NT) cp_async16(ksm + 4 * e, kh + 4 * e);
        load_tile_pair<H, NT>(X, src);
        cp_async_wait_all();
        __syncthreads();
        fft_fused<H, 1, NT, false, true>(X, stw, [&](int, int j, cpair* v) {
            constexpr int R = plan_radix(H, 0, PMR), NB = H / R;
#pragma unroll
            for (int m = 0; m < R; m++) {
                const int ky = j + m * NB, kk = ky <= H / 2 ? ky : H - ky;
                v[m] = cscale2(v[m], make_float2(ksm[kk], ksm[HQC + kk]));
            }
        });
        store_tile_pair<H, NT>(X, dst);
        return;
    }
    col_item_unchained_pair<H, NT>(X, stw, src, dst, wd.khat + (size_t)k * (W / 2 + 1) * HQ, HQ, W, t);
}

// Sizes built: each TU instantiates one group.  Threads per CTA: one first-stage butterfly per
// thread for the two sequences a CTA holds (2N / first radix), between 64 and 1024.
#define LENIA_SIZES_SMALL(X) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768)
#define LENIA_SIZES_LARGE(X) X(1024) X(1536) X(2048) X(3072) X(4096) X(6144) X(8192)
// (The column pass keeps one first-stage butterfly per thread at every size: at 768 the balanced count,
// 128 threads, made it slower, 66 -> 73 us a generation on the batched workload's class.)
template <int N, int MR = CMR> constexpr int nt_of() {
    constexpr int n = 2 * N / plan_radix(N, 0, MR);  // one first-stage butterfly per thread, two sequences
    return n < 64 ? 64 : (n > 1024 ? 1024 : n);
}
// whether the scalar column build's plan has radix 32 (1024, 3072, 8192): those sizes also build the
// radix-16 plan (launch variant 3)
template <int N> constexpr bool col_r32() { return plan_radix(N, 0, CMR) == 32; }
// variant 0: at most 64 registers per thread (80 for radix-32 plans: the 1024 build spilled 508 B at
// 64 and needs none at 80); variant 1: at most 128
template <int N, int V, int MR = CMR> constexpr int minb_threads() {
    return V == 0 ? (plan_radix(N, 0, MR) == 32 ? 768 : 1024) : 512;
}
template <int N, int V, int MR = CMR> constexpr int minb_of() {
    return minb_threads<N, V, MR>() / nt_of<N, MR>() < 1 ? 1 : minb_threads<N, V, MR>() / nt_of<N, MR>();
}
// paired column build: one first-stage butterfly per thread for the one (paired) sequence, at most
// 128 registers a thread
template <int N> constexpr int nt_pair_of() {
    constexpr int n = N / plan_radix(N, 0, PMR);
    return n < 64 ? 64 : (n > 1024 ? 1024 : n);
}
template <int N> constexpr int minb_pair_of() { return 512 / nt_pair_of<N>() < 1 ? 1 : 512 / nt_pair_of<N>(); }

// Launch one instantiation.  Dynamic shared memory above 48 KB must be enabled per kernel before
// its first launch and before any stream capture that contains it; a zero-item call does just that.
template <int H, int NT, int MINB, int MR = CMR>
bool col_go(const DevWorld* worlds, const ColItem* items, int nitems, const float2* tw, cudaStream_t s) {
    const size_t smem = (size_t)TC * seq_stride(H) * sizeof(float2) + stage_table_bytes<H, MR>() + col_khat_bytes<H>();
    static int attr_max = 0;
    if ((int)smem > attr_max) {
        if (cudaFuncSetAttribute(col_pass<H, NT, MINB, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return false;
        attr_max = (int)smem;
    }
    if (nitems > 0) col_pass<H, NT, MINB, MR><<<nitems, NT, smem, s>>>(worlds, items, tw);
    return true;
}

template <int H>
constexpr size_t col_pair_smem() {
    return (size_t)seq_stride(H) * sizeof(cpair) + (size_t)(tw_table_size(H, PMR) + 1) * sizeof(tw2) + col_khat_bytes<H>();
}

template <int H, int NT, int MINB>
bool col_go_pair(const DevWorld* worlds, const ColItem* items, int nitems, const float2* tw, cudaStream_t s) {
    const size_t smem = col_pair_smem<H>();
    static int attr_max = 0;
    if ((int)smem > attr_max) {
        if (cudaFuncSetAttribute(col_pass_pair<H, NT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return false;
        attr_max = (int)smem;
    }
    if (nitems > 0) col_pass_pair<H, NT, MINB><<<nitems, NT, smem, s>>>(worlds, items, tw);
    return true;
}

// Shared memory of a row-pass launch: sequences, stage tables, then the general path's
// accumulation planes.
template <int W, bool GEN>
constexpr size_t row_smem(int general, int planes) {
    const int rows = 2 * row_seqs(W, GEN);
    return (size_t)row_seqs(W, GEN) * seq_stride(W) * sizeof(float2) + stage_table_bytes<W>() +
           (size_t)(general ? planes : 0) * rows * W * sizeof(float);
}

template <int W, int NT, int MINB, bool GEN>
bool row_go(int mode, int general, int planes, const DevWorld* worlds, const RowItem* items, int nitems,
            const float2* tw, cudaStream_t s) {
    const size_t smem = row_smem<W, GEN>(general, planes);
    static int attr_max = 0;
    if ((int)smem > attr_max) {
        if (cudaFuncSetAttribute(row_pass<W, NT, MINB, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return false;
        attr_max = (int)smem;
    }
    if (nitems > 0) row_pass<W, NT, MINB, GEN><<<nitems, NT, smem, s>>>(worlds, items, mode, general, tw);
    return true;
}

// Column-pass builds: variant 0 and 1 are the scalar build at 64 (80 with a radix-32 plan) and 128
// registers a thread, variant 2 the paired build, variant 3 the scalar build with the radix-16 plan at
// 64 registers where the scalar plan has radix 32 (elsewhere variant 0).
template <int N>
bool col_go_variant(int variant, const DevWorld* worlds, const ColItem* items, int nitems, const float2* tw,
                    cudaStream_t s) {
    if (variant == 2) return col_go_pair<N, nt_pair_of<N>(), minb_pair_of<N>()>(worlds, items, nitems, tw, s);
    if (variant == 1) return col_go<N, nt_of<N>(), minb_of<N, 1>()>(worlds, items, nitems, tw, s);
    if constexpr (col_r32<N>())
        if (variant == 3) return col_go<N, nt_of<N, 16>(), minb_of<N, 0, 16>(), 16>(worlds, items, nitems, tw, s);
    return col_go<N, nt_of<N>(), minb_of<N, 0>()>(worlds, items, nitems, tw, s);
}
#define LENIA_COL_CASE(N) \
    case N: return col_go_variant<N>(variant, worlds, items, nitems, tw, s);

// Row-pass builds: variant bit 0 selects the register cap (row_minb); the single-kernel (GEN =
// false) and general (GEN = true) builds sit in separate translation units, which keeps each
// unit's compile time down.  (A paired row build, two packed sequences per thread as in the
// column pass, measured 15% slower at 4096 x 4096: its stores and growth had half the warps to
// hide behind.)
#define LENIA_ROW_CASE_G(N, G)                                                                                   \
    case N:                                                                                                      \
        return (variant & 1)                                                                                     \
                   ? row_go<N, row_nt<N, G>(), row_minb<N, 1, G>(), G>(mode, general, planes, worlds, items, nitems, tw, s) \
                   : row_go<N, row_nt<N, G>(), row_minb<N, 0, G>(), G>(mode, general, planes, worlds, items, nitems, tw, s);
#define LENIA_ROW_CASE_SIMPLE(N) LENIA_ROW_CASE_G(N, false)
#define LENIA_ROW_CASE_GENERAL(N) LENIA_ROW_CASE_G(N, true)

// Local memory (spills and stack) of one instantiation, bytes per thread; -1 if unknown.
template <class F>
int local_bytes_of(F* f) {
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, f) == cudaSuccess ? (int)a.localSizeBytes : -1;
}
template <int N>
int col_local_bytes_variant(int variant) {
    if (variant == 2) return local_bytes_of(col_pass_pair<N, nt_pair_of<N>(), minb_pair_of<N>()>);
    if (variant == 1) return local_bytes_of(col_pass<N, nt_of<N>(), minb_of<N, 1>()>);
    if constexpr (col_r32<N>())
        if (variant == 3) return local_bytes_of(col_pass<N, nt_of<N, 16>(), minb_of<N, 0, 16>(), 16>);
    return local_bytes_of(col_pass<N, nt_of<N>(), minb_of<N, 0>()>);
}
#define LENIA_COL_LOCAL_CASE(N) \
    case N: return col_local_bytes_variant<N>(variant);
#define LENIA_ROW_LOCAL_CASE_G(N, G)                                                    \
    case N:                                                                             \
        return (variant & 1) ? local_bytes_of(row_pass<N, row_nt<N, G>(), row_minb<N, 1, G>(), G>) \
                             : local_bytes_of(row_pass<N, row_nt<N, G>(), row_minb<N, 0, G>(), G>);
#define LENIA_ROW_LOCAL_CASE_SIMPLE(N) LENIA_ROW_LOCAL_CASE_G(N, false)
#define LENIA_ROW_LOCAL_CASE_GENERAL(N) LENIA_ROW_LOCAL_CASE_G(N, true)
int col_local_bytes_small(int H, int variant);
int col_local_bytes_large(int H, int variant);
// row builds: one function per (size group, single-kernel or general) translation unit
int row_local_bytes_small_simple(int W, int variant);
int row_local_bytes_small_general(int W, int variant);
int row_local_bytes_large_simple(int W, int variant);
int row_local_bytes_large_general(int W, int variant);

bool launch_col_group_small(int H, int variant, const DevWorld* worlds, const ColItem* items, int nitems,
                            const float2* tw, cudaStream_t s);
bool launch_col_group_large(int H, int variant, const DevWorld* worlds, const ColItem* items, int nitems,
                            const float2* tw, cudaStream_t s);
#define LENIA_ROW_GROUP_DECL(NAME)                                                                       \
    bool NAME(int W, int variant, int mode, int general, int planes, const DevWorld* worlds, const RowItem* items, \
              int nitems, const float2* tw, cudaStream_t s);
LENIA_ROW_GROUP_DECL(launch_row_group_small_simple)
LENIA_ROW_GROUP_DECL(launch_row_group_small_general)
LENIA_ROW_GROUP_DECL(launch_row_group_large_simple)
LENIA_ROW_GROUP_DECL(launch_row_group_large_general)

}  // namespace lenia
