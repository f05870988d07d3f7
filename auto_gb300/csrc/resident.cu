// Cluster-resident Lenia step for small square worlds: one persistent launch advances every world
// of a size class through all the generations of a step call, one thread-block cluster per world.
//
// The two-pass step (step_fp32.cuh) needs two grid-wide boundaries per generation: every world of
// the class waits for every other at each kernel boundary, and a world of 128 x 128 to 512 x 512
// gives each launch too little work to hide that.  Here the worlds progress independently:
//
//   cluster = one world of N x N (N = 128, 192, 256, 384, 512), G = N / 32 CTAs;
//   CTA q owns rows [32 q, 32 q + 32) and spectrum columns kx in [16 q, 16 q + 16);
//   its shared memory holds those 16 columns of the world's half-spectrum along x (all N rows),
//   for the whole launch -- the world's spectrum lives in the cluster's distributed shared memory.
//
// Per generation (the reference's pass order, crates/auto-core/src/automata/spectral.rs:199-264,
// regrouped as in the two-pass step):
//   column phase  each CTA transforms its 16 columns along y in place, multiplies by the kernel
//                 spectrum and transforms back (the column pass's arithmetic);
//   cluster sync
//   row phase     each CTA gathers its rows' spectrum from the 16-column slices of every CTA of the
//                 cluster (distributed shared memory loads), runs the inverse row FFT, the growth,
//                 dt update and clamp (spectral.rs:337-345) against the state in global memory, the
//                 forward row FFT, and scatters the new row spectrum back into the owners' slices
//                 (distributed shared memory stores);
//   cluster sync
// so the half-spectrum never leaves the chip between generations; the state (read and written once
// per generation, L2-resident for these sizes) and the kernel spectrum columns (read once per
// launch) are the only global traffic.  Each butterfly, twiddle, Hermitian (un)packing and growth
// evaluation is the two-pass step's own device code on the same values, so the results are those of
// the two-pass step.
//
// Cluster syncs are bounded: every CTA arrives (release, cluster scope) on an mbarrier in every CTA
// of the cluster and waits (acquire, cluster scope) on its own with a poll limit.  A CTA whose wait
// runs out sets the error flag and, so that its peers are not left waiting, keeps arriving at every
// later sync (with a short poll limit) while skipping its compute; the host reports the flag as
// LENIA_ECUDA.
#include <cuda_runtime.h>

#include <cstdio>

#include "engine.cuh"
#include "step_fp32.cuh"

namespace lenia {
namespace {

// -------------------------------------------------------------- cluster / DSMEM helpers (PTX)
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// The address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_rank(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
// No memory clobber: these loads are ordered after the peers' stores by the cluster sync (whose
// arrive and wait carry the clobber), and leaving them free lets a thread issue all of its remote
// loads before it uses the first.
__device__ __forceinline__ float2 ld_dsmem(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}
__device__ __forceinline__ void st_dsmem(uint32_t addr, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void remote_arrive(uint32_t addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(addr) : "memory");
}
__device__ __forceinline__ bool try_wait_cluster(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void cluster_barrier_hw() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

constexpr uint32_t SYNC_POLLS = 1u << 22;      // a cluster sync gives up after this many polls
constexpr uint32_t SYNC_POLLS_DEAD = 1u << 6;  // after one has given up: keep arriving, barely wait

// -------------------------------------------------------------- shape of one size class
// S: sequences a CTA transforms at once, S packed row pairs (2S rows) or S columns (16: all 32 rows
// and all 16 columns in one batch); MINB: resident CTAs per SM the registers are budgeted for.  Each
// size is built in a few (S, MINB) launch variants, which the autotuner times.
template <int N, int S_, int MINB_>
struct Res {
    static constexpr int G = N / 32;                 // CTAs per cluster (one world)
    static constexpr int ROWS = 32;                  // rows a CTA owns
    static constexpr int COLS = 16;                  // spectrum columns a CTA owns
    static constexpr int R0 = plan_radix(N, 0), NB = N / R0;
    static constexpr int S = S_, MINB = MINB_;
    static constexpr int NT = S * NB;                // one first-stage butterfly per thread
    static constexpr int GATHER = S * (N / 2) / NT;  // remote elements a thread gathers (and scatters) per batch
    static constexpr int SEQ = seq_stride(N);
    static constexpr int HQC = khat_cols_stride<N>();
    // shared memory: CS [COLS][SEQ] float2 | WK [S][SEQ] float2 | stage tables | KH [COLS][HQC] float | bars
    static constexpr size_t OFF_WK = (size_t)COLS * SEQ * sizeof(float2);
    static constexpr size_t OFF_TW = OFF_WK + (size_t)S * SEQ * sizeof(float2);
    static constexpr size_t OFF_KH = (OFF_TW + stage_table_bytes<N>() + 15) / 16 * 16;
    static constexpr size_t OFF_BAR = OFF_KH + (size_t)COLS * HQC * sizeof(float);
    static constexpr size_t SMEM = OFF_BAR + 16;
    static_assert(G * ROWS == N && G * COLS == N / 2, "32 rows and 16 spectrum columns per CTA");
    static_assert(ROWS % (2 * S) == 0 && COLS % S == 0 && S >= TC, "batches of S");
    static_assert(fusable<N>(), "chained transforms");
    static_assert(GATHER * NT == S * (N / 2), "gather loop without remainder");
};

// Cluster sync, bounded (see the file comment).  Returns false once a wait has run out, on every
// thread of the CTA.
struct ClusterSync {
    uint32_t bar;    // shared address of this CTA's mbarrier
    uint32_t phase;  // parity of the next phase to complete
    bool dead;
    template <int G>
    __device__ __forceinline__ bool sync() {
        __syncthreads();  // every thread's shared, distributed-shared and global writes precede the arrivals
        if (threadIdx.x == 0)
#pragma unroll 1
            for (int q = 0; q < G; q++) remote_arrive(map_rank(bar, (uint32_t)q));
        const uint32_t limit = dead ? SYNC_POLLS_DEAD : SYNC_POLLS;
        bool ok = false;
        for (uint32_t i = 0; i < limit && !ok; i++) ok = try_wait_cluster(bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) dead = true;
        return !dead;
    }
};

// -------------------------------------------------------------- the kernel
template <int N, int S_, int MINB_>
__global__ void __launch_bounds__(Res<N, S_, MINB_>::NT, MINB_)
    resident_step(const DevWorld* __restrict__ worlds, const int* __restrict__ world_ids, int gens,
                  const float2* __restrict__ tw, int* __restrict__ err) {
    using P = Res<N, S_, MINB_>;
    constexpr int S = P::S, NT = P::NT, SEQ = P::SEQ, COLS = P::COLS, HQC = P::HQC;
    extern __shared__ float4 smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>(smem_raw);
    float2* CS = reinterpret_cast<float2*>(base);
    float2* WK = reinterpret_cast<float2*>(base + P::OFF_WK);
    float2* stw = reinterpret_cast<float2*>(base + P::OFF_TW);
    float* KH = reinterpret_cast<float*>(base + P::OFF_KH);
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + P::OFF_BAR);

    const int q = (int)cluster_rank();
    const DevWorld& wd = worlds[world_ids[blockIdx.x / P::G]];
    const int kx0 = COLS * q, r0q = P::ROWS * q;
    const uint32_t cs_addr = tc::smem_u32(CS);

    fill_stage_twiddles<N>(stw, tw, threadIdx.x, NT);
    if (threadIdx.x == 0) {
        tc::mbar_init(bar, P::G);
        tc::fence_barrier_init();
    }
    // this CTA's kernel-spectrum columns, once for every generation (rows kx of khat, HQC floats each)
    {
        const float* kh = wd.khat + (size_t)kx0 * HQC;
        for (int e = threadIdx.x; e < COLS * HQC / 4; e += NT) cp_async16(KH + 4 * e, kh + 4 * e);
    }
    // this CTA's 16 spectrum columns from the tile layout ([tile][H][TC]), in column sequences
    for (int e = threadIdx.x; e < COLS * N; e += NT) {
        const int c = e / N, y = e - c * N, kx = kx0 + c;
        CS[c * SEQ + pad(y)] = wd.spec[((size_t)(kx / TC) * N + y) * TC + kx % TC];
    }
    cp_async_wait_all();
    cluster_barrier_hw();  // every CTA's mbarrier is initialised before anyone arrives on it
    ClusterSync cs{tc::smem_u32(bar), 0u, false};

    const DevKernel kp = wd.kern[0];
    const float dtw = wd.dt * kp.weight;
    const Growth growth(kp.mu, kp.sigma);
    const uint64_t stream = hint::policy_stream();
    constexpr int R = P::R0, NB = P::NB;

#pragma unroll 1
    for (int g = 0; g < gens; g++) {
        // ---------------- column phase: forward FFT along y, x khat, inverse FFT, in place
        if (!cs.dead) {
            if (q == 0) {
                // columns 0 and 1: column 0 packs the real DC and Nyquist columns, which pair ky with
                // N - ky in the khat multiply; they take the two-pass step's unchained form in WK
                for (int e = threadIdx.x; e < TC * N; e += NT) {
                    const int c = e / N, y = e - c * N;
                    WK[c * SEQ + pad(y)] = CS[c * SEQ + pad(y)];
                }
            }
#pragma unroll 1
            for (int b = 0; b < COLS / S; b++) {
                fft_fused<N, S, NT, false, true>(CS + b * S * SEQ, stw, [&](int s, int j, float2* v) {
                    const float* kc = KH + (b * S + s) * HQC;
#pragma unroll
                    for (int m = 0; m < R; m++) {
                        const int ky = j + m * NB;
                        v[m] = cscale(v[m], kc[ky <= N / 2 ? ky : N - ky]);
                    }
                });
            }
            if (q == 0) {
                fft_seqs<N, TC, NT, false>(WK, stw);
                multiply_khat<N, NT>(WK, WK, wd.khat, wd.HQ, N, 0);
                __syncthreads();
                fft_seqs<N, TC, NT, true>(WK, stw);
                for (int e = threadIdx.x; e < TC * N; e += NT) {
                    const int c = e / N, y = e - c * N;
                    CS[c * SEQ + pad(y)] = WK[c * SEQ + pad(y)];
                }
            }
        }
        cs.template sync<P::G>();
        // ---------------- row phase: gather, inverse row FFT, growth, forward row FFT, scatter
        if (!cs.dead) {
#pragma unroll 1
            for (int rb = 0; rb < P::ROWS; rb += 2 * S) {
                const int r0 = r0q + rb;
                float* st = wd.state + (size_t)r0 * N;
                if (threadIdx.x == 0) tc::bulk_prefetch_l2(st, 2 * S * N * (uint32_t)sizeof(float));
                // gather: Z_p = A + iB (A = row r0 + 2p, B = row r0 + 2p + 1) with Hermitian symmetry
                // for kx > N/2, the formulas of load_rows_spectrum; consecutive lanes on
                // consecutive kx.  Every remote load of the thread is issued before the first is used.
                float2 GA[P::GATHER], GB[P::GATHER];
#pragma unroll
                for (int i = 0; i < P::GATHER; i++) {
                    const int e = threadIdx.x + i * NT, p = e / (N / 2), kx = e - p * (N / 2);
                    // rows r0 + 2p and r0 + 2p + 1 of column kx in its owner's slice: r0 + 2p is even, so
                    // the two are neighbours (padding follows odd indices 15 mod 16 only)
                    const uint32_t off = cs_addr + (uint32_t)(((kx % COLS) * SEQ + pad(r0 + 2 * p)) * sizeof(float2));
                    const uint32_t src = map_rank(off, (uint32_t)(kx / COLS));
                    GA[i] = ld_dsmem(src);
                    GB[i] = ld_dsmem(src + (uint32_t)sizeof(float2));
                }
#pragma unroll
                for (int i = 0; i < P::GATHER; i++) {
                    const int e = threadIdx.x + i * NT, p = e / (N / 2), kx = e - p * (N / 2);
                    const float2 A = GA[i], B = GB[i];
                    float2* z = WK + p * SEQ;
                    if (kx == 0) {
                        z[pad(0)] = make_float2(A.x, B.x);
                        z[pad(N / 2)] = make_float2(A.y, B.y);
                    } else {
                        z[pad(kx)] = make_float2(A.x - B.y, A.y + B.x);
                        z[pad(N - kx)] = make_float2(A.x + B.y, B.x - A.y);
                    }
                }
                __syncthreads();
                float sa[R], sb[R];
                fft_fused<N, S, NT, true, false>(
                    WK, stw,
                    [&](int s, int j, float2* v) {
                        float* ga = st + (2 * s) * N + j;
                        static_for<0, R>([&](auto m) {
                            const float n0 = __saturatef(fmaf(dtw, growth(v[m].x), sa[m]));
                            const float n1 = __saturatef(fmaf(dtw, growth(v[m].y), sb[m]));
                            hint::st1_at<decltype(m)::value * NB * 4>(ga, n0, stream);
                            hint::st1_at<(N + decltype(m)::value * NB) * 4>(ga, n1, stream);
                            v[m] = make_float2(n0, n1);
                        });
                    },
                    [&](int s, int j) {
                        const float* ga = st + (2 * s) * N + j;
                        static_for<0, R>([&](auto m) {
                            sa[m] = hint::ld1_at<decltype(m)::value * NB * 4>(ga, stream);
                            sb[m] = hint::ld1_at<(N + decltype(m)::value * NB) * 4>(ga, stream);
                        });
                    });
                // scatter: the half-spectra of the 2S new rows into the owners' column slices (the
                // formulas of store_rows_spectrum)
#pragma unroll
                for (int i = 0; i < P::GATHER; i++) {
                    const int e = threadIdx.x + i * NT, p = e / (N / 2), kx = e - p * (N / 2);
                    const float2* z = WK + p * SEQ;
                    float2 A, B;
                    if (kx == 0) {
                        const float2 z0 = z[pad(0)], zn = z[pad(N / 2)];
                        A = make_float2(z0.x, zn.x);
                        B = make_float2(z0.y, zn.y);
                    } else {
                        const float2 a = z[pad(kx)], b = z[pad(N - kx)];
                        A = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
                        B = make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x));
                    }
                    const uint32_t off = cs_addr + (uint32_t)(((kx % COLS) * SEQ + pad(r0 + 2 * p)) * sizeof(float2));
                    const uint32_t dst = map_rank(off, (uint32_t)(kx / COLS));
                    st_dsmem(dst, A);
                    st_dsmem(dst + (uint32_t)sizeof(float2), B);
                }
                __syncthreads();  // WK is rewritten by the next batch
            }
        }
        cs.template sync<P::G>();
    }
    // the half-spectrum back to the tile layout, so the engine's other passes see the current one
    for (int e = threadIdx.x; e < COLS * N; e += NT) {
        const int c = e / N, y = e - c * N, kx = kx0 + c;
        wd.spec[((size_t)(kx / TC) * N + y) * TC + kx % TC] = CS[c * SEQ + pad(y)];
    }
    if (cs.dead && threadIdx.x == 0) atomicExch(err, 1);
}

template <int N, int S, int MINB>
bool launch_shape(const DevWorld* worlds, const int* world_ids, int nworlds, int gens, const float2* tw, int* err,
                  cudaStream_t s) {
    using P = Res<N, S, MINB>;
    static int configured = 0;
    if (!configured) {
        if (cudaFuncSetAttribute(resident_step<N, S, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)P::SMEM) != cudaSuccess ||
            (P::G > 8 && cudaFuncSetAttribute(resident_step<N, S, MINB>,
                                              cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess))
            return false;
        configured = 1;
    }
    if (nworlds <= 0 || gens <= 0) return true;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(P::G * nworlds));
    cfg.blockDim = dim3((unsigned)P::NT);
    cfg.dynamicSmemBytes = P::SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = P::G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, resident_step<N, S, MINB>, worlds, world_ids, gens, tw, err) == cudaSuccess;
}

template <int N, int S, int MINB>
int clusters_that_fit() {
    using P = Res<N, S, MINB>;
    if (!launch_shape<N, S, MINB>(nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr)) return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)P::G);
    cfg.blockDim = dim3((unsigned)P::NT);
    cfg.dynamicSmemBytes = P::SMEM;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = P::G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, resident_step<N, S, MINB>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// The launch variants of each size, (S, MINB): 0 = (16, 1), 1 = (8, 1), 2 = (4, 2).
#define LENIA_RESIDENT_VARIANT(N, F) (variant == 0 ? F<N, 16, 1> : variant == 1 ? F<N, 8, 1> : F<N, 4, 2>)

}  // namespace

bool resident_supported(int N) { return N == 128 || N == 192 || N == 256 || N == 384 || N == 512; }

int resident_clusters_that_fit(int N, int variant) {
    if (variant < 0 || variant >= RESIDENT_VARIANTS) return 0;
    switch (N) {
    case 128: return LENIA_RESIDENT_VARIANT(128, clusters_that_fit)();
    case 192: return LENIA_RESIDENT_VARIANT(192, clusters_that_fit)();
    case 256: return LENIA_RESIDENT_VARIANT(256, clusters_that_fit)();
    case 384: return LENIA_RESIDENT_VARIANT(384, clusters_that_fit)();
    case 512: return LENIA_RESIDENT_VARIANT(512, clusters_that_fit)();
    }
    return 0;
}

bool launch_resident(int N, int variant, const DevWorld* worlds, const int* world_ids, int nworlds, int gens,
                     const float2* tw, int* err, cudaStream_t s) {
    if (variant < 0 || variant >= RESIDENT_VARIANTS) return false;
    switch (N) {
    case 128: return LENIA_RESIDENT_VARIANT(128, launch_shape)(worlds, world_ids, nworlds, gens, tw, err, s);
    case 192: return LENIA_RESIDENT_VARIANT(192, launch_shape)(worlds, world_ids, nworlds, gens, tw, err, s);
    case 256: return LENIA_RESIDENT_VARIANT(256, launch_shape)(worlds, world_ids, nworlds, gens, tw, err, s);
    case 384: return LENIA_RESIDENT_VARIANT(384, launch_shape)(worlds, world_ids, nworlds, gens, tw, err, s);
    case 512: return LENIA_RESIDENT_VARIANT(512, launch_shape)(worlds, world_ids, nworlds, gens, tw, err, s);
    }
    return false;
}

}  // namespace lenia
