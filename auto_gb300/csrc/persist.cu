// Persistent step of one size class (FP32 path): one launch advances every world of a square,
// one-channel, one-kernel Lenia class through every generation of a step call.
//
// The two-pass step launches a column pass and a row pass per class and generation; a graph of 64
// generations is 128 launches a class, each with a tail where its last items leave SMs idle, and each
// world's half-spectrum goes to HBM between the passes when the class's spectra exceed L2.  Here a
// grid of resident CTAs takes the same column and row items, from the same item lists, in one
// sequence per generation in which each world's row items come L worlds after its column items:
//
//     col(w0) .. col(w_L-1)  col(w_L) row(w0)  col(w_L+1) row(w1)  ...  row(w_n-L) .. row(w_n-1)
//
// The lag L is the number of worlds whose items the resident grid holds at once, plus one, so a
// world's column items have finished by the time its row items are claimed (with a lag of one world
// the row items of a large class waited on column items still in flight: 1024 x 1024 ran at 0.6 of
// the two-pass rate, 128 x 128 at 0.06).
// A CTA claims items in that order with one atomic counter (the next item is claimed while the
// current one runs).  An item waits, if it must, for the items it depends on: a world's row items for
// all of its column items of the same generation, its column items for all of its row items of the
// previous generation, counted per world.  Because claims are in order and every dependency lies
// earlier in the sequence, the earliest unfinished item always has its inputs and its CTA is running,
// so the launch cannot deadlock, whatever the number of resident CTAs.  A world's spectrum written by
// its column items is read by its row items L worlds later, from L2 (L worlds' spectra are a few MB).
//
// The item bodies are the two-pass step's own device code (col_item, row_item_simple), with loads of
// the spectrum and state that bypass L1, since another SM of the same launch may have written them
// (L1 is not coherent across SMs); results are bit-identical to the two-pass step.  A producer
// publishes an item with __syncthreads, a device-scope fence and an atomic increment; a consumer
// spins (one thread, bounded: 2^22 polls) with acquire loads.  A wait that gives up sets the launch's
// abort word and the context's error flag, and every CTA then stops claiming items.  A test hook
// (err[1], lenia_persist_set_wait_limit) lowers the limit, down to every dependency wait giving up
// at once.
#include <cuda_runtime.h>

#include "engine.cuh"
#include "step_fp32.cuh"

namespace lenia {

// Control words of a persistent launch (zeroed before it): [0] next item, [1] abort,
// [2 .. 2+nw) column items done per world, [2+nw .. 2+2nw) row items done per world.
constexpr int PST_NEXT = 0, PST_ABORT = 1, PST_COUNTERS = 2;
constexpr uint32_t PST_WAIT_POLLS = 1u << 22;

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <int N, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    persist_class(const DevWorld* __restrict__ worlds, const ColItem* __restrict__ cols, const RowItem* __restrict__ rows,
                  int nw, int nc, int nr, int lag, int gens, const float2* __restrict__ tw, int* ctl, int* err) {
    extern __shared__ float4 smem_raw[];
    __shared__ long long s_item;
    __shared__ int s_stop;
    constexpr int SEQ = seq_stride(N), NSEQ = row_seqs(N, false) > TC ? row_seqs(N, false) : TC;
    float2* X = reinterpret_cast<float2*>(smem_raw);
    float2* stw = X + NSEQ * SEQ;  // after the column pass's tile sequences and the row pass's packed rows
    // the row items' stage tables, then the column items' (their plans may differ: CMR)
    float2* stwc = stw + tw_table_size(N) + 1;
    fill_stage_twiddles<N>(stw, tw, threadIdx.x, NT);
    fill_stage_twiddles<N, float2, 0, CMR>(stwc, tw, threadIdx.x, NT);
    int* cols_done = ctl + PST_COUNTERS;
    int* rows_done = cols_done + nw;
    const long long per_gen = (long long)nw * (nc + nr), total = per_gen * gens;
    // err[1]: the wait limit + 1 (0: the default; 1: every dependency wait gives up at once, met or not)
    const int lim1 = threadIdx.x == 0 ? err[1] : 0;
    const uint32_t max_polls = lim1 > 1 ? (uint32_t)(lim1 - 1) : PST_WAIT_POLLS;
    unsigned int* claim = reinterpret_cast<unsigned int*>(ctl + PST_NEXT);
    long long next = 0;
    if (threadIdx.x == 0) next = atomicAdd(claim, 1u);
    for (;;) {
        if (threadIdx.x == 0) {
            // claim the item after the current one while the current one runs
            const long long cur = next;
            next = atomicAdd(claim, 1u);
            s_item = cur;
        }
        __syncthreads();  // also: the previous item's shared-memory use is over
        const long long i = s_item;
        if (i >= total) break;
        const int g = (int)(i / per_gen);
        const int p = (int)(i - (long long)g * per_gen);
        bool is_col;
        int w, idx;
        if (p < lag * nc) {
            is_col = true, w = p / nc, idx = p - w * nc;
        } else {
            const int q = p - lag * nc, pr = q / (nc + nr);
            if (pr < nw - lag) {
                const int off = q - pr * (nc + nr);
                is_col = off < nc;
                w = is_col ? lag + pr : pr;
                idx = is_col ? off : off - nc;
            } else {
                const int q2 = q - (nw - lag) * (nc + nr);
                is_col = false, w = nw - lag + q2 / nr, idx = q2 % nr;
            }
        }
        if (threadIdx.x == 0) {
            // wait (bounded) for the items this one depends on
            const int* cnt = is_col ? rows_done + w : cols_done + w;
            const int target = is_col ? g * nr : (g + 1) * nc;
            int stop = lim1 == 1 && target > 0;
            for (uint32_t polls = 0; !stop && ld_acquire(cnt) < target; polls++) {
                if (ld_acquire(ctl + PST_ABORT) || polls >= max_polls) {
                    stop = 1;
                    break;
                }
                __nanosleep(32);
            }
            if (stop) {
                atomicExch(ctl + PST_ABORT, 1);
                atomicExch(err, 1);
            }
            s_stop = stop;
        }
        __syncthreads();
        if (s_stop) break;
        if (is_col) {
            const ColItem it = cols[(size_t)w * nc + idx];
            col_item<N, NT, true>(worlds[it.world], it, X, stwc);
        } else {
            const RowItem it = rows[(size_t)w * nr + idx];
            row_item_simple<N, NT, true>(worlds[it.world], it.row0, X, stw);
        }
        __syncthreads();  // every thread's stores of this item are issued
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(is_col ? cols_done + w : rows_done + w, 1);
        }
    }
}

// Sizes the persistent step is built for (square classes).
#define LENIA_PERSIST_SIZES(X) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(2048) X(4096)

namespace {

// the larger of the column and row items' thread counts (an item with fewer butterflies than threads
// leaves the rest idle in its stages)
template <int N>
constexpr int persist_nt() { return nt_of<N>() > row_nt<N, false>() ? nt_of<N>() : row_nt<N, false>(); }
// Two launch variants, as the two-pass step's: 0 caps registers at 64 a thread (twice the resident
// CTAs; the column and row item bodies in one kernel spill 24-52 bytes a thread at 512 and above, and
// 300-700 bytes below), 1 at 128 (no spills from 512 up).
template <int N, int V>
constexpr int persist_minb() { return (V == 0 ? 1024 : 512) / persist_nt<N>() < 1 ? 1 : (V == 0 ? 1024 : 512) / persist_nt<N>(); }

template <int N>
size_t persist_smem() {
    constexpr int NSEQ = row_seqs(N, false) > TC ? row_seqs(N, false) : TC;
    return (size_t)NSEQ * seq_stride(N) * sizeof(float2) + stage_table_bytes<N>() + stage_table_bytes<N, CMR>() +
           col_khat_bytes<N>();
}

template <int N, int V>
bool persist_go(const DevWorld* worlds, const ColItem* cols, const RowItem* rows, int nw, int nc, int nr, int gens,
                const float2* tw, int* ctl, int* err, cudaStream_t s, int* capacity) {
    constexpr int NT = persist_nt<N>(), MINB = persist_minb<N, V>();
    auto kern = persist_class<N, NT, MINB>;
    const size_t smem = persist_smem<N>();
    static int per_sm = -1, sms = 0;
    if (per_sm < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem) != cudaSuccess) {
            per_sm = -1;
            return false;
        }
    }
    if (capacity) *capacity = per_sm * sms;
    if (nw <= 0 || gens <= 0) return true;
    if (per_sm < 1) return false;
    const long long items = (long long)nw * (nc + nr) * gens;
    const int grid = (int)(items < (long long)per_sm * sms ? items : (long long)per_sm * sms);
    // worlds the grid holds at once, plus one; at least 1, at most every world
    int lag = (grid + nc + nr - 1) / (nc + nr) + 1;
    if (lag > nw) lag = nw;
    if (lag < 1) lag = 1;
    // Every CTA of the grid fits the GPU at once (grid <= the occupancy bound); launched cooperatively,
    // so that they are resident together.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, worlds, cols, rows, nw, nc, nr, lag, gens, tw, ctl, err) == cudaSuccess;
}

}  // namespace

bool persist_supported(int N) {
    switch (N) {
#define PS_CASE(n) case n: return true;
        LENIA_PERSIST_SIZES(PS_CASE)
#undef PS_CASE
    }
    return false;
}

int persist_ctl_words(int nworlds) { return PST_COUNTERS + 2 * nworlds; }

bool launch_persist(int N, int variant, const DevWorld* worlds, const ColItem* cols, const RowItem* rows, int nworlds,
                    int ncol, int nrow, int gens, const float2* tw, int* ctl, int* err, cudaStream_t s, int* capacity) {
    switch (N) {
#define PL_CASE(n)                                                                                                 \
    case n:                                                                                                        \
        return variant == 0 ? persist_go<n, 0>(worlds, cols, rows, nworlds, ncol, nrow, gens, tw, ctl, err, s, capacity) \
                            : persist_go<n, 1>(worlds, cols, rows, nworlds, ncol, nrow, gens, tw, ctl, err, s, capacity);
        LENIA_PERSIST_SIZES(PL_CASE)
#undef PL_CASE
    }
    return false;
}

}  // namespace lenia
