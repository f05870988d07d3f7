// Engine context and the C ABI (include/lenia_gb300.h).
//
// A context is the GB300 counterpart of the reference's Sim + Program pair
// (crates/auto-core/src/sim.rs:59-80, program.rs:102-129): it owns the device buffers of every
// world, the kernel spectra, the work lists of each size class and the CUDA graphs that replay
// steps.  Worlds of one grid size form a size class; each class is one column launch and one
// row launch per step over all of its worlds, and the graph runs the classes one after another.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "engine.cuh"
#include "fft_core.cuh"
#include "step_radix2.cuh"
#include "step_tc.cuh"

using namespace lenia;

namespace {

thread_local std::string g_create_error;

// A run of consecutive worlds of one size class (their items are consecutive in the class lists).
// The step graph advances a chunk through all of its steps before the next chunk starts, so a chunk
// small enough for L2 keeps its states, spectra and kernel spectra there across generations instead
// of streaming them from HBM twice per generation.
struct Chunk {
    int col0 = 0, ncol = 0, tcg0 = 0, ntcg = 0, row0 = 0, nrow = 0;
    size_t bytes = 0;
};

struct SizeClass {
    int W = 0, H = 0;
    std::vector<int> worlds;
    ColItem* d_col = nullptr;  // FP32 column items (tiles)
    int ncol = 0;
    ColItem* d_tcg = nullptr;  // tensor-core column groups (TF32 / BF16X3 paths)
    int ntcg = 0;
    RowItem* d_row = nullptr;
    int nrow = 0;
    int var_col = 0, var_row = 0;  // launch variants (see launch_col_fp32)
    int var_tc = 1;                // tensor-core column pass variant (launch_col_tc): 1 measured 4-7% faster
                                   // than 0 at 512 and 1024 (batched BF16x3), equal at 256
    int general = 0, planes = 0;
    size_t bytes = 0;          // device bytes the class's worlds touch in a step
    size_t chunk_budget = 0;   // largest chunk in bytes (0: the whole class is one chunk)
    std::vector<Chunk> chunks;
    int lanes = 1;             // concurrent lanes its chunks run on (enqueue_class)
    // cluster-resident step (resident.cu): possible for square one-channel, one-kernel Lenia classes
    // of 128..512 on the FP32 path; `resident` selects it over the two launches per generation
    int resident_ok = 0, resident = 0;
    int var_res = 0;                       // its launch variant (resident.cu)
    int res_fits[RESIDENT_VARIANTS] = {};  // clusters of each variant the GPU holds at once (0: cannot run)
    int* d_world_ids = nullptr;
    // tensor-core row pass (step_tc_row.cu): possible for one-channel, one-kernel Lenia classes on the
    // TF32 / BF16X3 paths whose row length it serves; `tc_rows` selects it over the FP32 row pass.
    // Its groups are tc_row_stride consecutive FP32 row items, or -tc_row_stride groups an item.
    int tc_rows_ok = 0, tc_rows = 0, tc_row_stride = 1;
    // persistent step (persist.cu): possible for square one-channel, one-kernel Lenia classes on the
    // FP32 path; `persist` selects one launch per class and step call over the two launches per
    // generation.  d_pctl: its control words.
    int persist_ok = 0, persist = 0;
    int var_per = 0;  // its launch variant (persist.cu)
    int* d_pctl = nullptr;
};

// Default chunk budget and lanes: a class of more than 32 MiB of per-step data runs in chunks of at
// most 32 MiB, four chunks at a time on concurrent lanes.  A chunk keeps its worlds in L2 across its
// generations (ncu on the 55 worlds of 1024 x 1024 in 32 MiB chunks: DRAM traffic 1.4 GB -> 23 MB per
// generation), but a launch over a few worlds fills the GPU less, and chunks one after another
// measured slower than one chunk (1024 x 1024: 2.07e11 cell-updates/s as one chunk, 1.87e11 in 8
// chunks of 64 MiB, 1.53e11 in 16 of 32 MiB).  On lanes the chunks' launches fill the GPU together:
// 1024 x 1024 2.35e11 in 16 chunks of 32 MiB on four lanes (2.22e11 in 8 of 64 MiB on two; 16 MiB
// on eight, 2.35e11, and 24 MiB on six, 2.32e11, no faster), 768 x 768 1.99e11 (1.93e11).  The
// autotuner tries other budgets and 1 to 4 lanes per class.
constexpr size_t DEFAULT_CHUNK_BUDGET = 32ull << 20;
constexpr int DEFAULT_LANES = 4;
// Whether a class the persistent step serves starts with it (the autotuner times it against the two
// launches per generation and keeps the faster).  Off: on the batched workload every class measured
// slower persistent (1024 x 1024: 1.73e11 cell-updates/s against 1.92e11; 128 x 128: 3.5e10 against
// 8.8e10; one 4096 x 4096 world: 1.31e11 against 1.54e11), the two-pass kernels' own register budgets
// and builds mattering more than the launches and HBM round trips it saves.
constexpr int PERSIST_DEFAULT = 0;
// Whether a class the tensor-core row pass serves starts with it.  Off: measured slower than the FP32
// row pass at every size it serves (1024 x 1024: 354 us a generation for the class of 55 worlds
// against 188 us), and its BF16x3 inverse feeds U's rounding error straight into the growth (about
// 3e-5 a step against FP64, where the FP32 row pass leaves 6e-6).  lenia_set_tc_rows turns it on;
// the autotuner times it and keeps it only where it is faster.
constexpr int TC_ROWS_DEFAULT = 0;
// Whether a class the cluster-resident step serves starts with it (the autotuner then times it
// against the two launches per generation and keeps the faster).
constexpr int RESIDENT_DEFAULT = 0;

struct WorldBuffers {
    ColItem* d_col = nullptr;  // this world's column items (inspection, U fields)
    int ncol = 0;
    ColItem* d_tcg = nullptr;
    int ntcg = 0;
    RowItem* d_row = nullptr;  // this world's row items (forward transform after writes)
    int nrow = 0;
    int cls = 0;
};

}  // namespace

struct LeniaCtx {
    std::string err;
    int device = 0;
    int path = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    // the tensor-core paths run a class's few FP32 column items beside the tensor-core launch
    cudaStream_t side = nullptr;
    // two-branch step graph (FP32 path): the size classes of at most `branch_cells` cells a world run
    // one after another on `branch`, beside the larger classes on `stream` (0: one branch)
    // with branch_each, every such class gets a branch of its own
    static constexpr int MAX_BRANCHES = 8;
    cudaStream_t branch[MAX_BRANCHES] = {};
    cudaEvent_t ev_bfork = nullptr, ev_bjoin[MAX_BRANCHES] = {};
    int64_t branch_cells = 0;
    int branch_each = 0;
    // chunk lanes: the chunks of a class on the main branch may run on up to MAX_LANES concurrent
    // graph branches (SizeClass::lanes), chunk c on lane c mod lanes
    static constexpr int MAX_LANES = 4;
    cudaStream_t lane[MAX_LANES] = {};
    cudaEvent_t ev_lfork = nullptr, ev_ljoin[MAX_LANES] = {};
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // asynchronous state copies (lenia_write_states_async / lenia_read_states_async): uploads on
    // `up`, downloads on `down`, through device staging buffers, so that they overlap the
    // generations on `stream` (one copy stream would queue the next upload behind the last
    // download, which waits for the last step)
    cudaStream_t up = nullptr, down = nullptr;
    float* stage_in = nullptr;
    float* stage_out = nullptr;
    cudaEvent_t ev_in_ready = nullptr, ev_in_free = nullptr, ev_out_ready = nullptr, ev_out_free = nullptr;
    std::vector<LeniaWorldDesc> desc;
    std::vector<DevWorld> hw;
    DevWorld* d_worlds = nullptr;
    float2* d_tw = nullptr;
    float* d_stats = nullptr;
    std::vector<SizeClass> classes;
    std::vector<WorldBuffers> wb;
    std::vector<R2World> r2;
    std::vector<void*> allocs;
    uint64_t tick = 0;
    uint64_t bytes = 0;
    // one device arena for all per-world buffers (many small worlds would otherwise cost one
    // cudaMalloc each): `arena_need` is summed in a sizing pass, then carved in order
    char* arena = nullptr;
    size_t arena_need = 0, arena_used = 0;
    bool sizing = false;
    int graph_steps = 64;
    cudaGraphExec_t graph_big = nullptr, graph_one = nullptr;
    TcPlan tc;
    // Worlds whose state changed since their half-spectrum was last formed.  The forward row
    // transforms run at the next call that reads spectra (flush_spectra), one launch per size class
    // when a whole class changed.
    std::vector<char> dirty;
    int ndirty = 0;
    // all states back to back in world order (fused paths): one copy for every world
    float* states = nullptr;
    size_t states_count = 0;
    // device error flag of the cluster-resident step (1: a cluster sync gave up)
    int* d_flags = nullptr;
};

namespace {

int fail(LeniaCtx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_create_error = buf;
    return code;
}

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(ctx, LENIA_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// Owners that release on every return path (the CK macro returns early on a CUDA error).
struct Events {
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    ~Events() {
        for (cudaEvent_t x : e)
            if (x) cudaEventDestroy(x);
    }
};
struct DeviceBuffer {
    void* p = nullptr;
    ~DeviceBuffer() {
        if (p) cudaFree(p);
    }
};

template <typename T>
int dalloc(LeniaCtx* ctx, T** p, size_t count) {
    const size_t bytes = (count * sizeof(T) + 255) / 256 * 256;
    if (ctx->sizing) {
        ctx->arena_need += bytes;
        *p = nullptr;
        return 0;
    }
    if (ctx->arena && ctx->arena_used + bytes <= ctx->arena_need) {
        *p = (T*)(ctx->arena + ctx->arena_used);
        ctx->arena_used += bytes;
        ctx->bytes += bytes;
        return 0;
    }
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, count * sizeof(T) > 0 ? count * sizeof(T) : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, LENIA_ENOMEM, "device allocation of %zu bytes failed: %s", count * sizeof(T),
                    cudaGetErrorString(e));
    }
    ctx->allocs.push_back(v);
    ctx->bytes += count * sizeof(T);
    *p = (T*)v;
    return 0;
}

bool supported_side(uint32_t n) {
    uint32_t m = (n % 3 == 0) ? n / 3 : n;
    if (m == 0 || (m & (m - 1)) != 0) return false;
    return n >= 32 && n <= 8192;
}
bool is_pow2(uint32_t n) { return n && !(n & (n - 1)); }

// ---------------------------------------------------------------- kernel shapes in FP64
double lenia_core64(double q) { return (q <= 0.0 || q >= 1.0) ? 0.0 : std::exp(4.0 - 1.0 / (q * (1.0 - q))); }

double shape64(const LeniaKernel& k, double r) {
    switch (k.shape) {
    case LENIA_SHAPE_LENIA: {
        int B = k.nshells < 1 ? 1 : k.nshells;
        double q = r / k.radius;
        if (q <= 0.0 || q >= 1.0) return 0.0;
        double bq = B * q;
        int i = (int)std::floor(bq);
        if (i >= B) return 0.0;
        return (double)k.beta[i] * lenia_core64(bq - i);
    }
    case LENIA_SHAPE_SL_INNER: {
        double ri = k.radius / 3.0, aa = 0.5;
        return std::min(std::max((ri + aa - r) / (2 * aa), 0.0), 1.0);
    }
    case LENIA_SHAPE_SL_OUTER: {
        double ra = k.radius, ri = k.radius / 3.0, aa = 0.5;
        return std::min(std::max((ra + aa - r) / (2 * aa), 0.0), 1.0) * std::min(std::max((r - ri + aa) / (2 * aa), 0.0), 1.0);
    }
    case LENIA_SHAPE_RING: return (r >= k.ring_lo && r < k.ring_hi) ? 1.0 : 0.0;
    }
    return 0.0;
}

// Kernel.reach of spectral.rs:111-116 (size guard) and a bound on the support.
int guard_reach(const LeniaKernel& k) {
    switch (k.shape) {
    case LENIA_SHAPE_LENIA: return (int)std::ceil(k.radius);
    case LENIA_SHAPE_SL_INNER:
    case LENIA_SHAPE_SL_OUTER: return (int)std::ceil(k.radius) + 2;
    case LENIA_SHAPE_RING: return (int)std::ceil(k.ring_hi);
    }
    return 0;
}

// Real, even kernel spectrum in FP64, rounded to f32, with 1/(W*H) folded in:
//   khat[kx][ky] = sum_{dx,dy} K(dx,dy) cos(2 pi kx dx / W) cos(2 pi ky dy / H) / (sum K * W * H)
// for kx in [0, W/2], ky in [0, H/2].  The kernel is even in dx and in dy (min-image
// placement), so this is its exact DFT; the reference computes the same spectrum with an f32
// FFT on the GPU (spectral.rs:150-181).
void compute_khat(const LeniaKernel& k, int W, int H, int HQ, float* out, bool threaded = true) {
    const int reach = guard_reach(k) + 1;
    const int nR = reach + 1;
    std::vector<double> v((size_t)nR * nR);
    double sum = 0.0;
    for (int dy = 0; dy <= reach; dy++)
        for (int dx = 0; dx <= reach; dx++) {
            double val = shape64(k, std::sqrt((double)dx * dx + (double)dy * dy));
            v[(size_t)dy * nR + dx] = val;
            sum += val * (dx ? 2.0 : 1.0) * (dy ? 2.0 : 1.0);
        }
    std::vector<double> cw(W), ch(H);
    for (int t = 0; t < W; t++) cw[t] = std::cos(2.0 * M_PI * t / W);
    for (int t = 0; t < H; t++) ch[t] = std::cos(2.0 * M_PI * t / H);
    const int KX = W / 2 + 1, KY = H / 2 + 1;
    std::vector<double> rw((size_t)nR * KX);
    for (int dy = 0; dy <= reach; dy++)
        for (int kx = 0; kx < KX; kx++) {
            double a = v[(size_t)dy * nR];
            for (int dx = 1; dx <= reach; dx++) a += 2.0 * v[(size_t)dy * nR + dx] * cw[((size_t)kx * dx) % W];
            rw[(size_t)dy * KX + kx] = a;
        }
    const double norm = 1.0 / (sum * (double)W * (double)H);
    unsigned nth = threaded ? std::max(1u, std::min(16u, std::thread::hardware_concurrency())) : 1u;
    auto work = [&](unsigned t) {
        for (int kx = (int)t; kx < KX; kx += (int)nth)
            for (int ky = 0; ky < KY; ky++) {
                double a = rw[kx];
                for (int dy = 1; dy <= reach; dy++) a += 2.0 * rw[(size_t)dy * KX + kx] * ch[((size_t)ky * dy) % H];
                out[(size_t)kx * HQ + ky] = (float)(a * norm);
            }
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nth; t++) th.emplace_back(work, t);
    work(0);
    for (auto& t : th) t.join();
}

// f64 sum of f32 shape values over [-reach, reach]^2 as f32 (spectral.rs:75-83), for the radix-2 path.
float kernel_sum_f32(const LeniaKernel& k) {
    int reach;
    switch (k.shape) {
    case LENIA_SHAPE_LENIA: reach = (int)std::ceil(k.radius) + 1; break;
    case LENIA_SHAPE_RING: reach = (int)std::ceil(k.ring_hi) + 1; break;
    default: reach = (int)std::ceil(k.radius) + 2;
    }
    double s = 0.0;
    for (int y = -reach; y <= reach; y++)
        for (int x = -reach; x <= reach; x++) s += (double)(float)shape64(k, (double)std::sqrt((float)(x * x + y * y)));
    return (float)s;
}

int validate(const LeniaWorldDesc& d, int i, int path) {
    if (!supported_side(d.width) || !supported_side(d.height))
        return fail(nullptr, LENIA_ESIZE, "world %d: %ux%u is not supported (sides 2^a or 3*2^a, 32..8192)", i, d.width,
                    d.height);
    if (path == LENIA_PATH_RADIX2 && (!is_pow2(d.width) || !is_pow2(d.height)))
        return fail(nullptr, LENIA_ESIZE, "world %d: FFT grids must be powers of two on the radix-2 path", i);
    if (d.channels < 1 || d.channels > LENIA_MAX_CHANNELS)
        return fail(nullptr, LENIA_EINVAL, "world %d: channels must be 1..%d", i, LENIA_MAX_CHANNELS);
    if (d.nkernels < 1 || d.nkernels > LENIA_MAX_KERNELS)
        return fail(nullptr, LENIA_EINVAL, "world %d: nkernels must be 1..%d", i, LENIA_MAX_KERNELS);
    if (d.rule < 0 || d.rule > 2) return fail(nullptr, LENIA_EINVAL, "world %d: unknown rule %d", i, d.rule);
    if (d.rule != LENIA_RULE_LENIA && (d.channels != 1 || d.nkernels != 2))
        return fail(nullptr, LENIA_EINVAL, "world %d: SmoothLife and MNCA need one channel and two kernels", i);
    if (path == LENIA_PATH_RADIX2 && (d.channels != 1 || d.nkernels > 3))
        return fail(nullptr, LENIA_EINVAL, "world %d: the radix-2 path runs one channel and 1-3 kernels", i);
    if (!(d.dt > 0.0f) && d.rule == LENIA_RULE_LENIA) return fail(nullptr, LENIA_EINVAL, "world %d: dt must be > 0", i);
    for (uint32_t k = 0; k < d.nkernels; k++) {
        const LeniaKernel& kk = d.kernels[k];
        if (kk.shape < 0 || kk.shape > 3) return fail(nullptr, LENIA_EINVAL, "world %d kernel %u: unknown shape", i, k);
        if (kk.src < 0 || kk.src >= (int)d.channels || kk.dst < 0 || kk.dst >= (int)d.channels)
            return fail(nullptr, LENIA_EINVAL, "world %d kernel %u: src/dst channel out of range", i, k);
        if (kk.shape == LENIA_SHAPE_LENIA && (kk.nshells < 1 || kk.nshells > 3 || !(kk.radius > 0.0f)))
            return fail(nullptr, LENIA_EINVAL, "world %d kernel %u: need R > 0 and 1..3 shells", i, k);
        if (kk.shape == LENIA_SHAPE_RING && !(kk.ring_hi > kk.ring_lo && kk.ring_lo >= 0.0f))
            return fail(nullptr, LENIA_EINVAL, "world %d kernel %u: ring needs 0 <= lo < hi", i, k);
        if (d.rule == LENIA_RULE_LENIA && !(kk.sigma > 0.0f))
            return fail(nullptr, LENIA_EINVAL, "world %d kernel %u: sigma must be > 0", i, k);
        // spectral.rs:111-116: the kernel is stored once per torus position, so it must fit.
        if (2 * guard_reach(kk) >= (int)std::min(d.width, d.height))
            return fail(nullptr, LENIA_ESIZE, "world %d kernel %u: world smaller than its kernel", i, k);
    }
    return 0;
}

int world_from_ctx(const LeniaCtx* ctx, int32_t w) { return (w >= 0 && w < (int)ctx->desc.size()) ? 0 : -1; }

size_t state_count(const LeniaWorldDesc& d) { return (size_t)d.channels * d.width * d.height; }

// A world's state changed: its half-spectrum is re-formed by the next flush_spectra.
int refresh_spectrum(LeniaCtx* ctx, int w) {
    if (ctx->path == LENIA_PATH_RADIX2) return 0;
    if (!ctx->dirty[w]) {
        ctx->dirty[w] = 1;
        ctx->ndirty++;
    }
    return 0;
}

// Forward row transforms (state -> half-spectrum) of every changed world: one launch for a size
// class whose worlds all changed, else one launch per changed world.
int flush_spectra(LeniaCtx* ctx) {
    if (ctx->ndirty == 0) return 0;
    for (const SizeClass& cl : ctx->classes) {
        size_t n = 0;
        for (int w : cl.worlds) n += ctx->dirty[w] ? 1 : 0;
        if (n == 0) continue;
        bool ok = true;
        if (n == cl.worlds.size()) {
            ok = launch_row_fp32(cl.W, cl.var_row, MODE_FORWARD, cl.general, ctx->d_worlds, cl.d_row, cl.nrow, cl.planes,
                                 ctx->d_tw, ctx->stream);
        } else {
            for (int w : cl.worlds) {
                if (!ctx->dirty[w]) continue;
                const WorldBuffers& b = ctx->wb[w];
                ok = ok && launch_row_fp32(cl.W, cl.var_row, MODE_FORWARD, cl.general, ctx->d_worlds, b.d_row, b.nrow,
                                           cl.planes, ctx->d_tw, ctx->stream);
            }
        }
        if (!ok) return fail(ctx, LENIA_ECUDA, "row transform launch failed for %dx%d", cl.W, cl.H);
    }
    CK(cudaGetLastError());
    std::fill(ctx->dirty.begin(), ctx->dirty.end(), 0);
    ctx->ndirty = 0;
    return 0;
}

// The column pass of one class (or one world's slice of it).
bool launch_columns(LeniaCtx* ctx, const SizeClass& cl, const ColItem* col, int ncol, const ColItem* tcg, int ntcg,
                    int variant, int var_tc, cudaStream_t s) {
    if (ntcg <= 0) return launch_col_fp32(cl.H, variant, ctx->d_worlds, col, ncol, ctx->d_tw, s);
    // Tensor-core paths: the FP32 items (each channel's first tile group, which holds the packed
    // DC/Nyquist column) are few.  After the tensor-core launch they ran on an otherwise idle GPU
    // (a 4096-point column item takes about as long as a quarter of the whole tensor-core launch),
    // so they run beside it on a side stream, on SMs the persistent tensor-core grid leaves free.
    const int reserve = (ncol + 1) / 2;
    // on a side branch of the step graph the FP32 items follow the tensor-core launch on the branch's
    // own stream: the fork to the context's side stream is the main branch's
    if (ncol <= 0 || reserve > ctx->sms / 16 || s != ctx->stream) {
        const bool ok = launch_col_tc(ctx->tc, ctx->path, cl.H, var_tc, ctx->d_worlds, tcg, ntcg, ctx->d_tw, s);
        return ok && launch_col_fp32(cl.H, variant, ctx->d_worlds, col, ncol, ctx->d_tw, s);
    }
    if (cudaEventRecord(ctx->ev_fork, s) != cudaSuccess || cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0) != cudaSuccess)
        return false;
    bool ok = launch_col_fp32(cl.H, variant, ctx->d_worlds, col, ncol, ctx->d_tw, ctx->side);
    ok = ok && cudaEventRecord(ctx->ev_join, ctx->side) == cudaSuccess;
    ok = ok && launch_col_tc(ctx->tc, ctx->path, cl.H, var_tc, ctx->d_worlds, tcg, ntcg, ctx->d_tw, s, reserve);
    return ok && cudaStreamWaitEvent(s, ctx->ev_join, 0) == cudaSuccess;
}

// The row pass of one step over a run of a class's row items: on the tensor cores where the class
// takes them, else the FP32 pass.
bool launch_rows_step(LeniaCtx* ctx, const SizeClass& cl, int variant, const RowItem* items, int nrow, cudaStream_t s) {
    if (cl.tc_rows) {
        const int st = cl.tc_row_stride, ngroups = st > 0 ? nrow / st : nrow * -st;
        return launch_row_tc(ctx->tc, ctx->path, cl.W, ctx->d_worlds, items, st, ngroups, ctx->d_tw, s);
    }
    return launch_row_fp32(cl.W, variant, MODE_STEP, cl.general, ctx->d_worlds, items, nrow, cl.planes, ctx->d_tw, s);
}

// A launch shape of one size class: launch variants, chunks and the lanes the chunks run on.
struct Shape {
    int var_col, var_row, var_tc;
    const std::vector<Chunk>* chunks;
    int lanes;
};
Shape shape_of(const SizeClass& cl) { return Shape{cl.var_col, cl.var_row, cl.var_tc, &cl.chunks, cl.lanes}; }

// `steps` steps of one size class, chunk after chunk, in the given launch shape; a resident class is
// one launch for all its worlds and steps.
int enqueue_class(LeniaCtx* ctx, const SizeClass& cl, const Shape& sh, int steps, cudaStream_t s) {
    if (cl.persist) {
        const int nw = (int)cl.worlds.size();
        CK(cudaMemsetAsync(cl.d_pctl, 0, persist_ctl_words(nw) * sizeof(int), s));
        if (!launch_persist(cl.W, cl.var_per, ctx->d_worlds, cl.d_col, cl.d_row, nw, cl.ncol / nw, cl.nrow / nw, steps,
                            ctx->d_tw, cl.d_pctl, ctx->d_flags, s))
            return fail(ctx, LENIA_ECUDA, "persistent launch failed (%dx%d)", cl.W, cl.H);
        return 0;
    }
    if (cl.resident) {
        if (!launch_resident(cl.W, cl.var_res, ctx->d_worlds, cl.d_world_ids, (int)cl.worlds.size(), steps, ctx->d_tw,
                             ctx->d_flags, s))
            return fail(ctx, LENIA_ECUDA, "resident launch failed (%dx%d)", cl.W, cl.H);
        return 0;
    }
    // chunks of a class on the main branch may run on concurrent lanes (each lane's chunks one after
    // another); lanes fork from and join into the class's stream
    const int nch = (int)sh.chunks->size();
    const int lanes = (s == ctx->stream && nch > 1) ? std::min(std::min(sh.lanes, nch), LeniaCtx::MAX_LANES) : 1;
    if (lanes > 1) {
        CK(cudaEventRecord(ctx->ev_lfork, s));
        for (int l = 0; l < lanes; l++) CK(cudaStreamWaitEvent(ctx->lane[l], ctx->ev_lfork, 0));
    }
    for (int c = 0; c < nch; c++) {
        const Chunk& ch = (*sh.chunks)[c];
        cudaStream_t on = lanes > 1 ? ctx->lane[c % lanes] : s;
        for (int st = 0; st < steps; st++) {
            bool ok = launch_columns(ctx, cl, cl.d_col + ch.col0, ch.ncol, cl.d_tcg + ch.tcg0, ch.ntcg, sh.var_col,
                                     sh.var_tc, on);
            if (!ok) return fail(ctx, LENIA_ECUDA, "column launch failed (H=%d)", cl.H);
            ok = launch_rows_step(ctx, cl, sh.var_row, cl.d_row + ch.row0, ch.nrow, on);
            if (!ok) return fail(ctx, LENIA_ECUDA, "row launch failed (W=%d)", cl.W);
        }
    }
    if (lanes > 1)
        for (int l = 0; l < lanes; l++) {
            CK(cudaEventRecord(ctx->ev_ljoin[l], ctx->lane[l]));
            CK(cudaStreamWaitEvent(s, ctx->ev_ljoin[l], 0));
        }
    return 0;
}

// Device bytes world w touches in one step: state, half-spectra, convolved spectra, kernel spectra.
size_t world_step_bytes(const LeniaWorldDesc& d) {
    const size_t cells = (size_t)d.width * d.height;
    const size_t spec = cells * 4;  // W/2 x H complex f32
    const size_t conv = (d.channels == 1 && d.nkernels == 1) ? 0 : spec * d.nkernels;
    const size_t khat = (size_t)(d.width / 2 + 1) * khat_stride(d.height) * 4 * d.nkernels;
    return cells * 4 * d.channels + spec * d.channels + conv + khat;
}

// Split a class into runs of consecutive worlds of at most `budget` bytes each, as even in world
// count as the budget allows (budget 0: one chunk).
std::vector<Chunk> make_chunks(const LeniaCtx* ctx, const SizeClass& cl, size_t budget) {
    const int n = (int)cl.worlds.size();
    int nchunks = 1;
    if (budget > 0 && cl.bytes > budget) nchunks = (int)std::min<size_t>((size_t)n, (cl.bytes + budget - 1) / budget);
    std::vector<Chunk> out;
    int col = 0, tcg = 0, row = 0, w = 0;
    for (int c = 0; c < nchunks; c++) {
        const int wend = (int)(((long long)(c + 1) * n) / nchunks);
        Chunk ch;
        ch.col0 = col;
        ch.tcg0 = tcg;
        ch.row0 = row;
        for (; w < wend; w++) {
            const int wi = cl.worlds[w];
            const WorldBuffers& b = ctx->wb[wi];
            ch.ncol += b.ncol;
            ch.ntcg += b.ntcg;
            ch.nrow += b.nrow;
            ch.bytes += world_step_bytes(ctx->desc[wi]);
        }
        col += ch.ncol;
        tcg += ch.ntcg;
        row += ch.nrow;
        if (ch.ncol + ch.ntcg + ch.nrow > 0) out.push_back(ch);
    }
    return out;
}

// Enqueue `steps` steps of every world on the context's streams (captured into graphs).
int enqueue_steps(LeniaCtx* ctx, int steps) {
    if (ctx->path == LENIA_PATH_RADIX2) {
        for (int s = 0; s < steps; s++)
            for (auto& r : ctx->r2) r2_enqueue_step(r, ctx->stream);
        CK(cudaGetLastError());
        return 0;
    }
    // Size classes one after another, and within a class its chunks one after another, each chunk for
    // all its steps: a chunk's states and spectra then stay in L2 across its generations.  Measured on
    // the 384-world batched workload, running every class as its own concurrent graph branch was 6%
    // slower than one after another.  With branch_cells set, the small classes (latency-bound: little
    // work a launch) run one after another on a second branch beside the large ones, whose launches
    // fill the GPU; lenia_autotune decides whether that pays.
    cudaStream_t s = ctx->stream;
    const bool split = ctx->branch_cells > 0;
    int used = 0;  // side branches in use
    if (split) CK(cudaEventRecord(ctx->ev_bfork, s));
    for (auto& cl : ctx->classes) {
        cudaStream_t on = s;
        if (split && (int64_t)cl.W * cl.H <= ctx->branch_cells) {
            const int b = ctx->branch_each ? std::min(used, LeniaCtx::MAX_BRANCHES - 1) : 0;
            if (b >= used) {
                CK(cudaStreamWaitEvent(ctx->branch[b], ctx->ev_bfork, 0));
                used = b + 1;
            }
            on = ctx->branch[b];
        }
        int rc = enqueue_class(ctx, cl, shape_of(cl), steps, on);
        if (rc) return rc;
    }
    for (int b = 0; b < used; b++) {
        CK(cudaEventRecord(ctx->ev_bjoin[b], ctx->branch[b]));
        CK(cudaStreamWaitEvent(s, ctx->ev_bjoin[b], 0));
    }
    CK(cudaGetLastError());
    return 0;
}

int capture(LeniaCtx* ctx, int steps, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_steps(ctx, steps);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(ctx, LENIA_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ctx, LENIA_ECUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    return 0;
}

int rebuild_graphs(LeniaCtx* ctx) {
    if (ctx->graph_big) cudaGraphExecDestroy(ctx->graph_big);
    if (ctx->graph_one) cudaGraphExecDestroy(ctx->graph_one);
    ctx->graph_big = ctx->graph_one = nullptr;
    int rc = capture(ctx, ctx->graph_steps, &ctx->graph_big);
    if (!rc) rc = capture(ctx, 1, &ctx->graph_one);
    return rc;
}

int setup_fused(LeniaCtx* ctx) {
    const int nw = (int)ctx->desc.size();
    ctx->hw.resize(nw);
    ctx->wb.resize(nw);
    // size classes by (W, H)
    for (int i = 0; i < nw; i++) {
        const LeniaWorldDesc& d = ctx->desc[i];
        int found = -1;
        for (size_t c = 0; c < ctx->classes.size(); c++)
            if (ctx->classes[c].W == (int)d.width && ctx->classes[c].H == (int)d.height) found = (int)c;
        if (found < 0) {
            SizeClass cl;
            cl.W = d.width;
            cl.H = d.height;
            ctx->classes.push_back(cl);
            found = (int)ctx->classes.size() - 1;
        }
        ctx->classes[found].worlds.push_back(i);
        ctx->wb[i].cls = found;
    }
    const int smem_max = max_smem_optin();
    // per-world buffers: a sizing pass, one arena, then the same calls carve it
    // every world's state first, back to back in world order (each a multiple of 256 bytes), so
    // that lenia_write_states / lenia_read_states are one copy each
    auto world_buffers = [&](void) -> int {
        for (int i = 0; i < nw; i++) {
            const LeniaWorldDesc& d = ctx->desc[i];
            int rc = dalloc(ctx, &ctx->hw[i].state, (size_t)d.width * d.height * d.channels);
            if (rc) return rc;
        }
        for (int i = 0; i < nw; i++) {
            const LeniaWorldDesc& d = ctx->desc[i];
            DevWorld& w = ctx->hw[i];
            int rc;
            if ((rc = dalloc(ctx, &w.spec, spec_elems(d.width, d.height) * d.channels))) return rc;
            if (d.channels == 1 && d.nkernels == 1) w.conv = w.spec;
            else if ((rc = dalloc(ctx, &w.conv, spec_elems(d.width, d.height) * d.nkernels))) return rc;
            float* kh;
            if ((rc = dalloc(ctx, &kh, (size_t)(d.width / 2 + 1) * khat_stride(d.height) * d.nkernels))) return rc;
            w.khat = kh;
        }
        return 0;
    };
    ctx->sizing = true;
    int rc0 = world_buffers();
    ctx->sizing = false;
    if (rc0) return rc0;
    {
        void* a = nullptr;
        cudaError_t e = cudaMalloc(&a, ctx->arena_need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, LENIA_ENOMEM, "device allocation of %zu bytes failed: %s", ctx->arena_need,
                        cudaGetErrorString(e));
        }
        ctx->allocs.push_back(a);
        ctx->arena = (char*)a;
    }
    if ((rc0 = world_buffers())) return rc0;
    // kernel spectra in FP64 on the host, in parallel across (world, kernel) pairs
    std::vector<std::pair<int, int>> jobs;
    size_t khat_total = 0;
    std::vector<size_t> khat_off(nw + 1, 0);
    for (int i = 0; i < nw; i++) {
        const LeniaWorldDesc& d = ctx->desc[i];
        khat_off[i] = khat_total;
        khat_total += (size_t)(d.width / 2 + 1) * khat_stride(d.height) * d.nkernels;
        for (uint32_t k = 0; k < d.nkernels; k++) jobs.push_back({i, (int)k});
    }
    std::vector<float> khat_host(khat_total, 0.0f);
    {
        const unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        std::atomic<size_t> next(0);
        auto worker = [&]() {
            for (size_t j = next++; j < jobs.size(); j = next++) {
                const LeniaWorldDesc& d = ctx->desc[jobs[j].first];
                const size_t khn = (size_t)(d.width / 2 + 1) * khat_stride(d.height);
                compute_khat(d.kernels[jobs[j].second], d.width, d.height, khat_stride(d.height),
                             khat_host.data() + khat_off[jobs[j].first] + khn * jobs[j].second, jobs.size() < nth);
            }
        };
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nth && t < jobs.size(); t++) th.emplace_back(worker);
        worker();
        for (auto& t : th) t.join();
    }
    for (int i = 0; i < nw; i++) {
        const LeniaWorldDesc& d = ctx->desc[i];
        DevWorld& w = ctx->hw[i];
        w.W = d.width;
        w.H = d.height;
        w.C = d.channels;
        w.K = d.nkernels;
        w.rule = d.rule;
        w.dt = d.dt;
        w.HQ = khat_stride(d.height);
        w.u_out = nullptr;
        for (uint32_t k = 0; k < d.nkernels; k++) {
            const LeniaKernel& kk = d.kernels[k];
            w.kern[k].src = kk.src;
            w.kern[k].dst = kk.dst;
            w.kern[k].mu = kk.mu;
            w.kern[k].sigma = kk.sigma;
            w.kern[k].weight = kk.weight;
        }
    }
    CK(cudaMemsetAsync(ctx->arena, 0, ctx->arena_need, ctx->stream));
    for (int i = 0; i < nw; i++) {
        const LeniaWorldDesc& d = ctx->desc[i];
        const size_t khn = (size_t)(d.width / 2 + 1) * khat_stride(d.height) * d.nkernels;
        CK(cudaMemcpyAsync((float*)ctx->hw[i].khat, khat_host.data() + khat_off[i], khn * sizeof(float),
                           cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    int rc;
    if ((rc = dalloc(ctx, &ctx->d_worlds, nw))) return rc;
    CK(cudaMemcpy(ctx->d_worlds, ctx->hw.data(), nw * sizeof(DevWorld), cudaMemcpyHostToDevice));
    // work lists
    const bool tc_path = ctx->path == LENIA_PATH_TF32 || ctx->path == LENIA_PATH_BF16X3;
    for (auto& cl : ctx->classes) {
        std::vector<ColItem> col, tcg;
        std::vector<RowItem> row;
        // a class takes the general step when any of its worlds needs it; every row launch of the class
        // then uses the general build, whose items are two rows each from W = 2048 up
        int general = 0;
        for (int wi : cl.worlds) {
            const LeniaWorldDesc& d = ctx->desc[wi];
            if (!(d.channels == 1 && d.nkernels == 1 && d.rule == LENIA_RULE_LENIA)) general = 1;
        }
        const int planes = general;  // the general step's one shared-memory plane
        const uint32_t item_rows = (uint32_t)row_item_rows(cl.W, general);
        // tensor-core groups of CT columns, except the first group of every channel: column 0
        // packs the DC and Nyquist columns, which the FP32 pass pairs up (ky with H - ky)
        const bool use_tc = tc_path && tc_supports(cl.H);
        const int tpg = use_tc ? tc_columns_per_group(cl.H) / TC : 0;
        for (int wi : cl.worlds) {
            const LeniaWorldDesc& d = ctx->desc[wi];
            const int first_col = (int)col.size(), first_row = (int)row.size(), first_tcg = (int)tcg.size();
            // FP32 column items: one per (channel tile, kernel reading that channel); the tensor-core
            // groups cover every kernel of a channel in one item
            for (uint32_t c = 0; c < d.channels; c++) {
                const int ntiles = spec_tiles(d.width);
                const bool tc_here = use_tc && ntiles % tpg == 0;
                bool read = false;
                for (uint32_t k = 0; k < d.nkernels; k++) {
                    if (d.kernels[k].src != (int)c) continue;
                    read = true;
                    for (int t = 0; t < (tc_here ? tpg : ntiles); t++) col.push_back(ColItem{wi, (int)c, t, (int)k});
                }
                if (read && tc_here)
                    for (int t = tpg; t < ntiles; t += tpg) tcg.push_back(ColItem{wi, (int)c, t, 0});
            }
            // Lenia: one row item per target channel (its kernels, update and forward transform), so a
            // multichannel world has C times the row items; other rules: one item for every channel
            const uint32_t split = d.rule == LENIA_RULE_LENIA ? d.channels : 1;
            for (uint32_t r = 0; r < d.height; r += item_rows)
                for (uint32_t c = 0; c < split; c++) row.push_back(RowItem{wi, (int)r, (int)c, 0});
            WorldBuffers& b = ctx->wb[wi];
            b.ncol = (int)col.size() - first_col;
            b.nrow = (int)row.size() - first_row;
            b.ntcg = (int)tcg.size() - first_tcg;
        }
        if ((int)col_smem_bytes(cl.H) > smem_max || (int)row_smem_bytes(cl.W, planes) > smem_max)
            return fail(ctx, LENIA_ESIZE, "%dx%d with %d planes needs more shared memory than a CTA has", cl.W, cl.H,
                        planes);
        cl.general = general;
        cl.planes = planes;
        // Default launch variant: the 64-register form (more resident CTAs) unless it spills more
        // than 128 bytes a thread and the 128-register form spills less than half as much.  Columns
        // of 4096 and more take the paired build (measured 8% faster at 4096 x 4096; at 128 to 1024
        // the scalar builds were faster); the autotuner times all three.
        auto pick = [](int v0, int v1) { return (v0 > 128 && v1 >= 0 && v1 < v0 / 2) ? 1 : 0; };
        cl.var_col = cl.H >= 4096 ? 2 : pick(fp32_local_bytes(0, cl.H, 0), fp32_local_bytes(0, cl.H, 1));
        const int g2 = general ? 2 : 0;
        cl.var_row = pick(fp32_local_bytes(1, cl.W, g2), fp32_local_bytes(1, cl.W, 1 | g2));
        cl.ncol = (int)col.size();
        cl.nrow = (int)row.size();
        cl.ntcg = (int)tcg.size();
        if ((rc = dalloc(ctx, &cl.d_col, col.size()))) return rc;
        if ((rc = dalloc(ctx, &cl.d_row, row.size()))) return rc;
        if ((rc = dalloc(ctx, &cl.d_tcg, tcg.size()))) return rc;
        CK(cudaMemcpy(cl.d_col, col.data(), col.size() * sizeof(ColItem), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(cl.d_row, row.data(), row.size() * sizeof(RowItem), cudaMemcpyHostToDevice));
        if (!tcg.empty()) CK(cudaMemcpy(cl.d_tcg, tcg.data(), tcg.size() * sizeof(ColItem), cudaMemcpyHostToDevice));
        if (use_tc) {
            int trc = tc_prepare_size(ctx->tc, ctx->path, cl.H, &ctx->err);
            if (trc) return trc;
        }
        // the tensor-core row pass, where the class's worlds all take the one-kernel Lenia step and
        // their heights are whole groups of its rows
        if (tc_path && !general && tc_row_supports(cl.W)) {
            const int rg = tc_row_group_rows(cl.W);
            bool fits = rg % (int)item_rows == 0 || (int)item_rows % rg == 0;
            for (int wi : cl.worlds) fits = fits && ctx->desc[wi].height % rg == 0;
            if (fits) {
                int trc = tc_row_prepare(ctx->tc, ctx->path, cl.W, &ctx->err);
                if (trc) return trc;
                // groups of rg rows: several items a group, or several groups an item (negative)
                cl.tc_row_stride = rg >= (int)item_rows ? rg / (int)item_rows : -((int)item_rows / rg);
                cl.tc_rows_ok = 1;
                cl.tc_rows = TC_ROWS_DEFAULT;
            }
        }
        // per-world slices of the class lists
        size_t co = 0, ro = 0, go = 0;
        cl.bytes = 0;
        for (int wi : cl.worlds) {
            WorldBuffers& b = ctx->wb[wi];
            b.d_col = cl.d_col + co;
            b.d_row = cl.d_row + ro;
            b.d_tcg = cl.d_tcg + go;
            co += b.ncol;
            ro += b.nrow;
            go += b.ntcg;
            cl.bytes += world_step_bytes(ctx->desc[wi]);
        }
        cl.chunk_budget = DEFAULT_CHUNK_BUDGET;
        cl.lanes = DEFAULT_LANES;
        cl.chunks = make_chunks(ctx, cl, cl.chunk_budget);
        // the cluster-resident step: square one-channel, one-kernel Lenia worlds of 128..512 on the
        // FP32 path, where the GPU can hold at least one of its clusters
        if (ctx->path == LENIA_PATH_FP32 && !general && cl.W == cl.H && resident_supported(cl.W)) {
            cl.var_res = -1;
            for (int v = 0; v < RESIDENT_VARIANTS; v++) {
                cl.res_fits[v] = resident_clusters_that_fit(cl.W, v);
                if (cl.res_fits[v] > 0 && cl.var_res < 0) cl.var_res = v;
            }
            cudaGetLastError();
            if (cl.var_res >= 0) {
                if ((rc = dalloc(ctx, &cl.d_world_ids, cl.worlds.size()))) return rc;
                CK(cudaMemcpy(cl.d_world_ids, cl.worlds.data(), cl.worlds.size() * sizeof(int), cudaMemcpyHostToDevice));
                cl.resident_ok = 1;
                cl.resident = RESIDENT_DEFAULT;
            } else {
                cl.var_res = 0;
            }
        }
        // the persistent step: square one-channel, one-kernel Lenia worlds on the FP32 path, every world of
        // the class with the same number of column and row items
        if (ctx->path == LENIA_PATH_FP32 && !general && cl.W == cl.H && persist_supported(cl.W)) {
            const int nw = (int)cl.worlds.size();
            bool even = cl.ncol % nw == 0 && cl.nrow % nw == 0;
            for (int wi : cl.worlds) even = even && ctx->wb[wi].ncol == cl.ncol / nw && ctx->wb[wi].nrow == cl.nrow / nw;
            int cap0 = 0, cap1 = 0;
            if (even &&
                launch_persist(cl.W, 0, ctx->d_worlds, cl.d_col, cl.d_row, 0, 0, 0, 0, ctx->d_tw, nullptr, nullptr,
                               ctx->stream, &cap0) &&
                launch_persist(cl.W, 1, ctx->d_worlds, cl.d_col, cl.d_row, 0, 0, 0, 0, ctx->d_tw, nullptr, nullptr,
                               ctx->stream, &cap1) &&
                cap0 > 0 && cap1 > 0) {
                if ((rc = dalloc(ctx, &cl.d_pctl, (size_t)persist_ctl_words(nw)))) return rc;
                cl.persist_ok = 1;
                cl.persist = PERSIST_DEFAULT;
            }
            cudaGetLastError();
        }
        // zero-item launches only set each kernel's shared-memory limit, outside any capture
        for (int v = 0; v < COL_VARIANTS; v++)
            if (!launch_col_fp32(cl.H, v, ctx->d_worlds, cl.d_col, 0, ctx->d_tw, ctx->stream))
                return fail(ctx, LENIA_ECUDA, "cannot configure launches for %dx%d", cl.W, cl.H);
        for (int v = 0; v < 2; v++)
            if (!launch_row_fp32(cl.W, v, MODE_STEP, cl.general, ctx->d_worlds, cl.d_row, 0, cl.planes, ctx->d_tw,
                                 ctx->stream))
                return fail(ctx, LENIA_ECUDA, "cannot configure launches for %dx%d", cl.W, cl.H);
        for (int v = 0; v < TC_COL_VARIANTS && cl.ntcg > 0; v++)
            if (!launch_col_tc(ctx->tc, ctx->path, cl.H, v, ctx->d_worlds, cl.d_tcg, 0, ctx->d_tw, ctx->stream))
                return fail(ctx, LENIA_ECUDA, "cannot configure the tensor-core pass for H=%d", cl.H);
        if (cl.tc_rows_ok &&
            !launch_row_tc(ctx->tc, ctx->path, cl.W, ctx->d_worlds, cl.d_row, cl.tc_row_stride, 0, ctx->d_tw, ctx->stream))
            return fail(ctx, LENIA_ECUDA, "cannot configure the tensor-core row pass for W=%d", cl.W);
    }
    return 0;
}

int setup_radix2(LeniaCtx* ctx) {
    const int nw = (int)ctx->desc.size();
    ctx->r2.resize(nw);
    for (int i = 0; i < nw; i++) {
        const LeniaWorldDesc& d = ctx->desc[i];
        R2World& r = ctx->r2[i];
        memset(&r, 0, sizeof(r));
        r.w = d.width;
        r.h = d.height;
        r.k = d.nkernels;
        r.rule = d.rule;
        r.mu = d.kernels[0].mu;
        r.sigma = d.kernels[0].sigma;
        r.dt = d.dt;
        const size_t n = (size_t)r.w * r.h;
        int rc;
        if ((rc = dalloc(ctx, &r.state, n))) return rc;
        if ((rc = dalloc(ctx, &r.work[0], n))) return rc;
        if ((rc = dalloc(ctx, &r.work[1], n))) return rc;
        if ((rc = dalloc(ctx, &r.spec, n))) return rc;
        R2Shape shapes[3];
        float sums[3];
        for (int k = 0; k < r.k; k++) {
            if ((rc = dalloc(ctx, &r.kern[k], n))) return rc;
            if ((rc = dalloc(ctx, &r.conv[k], n))) return rc;
            const LeniaKernel& kk = d.kernels[k];
            shapes[k] = R2Shape{kk.shape, kk.radius, kk.nshells, {kk.beta[0], kk.beta[1], kk.beta[2]}, kk.ring_lo, kk.ring_hi};
            sums[k] = kernel_sum_f32(kk);
        }
        CK(cudaMemset(r.state, 0, n * sizeof(float)));
        r2_enqueue_kernel_spectra(r, shapes, sums, ctx->stream);
        CK(cudaGetLastError());
    }
    // the stats kernel reads states through a world table
    ctx->hw.resize(nw);
    for (int i = 0; i < nw; i++) {
        DevWorld& w = ctx->hw[i];
        memset(&w, 0, sizeof(w));
        w.W = ctx->r2[i].w;
        w.H = ctx->r2[i].h;
        w.C = 1;
        w.K = ctx->r2[i].k;
        w.state = ctx->r2[i].state;
    }
    int rc;
    if ((rc = dalloc(ctx, &ctx->d_worlds, nw))) return rc;
    CK(cudaMemcpy(ctx->d_worlds, ctx->hw.data(), nw * sizeof(DevWorld), cudaMemcpyHostToDevice));
    return 0;
}

float* state_ptr(LeniaCtx* ctx, int w) { return ctx->path == LENIA_PATH_RADIX2 ? ctx->r2[w].state : ctx->hw[w].state; }

// Device time of `steps` steps of one size class in the graph's order (chunk after chunk, each for
// all its steps), split into its column and row launches: events around every launch, one
// synchronisation at the end.  var_col / var_row / chunks as given (the autotuner's candidates).
struct EventList {
    std::vector<cudaEvent_t> e;
    ~EventList() {
        for (cudaEvent_t x : e) cudaEventDestroy(x);
    }
};
int time_class(LeniaCtx* ctx, const SizeClass& cl, const Shape& sh, int steps, double* col_ms, double* row_ms) {
    if (cl.resident || cl.persist) {
        // one launch: its whole time is reported as the column share
        Events ev;
        CK(cudaEventCreate(&ev.e[0]));
        CK(cudaEventCreate(&ev.e[1]));
        CK(cudaEventRecord(ev.e[0], ctx->stream));
        int rc = enqueue_class(ctx, cl, sh, steps, ctx->stream);
        CK(cudaEventRecord(ev.e[1], ctx->stream));
        if (rc) return rc;
        CK(cudaEventSynchronize(ev.e[1]));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ev.e[0], ev.e[1]));
        *col_ms = ms;
        *row_ms = 0;
        return 0;
    }
    const std::vector<Chunk>& chunks = *sh.chunks;
    EventList ev;
    const size_t n = 1 + 2 * chunks.size() * (size_t)steps;
    ev.e.reserve(n);
    for (size_t i = 0; i < n; i++) {
        cudaEvent_t x;
        CK(cudaEventCreate(&x));
        ev.e.push_back(x);
    }
    size_t k = 0;
    CK(cudaEventRecord(ev.e[k++], ctx->stream));
    for (const Chunk& ch : chunks) {
        for (int st = 0; st < steps; st++) {
            bool ok = launch_columns(ctx, cl, cl.d_col + ch.col0, ch.ncol, cl.d_tcg + ch.tcg0, ch.ntcg, sh.var_col,
                                     sh.var_tc, ctx->stream);
            CK(cudaEventRecord(ev.e[k++], ctx->stream));
            ok = ok && launch_rows_step(ctx, cl, sh.var_row, cl.d_row + ch.row0, ch.nrow, ctx->stream);
            CK(cudaEventRecord(ev.e[k++], ctx->stream));
            if (!ok) {
                cudaStreamSynchronize(ctx->stream);
                cudaGetLastError();
                return fail(ctx, LENIA_ECUDA, "launch failed for %dx%d", cl.W, cl.H);
            }
        }
    }
    CK(cudaEventSynchronize(ev.e[k - 1]));
    double c = 0, r = 0;
    for (size_t i = 1; i < k; i += 2) {
        float a = 0, b = 0;
        CK(cudaEventElapsedTime(&a, ev.e[i - 1], ev.e[i]));
        CK(cudaEventElapsedTime(&b, ev.e[i], ev.e[i + 1]));
        c += a;
        r += b;
    }
    *col_ms = c;
    *row_ms = r;
    return 0;
}

// Device time of `steps` steps of one size class as the step graph runs them: the class's launches in
// `sh` captured into a graph, replayed once to warm up and once under events.  (Events around every
// launch, as in time_class, leave the GPU idle between small launches that a graph replays back to
// back, which would favour the one-launch resident step.)
template <class Enqueue>
int time_graph(LeniaCtx* ctx, Enqueue enqueue, double* ms) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue();
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : fail(ctx, LENIA_ECUDA, "autotune capture failed: %s", cudaGetErrorString(e));
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ctx, LENIA_ECUDA, "autotune instantiate failed: %s", cudaGetErrorString(e));
    Events ev;
    float t = 0;
    e = cudaEventCreate(&ev.e[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev.e[1]);
    if (e == cudaSuccess) e = cudaGraphLaunch(ge, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev.e[0], ctx->stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(ge, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev.e[1], ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev.e[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev.e[0], ev.e[1]);
    cudaGraphExecDestroy(ge);
    if (e != cudaSuccess) return fail(ctx, LENIA_ECUDA, "autotune timing failed: %s", cudaGetErrorString(e));
    *ms = t;
    return 0;
}

int time_class_graph(LeniaCtx* ctx, const SizeClass& cl, const Shape& sh, int steps, double* ms) {
    return time_graph(ctx, [&]() { return enqueue_class(ctx, cl, sh, steps, ctx->stream); }, ms);
}

// The device-side error flags of the context's kernels: the tensor-core passes' and the resident
// step's (set when a bounded barrier wait gave up).  Reading them synchronises with the device.
int check_device_errors(LeniaCtx* ctx) {
    int rc = tc_check_error(ctx->tc, &ctx->err);
    if (rc || !ctx->d_flags) return rc;
    int h = 0;
    CK(cudaMemcpy(&h, ctx->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        CK(cudaMemset(ctx->d_flags, 0, sizeof(int)));
        return fail(ctx, LENIA_ECUDA,
                    "a cluster-resident or persistent step gave up waiting on another CTA; results of that step are invalid");
    }
    return 0;
}

}  // namespace

void lenia::set_thread_error(const std::string& msg) { g_create_error = msg; }

extern "C" {

const char* lenia_last_error(const LeniaCtx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->err.c_str();
}

int lenia_create(const LeniaWorldDesc* worlds, int32_t nworlds, int32_t path, LeniaCtx** out) {
    if (!out) return fail(nullptr, LENIA_EINVAL, "out is NULL");
    *out = nullptr;
    if (!worlds || nworlds < 1) return fail(nullptr, LENIA_EINVAL, "need at least one world");
    if (path < LENIA_PATH_FP32 || path > LENIA_PATH_RADIX2) return fail(nullptr, LENIA_EINVAL, "unknown path %d", path);
    for (int i = 0; i < nworlds; i++) {
        int rc = validate(worlds[i], i, path);
        if (rc) return rc;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(nullptr, LENIA_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return fail(nullptr, LENIA_ENODEV, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
    if (prop.major != 10 || prop.minor != 3)
        return fail(nullptr, LENIA_ENODEV, "built for sm_103a (GB300); device is sm_%d%d", prop.major, prop.minor);

    LeniaCtx* ctx = new LeniaCtx();
    ctx->device = dev;
    ctx->path = path;
    ctx->desc.assign(worlds, worlds + nworlds);
    int rc = 0;
    auto bail = [&](int code) {
        std::string msg = ctx->err;
        lenia_destroy(ctx);
        g_create_error = msg;
        return code;
    };
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_bfork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->up, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->down, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_in_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_in_free, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_out_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_out_free, cudaEventDisableTiming) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess) {
        fail(ctx, LENIA_ECUDA, "stream creation failed");
        return bail(LENIA_ECUDA);
    }
    for (int b = 0; b < LeniaCtx::MAX_BRANCHES; b++)
        if (cudaStreamCreateWithFlags(&ctx->branch[b], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_bjoin[b], cudaEventDisableTiming) != cudaSuccess) {
            fail(ctx, LENIA_ECUDA, "stream creation failed");
            return bail(LENIA_ECUDA);
        }
    if (cudaEventCreateWithFlags(&ctx->ev_lfork, cudaEventDisableTiming) != cudaSuccess) {
        fail(ctx, LENIA_ECUDA, "stream creation failed");
        return bail(LENIA_ECUDA);
    }
    for (int l = 0; l < LeniaCtx::MAX_LANES; l++)
        if (cudaStreamCreateWithFlags(&ctx->lane[l], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_ljoin[l], cudaEventDisableTiming) != cudaSuccess) {
            fail(ctx, LENIA_ECUDA, "stream creation failed");
            return bail(LENIA_ECUDA);
        }
    // twiddles exp(-2 pi i t / TWN) from FP64
    {
        std::vector<float2> tw(lfft::TWN);
        for (int t = 0; t < lfft::TWN; t++) {
            double a = -2.0 * M_PI * (double)t / (double)lfft::TWN;
            tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        if ((rc = dalloc(ctx, &ctx->d_tw, tw.size()))) return bail(rc);
        if (cudaMemcpy(ctx->d_tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) {
            fail(ctx, LENIA_ECUDA, "twiddle upload failed");
            return bail(LENIA_ECUDA);
        }
    }
    if (path == LENIA_PATH_TF32 || path == LENIA_PATH_BF16X3) {
        rc = tc_setup(ctx->tc, path, &ctx->err);
        if (rc) return bail(rc);
    }
    ctx->dirty.assign(nworlds, 0);
    rc = (path == LENIA_PATH_RADIX2) ? setup_radix2(ctx) : setup_fused(ctx);
    if (rc) return bail(rc);
    if (path != LENIA_PATH_RADIX2) {
        // the states were carved back to back from the arena (checked, not assumed)
        bool packed = true;
        size_t off = 0;
        for (int w = 0; w < nworlds; w++) {
            packed = packed && ctx->hw[w].state == ctx->hw[0].state + off;
            off += state_count(ctx->desc[w]);
        }
        if (packed) ctx->states = ctx->hw[0].state, ctx->states_count = off;
    }
    if ((rc = dalloc(ctx, &ctx->d_stats, 3 * (size_t)nworlds))) return bail(rc);
    // [0] the device error flag, [1] the persistent step's wait limit + 1 (lenia_persist_set_wait_limit)
    if ((rc = dalloc(ctx, &ctx->d_flags, 2))) return bail(rc);
    if (cudaMemset(ctx->d_flags, 0, 2 * sizeof(int)) != cudaSuccess) {
        fail(ctx, LENIA_ECUDA, "flag initialisation failed");
        return bail(LENIA_ECUDA);
    }
    if ((rc = rebuild_graphs(ctx))) return bail(rc);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        fail(ctx, LENIA_ECUDA, "initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
        return bail(LENIA_ECUDA);
    }
    *out = ctx;
    return 0;
}

int lenia_destroy(LeniaCtx* ctx) {
    if (!ctx) return 0;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->up) cudaStreamSynchronize(ctx->up);
    if (ctx->down) cudaStreamSynchronize(ctx->down);
    if (ctx->graph_big) cudaGraphExecDestroy(ctx->graph_big);
    if (ctx->graph_one) cudaGraphExecDestroy(ctx->graph_one);
    tc_release(ctx->tc);
    for (void* p : ctx->allocs) cudaFree(p);
    for (cudaEvent_t e : {ctx->ev_in_ready, ctx->ev_in_free, ctx->ev_out_ready, ctx->ev_out_free})
        if (e) cudaEventDestroy(e);
    if (ctx->up) cudaStreamDestroy(ctx->up);
    if (ctx->down) cudaStreamDestroy(ctx->down);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    for (int b = 0; b < LeniaCtx::MAX_BRANCHES; b++) {
        if (ctx->branch[b]) cudaStreamSynchronize(ctx->branch[b]), cudaStreamDestroy(ctx->branch[b]);
        if (ctx->ev_bjoin[b]) cudaEventDestroy(ctx->ev_bjoin[b]);
    }
    if (ctx->ev_bfork) cudaEventDestroy(ctx->ev_bfork);
    for (int l = 0; l < LeniaCtx::MAX_LANES; l++) {
        if (ctx->lane[l]) cudaStreamSynchronize(ctx->lane[l]), cudaStreamDestroy(ctx->lane[l]);
        if (ctx->ev_ljoin[l]) cudaEventDestroy(ctx->ev_ljoin[l]);
    }
    if (ctx->ev_lfork) cudaEventDestroy(ctx->ev_lfork);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return 0;
}

int lenia_write_state(LeniaCtx* ctx, int32_t world, const float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (!host || count != state_count(ctx->desc[world]))
        return fail(ctx, LENIA_EINVAL, "state of world %d has %zu values, got %zu", world, state_count(ctx->desc[world]),
                    count);
    CK(cudaMemcpyAsync(state_ptr(ctx, world), host, count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    return refresh_spectrum(ctx, world);
}

int lenia_write_state_device(LeniaCtx* ctx, int32_t world, const float* dev, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (!dev || count != state_count(ctx->desc[world])) return fail(ctx, LENIA_EINVAL, "bad count for world %d", world);
    CK(cudaMemcpyAsync(state_ptr(ctx, world), dev, count * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    return refresh_spectrum(ctx, world);
}

int lenia_read_state(LeniaCtx* ctx, int32_t world, float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (!host || count != state_count(ctx->desc[world])) return fail(ctx, LENIA_EINVAL, "bad count for world %d", world);
    CK(cudaMemcpyAsync(host, state_ptr(ctx, world), count * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return check_device_errors(ctx);
}

int lenia_read_state_device(LeniaCtx* ctx, int32_t world, float* dev, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (!dev || count != state_count(ctx->desc[world])) return fail(ctx, LENIA_EINVAL, "bad count for world %d", world);
    CK(cudaMemcpyAsync(dev, state_ptr(ctx, world), count * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    return 0;
}

int lenia_write_states(LeniaCtx* ctx, const float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    size_t total = 0;
    for (const auto& d : ctx->desc) total += state_count(d);
    if (!host || count != total) return fail(ctx, LENIA_EINVAL, "the worlds hold %zu state values, got %zu", total, count);
    if (ctx->states) {
        CK(cudaMemcpyAsync(ctx->states, host, count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    } else {
        size_t off = 0;
        for (size_t w = 0; w < ctx->desc.size(); w++) {
            const size_t n = state_count(ctx->desc[w]);
            CK(cudaMemcpyAsync(state_ptr(ctx, (int)w), host + off, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
            off += n;
        }
    }
    for (size_t w = 0; w < ctx->desc.size(); w++) refresh_spectrum(ctx, (int)w);
    return 0;
}

int lenia_read_states(LeniaCtx* ctx, float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    size_t total = 0;
    for (const auto& d : ctx->desc) total += state_count(d);
    if (!host || count != total) return fail(ctx, LENIA_EINVAL, "the worlds hold %zu state values, got %zu", total, count);
    if (ctx->states) {
        CK(cudaMemcpyAsync(host, ctx->states, count * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    } else {
        size_t off = 0;
        for (size_t w = 0; w < ctx->desc.size(); w++) {
            const size_t n = state_count(ctx->desc[w]);
            CK(cudaMemcpyAsync(host + off, state_ptr(ctx, (int)w), n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
            off += n;
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return check_device_errors(ctx);
}

// Asynchronous whole-context state copies.  The host copy runs on the upload (download) stream
// into (out of) a device staging buffer; the compute stream moves the staging buffer into (or out of) the
// states with one device-to-device copy, in stream order with the steps.  So the upload of the
// next input and the download of the last result overlap the generations in between.
static int states_async_check(LeniaCtx* ctx, const void* host, size_t count) {
    size_t total = 0;
    for (const auto& d : ctx->desc) total += state_count(d);
    if (!host || count != total) return fail(ctx, LENIA_EINVAL, "the worlds hold %zu state values, got %zu", total, count);
    if (!ctx->states) return fail(ctx, LENIA_EINVAL, "asynchronous state copies need the fused paths' state arena");
    return 0;
}

int lenia_write_states_async(LeniaCtx* ctx, const float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    int rc = states_async_check(ctx, host, count);
    if (rc) return rc;
    if (!ctx->stage_in && (rc = dalloc(ctx, &ctx->stage_in, count))) return rc;
    const size_t bytes = count * sizeof(float);
    CK(cudaStreamWaitEvent(ctx->up, ctx->ev_in_free, 0));  // the previous input has left the buffer
    CK(cudaMemcpyAsync(ctx->stage_in, host, bytes, cudaMemcpyHostToDevice, ctx->up));
    CK(cudaEventRecord(ctx->ev_in_ready, ctx->up));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_in_ready, 0));
    CK(cudaMemcpyAsync(ctx->states, ctx->stage_in, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->ev_in_free, ctx->stream));
    for (size_t w = 0; w < ctx->desc.size(); w++) refresh_spectrum(ctx, (int)w);
    return 0;
}

int lenia_read_states_async(LeniaCtx* ctx, float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    int rc = states_async_check(ctx, host, count);
    if (rc) return rc;
    if (!ctx->stage_out && (rc = dalloc(ctx, &ctx->stage_out, count))) return rc;
    const size_t bytes = count * sizeof(float);
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_out_free, 0));  // the previous result has left the buffer
    CK(cudaMemcpyAsync(ctx->stage_out, ctx->states, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->ev_out_ready, ctx->stream));
    CK(cudaStreamWaitEvent(ctx->down, ctx->ev_out_ready, 0));
    CK(cudaMemcpyAsync(host, ctx->stage_out, bytes, cudaMemcpyDeviceToHost, ctx->down));
    CK(cudaEventRecord(ctx->ev_out_free, ctx->down));
    return 0;
}

int lenia_step(LeniaCtx* ctx, uint32_t steps) {
    if (!ctx) return LENIA_EINVAL;
    int frc = flush_spectra(ctx);
    if (frc) return frc;
    uint32_t full = steps / ctx->graph_steps, rem = steps % ctx->graph_steps;
    for (uint32_t i = 0; i < full; i++) CK(cudaGraphLaunch(ctx->graph_big, ctx->stream));
    for (uint32_t i = 0; i < rem; i++) CK(cudaGraphLaunch(ctx->graph_one, ctx->stream));
    ctx->tick += steps;
    return 0;
}

int lenia_step_timed(LeniaCtx* ctx, uint32_t steps, float* ms) {
    if (!ctx || !ms) return LENIA_EINVAL;
    int frc = flush_spectra(ctx);  // outside the timed region
    if (frc) return frc;
    Events ev;
    CK(cudaEventCreate(&ev.e[0]));
    CK(cudaEventCreate(&ev.e[1]));
    CK(cudaEventRecord(ev.e[0], ctx->stream));
    int rc = lenia_step(ctx, steps);
    CK(cudaEventRecord(ev.e[1], ctx->stream));
    CK(cudaEventSynchronize(ev.e[1]));
    CK(cudaEventElapsedTime(ms, ev.e[0], ev.e[1]));
    if (!rc) rc = check_device_errors(ctx);
    return rc;
}

int lenia_sync(LeniaCtx* ctx) {
    if (!ctx) return LENIA_EINVAL;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaStreamSynchronize(ctx->up));
    CK(cudaStreamSynchronize(ctx->down));
    int rc = check_device_errors(ctx);
    return rc;
}

int lenia_tick(const LeniaCtx* ctx, uint64_t* tick) {
    if (!ctx || !tick) return LENIA_EINVAL;
    *tick = ctx->tick;
    return 0;
}

int lenia_seed_patches(LeniaCtx* ctx, int32_t world, uint32_t seed, const int32_t* patches, int32_t npatches) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (npatches < 0 || npatches > 4096 || (npatches > 0 && !patches))
        return fail(ctx, LENIA_EINVAL, "npatches must be 0..4096");
    const LeniaWorldDesc& d = ctx->desc[world];
    int4* dp = nullptr;
    CK(cudaMallocAsync((void**)&dp, std::max(1, npatches) * sizeof(int4), ctx->stream));
    if (npatches) CK(cudaMemcpyAsync(dp, patches, npatches * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
    for (uint32_t c = 0; c < d.channels; c++)
        launch_seed_patches(state_ptr(ctx, world) + (size_t)c * d.width * d.height, d.width, d.height, seed + c, dp,
                            npatches, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaFreeAsync(dp, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return refresh_spectrum(ctx, world);
}

int lenia_seed_tiles(LeniaCtx* ctx, int32_t world, uint32_t seed, const float* pattern, int32_t pw, int32_t ph,
                     int32_t spacing) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (!pattern || pw < 1 || ph < 1 || pw != ph || spacing < pw || pw > 1024)
        return fail(ctx, LENIA_EINVAL, "pattern must be square, 1..1024 cells, and fit in its tile");
    const LeniaWorldDesc& d = ctx->desc[world];
    float* dp = nullptr;
    CK(cudaMallocAsync((void**)&dp, (size_t)pw * ph * sizeof(float), ctx->stream));
    CK(cudaMemcpyAsync(dp, pattern, (size_t)pw * ph * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    for (uint32_t c = 0; c < d.channels; c++)
        launch_seed_tiles(state_ptr(ctx, world) + (size_t)c * d.width * d.height, d.width, d.height, seed + c, dp, pw, ph,
                          spacing, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaFreeAsync(dp, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return refresh_spectrum(ctx, world);
}

int lenia_seed_rule(LeniaCtx* ctx, int32_t world, uint32_t seed, int32_t kind) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (kind != LENIA_SEED_SL_DISCS && kind != LENIA_SEED_MNCA_BLOCKS) return fail(ctx, LENIA_EINVAL, "unknown seed %d", kind);
    const LeniaWorldDesc& d = ctx->desc[world];
    for (uint32_t c = 0; c < d.channels; c++)
        launch_seed_rule(state_ptr(ctx, world) + (size_t)c * d.width * d.height, d.width, d.height, seed + c, kind,
                         ctx->stream);
    CK(cudaGetLastError());
    return refresh_spectrum(ctx, world);
}

int lenia_render(LeniaCtx* ctx, int32_t world, int32_t channel, float origin_x, float origin_y, float scale,
                 uint32_t samples, uint32_t out_w, uint32_t out_h, int32_t palette, uint8_t* rgba) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    const LeniaWorldDesc& d = ctx->desc[world];
    if (channel < 0 || channel >= (int)d.channels) return fail(ctx, LENIA_EINVAL, "no channel %d", channel);
    if (!rgba || out_w < 1 || out_h < 1 || out_w > 16384 || out_h > 16384 || samples < 1 || samples > 16 ||
        !(scale > 0.0f) || palette < 0 || palette > 2)
        return fail(ctx, LENIA_EINVAL, "render: bad output size, samples, scale or palette");
    uchar4* dev = nullptr;
    const size_t bytes = (size_t)out_w * out_h * 4;
    CK(cudaMallocAsync((void**)&dev, bytes, ctx->stream));
    launch_render(state_ptr(ctx, world) + (size_t)channel * d.width * d.height, d.width, d.height, origin_x, origin_y,
                  scale, (int)samples, (int)out_w, (int)out_h, palette, dev, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rgba, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(dev, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_cells_per_step(const LeniaCtx* ctx, uint64_t* cells) {
    if (!ctx || !cells) return LENIA_EINVAL;
    uint64_t n = 0;
    for (const auto& d : ctx->desc) n += (uint64_t)d.width * d.height * d.channels;
    *cells = n;
    return 0;
}

int lenia_memory_bytes(const LeniaCtx* ctx, uint64_t* bytes) {
    if (!ctx || !bytes) return LENIA_EINVAL;
    *bytes = ctx->bytes;
    return 0;
}

int lenia_read_field_u(LeniaCtx* ctx, int32_t world, int32_t kernel, float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    const LeniaWorldDesc& d = ctx->desc[world];
    if (kernel < 0 || kernel >= (int)d.nkernels) return fail(ctx, LENIA_EINVAL, "no kernel %d", kernel);
    const size_t cells = (size_t)d.width * d.height;
    if (!host || count != cells) return fail(ctx, LENIA_EINVAL, "U field has %zu values", cells);
    if (ctx->path == LENIA_PATH_RADIX2) {
        r2_enqueue_convolve(ctx->r2[world], ctx->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(host, ctx->r2[world].conv[kernel], cells * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return 0;
    }
    int frc = flush_spectra(ctx);
    if (frc) return frc;
    DevWorld& w = ctx->hw[world];
    if (!w.u_out) {
        int rc = dalloc(ctx, &w.u_out, cells * d.nkernels);
        if (rc) return rc;
        CK(cudaMemcpy(ctx->d_worlds + world, &w, sizeof(DevWorld), cudaMemcpyHostToDevice));
    }
    const WorldBuffers& b = ctx->wb[world];
    const SizeClass& cl = ctx->classes[b.cls];
    bool ok = launch_columns(ctx, cl, b.d_col, b.ncol, b.d_tcg, b.ntcg, cl.var_col, cl.var_tc, ctx->stream);
    ok = ok && launch_row_fp32(cl.W, cl.var_row, MODE_U, cl.general, ctx->d_worlds, b.d_row, b.nrow, cl.planes, ctx->d_tw,
                               ctx->stream);
    if (!ok) return fail(ctx, LENIA_ECUDA, "U launch failed");
    CK(cudaGetLastError());
    int rc = refresh_spectrum(ctx, world);
    if (rc) return rc;
    CK(cudaMemcpyAsync(host, w.u_out + (size_t)kernel * cells, cells * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_read_spectrum(LeniaCtx* ctx, int32_t world, int32_t channel, float* host, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (world_from_ctx(ctx, world)) return fail(ctx, LENIA_EINVAL, "no world %d", world);
    if (ctx->path == LENIA_PATH_RADIX2) return fail(ctx, LENIA_ESTATE, "the radix-2 path keeps no half-spectrum");
    const LeniaWorldDesc& d = ctx->desc[world];
    if (channel < 0 || channel >= (int)d.channels) return fail(ctx, LENIA_EINVAL, "no channel %d", channel);
    const int W = d.width, H = d.height, KX = W / 2 + 1;
    if (!host || count != (size_t)H * KX * 2) return fail(ctx, LENIA_EINVAL, "spectrum has %d values", H * KX * 2);
    int frc = flush_spectra(ctx);
    if (frc) return frc;
    std::vector<float2> tiles(spec_elems(W, H));
    CK(cudaMemcpyAsync(tiles.data(), ctx->hw[world].spec + (size_t)channel * spec_elems(W, H), tiles.size() * sizeof(float2),
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int y = 0; y < H; y++)
        for (int kx = 0; kx < W / 2; kx++) {
            const float2 v = tiles[((size_t)(kx / TC) * H + y) * TC + (kx % TC)];
            float* o = host + ((size_t)y * KX + kx) * 2;
            if (kx == 0) {
                o[0] = v.x;
                o[1] = 0.0f;
                float* n = host + ((size_t)y * KX + W / 2) * 2;
                n[0] = v.y;
                n[1] = 0.0f;
            } else {
                o[0] = v.x;
                o[1] = v.y;
            }
        }
    return 0;
}

int lenia_world_stats(LeniaCtx* ctx, float* host_out, size_t count) {
    if (!ctx) return LENIA_EINVAL;
    if (!host_out || count != 3 * ctx->desc.size()) return fail(ctx, LENIA_EINVAL, "need 3 floats per world");
    launch_world_stats(ctx->d_worlds, (int)ctx->desc.size(), ctx->d_stats, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host_out, ctx->d_stats, count * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_profile_step(LeniaCtx* ctx, uint32_t steps, float* out3) {
    if (!ctx || !out3 || steps == 0) return LENIA_EINVAL;
    {
        int frc = flush_spectra(ctx);
        if (frc) return frc;
    }
    if (ctx->path == LENIA_PATH_RADIX2) {
        Events ev;
        CK(cudaEventCreate(&ev.e[0]));
        CK(cudaEventCreate(&ev.e[1]));
        CK(cudaEventRecord(ev.e[0], ctx->stream));
        for (uint32_t s = 0; s < steps; s++) CK(cudaGraphLaunch(ctx->graph_one, ctx->stream));
        CK(cudaEventRecord(ev.e[1], ctx->stream));
        CK(cudaEventSynchronize(ev.e[1]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ev.e[0], ev.e[1]);
        out3[0] = out3[1] = 0.0f;
        out3[2] = ms / steps;
        ctx->tick += steps;
        return 0;
    }
    // every class's column and row launches on the context stream, in the graph's order
    double col_ms = 0, row_ms = 0;
    for (auto& cl : ctx->classes) {
        double c = 0, r = 0;
        int rc = time_class(ctx, cl, shape_of(cl), (int)steps, &c, &r);
        if (rc) return rc;
        col_ms += c;
        row_ms += r;
    }
    out3[0] = (float)(col_ms / steps);
    out3[1] = (float)(row_ms / steps);
    out3[2] = (float)((col_ms + row_ms) / steps);
    ctx->tick += steps;
    return 0;
}

int lenia_profile_classes(LeniaCtx* ctx, uint32_t steps, float* out, size_t count, size_t* nclasses) {
    if (!ctx || !nclasses) return LENIA_EINVAL;
    *nclasses = ctx->classes.size();
    if (!out) return 0;
    if (steps == 0 || count < 5 * ctx->classes.size()) return fail(ctx, LENIA_EINVAL, "need steps > 0 and 5 floats per class");
    if (ctx->path == LENIA_PATH_RADIX2) return fail(ctx, LENIA_ESTATE, "the radix-2 path has no size classes");
    int frc = flush_spectra(ctx);
    if (frc) return frc;
    for (size_t c = 0; c < ctx->classes.size(); c++) {
        const SizeClass& cl = ctx->classes[c];
        double col_ms = 0, row_ms = 0;
        int rc = time_class(ctx, cl, shape_of(cl), (int)steps, &col_ms, &row_ms);
        if (rc) return rc;
        // the class as the step graph runs it: launches back to back, chunks on their lanes (replayed
        // twice, the second timed)
        double graph_ms = 0;
        rc = time_class_graph(ctx, cl, shape_of(cl), (int)steps, &graph_ms);
        if (rc) return rc;
        out[5 * c] = (float)cl.W;
        out[5 * c + 1] = (float)cl.H;
        out[5 * c + 2] = (float)(col_ms / steps);
        out[5 * c + 3] = (float)(row_ms / steps);
        out[5 * c + 4] = (float)(graph_ms / steps);
    }
    ctx->tick += 3 * steps;
    return check_device_errors(ctx);
}

int lenia_kernel_spectrum(const LeniaKernel* kernel, uint32_t width, uint32_t height, float* out, size_t count) {
    if (!kernel || !out) return fail(nullptr, LENIA_EINVAL, "NULL argument");
    LeniaWorldDesc d;
    memset(&d, 0, sizeof(d));
    d.width = width;
    d.height = height;
    d.channels = 1;
    d.nkernels = 1;
    d.rule = LENIA_RULE_LENIA;
    d.dt = 1.0f;
    d.kernels[0] = *kernel;
    d.kernels[0].src = d.kernels[0].dst = 0;
    if (!(d.kernels[0].sigma > 0.0f)) d.kernels[0].sigma = 1.0f;
    int rc = validate(d, 0, LENIA_PATH_FP32);
    if (rc) return rc;
    const size_t need = (size_t)(width / 2 + 1) * (height / 2 + 1);
    if (count != need) return fail(nullptr, LENIA_EINVAL, "spectrum has %zu values, got %zu", need, count);
    compute_khat(*kernel, (int)width, (int)height, (int)(height / 2 + 1), out);
    return 0;
}

int lenia_tc_selftest(int32_t path, int32_t n, int32_t k, const float* a, const float* b, float* d) {
    if (!a || !b || !d) return fail(nullptr, LENIA_EINVAL, "NULL argument");
    std::string err;
    int rc = tc_selftest(path, n, k, a, b, d, &err);
    if (rc) return fail(nullptr, rc, "%s", err.c_str());
    return 0;
}

int lenia_tc_set_wait_limit(LeniaCtx* ctx, int32_t polls_plus_one) {
    if (!ctx) return LENIA_EINVAL;
    if (polls_plus_one < 0) return fail(ctx, LENIA_EINVAL, "polls_plus_one must be >= 0");
    if (ctx->path != LENIA_PATH_TF32 && ctx->path != LENIA_PATH_BF16X3)
        return fail(ctx, LENIA_ESTATE, "the context has no tensor-core path");
    CK(cudaStreamSynchronize(ctx->stream));
    std::string err;
    int rc = tc_set_wait_limit(ctx->tc, polls_plus_one, &err);
    if (rc) return fail(ctx, rc, "%s", err.c_str());
    return 0;
}

int lenia_persist_set_wait_limit(LeniaCtx* ctx, int32_t polls_plus_one) {
    if (!ctx) return LENIA_EINVAL;
    if (polls_plus_one < 0) return fail(ctx, LENIA_EINVAL, "polls_plus_one must be >= 0");
    if (!ctx->d_flags) return fail(ctx, LENIA_ESTATE, "the context has no persistent step");
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(ctx->d_flags + 1, &polls_plus_one, sizeof(int), cudaMemcpyHostToDevice));
    return 0;
}

int lenia_class_variants(const LeniaCtx* ctx, int32_t* out, size_t count, size_t* nclasses) {
    if (!ctx || !nclasses) return LENIA_EINVAL;
    *nclasses = ctx->classes.size();
    if (!out) return 0;
    if (count < 4 * ctx->classes.size()) return LENIA_EINVAL;
    for (size_t i = 0; i < ctx->classes.size(); i++) {
        const auto& cl = ctx->classes[i];
        out[4 * i] = cl.W;
        out[4 * i + 1] = cl.H;
        out[4 * i + 2] = cl.var_col;
        out[4 * i + 3] = cl.var_row;
    }
    return 0;
}

int lenia_set_chunk_budget(LeniaCtx* ctx, uint32_t mib) {
    if (!ctx) return LENIA_EINVAL;
    if (mib > (1u << 20)) return fail(ctx, LENIA_EINVAL, "chunk budget above 1 TiB");
    if (ctx->path == LENIA_PATH_RADIX2) return 0;  // no size classes
    for (auto& cl : ctx->classes) {
        cl.chunk_budget = (size_t)mib << 20;
        cl.chunks = make_chunks(ctx, cl, cl.chunk_budget);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_set_chunk_lanes(LeniaCtx* ctx, int32_t lanes) {
    if (!ctx) return LENIA_EINVAL;
    if (lanes < 1 || lanes > LeniaCtx::MAX_LANES)
        return fail(ctx, LENIA_EINVAL, "lanes must be 1..%d, got %d", LeniaCtx::MAX_LANES, lanes);
    if (ctx->path == LENIA_PATH_RADIX2) return 0;  // no size classes
    for (auto& cl : ctx->classes) cl.lanes = lanes;
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_set_resident(LeniaCtx* ctx, int32_t mode) {
    if (!ctx) return LENIA_EINVAL;
    if (mode < 0 || mode > 1 + RESIDENT_VARIANTS)
        return fail(ctx, LENIA_EINVAL, "mode must be 0 (off), 1 (on) or 2..%d (on, launch variant mode - 2)",
                    1 + RESIDENT_VARIANTS);
    for (auto& cl : ctx->classes) {
        const int v = mode >= 2 ? mode - 2 : cl.var_res;
        cl.resident = mode != 0 && cl.resident_ok && cl.res_fits[v] > 0;
        if (cl.resident) cl.var_res = v, cl.persist = 0;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_set_persistent(LeniaCtx* ctx, int32_t mode) {
    if (!ctx) return LENIA_EINVAL;
    if (mode < 0 || mode > 1 + PERSIST_VARIANTS)
        return fail(ctx, LENIA_EINVAL, "mode must be 0 (off), 1 (on) or 2..%d (on, launch variant mode - 2)",
                    1 + PERSIST_VARIANTS);
    for (auto& cl : ctx->classes) {
        cl.persist = mode != 0 && cl.persist_ok;
        if (cl.persist) {
            cl.resident = 0;
            if (mode >= 2) cl.var_per = mode - 2;
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_set_tc_variant(LeniaCtx* ctx, int32_t variant) {
    if (!ctx) return LENIA_EINVAL;
    if (variant < 0 || variant >= TC_COL_VARIANTS)
        return fail(ctx, LENIA_EINVAL, "tensor-core column variants are 0..%d", TC_COL_VARIANTS - 1);
    for (auto& cl : ctx->classes) cl.var_tc = variant;
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_set_tc_rows(LeniaCtx* ctx, int32_t on) {
    if (!ctx) return LENIA_EINVAL;
    if (on != 0 && on != 1) return fail(ctx, LENIA_EINVAL, "on must be 0 or 1");
    for (auto& cl : ctx->classes) cl.tc_rows = on && cl.tc_rows_ok;
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_set_branch_split(LeniaCtx* ctx, int64_t cells, int32_t each) {
    if (!ctx) return LENIA_EINVAL;
    if (cells < 0 || (each != 0 && each != 1)) return fail(ctx, LENIA_EINVAL, "cells must be >= 0, each 0 or 1");
    if (ctx->path == LENIA_PATH_RADIX2) return 0;  // no size classes
    ctx->branch_cells = cells;
    ctx->branch_each = each;
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int lenia_branch_split(const LeniaCtx* ctx, int64_t* cells, int32_t* each) {
    if (!ctx || !cells || !each) return LENIA_EINVAL;
    *cells = ctx->branch_cells;
    *each = ctx->branch_each;
    return 0;
}

int lenia_class_shapes(const LeniaCtx* ctx, int32_t* out, size_t count, size_t* nclasses) {
    if (!ctx || !nclasses) return LENIA_EINVAL;
    *nclasses = ctx->classes.size();
    if (!out) return 0;
    if (count < 14 * ctx->classes.size()) return LENIA_EINVAL;
    for (size_t i = 0; i < ctx->classes.size(); i++) {
        const auto& cl = ctx->classes[i];
        int32_t* o = out + 14 * i;
        o[0] = cl.W;
        o[1] = cl.H;
        o[2] = cl.var_col;
        o[3] = cl.var_row;
        o[4] = (int32_t)cl.chunks.size();
        o[5] = (int32_t)cl.worlds.size();
        o[6] = (int32_t)(cl.chunk_budget >> 20);
        o[7] = row_item_rows(cl.W, cl.general);
        o[8] = cl.resident;
        o[9] = cl.var_res;
        o[10] = cl.tc_rows;
        o[11] = cl.ntcg > 0 ? cl.var_tc : -1;
        o[12] = cl.persist ? cl.var_per : -1;
        o[13] = cl.lanes;
    }
    return 0;
}

int lenia_set_variants(LeniaCtx* ctx, int32_t col_variant, int32_t row_variant) {
    if (!ctx) return LENIA_EINVAL;
    if (col_variant < -1 || col_variant >= COL_VARIANTS || row_variant < -1 || row_variant > 1)
        return fail(ctx, LENIA_EINVAL, "launch variants are -1..%d (column) and -1..1 (row), got %d and %d",
                    COL_VARIANTS - 1, col_variant, row_variant);
    if (ctx->path == LENIA_PATH_RADIX2) return 0;  // one build per stage: nothing to choose
    for (auto& cl : ctx->classes) {
        if (col_variant >= 0) cl.var_col = col_variant;
        if (row_variant >= 0) cl.var_row = row_variant;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = rebuild_graphs(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

// The autotuner's search, on states it may advance.  For every size class, in turn: the cluster-
// resident and persistent steps against two launches a generation (FP32 path, where they apply), the
// tensor-core row
// pass against the FP32 one (TF32 / BF16X3 paths, where it applies), then every pair of column and
// row launch variants jointly with every chunk budget that gives a different number of chunks, the
// chunks one after another or on 2..MAX_LANES concurrent lanes.
// Each candidate is timed as a captured graph of a few steps (time_class_graph), and a class keeps
// its current choice of a dimension unless another is at least 3% faster, so that timing noise does
// not flip it.
static int autotune_search(LeniaCtx* ctx) {
    const size_t budgets[] = {0, 128ull << 20, 96ull << 20, 64ull << 20, 32ull << 20};
    constexpr int REPS = 8;
    for (auto& cl : ctx->classes) {
        auto timed = [&](const Shape& sh, double* t) { return time_class_graph(ctx, cl, sh, REPS, t); };
        // pick among candidate shapes; the first candidate is the current shape
        auto pick = [&](std::vector<Shape>& cands, int* best_i) {
            std::vector<double> t(cands.size());
            for (size_t i = 0; i < cands.size(); i++) {
                int rc = timed(cands[i], &t[i]);
                if (rc) return rc;
            }
            int b = 0;
            for (size_t i = 1; i < cands.size(); i++)
                if (t[i] < t[b]) b = (int)i;
            *best_i = t[b] < 0.97 * t[0] ? b : 0;
            return 0;
        };
        int bi = 0, rc = 0;
        if (cl.resident_ok || cl.persist_ok) {
            // one launch per class and step call -- every variant of the cluster-resident step that fits,
            // and the persistent step -- against the two-pass step in its current shape; candidate 0 is
            // the current choice
            struct Cand {
                int res, var, per, pvar;
            };
            const Cand was{cl.resident, cl.var_res, cl.persist, cl.var_per};
            std::vector<Cand> cands{was};
            if (was.res || was.per) cands.push_back({0, was.var, 0, was.pvar});
            for (int v = 0; v < RESIDENT_VARIANTS && cl.resident_ok; v++)
                if (cl.res_fits[v] > 0 && !(was.res && v == was.var)) cands.push_back({1, v, 0, was.pvar});
            for (int v = 0; v < PERSIST_VARIANTS && cl.persist_ok; v++)
                if (!(was.per && v == was.pvar)) cands.push_back({0, was.var, 1, v});
            std::vector<double> t(cands.size());
            for (size_t i = 0; i < cands.size() && !rc; i++) {
                cl.resident = cands[i].res;
                cl.var_res = cands[i].var;
                cl.persist = cands[i].per;
                cl.var_per = cands[i].pvar;
                rc = timed(shape_of(cl), &t[i]);
            }
            cl.resident = was.res;
            cl.var_res = was.var;
            cl.persist = was.per;
            cl.var_per = was.pvar;
            if (rc) return rc;
            size_t b = 0;
            for (size_t i = 1; i < cands.size(); i++)
                if (t[i] < t[b]) b = i;
            if (t[b] < 0.97 * t[0]) {
                cl.resident = cands[b].res;
                cl.var_res = cands[b].var;
                cl.persist = cands[b].per;
                cl.var_per = cands[b].pvar;
            }
            if (cl.resident || cl.persist) continue;  // launch variants and chunks do not apply to them
        }
        if (cl.ntcg > 0) {
            // the tensor-core column pass's variants (staged tile groups, or L2-prefetched loads with more
            // CTAs an SM); candidate 0 is the current choice
            std::vector<Shape> c{shape_of(cl)};
            for (int v = 0; v < TC_COL_VARIANTS; v++)
                if (v != cl.var_tc) c.push_back(Shape{cl.var_col, cl.var_row, v, &cl.chunks, cl.lanes});
            if ((rc = pick(c, &bi))) return rc;
            cl.var_tc = c[bi].var_tc;
        }
        if (cl.tc_rows_ok) {
            // the tensor-core row pass against the FP32 row pass (TF32 / BF16X3 paths); candidate 0 is
            // the current choice
            const int was = cl.tc_rows;
            double t[2] = {0, 0};
            for (int i = 0; i < 2 && !rc; i++) {
                cl.tc_rows = i == 0 ? was : !was;
                rc = timed(shape_of(cl), &t[i]);
            }
            cl.tc_rows = was;
            if (rc) return rc;
            if (t[1] < 0.97 * t[0]) cl.tc_rows = !was;
        }
        {
            // launch variants jointly with the chunk budget and lanes: their best pairs differ (on the
            // batched workload's 1024 x 1024 class the radix-32 column build was fastest in 32 MiB chunks
            // on four lanes, the paired build in 64 MiB chunks on two).  Every pair of column and row
            // variants, for every list of chunks (each budget that changes the number of chunks) one
            // after another and on 2..MAX_LANES lanes; candidate 0 is the current shape.
            std::vector<std::vector<Chunk>> lists{cl.chunks};
            std::vector<size_t> bud{cl.chunk_budget};
            for (size_t b : budgets) {
                std::vector<Chunk> ch = make_chunks(ctx, cl, b);
                bool seen = false;
                for (auto& l : lists) seen = seen || l.size() == ch.size();
                if (!seen) lists.push_back(ch), bud.push_back(b);
            }
            std::vector<Shape> c{Shape{cl.var_col, cl.var_row, cl.var_tc, &lists[0], cl.lanes}};
            std::vector<size_t> which{0};
            for (size_t li = 0; li < lists.size(); li++)
                for (int ln = 1; ln <= LeniaCtx::MAX_LANES && ln <= (int)lists[li].size(); ln++)
                    for (int vc = 0; vc < COL_VARIANTS; vc++)
                        for (int vr = 0; vr < 2; vr++)
                            if (!(li == 0 && ln == c[0].lanes && vc == c[0].var_col && vr == c[0].var_row) &&
                                (vc != 3 || col_has_r16_variant(cl.H))) {
                                c.push_back(Shape{vc, vr, cl.var_tc, &lists[li], ln});
                                which.push_back(li);
                            }
            if ((rc = pick(c, &bi))) return rc;
            cl.var_col = c[bi].var_col;
            cl.var_row = c[bi].var_row;
            cl.chunk_budget = bud[which[bi]];
            cl.lanes = c[bi].lanes;
            cl.chunks = lists[which[bi]];
        }
    }
    // The whole step: the small classes on a second graph branch beside the large ones, for every
    // split point between class sizes, against one branch (kept unless another is 3% faster).
    if (ctx->classes.size() > 1) {
        std::vector<int64_t> sizes;
        for (auto& cl : ctx->classes) sizes.push_back((int64_t)cl.W * cl.H);
        std::sort(sizes.begin(), sizes.end());
        sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
        // (split, each): candidate 0 is the current choice
        std::vector<std::pair<int64_t, int>> cands{{ctx->branch_cells, ctx->branch_each}};
        if (ctx->branch_cells) cands.push_back({0, 0});
        for (size_t i = 0; i + 1 < sizes.size(); i++)
            for (int each = 0; each < 2; each++)
                if (!(sizes[i] == ctx->branch_cells && each == ctx->branch_each) && !(each && i == 0))
                    cands.push_back({sizes[i], each});
        const auto was = cands[0];
        std::vector<double> t(cands.size());
        int rc = 0;
        for (size_t i = 0; i < cands.size() && !rc; i++) {
            ctx->branch_cells = cands[i].first;
            ctx->branch_each = cands[i].second;
            rc = time_graph(ctx, [&]() { return enqueue_steps(ctx, REPS); }, &t[i]);
        }
        ctx->branch_cells = was.first;
        ctx->branch_each = was.second;
        if (rc) return rc;
        size_t b = 0;
        for (size_t i = 1; i < cands.size(); i++)
            if (t[i] < t[b]) b = i;
        if (t[b] < 0.97 * t[0]) ctx->branch_cells = cands[b].first, ctx->branch_each = cands[b].second;
    }
    return 0;
}

int lenia_autotune(LeniaCtx* ctx) {
    if (!ctx) return LENIA_EINVAL;
    if (ctx->path == LENIA_PATH_RADIX2) return 0;
    {
        int frc = flush_spectra(ctx);
        if (frc) return frc;
    }
    // The trial steps advance the worlds, so every state is saved to a device buffer first and
    // restored afterwards, also when the search fails.
    size_t total = 0;
    for (const auto& d : ctx->desc) total += state_count(d);
    DeviceBuffer save_buf;
    CK(cudaMalloc(&save_buf.p, total * sizeof(float)));
    float* saved = static_cast<float*>(save_buf.p);
    auto copy_states = [&](bool restore) -> cudaError_t {
        size_t off = 0;
        for (size_t w = 0; w < ctx->desc.size(); w++) {
            const size_t n = state_count(ctx->desc[w]);
            if (!ctx->states || w == 0) {
                float* dev = state_ptr(ctx, (int)w);
                const size_t cnt = (ctx->states ? total : n) * sizeof(float);
                cudaError_t e = restore ? cudaMemcpyAsync(dev, saved + off, cnt, cudaMemcpyDeviceToDevice, ctx->stream)
                                        : cudaMemcpyAsync(saved + off, dev, cnt, cudaMemcpyDeviceToDevice, ctx->stream);
                if (e != cudaSuccess) return e;
            }
            off += n;
        }
        return cudaSuccess;
    };
    CK(copy_states(false));
    const int rc = autotune_search(ctx);
    const cudaError_t e = copy_states(true);
    for (size_t w = 0; w < ctx->desc.size(); w++) refresh_spectrum(ctx, (int)w);
    if (rc) return rc;
    CK(e);
    CK(cudaStreamSynchronize(ctx->stream));
    int grc = rebuild_graphs(ctx);
    if (grc) return grc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

}  // extern "C"
