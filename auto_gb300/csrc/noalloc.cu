// lenia_step_noalloc: the fused FP32 Lenia step for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc when they want to step a world: a host application that
// has handed all device memory to its own pool allocator (so a cudaMalloc fails or is not allowed
// to take memory behind the pool's back), or a real-time frame loop in which a cudaMalloc, which
// may synchronize the device, would stall the frame.  This entry point allocates nothing.  The
// caller passes the state (input and output) and the kernel spectrum; the half-spectrum the step
// needs between its two launches, the twiddle table, the world descriptor and the work lists live
// in one file-scope __device__ array of fixed size.
//
// Limits and behaviour:
//   * at most NOALLOC_MAX_CELLS = 1,048,576 cells (width * height), each side a size the engine
//     supports; larger worlds are rejected with LENIA_ESIZE and a message;
//   * every GPU that loads this library holds the array (about 4.2 MiB) until the process exits;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) and
//     fills the twiddle table; make that first call before any stream capture;
//   * every call shares the array and it keeps the last call's contents; each call rewrites all of
//     it that it reads, so nothing carries over, but calls that overlap on the GPU (different
//     streams, or threads racing) race on it and must be serialised by the caller;
//   * the address is cached per device ordinal for the life of the process: the primary context
//     is assumed, so cudaDeviceReset, or a non-primary driver-API context made current, is not
//     supported between calls;
//   * the kernel spectrum arrives with lenia_kernel_spectrum's row stride H/2+1, not the 16-byte
//     aligned stride the engine's own contexts use, so every column item takes the column pass's
//     unchained form (transform, multiply, transform in three sweeps) instead of the chained one.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "engine.cuh"
#include "fft_core.cuh"

namespace lenia {
namespace {

constexpr size_t NOALLOC_MAX_CELLS = 1024 * 1024;
constexpr int NOALLOC_MAX_SIDE = 4096;
constexpr size_t SPEC_BYTES = NOALLOC_MAX_CELLS / 2 * sizeof(float2);
constexpr size_t TW_BYTES = (size_t)lfft::TWN * sizeof(float2);
constexpr size_t WORLD_BYTES = (sizeof(DevWorld) + 255) / 256 * 256;
constexpr size_t COL_BYTES = (size_t)(NOALLOC_MAX_SIDE / (2 * TC)) * sizeof(ColItem);
constexpr size_t ROW_BYTES = (size_t)(NOALLOC_MAX_SIDE / 2) * sizeof(RowItem);  // items of >= 2 rows
constexpr size_t OFF_TW = SPEC_BYTES, OFF_WORLD = OFF_TW + TW_BYTES, OFF_COL = OFF_WORLD + WORLD_BYTES,
                 OFF_ROW = OFF_COL + COL_BYTES, SCRATCH_BYTES = OFF_ROW + ROW_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
unsigned char* g_base[MAX_DEVICES] = {};
// Failures are reported through lenia_last_error(NULL), like those of lenia_create.
int set_error(int code, const std::string& msg) {
    set_thread_error(msg);
    return code;
}

bool side_ok(uint32_t n) {
    const uint32_t m = (n % 3 == 0) ? n / 3 : n;
    return m && !(m & (m - 1)) && n >= 32 && n <= (uint32_t)NOALLOC_MAX_SIDE;
}

// Once per device, with that device current: the array's device address and the twiddle table.
int setup_device(int dev, unsigned char** base) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_base[dev]) {
        *base = g_base[dev];
        return 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return set_error(LENIA_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    std::vector<float2> tw(lfft::TWN);
    for (int t = 0; t < lfft::TWN; t++) {
        const double a = -2.0 * M_PI * (double)t / (double)lfft::TWN;
        tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    e = cudaMemcpy((unsigned char*)p + OFF_TW, tw.data(), TW_BYTES, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return set_error(LENIA_ECUDA, std::string("twiddle upload: ") + cudaGetErrorString(e));
    g_base[dev] = (unsigned char*)p;
    *base = g_base[dev];
    return 0;
}

// Writes the world descriptor and the work lists into the array on the caller's stream.
__global__ void noalloc_prepare(DevWorld* w, DevWorld value, ColItem* col, int ncol, RowItem* row, int nrow, int rows) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *w = value;
    if (i < ncol) col[i] = ColItem{0, 0, i, 0};
    if (i < nrow) row[i] = RowItem{0, rows * i};
}

}  // namespace
}  // namespace lenia

using namespace lenia;

extern "C" {

LENIA_API int lenia_step_noalloc(float* state, uint32_t width, uint32_t height, const float* khat, float mu,
                                 float sigma, float dt, uint32_t steps, void* stream) {
    if (!state || !khat) return set_error(LENIA_EINVAL, "state and khat must be device pointers");
    if (!side_ok(width) || !side_ok(height))
        return set_error(LENIA_ESIZE, "sides must be 2^a or 3*2^a, 32..4096");
    if ((size_t)width * height > NOALLOC_MAX_CELLS) {
        char m[160];
        snprintf(m, sizeof m, "%ux%u has %zu cells; lenia_step_noalloc holds at most %zu (use lenia_create)", width,
                 height, (size_t)width * height, NOALLOC_MAX_CELLS);
        return set_error(LENIA_ESIZE, m);
    }
    if (!(sigma > 0.0f) || !(dt > 0.0f)) return set_error(LENIA_EINVAL, "sigma and dt must be > 0");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(LENIA_ENODEV, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return set_error(LENIA_ENODEV, "device ordinal out of range");
    unsigned char* base = nullptr;
    int rc = setup_device(dev, &base);
    if (rc) return rc;

    cudaStream_t s = (cudaStream_t)stream;
    DevWorld w;
    memset(&w, 0, sizeof(w));
    w.W = (int)width;
    w.H = (int)height;
    w.C = 1;
    w.K = 1;
    w.rule = LENIA_RULE_LENIA;
    w.dt = dt;
    w.HQ = (int)height / 2 + 1;
    w.state = state;
    w.spec = reinterpret_cast<float2*>(base);
    w.conv = w.spec;
    w.khat = khat;
    w.kern[0] = DevKernel{0, 0, mu, sigma, 1.0f};
    DevWorld* dw = reinterpret_cast<DevWorld*>(base + OFF_WORLD);
    ColItem* col = reinterpret_cast<ColItem*>(base + OFF_COL);
    RowItem* row = reinterpret_cast<RowItem*>(base + OFF_ROW);
    const float2* tw = reinterpret_cast<const float2*>(base + OFF_TW);
    const int rows = row_item_rows((int)width, 0);
    const int ncol = spec_tiles((int)width), nrow = (int)height / rows;
    const int n = ncol > nrow ? ncol : nrow;
    // Zero-item launches configure both passes (shared-memory limits) before anything is enqueued,
    // so a size the passes cannot run is reported without having advanced the state.
    if (!launch_col_fp32((int)height, 0, dw, col, 0, tw, s) || !launch_row_fp32((int)width, 0, MODE_STEP, 0, dw, row, 0, 0, tw, s))
        return set_error(LENIA_ECUDA, "launch configuration failed; the state is unchanged");
    noalloc_prepare<<<(n + 255) / 256, 256, 0, s>>>(dw, w, col, ncol, row, nrow, rows);
    bool ok = launch_row_fp32((int)width, 0, MODE_FORWARD, 0, dw, row, nrow, 0, tw, s);
    for (uint32_t i = 0; ok && i < steps; i++) {
        ok = launch_col_fp32((int)height, 0, dw, col, ncol, tw, s) &&
             launch_row_fp32((int)width, 0, MODE_STEP, 0, dw, row, nrow, 0, tw, s);
    }
    if (!ok) return set_error(LENIA_ECUDA, "launch configuration failed");
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(LENIA_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
