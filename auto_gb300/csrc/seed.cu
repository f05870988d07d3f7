// On-device initial states and per-world statistics.
//
// The reference seeds worlds on the GPU in its init passes so that large worlds never need a
// host copy (crates/auto-core/src/sim.rs:284-294, spectral.rs:183-197).  The random source is
// the PCG hash of program.rs:140-147; the tile seeder follows spectral.rs:313-335 with the
// pattern passed in by the caller.
#include <cuda_runtime.h>

#include "engine.cuh"

namespace lenia {

__device__ __forceinline__ uint32_t pcg(uint32_t v) {
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
__device__ __forceinline__ uint32_t rand3(uint32_t a, uint32_t b, uint32_t c) { return pcg(pcg(pcg(a) ^ b) ^ c); }
__device__ __forceinline__ float unit_f(uint32_t r) { return (float)r * (1.0f / 4294967296.0f); }

// unit_f(rand3(x, y, seed)) inside any of the torus-wrapped patches, zero elsewhere.
__global__ void seed_patches_kernel(float* state, int W, int H, uint32_t seed, const int4* __restrict__ patches,
                                    int npatch) {
    const size_t n = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % W), y = (int)(i / W);
        bool inside = false;
        for (int p = 0; p < npatch && !inside; p++) {
            const int4 q = patches[p];
            const int dx = ((x - q.x) % W + W) % W, dy = ((y - q.y) % H + H) % H;
            inside = dx < q.z && dy < q.w;
        }
        state[i] = inside ? unit_f(rand3((uint32_t)x, (uint32_t)y, seed)) : 0.0f;
    }
}

// spectral.rs:318-335: tiles of `spacing` cells; a tile whose rand3(tx, ty, seed) is even gets
// the pattern, turned by (r >> 8) & 3 quarter turns.
__global__ void seed_tiles_kernel(float* state, int W, int H, uint32_t seed, const float* __restrict__ pattern,
                                  int pw, int ph, int spacing) {
    const size_t n = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(i % W), y = (uint32_t)(i / W);
        const uint32_t r = rand3(x / spacing, y / spacing, seed);
        float v = 0.0f;
        const uint32_t px = x % spacing, py = y % spacing;
        if ((r & 1u) == 0u && px < (uint32_t)pw && py < (uint32_t)ph) {
            uint32_t ix = px, iy = py;
            switch ((r >> 8u) & 3u) {
            case 1u: ix = py; iy = (uint32_t)pw - 1u - px; break;
            case 2u: ix = (uint32_t)pw - 1u - px; iy = (uint32_t)ph - 1u - py; break;
            case 3u: ix = (uint32_t)ph - 1u - py; iy = px; break;
            default: break;
            }
            v = pattern[iy * (uint32_t)pw + ix];
        }
        state[i] = v;
    }
}

// Mass of channel 0 and toroidal centroid (circular mean per axis), one CTA per world.
__global__ void world_stats_kernel(const DevWorld* __restrict__ worlds, float* out) {
    const DevWorld& wd = worlds[blockIdx.x];
    const int W = wd.W, H = wd.H;
    const size_t n = (size_t)W * H;
    float m = 0.f, cxs = 0.f, cxc = 0.f, cys = 0.f, cyc = 0.f;
    const float ax = 2.0f / W, ay = 2.0f / H;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float s = wd.state[i];
        if (s == 0.0f) continue;
        const int x = (int)(i % W), y = (int)(i / W);
        float sx, cx, sy, cy;
        sincospif(ax * x, &sx, &cx);
        sincospif(ay * y, &sy, &cy);
        m += s; cxs += s * sx; cxc += s * cx; cys += s * sy; cyc += s * cy;
    }
    __shared__ double red[5][32];
    double v[5] = {m, cxs, cxc, cys, cyc};
    for (int q = 0; q < 5; q++) {
        double a = v[q];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[5] = {0, 0, 0, 0, 0};
        for (int q = 0; q < 5; q++)
            for (int wi = 0; wi < (int)(blockDim.x >> 5); wi++) t[q] += red[q][wi];
        const double two_pi = 6.283185307179586;
        double cx = atan2(t[1], t[2]) / two_pi * W, cy = atan2(t[3], t[4]) / two_pi * H;
        if (cx < 0) cx += W;
        if (cy < 0) cy += H;
        out[3 * blockIdx.x + 0] = (float)t[0];
        out[3 * blockIdx.x + 1] = (float)cx;
        out[3 * blockIdx.x + 2] = (float)cy;
    }
}

static int grid_for(size_t n) {
    size_t g = (n + 255) / 256;
    return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

void launch_seed_patches(float* state, int W, int H, uint32_t seed, const int4* patches, int npatch, cudaStream_t s) {
    seed_patches_kernel<<<grid_for((size_t)W * H), 256, 0, s>>>(state, W, H, seed, patches, npatch);
}

void launch_seed_tiles(float* state, int W, int H, uint32_t seed, const float* pattern, int pw, int ph, int spacing,
                       cudaStream_t s) {
    seed_tiles_kernel<<<grid_for((size_t)W * H), 256, 0, s>>>(state, W, H, seed, pattern, pw, ph, spacing);
}

void launch_world_stats(const DevWorld* worlds, int nworlds, float* out, cudaStream_t s) {
    world_stats_kernel<<<nworlds, 1024, 0, s>>>(worlds, out);
}

}  // namespace lenia
