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

// The reference's other seeders: SmoothLife's scattered discs (spectral.rs:385-395) and MNCA's
// random 3x3 blocks (spectral.rs:456-460).
__global__ void seed_rule_kernel(float* state, int W, int H, uint32_t seed, int kind) {
    const size_t n = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(i % W), y = (uint32_t)(i / W);
        float v = 0.0f;
        if (kind == LENIA_SEED_SL_DISCS) {
            const uint32_t tile = 96u;
            const uint32_t c = rand3(x / tile, y / tile, seed);
            if ((c & 1u) != 0u) {
                const float dx = (float)(x % tile) - (float)tile / 2.0f, dy = (float)(y % tile) - (float)tile / 2.0f;
                v = (dx * dx + dy * dy < 24.0f * 24.0f) ? 1.0f : 0.0f;
            }
        } else {
            v = unit_f(rand3(x / 3u, y / 3u, seed)) < 0.32f ? 1.0f : 0.0f;
        }
        state[i] = v;
    }
}

// sim.rs:17-41 (view_main) with the shade functions of spectral.rs:347-349, 410-412, 475-477 and
// the ramp/mix3 helpers of program.rs:148-157: an n x n supersampled average in light (squares,
// then the square root) of the state's colours, outside the world black; rgba8 output.
__device__ __forceinline__ float3 mix3f(float3 a, float3 b, float t) {
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return make_float3(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t);
}
__device__ float3 shade(float t, int palette) {
    if (palette == LENIA_PALETTE_MNCA) return mix3f(make_float3(0.02f, 0.02f, 0.07f), make_float3(0.75f, 0.95f, 0.85f), t);
    float3 c[5];
    if (palette == LENIA_PALETTE_SMOOTHLIFE) {
        c[0] = make_float3(0.02f, 0.02f, 0.03f); c[1] = make_float3(0.3f, 0.07f, 0.25f); c[2] = make_float3(0.85f, 0.25f, 0.25f);
        c[3] = make_float3(0.98f, 0.7f, 0.3f); c[4] = make_float3(1.0f, 0.98f, 0.85f);
    } else {
        c[0] = make_float3(0.01f, 0.01f, 0.05f); c[1] = make_float3(0.08f, 0.12f, 0.45f); c[2] = make_float3(0.1f, 0.6f, 0.7f);
        c[3] = make_float3(0.95f, 0.85f, 0.4f); c[4] = make_float3(1.0f, 0.98f, 0.9f);
    }
    const float s = fminf(fmaxf(t, 0.0f), 1.0f) * 4.0f;
    if (s < 1.0f) return mix3f(c[0], c[1], s);
    if (s < 2.0f) return mix3f(c[1], c[2], s - 1.0f);
    if (s < 3.0f) return mix3f(c[2], c[3], s - 2.0f);
    return mix3f(c[3], c[4], s - 3.0f);
}

__global__ void render_kernel(const float* __restrict__ state, int W, int H, float ox, float oy, float scale, int n,
                              int out_w, int out_h, int palette, uchar4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= out_w || py >= out_h) return;
    float ar = 0.f, ag = 0.f, ab = 0.f;
    for (int sy = 0; sy < n; sy++)
        for (int sx = 0; sx < n; sx++) {
            const float subx = ((float)sx + 0.5f) / (float)n, suby = ((float)sy + 0.5f) / (float)n;
            const float x = ox + ((float)px + subx) * scale, y = oy + ((float)py + suby) * scale;
            if (x >= 0.0f && y >= 0.0f && x < (float)W && y < (float)H) {
                const int cx = min((int)x, W - 1), cy = min((int)y, H - 1);
                const float3 c = shade(state[(size_t)cy * W + cx], palette);
                ar += c.x * c.x;
                ag += c.y * c.y;
                ab += c.z * c.z;
            }
        }
    const float inv = 1.0f / (float)(n * n);
    auto u8 = [](float v) { return (unsigned char)__float2int_rn(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f); };
    out[(size_t)py * out_w + px] = make_uchar4(u8(sqrtf(ar * inv)), u8(sqrtf(ag * inv)), u8(sqrtf(ab * inv)), 255);
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

void launch_seed_rule(float* state, int W, int H, uint32_t seed, int kind, cudaStream_t s) {
    seed_rule_kernel<<<grid_for((size_t)W * H), 256, 0, s>>>(state, W, H, seed, kind);
}

void launch_render(const float* state, int W, int H, float ox, float oy, float scale, int n, int out_w, int out_h,
                   int palette, uchar4* out, cudaStream_t s) {
    const dim3 blk(16, 16), grd((out_w + 15) / 16, (out_h + 15) / 16);
    render_kernel<<<grd, blk, 0, s>>>(state, W, H, ox, oy, scale, n, out_w, out_h, palette, out);
}

void launch_world_stats(const DevWorld* worlds, int nworlds, float* out, cudaStream_t s) {
    world_stats_kernel<<<nworlds, 1024, 0, s>>>(worlds, out);
}

}  // namespace lenia
