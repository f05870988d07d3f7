// The reference's own pass structure on CUDA: LENIA_PATH_RADIX2.
//
// This is the "plain FP32 GPU FFT step" that the tensor-core and fused paths are compared
// against.  It keeps spectral.rs:101-283 pass for pass -- one launch per radix-2 Stockham
// stage over global memory, a complex FFT of the real state, f32 twiddles computed per
// butterfly as cos/sin(sign * 3.14159265358979 * k / m), the kernel spectrum built on the
// device by the same FFT, and separate multiply / convolved / update sweeps -- so its results
// track the reference's f32 arithmetic and its memory traffic shows what the fused design saves.
#include <cuda_runtime.h>
#include <math.h>

#include "step_radix2.cuh"

namespace lenia {

constexpr int R2_WG = 256;

__device__ __forceinline__ float clamp01_r2(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// spectral.rs:288-295 (Lenia core with shells), 356-359 (SmoothLife), 427-433 (MNCA ring), f32
__device__ float shape_f32(const R2Shape& k, float r) {
    switch (k.shape) {
    case LENIA_SHAPE_LENIA: {
        float q = r / k.radius;
        int B = k.nshells < 1 ? 1 : k.nshells;
        if (q <= 0.0f || q >= 1.0f) return 0.0f;
        float bq = (float)B * q;
        int i = B == 1 ? 0 : (int)floorf(bq);
        if (i >= B) return 0.0f;
        float f = B == 1 ? q : bq - (float)i;
        if (f <= 0.0f || f >= 1.0f) return 0.0f;
        return k.beta[i] * expf(4.0f - 1.0f / (f * (1.0f - f)));
    }
    case LENIA_SHAPE_SL_INNER: {
        float ri = k.radius / 3.0f, aa = 0.5f;
        return fminf(fmaxf((ri + aa - r) / (2.0f * aa), 0.0f), 1.0f);
    }
    case LENIA_SHAPE_SL_OUTER: {
        float ra = k.radius, ri = k.radius / 3.0f, aa = 0.5f;
        return fminf(fmaxf((ra + aa - r) / (2.0f * aa), 0.0f), 1.0f) * fminf(fmaxf((r - ri + aa) / (2.0f * aa), 0.0f), 1.0f);
    }
    case LENIA_SHAPE_RING: return (r >= k.lo && r < k.hi) ? 1.0f : 0.0f;
    }
    return 0.0f;
}

// spectral.rs:150-171: kernel at min-image distance / sum, as complex
__global__ void r2_kernel_init(float2* next, int w, int h, R2Shape k, float sum) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    const float dx = (float)min(x, w - x), dy = (float)min(y, h - y);
    next[(size_t)y * w + x] = make_float2(shape_f32(k, sqrtf(dx * dx + dy * dy)) / sum, 0.0f);
}

// spectral.rs:201-206 (load)
__global__ void r2_load(const float* __restrict__ state, float2* __restrict__ next, int w, int h) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    const size_t i = (size_t)y * w + x;
    next[i] = make_float2(state[i], 0.0f);
}

// spectral.rs:14-64 (fft_pass), one stage
__global__ void r2_stage(const float2* __restrict__ cur, float2* __restrict__ next, int w, int h, int axis_x, int inverse,
                         int phase) {
    const int n = axis_x ? w : h, rows = axis_x ? h : w, half = n / 2;
    const int p = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (p >= half || r >= rows) return;
    const int m = 1 << phase, k = p & (m - 1);
    auto idx = [&](int q) -> size_t { return axis_x ? (size_t)r * w + q : (size_t)q * w + r; };
    const float2 a = cur[idx(p)], b = cur[idx(p + half)];
    const float spi = inverse ? 3.14159265358979f : -3.14159265358979f;
    const float angle = __fdiv_rn(__fmul_rn(spi, (float)k), (float)m);
    const float2 tw = make_float2(cosf(angle), sinf(angle));
    const float2 t = make_float2(b.x * tw.x - b.y * tw.y, b.x * tw.y + b.y * tw.x);
    next[idx(2 * p - k)] = make_float2(a.x + t.x, a.y + t.y);
    next[idx(2 * p - k + m)] = make_float2(a.x - t.x, a.y - t.y);
}

// spectral.rs:209-213 (spectrum), 174-181 (keep)
__global__ void r2_copy(const float2* __restrict__ a, float2* __restrict__ b, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// spectral.rs:217-224 (multiply)
__global__ void r2_multiply(const float2* __restrict__ spec, const float2* __restrict__ kern, float2* __restrict__ next,
                            size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 a = spec[i], b = kern[i];
    next[i] = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// spectral.rs:227-234 (convolved)
__global__ void r2_convolved(const float2* __restrict__ cur, float* __restrict__ out, float scale, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = cur[i].x * scale;
}

// spectral.rs:246-264 with the bodies of :337-345 (Lenia), :396-407 (SmoothLife), :461-472 (MNCA)
__global__ void r2_update(float* __restrict__ state, const float* __restrict__ c0, const float* __restrict__ c1,
                          int rule, float mu, float sigma, float dt, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float s = state[i];
    float o;
    if (rule == LENIA_RULE_LENIA) {
        const float d = (c0[i] - mu) / sigma;
        o = clamp01_r2(s + dt * (2.0f * expf(-0.5f * d * d) - 1.0f));
    } else if (rule == LENIA_RULE_SMOOTHLIFE) {
        const float B1 = 0.278f, B2 = 0.365f, D1 = 0.267f, D2 = 0.445f, AN = 0.028f, AM = 0.147f, DT = 0.1f;
        const float a = c0[i], b = c1[i];
        const float m = 1.0f / (1.0f + expf((0.5f - a) * 4.0f / AM));
        const float lo = B1 * (1.0f - m) + D1 * m, hi = B2 * (1.0f - m) + D2 * m;
        const float target = (1.0f / (1.0f + expf((lo - b) * 4.0f / AN))) * (1.0f - 1.0f / (1.0f + expf((hi - b) * 4.0f / AN)));
        o = clamp01_r2(s + DT * (2.0f * target - 1.0f));
    } else {
        const float a = c0[i], b = c1[i];
        o = s;
        if (a >= 0.210f && a <= 0.220f) o = 1.0f;
        if (a >= 0.350f && a <= 0.500f) o = 0.0f;
        if (a >= 0.750f && a <= 0.850f) o = 0.0f;
        if (a >= 0.120f && a <= 0.150f) o = 0.0f;
        if (b >= 0.100f && b <= 0.280f) o = 0.0f;
        if (b >= 0.430f && b <= 0.550f) o = 1.0f;
    }
    state[i] = o;
}

static int ilog2i(int n) { int l = 0; while ((1 << l) < n) l++; return l; }

// log2(n) stages along one axis with ping-pong; returns the index of the buffer holding the result.
static int r2_fft_axis(float2* buf[2], int cur, int w, int h, bool axis_x, bool inverse, cudaStream_t s) {
    const int n = axis_x ? w : h, rows = axis_x ? h : w;
    const dim3 grid((n / 2 + R2_WG - 1) / R2_WG, rows);
    for (int ph = 0; ph < ilog2i(n); ph++) {
        r2_stage<<<grid, R2_WG, 0, s>>>(buf[cur], buf[cur ^ 1], w, h, axis_x ? 1 : 0, inverse ? 1 : 0, ph);
        cur ^= 1;
    }
    return cur;
}

int r2_launches_per_step(const R2World& r) {
    return 1 + ilog2i(r.w) + ilog2i(r.h) + 1 + r.k * (1 + ilog2i(r.h) + ilog2i(r.w) + 1) + 1;
}

void r2_enqueue_kernel_spectra(R2World& r, const R2Shape* shapes, const float* sums, cudaStream_t s) {
    const dim3 g((r.w + R2_WG - 1) / R2_WG, r.h);
    const size_t n = (size_t)r.w * r.h;
    for (int i = 0; i < r.k; i++) {
        r2_kernel_init<<<g, R2_WG, 0, s>>>(r.work[0], r.w, r.h, shapes[i], sums[i]);
        int cur = r2_fft_axis(r.work, 0, r.w, r.h, true, false, s);
        cur = r2_fft_axis(r.work, cur, r.w, r.h, false, false, s);
        r2_copy<<<(unsigned)((n + R2_WG - 1) / R2_WG), R2_WG, 0, s>>>(r.work[cur], r.kern[i], n);
    }
}

void r2_enqueue_convolve(R2World& r, cudaStream_t s) {
    const dim3 g((r.w + R2_WG - 1) / R2_WG, r.h);
    const size_t n = (size_t)r.w * r.h;
    const unsigned g1 = (unsigned)((n + R2_WG - 1) / R2_WG);
    r2_load<<<g, R2_WG, 0, s>>>(r.state, r.work[0], r.w, r.h);
    int cur = r2_fft_axis(r.work, 0, r.w, r.h, true, false, s);
    cur = r2_fft_axis(r.work, cur, r.w, r.h, false, false, s);
    r2_copy<<<g1, R2_WG, 0, s>>>(r.work[cur], r.spec, n);
    const float scale = 1.0f / (float)n;  // spectral.rs:215
    for (int i = 0; i < r.k; i++) {
        r2_multiply<<<g1, R2_WG, 0, s>>>(r.spec, r.kern[i], r.work[0], n);
        int c = r2_fft_axis(r.work, 0, r.w, r.h, false, true, s);
        c = r2_fft_axis(r.work, c, r.w, r.h, true, true, s);
        r2_convolved<<<g1, R2_WG, 0, s>>>(r.work[c], r.conv[i], scale, n);
    }
}

void r2_enqueue_step(R2World& r, cudaStream_t s) {
    const size_t n = (size_t)r.w * r.h;
    r2_enqueue_convolve(r, s);
    r2_update<<<(unsigned)((n + R2_WG - 1) / R2_WG), R2_WG, 0, s>>>(r.state, r.conv[0], r.k > 1 ? r.conv[1] : r.conv[0],
                                                                    r.rule, r.mu, r.sigma, r.dt, n);
}

}  // namespace lenia
