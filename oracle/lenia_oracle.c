/*
 * CPU oracle for the Lenia-family FFT step.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C and f32, the pass sequence of the reference's
 * spectral automata (ErikFrankling/auto, crates/auto-core/src/automata/spectral.rs).
 * It is the checker for the CUDA engine and the timed CPU baseline; nothing in the
 * shipped library links it.  Only tests/, the smoke check and the bench's CPU leg
 * may load it.
 *
 * Followed line by line (paths relative to the reference project):
 *   - PCG hash, rand3, unit_f ............ crates/auto-core/src/program.rs:140-147
 *   - radix-2 Stockham stage ............. spectral.rs:14-64 (fft_pass)
 *   - kernel_sum (f64 sum of f32 shape) .. spectral.rs:75-83
 *   - kernel placement at min-image dist . spectral.rs:150-171
 *   - step pass order .................... spectral.rs:199-264
 *       load (state,0) -> fft x -> fft y -> spectrum -> per kernel
 *       [multiply -> ifft y -> ifft x -> convolved (x 1/(w*h))] -> update
 *   - Lenia shape, sum, update ........... spectral.rs:288-303, 337-345
 *   - SmoothLife shapes and update ....... spectral.rs:355-407
 *   - MNCA rings and update .............. spectral.rs:426-472
 *   - Orbium tile seeding ................ spectral.rs:313-335 (pattern supplied by caller)
 *   - SmoothLife and MNCA seeds .......... spectral.rs:385-395, 456-460
 *   - view pass (colour ramps) ........... sim.rs:17-41, program.rs:148-157,
 *                                          spectral.rs:347-349, 410-412, 475-477
 *   - size guards ........................ spectral.rs:103-116
 *
 * The multi-shell kernel (beta shells) has no reference code: it follows Chan's
 * Lenia definition K(r) = beta[floor(B q)] * core(frac(B q)), q = r / R, and
 * reduces to the reference's single-shell kernel for beta = [1].
 *
 * Build: see oracle/build.py (gcc -O2 -ffp-contract=off -pthread -shared).
 * -ffp-contract=off keeps a*b - c*d unfused so x86 and Arm hosts give the same bits.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_SHAPE_LENIA 0      /* exponential core with beta shells */
#define ORC_SHAPE_SL_INNER 1   /* SmoothLife inner disc, radius ra/3 */
#define ORC_SHAPE_SL_OUTER 2   /* SmoothLife outer ring, radius ra */
#define ORC_SHAPE_RING 3       /* MNCA hard ring lo <= r < hi */

#define ORC_RULE_LENIA 0
#define ORC_RULE_SMOOTHLIFE 1
#define ORC_RULE_MNCA 2

typedef struct {
    int32_t shape;
    float radius;
    int32_t nshells;
    float beta[3];
    float lo, hi;
} OrcKernel;

typedef struct {
    int32_t rule;
    float mu, sigma, dt; /* Lenia growth; ignored by SmoothLife and MNCA */
} OrcRule;

/* ---------------------------------------------------------------- RNG */
/* program.rs:140-147 */
uint32_t orc_pcg(uint32_t v) {
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
uint32_t orc_rand3(uint32_t a, uint32_t b, uint32_t c) { return orc_pcg(orc_pcg(orc_pcg(a) ^ b) ^ c); }
float orc_unit_f(uint32_t r) { return (float)r * (1.0f / 4294967296.0f); }

/* ------------------------------------------------------- kernel shapes */
static float lenia_core(float q) {
    /* spectral.rs:288-295: exp(4 - 1/(q(1-q))) on (0,1), else 0 */
    if (q <= 0.0f || q >= 1.0f) return 0.0f;
    return expf(4.0f - 1.0f / (q * (1.0f - q)));
}

static float clampf01(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

float orc_shape(const OrcKernel* k, float r) {
    switch (k->shape) {
    case ORC_SHAPE_LENIA: {
        float q = r / k->radius;
        if (k->nshells <= 1) return lenia_core(q) * (k->nshells == 1 ? k->beta[0] : 1.0f);
        if (q <= 0.0f || q >= 1.0f) return 0.0f;
        float bq = (float)k->nshells * q;
        int i = (int)floorf(bq);
        if (i >= k->nshells) return 0.0f;
        return k->beta[i] * lenia_core(bq - (float)i);
    }
    case ORC_SHAPE_SL_INNER: {
        /* spectral.rs:356-359: ri = ra/3, aa = 0.5 */
        float ri = k->radius / 3.0f, aa = 0.5f;
        return clampf01((ri + aa - r) / (2.0f * aa), 0.0f, 1.0f);
    }
    case ORC_SHAPE_SL_OUTER: {
        float ra = k->radius, ri = k->radius / 3.0f, aa = 0.5f;
        return clampf01((ra + aa - r) / (2.0f * aa), 0.0f, 1.0f) *
               clampf01((r - ri + aa) / (2.0f * aa), 0.0f, 1.0f);
    }
    case ORC_SHAPE_RING:
        /* spectral.rs:427-433 */
        return (r >= k->lo && r < k->hi) ? 1.0f : 0.0f;
    }
    return 0.0f;
}

/* Distance out to which the reference sums a kernel (spectral.rs:296, 362, 434). */
int orc_sum_reach(const OrcKernel* k) {
    switch (k->shape) {
    case ORC_SHAPE_LENIA: return (int)ceilf(k->radius) + 1;
    case ORC_SHAPE_SL_INNER:
    case ORC_SHAPE_SL_OUTER: return (int)ceilf(k->radius) + 2;
    case ORC_SHAPE_RING: return (int)ceilf(k->hi) + 1;
    }
    return 0;
}

/* Kernel.reach, the size guard's radius (spectral.rs:111-116, 311, 374, 448). */
int orc_guard_reach(const OrcKernel* k) {
    switch (k->shape) {
    case ORC_SHAPE_LENIA: return (int)ceilf(k->radius);
    case ORC_SHAPE_SL_INNER:
    case ORC_SHAPE_SL_OUTER: return (int)ceilf(k->radius) + 2;
    case ORC_SHAPE_RING: return (int)ceilf(k->hi);
    }
    return 0;
}

/* spectral.rs:75-83: f64 sum of f32 shape values over [-reach, reach]^2, returned as f32. */
float orc_kernel_sum(const OrcKernel* k) {
    int reach = orc_sum_reach(k);
    double sum = 0.0;
    for (int y = -reach; y <= reach; y++)
        for (int x = -reach; x <= reach; x++)
            sum += (double)orc_shape(k, sqrtf((float)(x * x + y * y)));
    return (float)sum;
}

/* spectral.rs:150-171: kernel at min-image torus distance, divided by its sum, as f32. */
int orc_kernel_spatial(int w, int h, const OrcKernel* k, float* out) {
    if (w <= 0 || h <= 0) return -1;
    float sum = orc_kernel_sum(k);
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            float dx = (float)(x < w - x ? x : w - x);
            float dy = (float)(y < h - y ? y : h - y);
            out[(size_t)y * w + x] = orc_shape(k, sqrtf(dx * dx + dy * dy)) / sum;
        }
    }
    return 0;
}

/* ------------------------------------------------------- thread pool-less parallel for */
typedef void (*orc_range_fn)(void* ctx, long lo, long hi);
typedef struct { orc_range_fn fn; void* ctx; long lo, hi; } orc_job;

static void* orc_job_run(void* p) {
    orc_job* j = (orc_job*)p;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static void parallel_for(long n, int threads, orc_range_fn fn, void* ctx) {
    if (threads <= 1 || n < 2) { fn(ctx, 0, n); return; }
    if (threads > 256) threads = 256;
    if (threads > n) threads = (int)n;
    pthread_t tid[256];
    orc_job jobs[256];
    int started[256];
    for (int t = 0; t < threads; t++) {
        jobs[t].fn = fn; jobs[t].ctx = ctx;
        jobs[t].lo = n * t / threads; jobs[t].hi = n * (t + 1) / threads;
        started[t] = (t > 0) && pthread_create(&tid[t], NULL, orc_job_run, &jobs[t]) == 0;
        if (t > 0 && !started[t]) orc_job_run(&jobs[t]);
    }
    orc_job_run(&jobs[0]);
    for (int t = 1; t < threads; t++)
        if (started[t]) pthread_join(tid[t], NULL);
}

/* ------------------------------------------------------- radix-2 Stockham stage */
/* spectral.rs:14-64.  One stage (frame.phase = phase) over every row (axis x) or column
 * (axis y).  cur/next are interleaved complex f32 (re, im), row-major y*w + x. */
typedef struct {
    const float* cur; float* next; int w, h, axis_x, phase; const float* tw; /* 2*m twiddles */
} StageCtx;

static void stage_x(void* p, long lo, long hi) {
    StageCtx* c = (StageCtx*)p;
    int n = c->w, half = n / 2, m = 1 << c->phase;
    for (long r = lo; r < hi; r++) {
        const float* row = c->cur + 2 * (size_t)r * n;
        float* out = c->next + 2 * (size_t)r * n;
        for (int q = 0; q < half; q++) {
            int k = q & (m - 1);
            float ax = row[2 * q], ay = row[2 * q + 1];
            float bx = row[2 * (q + half)], by = row[2 * (q + half) + 1];
            float tx = c->tw[2 * k], ty = c->tw[2 * k + 1];
            float t0 = bx * tx - by * ty, t1 = bx * ty + by * tx;
            int d0 = 2 * q - k, d1 = 2 * q - k + m;
            out[2 * d0] = ax + t0; out[2 * d0 + 1] = ay + t1;
            out[2 * d1] = ax - t0; out[2 * d1 + 1] = ay - t1;
        }
    }
}

static void stage_y(void* p, long lo, long hi) {
    /* parallel over q (the butterfly index along y); inner loop runs along a row */
    StageCtx* c = (StageCtx*)p;
    int w = c->w, n = c->h, half = n / 2, m = 1 << c->phase;
    for (long q = lo; q < hi; q++) {
        int k = (int)q & (m - 1);
        float tx = c->tw[2 * k], ty = c->tw[2 * k + 1];
        const float* a = c->cur + 2 * (size_t)q * w;
        const float* b = c->cur + 2 * (size_t)(q + half) * w;
        float* o0 = c->next + 2 * (size_t)(2 * q - k) * w;
        float* o1 = c->next + 2 * (size_t)(2 * q - k + m) * w;
        for (int r = 0; r < w; r++) {
            float ax = a[2 * r], ay = a[2 * r + 1], bx = b[2 * r], by = b[2 * r + 1];
            float t0 = bx * tx - by * ty, t1 = bx * ty + by * tx;
            o0[2 * r] = ax + t0; o0[2 * r + 1] = ay + t1;
            o1[2 * r] = ax - t0; o1[2 * r + 1] = ay - t1;
        }
    }
}

/* Twiddles of one stage: angle = sign * 3.14159265358979 * f32(k) / f32(m) in f32, as the
 * WGSL does per butterfly (spectral.rs:43-51); cached per k since they depend on (k, m) only. */
static void stage_twiddles(float* tw, int m, int inverse) {
    const float spi = inverse ? (float)3.14159265358979 : (float)(-3.14159265358979);
    for (int k = 0; k < m; k++) {
        volatile float a = spi * (float)k;
        float angle = a / (float)m;
        tw[2 * k] = cosf(angle);
        tw[2 * k + 1] = sinf(angle);
    }
}

static int ilog2(int n) { int l = 0; while ((1 << l) < n) l++; return l; }
static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* fft over one axis: log2(n) stages with ping-pong; returns the buffer holding the result */
static float* fft_axis(float* a, float* b, int w, int h, int axis_x, int inverse, int threads) {
    int n = axis_x ? w : h;
    int stages = ilog2(n);
    float* tw = (float*)malloc(sizeof(float) * 2 * (size_t)n);
    for (int s = 0; s < stages; s++) {
        int m = 1 << s;
        stage_twiddles(tw, m, inverse);
        StageCtx c = {a, b, w, h, axis_x, s, tw};
        if (axis_x) parallel_for(h, threads, stage_x, &c);
        else parallel_for(n / 2, threads, stage_y, &c);
        float* t = a; a = b; b = t;
    }
    free(tw);
    return a;
}

/* spectral.rs:150-181: transform a spatial kernel (already divided by its sum) forward
 * along x then y, f32.  out: 2*w*h floats (interleaved complex). */
int orc_kernel_spectrum(int w, int h, const float* spatial, float* out, int threads) {
    if (!is_pow2(w) || !is_pow2(h)) return -1;
    size_t cells = (size_t)w * h;
    float* a = (float*)malloc(sizeof(float) * 2 * cells);
    float* b = (float*)malloc(sizeof(float) * 2 * cells);
    if (!a || !b) { free(a); free(b); return -2; }
    for (size_t i = 0; i < cells; i++) { a[2 * i] = spatial[i]; a[2 * i + 1] = 0.0f; }
    float* r = fft_axis(a, b, w, h, 1, 0, threads);
    float* o = (r == a) ? b : a;
    r = fft_axis(r, o, w, h, 0, 0, threads);
    memcpy(out, r, sizeof(float) * 2 * cells);
    free(a); free(b);
    return 0;
}

/* ------------------------------------------------------- update rules */
static float rule_update(const OrcRule* rule, float s, const float* c) {
    switch (rule->rule) {
    case ORC_RULE_LENIA: {
        /* spectral.rs:337-345 */
        float d = (c[0] - rule->mu) / rule->sigma;
        return clampf01(s + rule->dt * (2.0f * expf(-0.5f * d * d) - 1.0f), 0.0f, 1.0f);
    }
    case ORC_RULE_SMOOTHLIFE: {
        /* spectral.rs:396-407 */
        const float B1 = 0.278f, B2 = 0.365f, D1 = 0.267f, D2 = 0.445f;
        const float AN = 0.028f, AM = 0.147f, DT = 0.1f;
#define SIG(x, a, alpha) (1.0f / (1.0f + expf(((a) - (x)) * 4.0f / (alpha))))
        float m = SIG(c[0], 0.5f, AM);
        float lo = B1 * (1.0f - m) + D1 * m, hi = B2 * (1.0f - m) + D2 * m;
        float target = SIG(c[1], lo, AN) * (1.0f - SIG(c[1], hi, AN));
#undef SIG
        return clampf01(s + DT * (2.0f * target - 1.0f), 0.0f, 1.0f);
    }
    case ORC_RULE_MNCA: {
        /* spectral.rs:461-472 */
#define BAND(v, lo, hi) ((v) >= (lo) && (v) <= (hi))
        float o = s;
        if (BAND(c[0], 0.210f, 0.220f)) o = 1.0f;
        if (BAND(c[0], 0.350f, 0.500f)) o = 0.0f;
        if (BAND(c[0], 0.750f, 0.850f)) o = 0.0f;
        if (BAND(c[0], 0.120f, 0.150f)) o = 0.0f;
        if (BAND(c[1], 0.100f, 0.280f)) o = 0.0f;
        if (BAND(c[1], 0.430f, 0.550f)) o = 1.0f;
#undef BAND
        return o;
    }
    }
    return s;
}

/* ------------------------------------------------------- the step */
/* spectral.rs:199-264.  kern_spec: nk spectra of 2*w*h floats each (from orc_kernel_spectrum).
 * conv_out (optional): nk * w*h convolved fields of the last step. */
int orc_step(int w, int h, int nk, const float* kern_spec, const OrcRule* rule,
             const float* state_in, float* state_out, float* conv_out, int steps, int threads) {
    if (!is_pow2(w) || !is_pow2(h)) return -1;
    if (nk < 1 || nk > 3) return -1;
    size_t cells = (size_t)w * h;
    float* a = (float*)malloc(sizeof(float) * 2 * cells);
    float* b = (float*)malloc(sizeof(float) * 2 * cells);
    float* spec = (float*)malloc(sizeof(float) * 2 * cells);
    float* conv = (float*)malloc(sizeof(float) * cells * (size_t)nk);
    float* s = (float*)malloc(sizeof(float) * cells);
    if (!a || !b || !spec || !conv || !s) { free(a); free(b); free(spec); free(conv); free(s); return -2; }
    const float scale = 1.0f / (float)cells; /* spectral.rs:215 */
    memcpy(s, state_in, sizeof(float) * cells);
    for (int st = 0; st < steps; st++) {
        for (size_t i = 0; i < cells; i++) { a[2 * i] = s[i]; a[2 * i + 1] = 0.0f; } /* load */
        float* r = fft_axis(a, b, w, h, 1, 0, threads);                             /* fft x */
        float* o = (r == a) ? b : a;
        r = fft_axis(r, o, w, h, 0, 0, threads);                                    /* fft y */
        memcpy(spec, r, sizeof(float) * 2 * cells);                                 /* spectrum */
        for (int k = 0; k < nk; k++) {
            const float* kk = kern_spec + (size_t)k * 2 * cells;
            for (size_t i = 0; i < cells; i++) {                                     /* multiply */
                float ax = spec[2 * i], ay = spec[2 * i + 1], bx = kk[2 * i], by = kk[2 * i + 1];
                a[2 * i] = ax * bx - ay * by;
                a[2 * i + 1] = ax * by + ay * bx;
            }
            r = fft_axis(a, b, w, h, 0, 1, threads);                                /* ifft y */
            o = (r == a) ? b : a;
            r = fft_axis(r, o, w, h, 1, 1, threads);                                /* ifft x */
            for (size_t i = 0; i < cells; i++) conv[(size_t)k * cells + i] = r[2 * i] * scale; /* convolved */
        }
        for (size_t i = 0; i < cells; i++) {                                         /* update */
            float c[3];
            for (int k = 0; k < nk; k++) c[k] = conv[(size_t)k * cells + i];
            s[i] = rule_update(rule, s[i], c);
        }
    }
    memcpy(state_out, s, sizeof(float) * cells);
    if (conv_out) memcpy(conv_out, conv, sizeof(float) * cells * (size_t)nk);
    free(a); free(b); free(spec); free(conv); free(s);
    return 0;
}

/* ------------------------------------------------------- direct convolution (f64) */
/* crates/auto-core/tests/automata.rs:300-362: f64 core, f64 sum over a [-reach, reach]^2
 * window, torus wrap, one Lenia step.  Used only as the known-answer check. */
int orc_direct_lenia_step(int w, int h, float radius, int reach, double mu, double sigma, double dt,
                          const float* start, float* out) {
    double sum = 0.0;
    for (int dy = -reach; dy <= reach; dy++)
        for (int dx = -reach; dx <= reach; dx++) {
            double q = sqrt((double)(dx * dx + dy * dy)) / (double)radius;
            if (q > 0.0 && q < 1.0) sum += exp(4.0 - 1.0 / (q * (1.0 - q)));
        }
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double u = 0.0;
            for (int dy = -reach; dy <= reach; dy++)
                for (int dx = -reach; dx <= reach; dx++) {
                    double q = sqrt((double)(dx * dx + dy * dy)) / (double)radius;
                    if (!(q > 0.0 && q < 1.0)) continue;
                    double k = exp(4.0 - 1.0 / (q * (1.0 - q)));
                    int yy = ((y + dy) % h + h) % h, xx = ((x + dx) % w + w) % w;
                    u += k * (double)start[(size_t)yy * w + xx];
                }
            double d = (u / sum - mu) / sigma;
            double g = 2.0 * exp(-0.5 * d * d) - 1.0;
            double v = (double)start[(size_t)y * w + x] + dt * g;
            out[(size_t)y * w + x] = (float)(v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v));
        }
    return 0;
}

/* ------------------------------------------------------- seeds */
/* spectral.rs:313-335 with the pattern passed in (pw x ph u8/255 values as f32). */
void orc_seed_tiles(int w, int h, uint32_t seed, const float* pattern, int pw, int ph, int spacing,
                    float* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            uint32_t tx = (uint32_t)x / spacing, ty = (uint32_t)y / spacing;
            uint32_t r = orc_rand3(tx, ty, seed);
            float v = 0.0f;
            uint32_t px = (uint32_t)x % spacing, py = (uint32_t)y % spacing;
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
            out[(size_t)y * w + x] = v;
        }
}

/* U[0,1] from unit_f(rand3(x, y, seed)) inside axis-aligned patches (x0, y0, pw, ph) with
 * torus wrap, zero elsewhere: the synthetic initial states of the benchmark configurations. */
void orc_seed_patches(int w, int h, uint32_t seed, const int32_t* patches, int npatch, float* out) {
    memset(out, 0, sizeof(float) * (size_t)w * h);
    for (int p = 0; p < npatch; p++) {
        int x0 = patches[4 * p], y0 = patches[4 * p + 1], pw = patches[4 * p + 2], ph = patches[4 * p + 3];
        for (int j = 0; j < ph; j++)
            for (int i = 0; i < pw; i++) {
                int x = ((x0 + i) % w + w) % w, y = ((y0 + j) % h + h) % h;
                out[(size_t)y * w + x] = orc_unit_f(orc_rand3((uint32_t)x, (uint32_t)y, seed));
            }
    }
}

/* spectral.rs:385-395: SmoothLife's seed, discs of radius 24 in the 96-cell tiles whose
 * rand3(tx, ty, seed) is odd. */
void orc_seed_sl_discs(int w, int h, uint32_t seed, float* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const uint32_t tile = 96u;
            uint32_t c = orc_rand3((uint32_t)x / tile, (uint32_t)y / tile, seed);
            float v = 0.0f;
            if ((c & 1u) != 0u) {
                float dx = (float)((uint32_t)x % tile) - (float)tile / 2.0f;
                float dy = (float)((uint32_t)y % tile) - (float)tile / 2.0f;
                v = (dx * dx + dy * dy < 24.0f * 24.0f) ? 1.0f : 0.0f;
            }
            out[(size_t)y * w + x] = v;
        }
}

/* spectral.rs:456-460: MNCA's seed, 3x3 blocks set where unit_f(rand3(x/3, y/3, seed)) < 0.32. */
void orc_seed_mnca_blocks(int w, int h, uint32_t seed, float* out) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            out[(size_t)y * w + x] = orc_unit_f(orc_rand3((uint32_t)x / 3u, (uint32_t)y / 3u, seed)) < 0.32f ? 1.0f : 0.0f;
}

/* program.rs:148-157 (mix3, ramp) and the shade functions of spectral.rs:347-349, 410-412, 475-477 */
static void mix3(const float* a, const float* b, float t, float* o) {
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    for (int i = 0; i < 3; i++) o[i] = a[i] + (b[i] - a[i]) * t;
}
static void shade(float t, int palette, float* o) {
    static const float L[5][3] = {{0.01f, 0.01f, 0.05f}, {0.08f, 0.12f, 0.45f}, {0.1f, 0.6f, 0.7f},
                                  {0.95f, 0.85f, 0.4f}, {1.0f, 0.98f, 0.9f}};
    static const float S[5][3] = {{0.02f, 0.02f, 0.03f}, {0.3f, 0.07f, 0.25f}, {0.85f, 0.25f, 0.25f},
                                  {0.98f, 0.7f, 0.3f}, {1.0f, 0.98f, 0.85f}};
    static const float M[2][3] = {{0.02f, 0.02f, 0.07f}, {0.75f, 0.95f, 0.85f}};
    if (palette == 2) { mix3(M[0], M[1], t, o); return; }
    const float (*c)[3] = palette == 1 ? S : L;
    float s = (t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t)) * 4.0f;
    if (s < 1.0f) mix3(c[0], c[1], s, o);
    else if (s < 2.0f) mix3(c[1], c[2], s - 1.0f, o);
    else if (s < 3.0f) mix3(c[2], c[3], s - 2.0f, o);
    else mix3(c[3], c[4], s - 3.0f, o);
}

/* crates/auto-core/src/sim.rs:17-41 (view_main): n x n supersampling, averaging c*c, then sqrt. */
void orc_render(const float* state, int w, int h, float ox, float oy, float scale, int n, int out_w, int out_h,
                int palette, uint8_t* out) {
    for (int py = 0; py < out_h; py++)
        for (int px = 0; px < out_w; px++) {
            float acc[3] = {0.0f, 0.0f, 0.0f};
            for (int sy = 0; sy < n; sy++)
                for (int sx = 0; sx < n; sx++) {
                    float subx = ((float)sx + 0.5f) / (float)n, suby = ((float)sy + 0.5f) / (float)n;
                    float x = ox + ((float)px + subx) * scale, y = oy + ((float)py + suby) * scale;
                    if (x >= 0.0f && y >= 0.0f && x < (float)w && y < (float)h) {
                        int cx = (int)x < w - 1 ? (int)x : w - 1, cy = (int)y < h - 1 ? (int)y : h - 1;
                        float c[3];
                        shade(state[(size_t)cy * w + cx], palette, c);
                        for (int i = 0; i < 3; i++) acc[i] += c[i] * c[i];
                    }
                }
            uint8_t* o = out + 4 * ((size_t)py * out_w + px);
            for (int i = 0; i < 3; i++) {
                float v = sqrtf(acc[i] / (float)(n * n));
                v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
                o[i] = (uint8_t)lrintf(v * 255.0f);
            }
            o[3] = 255;
        }
}
