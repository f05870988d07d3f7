// Shared-memory Stockham FFT building blocks (mixed radix 2/3/4/8/16), FP32.
//
// The reference runs one radix-2 Stockham stage per dispatch over global memory
// (crates/auto-core/src/automata/spectral.rs:14-64: src p and p+n/2, dst 2p-k and 2p-k+m,
// twiddle exp(sign*i*pi*k/m)).  Here the same autosort formulation is generalised to radix R:
// with L the length of the sub-transforms already done,
//     butterfly j in [0, N/R), k = j mod L
//     v[m]   = x[j + m*N/R] * exp(sign*2*pi*i*k*m/(L*R))     m = 0..R-1
//     v      = DFT_R(v)
//     y[(j-k)*R + k + m*L] = v[m]
// which is the reference's stage for R = 2 (m there is L here).  Whole sequences live in
// shared memory and each thread keeps its butterflies in registers across a barrier, so a
// 4096-point transform costs 3 radix-16 passes over shared memory instead of 12 over HBM.
//
// Everything here is plain C++ on float2 so that the same templates compile for the host
// unit test (tests compile this header with g++ and compare against numpy's FFT).
#pragma once

#if defined(__CUDACC__)
#define FFT_HD __host__ __device__ __forceinline__
#define FFT_CHD __host__ __device__
#else
#include <math.h>
#define FFT_HD inline
#define FFT_CHD
#ifndef FFT_HOST_FLOAT2
#define FFT_HOST_FLOAT2
struct float2 { float x, y; };
static inline float2 make_float2(float x, float y) { float2 r; r.x = x; r.y = y; return r; }
#endif
#endif

namespace lfft {

// Twiddle table length: exp(-2*pi*i*t/TWN) for t in [0, TWN).  Every supported transform
// length (2^a * 3^b, a <= 13, b <= 1) divides TWN.
constexpr int TWN = 24576;

// cos/sin(2*pi*t/16), t = 0..15 (exact values rounded to float); folds to a constant when t is.
FFT_CHD constexpr float c16(int t) {
    return t == 0 ? 1.0f : t == 1 ? 0.92387953251128674f : t == 2 ? 0.70710678118654752f
         : t == 3 ? 0.38268343236508978f : t == 4 ? 0.0f : t == 5 ? -0.38268343236508978f
         : t == 6 ? -0.70710678118654752f : t == 7 ? -0.92387953251128674f : t == 8 ? -1.0f
         : t == 9 ? -0.92387953251128674f : t == 10 ? -0.70710678118654752f : t == 11 ? -0.38268343236508978f
         : t == 12 ? 0.0f : t == 13 ? 0.38268343236508978f : t == 14 ? 0.70710678118654752f
         : 0.92387953251128674f;
}
FFT_CHD constexpr float s16(int t) { return c16((t + 12) & 15); }  // sin(x) = cos(x - pi/2)
// cos/sin(2*pi*t/32), t = 0..31, from cos(pi*q/16) for q = 0..8 and the quadrant symmetries; the even
// t are c16(t/2)'s values
FFT_CHD constexpr float c32q(int q) {
    return q == 0 ? 1.0f : q == 1 ? 0.98078528040323044913f : q == 2 ? 0.92387953251128675613f
         : q == 3 ? 0.83146961230254523708f : q == 4 ? 0.70710678118654752440f : q == 5 ? 0.55557023301960222474f
         : q == 6 ? 0.38268343236508977173f : q == 7 ? 0.19509032201612826785f : 0.0f;
}
FFT_CHD constexpr float c32(int t) {
    return (t & 31) <= 8 ? c32q(t & 31) : (t & 31) <= 16 ? -c32q(16 - (t & 31)) : (t & 31) <= 24 ? -c32q((t & 31) - 16)
                                                                                                  : c32q(32 - (t & 31));
}
FFT_CHD constexpr float s32(int t) { return c32((t + 24) & 31); }
constexpr float SQRT3_2 = 0.86602540378443865f;

FFT_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
FFT_HD float2 cmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); } // a*conj(b)
FFT_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
FFT_HD float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
FFT_HD float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }
// multiply by exp(sign * i * pi/2): -i for the forward transform, +i for the inverse
template <bool INV> FFT_HD float2 rot90(float2 z) { return INV ? make_float2(-z.y, z.x) : make_float2(z.y, -z.x); }

// ------------------------------------------------------------------ paired sequences
// Two sequences transformed side by side, component-paired: re = (a.re, b.re), im = (a.im, b.im).
// The two always share their twiddles (same butterfly of the same stage), so on sm_100 and later
// every add, multiply and fma of a pair is one f32x2 instruction, and one 16-byte shared-memory
// access moves an element of both sequences: the instruction count of one sequence for two.
struct alignas(16) cpair {
    float2 re, im;
};
// a twiddle held in both halves: rr = (wr, wr), ii = (wi, wi)
struct alignas(16) tw2 {
    float2 rr, ii;
};
// Largest radix of a plan, by element (or twiddle) type: 16 for scalar and paired elements alike
// (paired elements with radix-8 plans, 8 registers of data a thread instead of 16, measured 50%
// slower at 4096: more stages, spills at 64 registers, bank conflicts of 16-byte elements).  A pass
// may ask for radix-32 plans where they save a stage (make_plan).
template <class T> FFT_CHD constexpr int max_radix() { return 16; }
FFT_HD float2 f2(float v) { return make_float2(v, v); }
FFT_HD float2 f2add(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
FFT_HD float2 f2sub(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(*reinterpret_cast<unsigned long long*>(&a)),
        "l"(*reinterpret_cast<unsigned long long*>(&b)));
    return *reinterpret_cast<float2*>(&r);
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
FFT_HD float2 f2mul(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __fmul2_rn(a, b);
#else
    return make_float2(a.x * b.x, a.y * b.y);
#endif
}
FFT_HD float2 f2fma(float2 a, float2 b, float2 c) {  // a * b + c, one rounding
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __ffma2_rn(a, b, c);
#else
    return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}
// a complex add or subtract of one float2 is one f32x2 instruction (two IEEE adds, so the results
// are those of the two scalar adds)
FFT_HD float2 cadd(float2 a, float2 b) { return f2add(a, b); }
FFT_HD float2 csub(float2 a, float2 b) { return f2add(a, make_float2(-b.x, -b.y)); }
FFT_HD cpair cadd(cpair a, cpair b) { return {f2add(a.re, b.re), f2add(a.im, b.im)}; }
FFT_HD cpair csub(cpair a, cpair b) { return {f2sub(a.re, b.re), f2sub(a.im, b.im)}; }
FFT_HD cpair cscale(cpair a, float s) { return {f2mul(a.re, f2(s)), f2mul(a.im, f2(s))}; }
FFT_HD cpair cscale2(cpair a, float2 s) { return {f2mul(a.re, s), f2mul(a.im, s)}; }  // sequence a by s.x, b by s.y
FFT_HD cpair cneg(cpair a) { return {f2sub(f2(0.0f), a.re), f2sub(f2(0.0f), a.im)}; }
template <bool INV> FFT_HD cpair rot90(cpair z) {
    return INV ? cpair{f2sub(f2(0.0f), z.im), z.re} : cpair{z.im, f2sub(f2(0.0f), z.re)};
}
FFT_HD tw2 splat(float2 w) { return {f2(w.x), f2(w.y)}; }
FFT_HD cpair cmul(cpair a, tw2 w) { return {f2sub(f2mul(a.re, w.rr), f2mul(a.im, w.ii)), f2fma(a.re, w.ii, f2mul(a.im, w.rr))}; }
FFT_HD cpair cmulc(cpair a, tw2 w) { return {f2fma(a.im, w.ii, f2mul(a.re, w.rr)), f2sub(f2mul(a.im, w.rr), f2mul(a.re, w.ii))}; }
FFT_HD cpair cmul(cpair a, float2 w) { return cmul(a, splat(w)); }
FFT_HD tw2 cmul(tw2 a, tw2 b) { return {f2sub(f2mul(a.rr, b.rr), f2mul(a.ii, b.ii)), f2fma(a.rr, b.ii, f2mul(a.ii, b.rr))}; }

// exp(sign*2*pi*i*j/R) for compile-time R in {2,4,8,16,32} and j, via the 16- or 32-entry table
template <int R, bool INV> FFT_HD float2 wR(int j) {
    if constexpr (R == 32) {
        const int t = j & 31;
        return make_float2(c32(t), INV ? s32(t) : -s32(t));
    } else {
        const int t = (j * (16 / R)) & 15;
        return make_float2(c16(t), INV ? s16(t) : -s16(t));
    }
}

// z * exp(sign*2*pi*i*j/R) for compile-time j: quarter turns are exact swaps and negations
// (a general complex multiply by 0 and +-1 would cost four instructions under IEEE rules).
template <int R, bool INV, class T> FFT_HD T cmul_wR(T z, int j) {
    const int t = R == 32 ? (j & 31) : 2 * ((j * (16 / R)) & 15);  // in 32nds of a turn
    if (t == 0) return z;
    if (t == 16) return cneg(z);
    if (t == 8) return rot90<INV>(z);
    if (t == 24) return rot90<!INV>(z);
    return cmul(z, wR<R, INV>(j));
}

// ------------------------------------------------------------------ register DFTs
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
    template <class T> FFT_HD static void run(T* v) {
        T a = v[0], b = v[1];
        v[0] = cadd(a, b); v[1] = csub(a, b);
    }
};

// t -/+ sign*i*c*d for a complex pair of sequences, without a separate negation
template <bool INV> FFT_HD void rot_pm(cpair t, cpair d, float c, cpair& p, cpair& q) {
    // forward: sign*i*c*d = (c d.im, -c d.re); inverse: (-c d.im, c d.re)
    const float2 cc = f2(INV ? -c : c);
    p = {f2fma(d.im, cc, t.re), f2sub(t.im, f2mul(d.re, cc))};
    q = {f2sub(t.re, f2mul(d.im, cc)), f2fma(d.re, cc, t.im)};
}

template <bool INV> struct Dft<3, INV> {
    FFT_HD static void run(float2* v) {
        float2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        float2 t = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
        // sign*i*(sqrt(3)/2)*d
        float2 r = INV ? make_float2(-SQRT3_2 * d.y, SQRT3_2 * d.x) : make_float2(SQRT3_2 * d.y, -SQRT3_2 * d.x);
        v[0] = cadd(v[0], s);
        v[1] = cadd(t, r);
        v[2] = csub(t, r);
    }
    FFT_HD static void run(cpair* v) {
        const cpair s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        const cpair t = {f2fma(s.re, f2(-0.5f), v[0].re), f2fma(s.im, f2(-0.5f), v[0].im)};
        v[0] = cadd(v[0], s);
        rot_pm<INV>(t, d, SQRT3_2, v[1], v[2]);
    }
};

template <bool INV> struct Dft<4, INV> {
    FFT_HD static void run(float2* v) {
        float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        float2 t2 = cadd(v[1], v[3]), t3 = rot90<INV>(csub(v[1], v[3]));
        v[0] = cadd(t0, t2); v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3); v[3] = csub(t1, t3);
    }
    FFT_HD static void run(cpair* v) {
        const cpair t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        const cpair t2 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        v[0] = cadd(t0, t2); v[2] = csub(t0, t2);
        // v1 = t1 + sign*i*d, v3 = t1 - sign*i*d: adds and subtracts of swapped planes
        if (INV) {
            v[1] = {f2sub(t1.re, d.im), f2add(t1.im, d.re)};
            v[3] = {f2add(t1.re, d.im), f2sub(t1.im, d.re)};
        } else {
            v[1] = {f2add(t1.re, d.im), f2sub(t1.im, d.re)};
            v[3] = {f2sub(t1.re, d.im), f2add(t1.im, d.re)};
        }
    }
};

// R = R1 * R2 with m = R2*m1 + m2 and q = q1 + R1*q2:
//   u[m2][q1] = DFT_R1 over m1 of v[R2*m1 + m2];  u *= w_R^(m2*q1);  y[q1 + R1*q2] = DFT_R2 over m2.
template <int R1, int R2, bool INV, class T> FFT_HD void dft_split(T* v) {
    constexpr int R = R1 * R2;
    T u[R];
#pragma unroll
    for (int m2 = 0; m2 < R2; m2++) {
        T a[R1];
#pragma unroll
        for (int m1 = 0; m1 < R1; m1++) a[m1] = v[R2 * m1 + m2];
        Dft<R1, INV>::run(a);
#pragma unroll
        for (int q1 = 0; q1 < R1; q1++) u[m2 * R1 + q1] = cmul_wR<R, INV>(a[q1], m2 * q1);
    }
#pragma unroll
    for (int q1 = 0; q1 < R1; q1++) {
        T b[R2];
#pragma unroll
        for (int m2 = 0; m2 < R2; m2++) b[m2] = u[m2 * R1 + q1];
        Dft<R2, INV>::run(b);
#pragma unroll
        for (int q2 = 0; q2 < R2; q2++) v[q1 + R1 * q2] = b[q2];
    }
}

template <bool INV> struct Dft<8, INV> { template <class T> FFT_HD static void run(T* v) { dft_split<4, 2, INV>(v); } };
template <bool INV> struct Dft<16, INV> { template <class T> FFT_HD static void run(T* v) { dft_split<4, 4, INV>(v); } };
template <bool INV> struct Dft<32, INV> { template <class T> FFT_HD static void run(T* v) { dft_split<8, 4, INV>(v); } };

// ------------------------------------------------------------------ radix plans
// N = 2^a * 3^b (b <= 1).  Every plan starts and ends with the same "outer" radix -- 16 when the
// power-of-two part p is at least 256, else 8 (p >= 64), 4 (p >= 16) or 2 -- with the 3, the
// remaining factor of two and any further 16s in between: 4096 = 16.16.16, 3072 = 16.3.4.16,
// 384 = 8.3.2.8, 96 = 4.3.2.4.  Equal first and last radix let two transforms be chained in
// registers (fft_fused), which every size then does.
// maxr caps the radix (16: 4096 = 16.16.16; 8: 4096 = 8.8.8.8, 2048 = 8.4.8.8).  With maxr = 32 the
// radix-32 plan is taken only where it has fewer stages than the radix-16 one (1024 = 32.32 against
// 16.4.16, 3072 = 32.3.32, 8192 = 32.8.32): one shared-memory round trip fewer per transform, for 32
// elements a thread in registers.
struct Plan {
    int len;
    int r[14];
};
FFT_CHD constexpr Plan make_plan_capped(int n, int maxr) {
    Plan P = {0, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
    const bool three = n % 3 == 0;
    const int p = three ? n / 3 : n;
    int outer = 0;
    for (int r = 2; r <= maxr; r *= 2)
        if (r * r <= p) outer = r;
    if (outer == 0) {  // p = 1 or 2: no pair of equal radices
        if (three) P.r[P.len++] = 3;
        if (p == 2) P.r[P.len++] = 2;
        return P;
    }
    int q = p / (outer * outer), inner = 0;
    while (outer == maxr && q >= maxr && q % maxr == 0) {
        inner++;
        q /= maxr;
    }
    P.r[P.len++] = outer;
    if (three) P.r[P.len++] = 3;
    if (q > 1) P.r[P.len++] = q;  // below maxr
    for (int i = 0; i < inner; i++) P.r[P.len++] = maxr;
    P.r[P.len++] = outer;
    return P;
}
FFT_CHD constexpr Plan make_plan(int n, int maxr = 16) {
    return maxr <= 16 ? make_plan_capped(n, maxr)
         : (make_plan_capped(n, 32).len < make_plan_capped(n, 16).len ? make_plan_capped(n, 32)
                                                                      : make_plan_capped(n, 16));
}
FFT_CHD constexpr int plan_len(int n, int maxr = 16) { return make_plan(n, maxr).len; }
FFT_CHD constexpr int plan_radix(int n, int i, int maxr = 16) { return make_plan(n, maxr).r[i]; }
FFT_CHD constexpr int plan_L(int n, int i, int maxr = 16) {  // product of the radices before stage i
    int l = 1;
    for (int s = 0; s < i; s++) l *= plan_radix(n, s, maxr);
    return l;
}
FFT_CHD constexpr bool size_ok(int n) {
    if (n % 3 == 0) n /= 3;
    return n >= 2 && (n & (n - 1)) == 0 && n <= 8192;
}

// Per-stage twiddle tables.  A stage with L > 1 needs w = exp(-2 pi i k / (L R)) for k < L and,
// when R >= 8, w^4 (and when R >= 32, w^16); they are copied once per CTA from the global table into
// shared memory.
FFT_CHD constexpr int stage_tw_count(int n, int i, int maxr = 16) {
    return plan_L(n, i, maxr) > 1
               ? (plan_radix(n, i, maxr) >= 32 ? 3 : plan_radix(n, i, maxr) >= 8 ? 2 : 1) * plan_L(n, i, maxr)
               : 0;
}
FFT_CHD constexpr int stage_tw_offset(int n, int i, int maxr = 16) {
    int o = 0;
    for (int s = 0; s < i; s++) o += stage_tw_count(n, s, maxr);
    return o;
}
FFT_CHD constexpr int tw_table_size(int n, int maxr = 16) { return stage_tw_offset(n, plan_len(n, maxr), maxr); }

// Fill the per-stage tables of transform length N from the global table (threads tid of nth);
// a tw2 table holds each twiddle in both halves, for paired sequences.
FFT_HD void set_twiddle(float2& d, float2 w) { d = w; }
FFT_HD void set_twiddle(tw2& d, float2 w) { d = splat(w); }
// One stage per template instance, so that each stage's L, R and table offset are compile-time
// constants (a runtime loop over the stages would evaluate the plan in every thread).
template <int N, class W, int I = 0, int MR = max_radix<W>()>
FFT_HD void fill_stage_twiddles(W* stw, const float2* tw, int tid, int nth) {
    if constexpr (I < plan_len(N, MR)) {
        constexpr int L = plan_L(N, I, MR), R = plan_radix(N, I, MR), off = stage_tw_offset(N, I, MR);
        if constexpr (L > 1) {
            constexpr int step = TWN / (L * R);
            for (int k = tid; k < L; k += nth) {
                set_twiddle(stw[off + k], tw[k * step]);
                if (R >= 8) set_twiddle(stw[off + L + k], tw[4 * k * step]);
                if (R >= 32) set_twiddle(stw[off + 2 * L + k], tw[16 * k * step]);
            }
        }
        fill_stage_twiddles<N, W, I + 1, MR>(stw, tw, tid, nth);
    }
}

// padded shared-memory index: one float2 of padding per 16 keeps radix-16 stores conflict-free
FFT_HD int pad(int i) { return i + (i >> 4); }
// stride between sequences held in one shared buffer: padded length, +4 so that loads of
// 4 interleaved columns fall into different banks
FFT_CHD constexpr int seq_stride(int n) { return n + n / 16 + 4; }

// Twiddles w^m, m = 1..R-1, of one butterfly from w, (R >= 8) w^4 and (R >= 32) w^16; the other
// powers are products of at most four factors, so each stays within a few float ulps of the exactly
// rounded value (checked against numpy by the host test).
template <int R, class W>
FFT_HD void twiddle_powers(W w1, W w4, W w16, W* w) {
    w[1] = w1;
    if (R >= 3) w[2] = cmul(w[1], w[1]);
    if (R >= 4) w[3] = cmul(w[2], w[1]);
    if (R >= 8) {
        w[4] = w4;
        w[5] = cmul(w[4], w[1]);
        w[6] = cmul(w[4], w[2]);
        w[7] = cmul(w[4], w[3]);
    }
    if (R >= 16) {
        w[8] = cmul(w[4], w[4]);
#pragma unroll
        for (int m = 9; m < 12; m++) w[m] = cmul(w[8], w[m - 8]);
        w[12] = cmul(w[8], w[4]);
#pragma unroll
        for (int m = 13; m < 16; m++) w[m] = cmul(w[12], w[m - 12]);
    }
    if (R >= 32) {
        w[16] = w16;
        w[24] = cmul(w[16], w[8]);
#pragma unroll
        for (int m = 17; m < 24; m++) w[m] = cmul(w[16], w[m - 16]);
#pragma unroll
        for (int m = 25; m < 32; m++) w[m] = cmul(w[24], w[m - 24]);
    }
}

// Load butterfly j of a stage (with its inter-stage twiddle) from one sequence; stw is the
// stage's twiddle table (see fill_stage_twiddles).
template <int N, int R, int L, bool INV, class T, class W>
FFT_HD void stage_load(const T* seq, int j, T* v, const W* stw) {
    constexpr int NB = N / R;
    const int k = j % L;
    if constexpr (NB % 16 == 0) {
        // pad(j + m NB) = pad(j) + m (NB + NB / 16): one base, compile-time offsets (evaluating
        // pad per element cost about 40% of the row pass's integer instructions)
        const T* p = seq + pad(j);
#pragma unroll
        for (int m = 0; m < R; m++) v[m] = p[m * (NB + NB / 16)];
    } else {
#pragma unroll
        for (int m = 0; m < R; m++) v[m] = seq[pad(j + m * NB)];
    }
    if (L > 1) {
        W w[R];
        twiddle_powers<R>(stw[k], R >= 8 ? stw[L + k] : stw[k], R >= 32 ? stw[2 * L + k] : stw[k], w);
#pragma unroll
        for (int m = 1; m < R; m++) v[m] = INV ? cmulc(v[m], w[m]) : cmul(v[m], w[m]);
    }
    Dft<R, INV>::run(v);
}

template <int N, int R, int L, class T>
FFT_HD void stage_store(T* seq, int j, const T* v) {
    const int k = j % L;
    const int base = (j - k) * R + k;
    if constexpr (L % 16 == 0 || (L == 1 && 16 % R == 0)) {
        // L a multiple of 16: pad(base + m L) = pad(base) + m (L + L / 16); L = 1 with R | 16: the
        // R elements from base = R j stay within one group of 16
        constexpr int STEP = L == 1 ? 1 : L + L / 16;
        T* p = seq + pad(base);
#pragma unroll
        for (int m = 0; m < R; m++) p[m * STEP] = v[m];
    } else if constexpr (L == 1 && R % 16 == 0) {
        // L = 1, R = 32: base = R j is a multiple of 16, so pad(base + m) = pad(base) + m + m / 16
        T* p = seq + pad(base);
#pragma unroll
        for (int m = 0; m < R; m++) p[m + m / 16] = v[m];
    } else {
#pragma unroll
        for (int m = 0; m < R; m++) seq[pad(base + m * L)] = v[m];
    }
}

}  // namespace lfft
