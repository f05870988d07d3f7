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
constexpr float SQRT3_2 = 0.86602540378443865f;

FFT_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FFT_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
FFT_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
FFT_HD float2 cmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); } // a*conj(b)
FFT_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
FFT_HD float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// multiply by exp(sign * i * pi/2): -i for the forward transform, +i for the inverse
template <bool INV> FFT_HD float2 rot90(float2 z) { return INV ? make_float2(-z.y, z.x) : make_float2(z.y, -z.x); }

// exp(sign*2*pi*i*j/R) for compile-time R in {2,4,8,16} and j, via the 16-entry table
template <int R, bool INV> FFT_HD float2 wR(int j) {
    int t = (j * (16 / R)) & 15;
    return make_float2(c16(t), INV ? s16(t) : -s16(t));
}

// z * exp(sign*2*pi*i*j/R) for compile-time j: quarter turns are exact swaps and negations
// (a general complex multiply by 0 and +-1 would cost four instructions under IEEE rules).
template <int R, bool INV> FFT_HD float2 cmul_wR(float2 z, int j) {
    const int t = (j * (16 / R)) & 15;
    if (t == 0) return z;
    if (t == 8) return make_float2(-z.x, -z.y);
    if (t == 4) return rot90<INV>(z);
    if (t == 12) return rot90<!INV>(z);
    return cmul(z, wR<R, INV>(j));
}

// ------------------------------------------------------------------ register DFTs
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
    FFT_HD static void run(float2* v) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b); v[1] = csub(a, b);
    }
};

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
};

template <bool INV> struct Dft<4, INV> {
    FFT_HD static void run(float2* v) {
        float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        float2 t2 = cadd(v[1], v[3]), t3 = rot90<INV>(csub(v[1], v[3]));
        v[0] = cadd(t0, t2); v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3); v[3] = csub(t1, t3);
    }
};

// R = R1 * R2 with m = R2*m1 + m2 and q = q1 + R1*q2:
//   u[m2][q1] = DFT_R1 over m1 of v[R2*m1 + m2];  u *= w_R^(m2*q1);  y[q1 + R1*q2] = DFT_R2 over m2.
template <int R1, int R2, bool INV> FFT_HD void dft_split(float2* v) {
    constexpr int R = R1 * R2;
    float2 u[R];
#pragma unroll
    for (int m2 = 0; m2 < R2; m2++) {
        float2 a[R1];
#pragma unroll
        for (int m1 = 0; m1 < R1; m1++) a[m1] = v[R2 * m1 + m2];
        Dft<R1, INV>::run(a);
#pragma unroll
        for (int q1 = 0; q1 < R1; q1++) u[m2 * R1 + q1] = cmul_wR<R, INV>(a[q1], m2 * q1);
    }
#pragma unroll
    for (int q1 = 0; q1 < R1; q1++) {
        float2 b[R2];
#pragma unroll
        for (int m2 = 0; m2 < R2; m2++) b[m2] = u[m2 * R1 + q1];
        Dft<R2, INV>::run(b);
#pragma unroll
        for (int q2 = 0; q2 < R2; q2++) v[q1 + R1 * q2] = b[q2];
    }
}

template <bool INV> struct Dft<8, INV> { FFT_HD static void run(float2* v) { dft_split<4, 2, INV>(v); } };
template <bool INV> struct Dft<16, INV> { FFT_HD static void run(float2* v) { dft_split<4, 4, INV>(v); } };

// ------------------------------------------------------------------ radix plans
// N = 2^a * 3^b (b <= 1).  Every plan starts and ends with the same "outer" radix -- 16 when the
// power-of-two part p is at least 256, else 8 (p >= 64), 4 (p >= 16) or 2 -- with the 3, the
// remaining factor of two and any further 16s in between: 4096 = 16.16.16, 3072 = 16.3.4.16,
// 384 = 8.3.2.8, 96 = 4.3.2.4.  Equal first and last radix let two transforms be chained in
// registers (fft_fused), which every size then does.
struct Plan {
    int len;
    int r[12];
};
FFT_CHD constexpr Plan make_plan(int n) {
    Plan P = {0, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
    const bool three = n % 3 == 0;
    const int p = three ? n / 3 : n;
    const int outer = p >= 256 ? 16 : p >= 64 ? 8 : p >= 16 ? 4 : p >= 4 ? 2 : 0;
    if (outer == 0) {  // p = 1 or 2: no pair of equal radices
        if (three) P.r[P.len++] = 3;
        if (p == 2) P.r[P.len++] = 2;
        return P;
    }
    int q = p / (outer * outer), inner16 = 0;
    while (outer == 16 && q >= 16 && q % 16 == 0) {
        inner16++;
        q /= 16;
    }
    P.r[P.len++] = outer;
    if (three) P.r[P.len++] = 3;
    if (q > 1) P.r[P.len++] = q;  // 2, 4 or 8
    for (int i = 0; i < inner16; i++) P.r[P.len++] = 16;
    P.r[P.len++] = outer;
    return P;
}
FFT_CHD constexpr int plan_len(int n) { return make_plan(n).len; }
FFT_CHD constexpr int plan_radix(int n, int i) { return make_plan(n).r[i]; }
FFT_CHD constexpr int plan_L(int n, int i) {  // product of the radices before stage i
    int l = 1;
    for (int s = 0; s < i; s++) l *= plan_radix(n, s);
    return l;
}
FFT_CHD constexpr bool size_ok(int n) {
    if (n % 3 == 0) n /= 3;
    return n >= 2 && (n & (n - 1)) == 0 && n <= 8192;
}

// Per-stage twiddle tables.  A stage with L > 1 needs w = exp(-2 pi i k / (L R)) for k < L and,
// when R >= 8, w^4; they are copied once per CTA from the global table into shared memory.
FFT_CHD constexpr int stage_tw_count(int n, int i) {
    return plan_L(n, i) > 1 ? (plan_radix(n, i) >= 8 ? 2 : 1) * plan_L(n, i) : 0;
}
FFT_CHD constexpr int stage_tw_offset(int n, int i) {
    int o = 0;
    for (int s = 0; s < i; s++) o += stage_tw_count(n, s);
    return o;
}
FFT_CHD constexpr int tw_table_size(int n) { return stage_tw_offset(n, plan_len(n)); }

// Fill the per-stage tables of transform length N from the global table (threads tid of nth).
template <int N>
FFT_HD void fill_stage_twiddles(float2* stw, const float2* tw, int tid, int nth) {
    for (int i = 0; i < plan_len(N); i++) {
        const int L = plan_L(N, i), R = plan_radix(N, i), off = stage_tw_offset(N, i);
        if (L == 1) continue;
        const int step = TWN / (L * R);
        for (int k = tid; k < L; k += nth) {
            stw[off + k] = tw[k * step];
            if (R >= 8) stw[off + L + k] = tw[4 * k * step];
        }
    }
}

// padded shared-memory index: one float2 of padding per 16 keeps radix-16 stores conflict-free
FFT_HD int pad(int i) { return i + (i >> 4); }
// stride between sequences held in one shared buffer: padded length, +4 so that loads of
// 4 interleaved columns fall into different banks
FFT_CHD constexpr int seq_stride(int n) { return n + n / 16 + 4; }

// Twiddles w^m, m = 1..R-1, of one butterfly from w and (R >= 8) w^4; the other powers are
// products of at most three factors, so each stays within a few float ulps of the exactly rounded
// value (checked against numpy by the host test).
template <int R>
FFT_HD void twiddle_powers(float2 w1, float2 w4, float2* w) {
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
}

// Load butterfly j of a stage (with its inter-stage twiddle) from one sequence; stw is the
// stage's twiddle table (see fill_stage_twiddles).
template <int N, int R, int L, bool INV>
FFT_HD void stage_load(const float2* seq, int j, float2* v, const float2* stw) {
    constexpr int NB = N / R;
    const int k = j % L;
#pragma unroll
    for (int m = 0; m < R; m++) v[m] = seq[pad(j + m * NB)];
    if (L > 1) {
        float2 w[R];
        twiddle_powers<R>(stw[k], R >= 8 ? stw[L + k] : stw[k], w);
#pragma unroll
        for (int m = 1; m < R; m++) v[m] = INV ? cmulc(v[m], w[m]) : cmul(v[m], w[m]);
    }
    Dft<R, INV>::run(v);
}

template <int N, int R, int L>
FFT_HD void stage_store(float2* seq, int j, const float2* v) {
    const int k = j % L;
    const int base = (j - k) * R + k;
#pragma unroll
    for (int m = 0; m < R; m++) seq[pad(base + m * L)] = v[m];
}

}  // namespace lfft
