// Host build of auto_gb300/csrc/fft_core.cuh: runs every Stockham stage of a plan serially
// (all butterfly loads of a stage, then all stores, as the GPU does across its barrier) so the
// radix plans, register DFTs, twiddle indexing and padding can be checked against numpy on a
// machine without a GPU.
#include <cmath>
#include <vector>
#include "../../auto_gb300/csrc/fft_core.cuh"

using namespace lfft;

template <int N, int I, bool INV, int MR = 16>
static void run_stage(float2* seq, const float2* tw) {
    if constexpr (I < plan_len(N, MR)) {
        constexpr int R = plan_radix(N, I, MR);
        constexpr int L = plan_L(N, I, MR);
        std::vector<float2> v((N / R) * R);
        for (int j = 0; j < N / R; j++) stage_load<N, R, L, INV>(seq, j, &v[j * R], tw + stage_tw_offset(N, I, MR));
        for (int j = 0; j < N / R; j++) stage_store<N, R, L>(seq, j, &v[j * R]);
        run_stage<N, I + 1, INV, MR>(seq, tw);
    }
}

// MR = 32: the plans a pass that asks for radix 32 gets (radix 32 where it saves a stage)
template <int N, int MR = 16>
static int fft_n(int inverse, const float* in, float* out, const float2* tw) {
    std::vector<float2> seq(seq_stride(N));
    std::vector<float2> stw(tw_table_size(N, MR) + 1);
    fill_stage_twiddles<N, float2, 0, MR>(stw.data(), tw, 0, 1);
    for (int i = 0; i < N; i++) seq[pad(i)] = make_float2(in[2 * i], in[2 * i + 1]);
    if (inverse) run_stage<N, 0, true, MR>(seq.data(), stw.data());
    else run_stage<N, 0, false, MR>(seq.data(), stw.data());
    for (int i = 0; i < N; i++) { out[2 * i] = seq[pad(i)].x; out[2 * i + 1] = seq[pad(i)].y; }
    return 0;
}

// Two sequences at once, component-paired (cpair elements, tw2 stage tables), as the paired
// GPU builds run them.
template <int N, int I, bool INV>
static void run_stage_pair(cpair* seq, const tw2* tw) {
    constexpr int MR = max_radix<cpair>();
    if constexpr (I < plan_len(N, MR)) {
        constexpr int R = plan_radix(N, I, MR);
        constexpr int L = plan_L(N, I, MR);
        std::vector<cpair> v((N / R) * R);
        for (int j = 0; j < N / R; j++) stage_load<N, R, L, INV>(seq, j, &v[j * R], tw + stage_tw_offset(N, I, MR));
        for (int j = 0; j < N / R; j++) stage_store<N, R, L>(seq, j, &v[j * R]);
        run_stage_pair<N, I + 1, INV>(seq, tw);
    }
}

template <int N>
static int fft_pair_n(int inverse, const float* a, const float* b, float* oa, float* ob, const float2* tw) {
    std::vector<cpair> seq(seq_stride(N));
    std::vector<tw2> stw(tw_table_size(N, max_radix<cpair>()) + 1);
    fill_stage_twiddles<N>(stw.data(), tw, 0, 1);
    for (int i = 0; i < N; i++)
        seq[pad(i)] = cpair{make_float2(a[2 * i], b[2 * i]), make_float2(a[2 * i + 1], b[2 * i + 1])};
    if (inverse) run_stage_pair<N, 0, true>(seq.data(), stw.data());
    else run_stage_pair<N, 0, false>(seq.data(), stw.data());
    for (int i = 0; i < N; i++) {
        const cpair z = seq[pad(i)];
        oa[2 * i] = z.re.x; oa[2 * i + 1] = z.im.x;
        ob[2 * i] = z.re.y; ob[2 * i + 1] = z.im.y;
    }
    return 0;
}

static const float2* table() {
    static std::vector<float2> tw;
    if (tw.empty()) {
        tw.resize(TWN);
        for (int t = 0; t < TWN; t++) {
            double a = -2.0 * M_PI * (double)t / (double)TWN;
            tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
    }
    return tw.data();
}

#define FFT_SIZES(CASE)                                                                                 \
    CASE(16) CASE(32) CASE(48) CASE(64) CASE(96) CASE(128) CASE(192) CASE(256) CASE(384) CASE(512) \
    CASE(768) CASE(1024) CASE(1536) CASE(2048) CASE(3072) CASE(4096) CASE(8192)

extern "C" int fft_host(int n, int inverse, const float* in, float* out) {
    switch (n) {
#define CASE(N) case N: return fft_n<N>(inverse, in, out, table());
        FFT_SIZES(CASE)
#undef CASE
    }
    return -1;
}

extern "C" int fft_host_r32(int n, int inverse, const float* in, float* out) {
    switch (n) {
#define CASE(N) case N: return fft_n<N, 32>(inverse, in, out, table());
        FFT_SIZES(CASE)
#undef CASE
    }
    return -1;
}

extern "C" int fft_host_pair(int n, int inverse, const float* a, const float* b, float* oa, float* ob) {
    switch (n) {
#define CASE(N) case N: return fft_pair_n<N>(inverse, a, b, oa, ob, table());
        FFT_SIZES(CASE)
#undef CASE
    }
    return -1;
}

// The radix plan of length n with radix cap maxr: its radices into out (at most 14); returns the
// number of stages.
extern "C" int plan_host(int n, int maxr, int* out) {
    const Plan p = make_plan(n, maxr);
    for (int i = 0; i < p.len; i++) out[i] = p.r[i];
    return p.len;
}
