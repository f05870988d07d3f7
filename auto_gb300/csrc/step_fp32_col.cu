// Column-pass instantiations of the fused FP32 step (templates in step_fp32.cuh).
#include "step_fp32.cuh"

namespace lenia {
using namespace lfft;

size_t col_smem_bytes(int H, int nbuf) { return (size_t)nbuf * 4 * seq_stride(H) * sizeof(float2); }
size_t row_smem_bytes(int W, int acc_planes) {
    return (size_t)2 * seq_stride(W) * sizeof(float2) + (size_t)acc_planes * 4 * W * sizeof(float);
}

int max_smem_optin() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

// Dynamic shared memory above 48 KB must be enabled per kernel before the first launch (and
// before any stream capture that contains it); done once per instantiation and size.
template <int H, int NT>
static bool col_attr(size_t smem) {
    static int attr_max = 0;
    if ((int)smem > attr_max) {
        if (cudaFuncSetAttribute(col_pass<H, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return false;
        attr_max = (int)smem;
    }
    return true;
}

template <int H, int NT>
static bool col_go(int nbuf, const DevWorld* worlds, const ColItem* items, int nitems, const float2* tw, cudaStream_t s) {
    const size_t smem = col_smem_bytes(H, nbuf);
    if (!col_attr<H, NT>(smem)) return false;
    if (nitems > 0) col_pass<H, NT><<<nitems, NT, smem, s>>>(worlds, items, nbuf, tw);
    return true;
}

bool launch_col_fp32(int H, int nt, int nbuf, const DevWorld* worlds, const ColItem* items, int nitems,
                     const float2* tw, cudaStream_t s) {
    switch (H) {
#define COL_CASE(N)                                                                      \
    case N:                                                                              \
        if (nt == nt_lo<N>()) return col_go<N, nt_lo<N>()>(nbuf, worlds, items, nitems, tw, s); \
        if (nt == nt_hi<N>()) return col_go<N, nt_hi<N>()>(nbuf, worlds, items, nitems, tw, s); \
        return false;
        LENIA_SIZES(COL_CASE)
#undef COL_CASE
    }
    return false;
}

int nt_choice(int n, int which) {
    switch (n) {
#define NT_CASE(N) case N: return which ? nt_hi<N>() : nt_lo<N>();
        LENIA_SIZES(NT_CASE)
#undef NT_CASE
    }
    return 0;
}

}  // namespace lenia
