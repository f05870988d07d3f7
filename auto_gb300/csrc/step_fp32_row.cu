// Row-pass instantiations of the fused FP32 step (templates in step_fp32.cuh).
#include "step_fp32.cuh"

namespace lenia {
using namespace lfft;

template <int W, int NT>
static bool row_go(int mode, int general, int planes, const DevWorld* worlds, const RowItem* items, int nitems,
                   const float2* tw, cudaStream_t s) {
    const size_t smem = row_smem_bytes(W, planes);
    static int attr_max = 0;
    if ((int)smem > attr_max) {
        if (cudaFuncSetAttribute(row_pass<W, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return false;
        attr_max = (int)smem;
    }
    if (nitems > 0) row_pass<W, NT><<<nitems, NT, smem, s>>>(worlds, items, mode, general, tw);
    return true;
}

bool launch_row_fp32(int W, int nt, int mode, int general, const DevWorld* worlds, const RowItem* items, int nitems,
                     int acc_planes, const float2* tw, cudaStream_t s) {
    switch (W) {
#define ROW_CASE(N)                                                                                    \
    case N:                                                                                            \
        if (nt == nt_lo<N>()) return row_go<N, nt_lo<N>()>(mode, general, acc_planes, worlds, items, nitems, tw, s); \
        if (nt == nt_hi<N>()) return row_go<N, nt_hi<N>()>(mode, general, acc_planes, worlds, items, nitems, tw, s); \
        return false;
        LENIA_SIZES(ROW_CASE)
#undef ROW_CASE
    }
    return false;
}

}  // namespace lenia
