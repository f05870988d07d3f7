// Row-pass instantiations of the fused FP32 step, large sizes, general step (several channels or kernels, SmoothLife, MNCA) (templates in
// step_fp32.cuh).
#include "step_fp32.cuh"

namespace lenia {

bool launch_row_group_large_general(int W, int variant, int mode, int general, int planes, const DevWorld* worlds,
                                const RowItem* items, int nitems, const float2* tw, cudaStream_t s) {
    switch (W) { LENIA_SIZES_LARGE(LENIA_ROW_CASE_GENERAL) }
    return false;
}

int row_local_bytes_large_general(int W, int variant) {
    switch (W) { LENIA_SIZES_LARGE(LENIA_ROW_LOCAL_CASE_GENERAL) }
    return -1;
}

}  // namespace lenia
