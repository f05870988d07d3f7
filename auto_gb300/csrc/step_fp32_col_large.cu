// Column-pass instantiations of the fused FP32 step, large sizes (templates in step_fp32.cuh).
#include "step_fp32.cuh"

namespace lenia {

bool launch_col_group_large(int H, int variant, const DevWorld* worlds, const ColItem* items, int nitems,
                            const float2* tw, cudaStream_t s) {
    switch (H) { LENIA_SIZES_LARGE(LENIA_COL_CASE) }
    return false;
}

int col_local_bytes_large(int H, int variant) {
    switch (H) { LENIA_SIZES_LARGE(LENIA_COL_LOCAL_CASE) }
    return -1;
}

}  // namespace lenia
