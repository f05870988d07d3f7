// Dispatch of the fused FP32 step's launches to the per-size instantiations.
#include "step_fp32.cuh"

namespace lenia {

static size_t col_khat_bytes_of(int H) {
    switch (H) {
#define KB_CASE(N) case N: return col_khat_bytes<N>();
        LENIA_SIZES_SMALL(KB_CASE) LENIA_SIZES_LARGE(KB_CASE)
#undef KB_CASE
    }
    return 0;
}

// the largest of the scalar builds' (radix-32 and radix-16 plans) and the paired build's (same
// sequence bytes; the paired stage tables hold each twiddle twice)
size_t col_smem_bytes(int H) {
    const int t32 = lfft::tw_table_size(H, CMR), t16 = lfft::tw_table_size(H);
    const size_t scalar_tables = ((t32 > t16 ? t32 : t16) + 1) * sizeof(float2);
    const size_t paired_tables = (lfft::tw_table_size(H, PMR) + 1) * sizeof(lfft::tw2);
    return (size_t)TC * lfft::seq_stride(H) * sizeof(float2) + (scalar_tables > paired_tables ? scalar_tables : paired_tables) +
           col_khat_bytes_of(H);
}
size_t row_smem_bytes(int W, int acc_planes) {
    switch (W) {
#define RS_CASE(N) \
    case N: return acc_planes > 0 ? row_smem<N, true>(1, acc_planes) : row_smem<N, false>(0, 0);
        LENIA_SIZES_SMALL(RS_CASE) LENIA_SIZES_LARGE(RS_CASE)
#undef RS_CASE
    }
    return 0;
}

int row_item_rows(int W, int general) { return 2 * row_seqs(W, general != 0); }

bool col_has_r16_variant(int H) { return lfft::plan_radix(H, 0, CMR) == 32; }

int max_smem_optin() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

bool launch_col_fp32(int H, int variant, const DevWorld* worlds, const ColItem* items, int nitems,
                     const float2* tw, cudaStream_t s) {
    return launch_col_group_small(H, variant, worlds, items, nitems, tw, s) ||
           launch_col_group_large(H, variant, worlds, items, nitems, tw, s);
}

bool launch_row_fp32(int W, int variant, int mode, int general, const DevWorld* worlds, const RowItem* items,
                     int nitems, int acc_planes, const float2* tw, cudaStream_t s) {
    if (general)
        return launch_row_group_small_general(W, variant, mode, general, acc_planes, worlds, items, nitems, tw, s) ||
               launch_row_group_large_general(W, variant, mode, general, acc_planes, worlds, items, nitems, tw, s);
    return launch_row_group_small_simple(W, variant, mode, general, acc_planes, worlds, items, nitems, tw, s) ||
           launch_row_group_large_simple(W, variant, mode, general, acc_planes, worlds, items, nitems, tw, s);
}

int fp32_local_bytes(int row, int n, int variant) {
    if (!row) {
        const int a = col_local_bytes_small(n, variant);
        return a >= 0 ? a : col_local_bytes_large(n, variant);
    }
    // row: variant bit 1 asks for the general build
    const int a = (variant & 2) ? row_local_bytes_small_general(n, variant) : row_local_bytes_small_simple(n, variant);
    return a >= 0 ? a : ((variant & 2) ? row_local_bytes_large_general(n, variant) : row_local_bytes_large_simple(n, variant));
}

}  // namespace lenia
