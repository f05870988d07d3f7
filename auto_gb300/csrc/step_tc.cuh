// Tensor-core (tcgen05) DFT-as-GEMM column pass: LENIA_PATH_TF32 and LENIA_PATH_BF16X3.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "engine.cuh"

namespace lenia {

// Per-context device data of the tensor-core path: the DFT matrices per column length, and the
// control words (tc_ptx.cuh: CTL_*): an error flag a kernel sets if it gives up waiting on a
// barrier, and a test hook on the poll limit of one wait.
struct TcPlan {
    int ready = 0;
    int path = 0;
    void* mats[16] = {};
    int sizes[16] = {};
    int nsizes = 0;
    void* rmats[16] = {};  // the row pass's DFT matrices per row length
    int rsizes[16] = {};
    int nrsizes = 0;
    void* d_err = nullptr;
};

// Column lengths the tensor-core pass serves (256..4096, powers of two); others use the FP32 pass.
bool tc_supports(int H);
// Spectrum columns one tensor-core CTA transforms at a time (a multiple of TC).
int tc_columns_per_group(int H);
int tc_setup(TcPlan& plan, int path, std::string* err);
int tc_prepare_size(TcPlan& plan, int path, int H, std::string* err);
// groups: (world, channel, first tile) items, each covering tc_columns_per_group(H) columns.
// variant (BF16x3, columns of 256..1024; other shapes ignore it): 0 stages each tile group by a bulk copy into shared memory a
// group ahead; 1 reads it from global memory after an L2 prefetch, with 32 KB less shared memory a
// CTA and so more CTAs an SM.  reserve_sms: SMs the persistent grid leaves free for a launch that
// runs beside it.
constexpr int TC_COL_VARIANTS = 2;
bool launch_col_tc(const TcPlan& plan, int path, int H, int variant, const DevWorld* worlds, const ColItem* groups,
                   int ngroups, const float2* tw, cudaStream_t s, int reserve_sms = 0);
int tc_check_error(TcPlan& plan, std::string* err);
// Test hook: limit_plus_one = 0 keeps the default poll limit of the DFT-matrix wait, n > 0 makes it
// n - 1 polls (1: the wait gives up at once and the pass exits early with the error flag set).
int tc_set_wait_limit(TcPlan& plan, int limit_plus_one, std::string* err);
// The 4096-point column pass with two pipelines per SM (step_tc64.cu); fmat = the 64-point DFT matrix.
bool launch_col_tc64(bool x3, const void* fmat, const DevWorld* worlds, const ColItem* groups, int ngroups,
                     const float2* tw, int* err, cudaStream_t s, int reserve_sms = 0);
void tc_release(TcPlan& plan);

// Tensor-core row pass (step_tc_row.cu) of the one-channel, one-kernel Lenia step: inverse row DFT,
// growth / dt / clamp, forward row DFT, as GEMMs.  Row lengths served: 256, 512, 1024.
bool tc_row_supports(int W);
int tc_row_group_rows(int W);  // rows per group (a multiple of the FP32 row item's 4)
int tc_row_prepare(TcPlan& plan, int path, int W, std::string* err);
// items: the FP32 row pass's items; item_stride > 0: group g starts at items[g * item_stride]; < 0: an
// item holds -item_stride groups of tc_row_group_rows(W) rows.
bool launch_row_tc(const TcPlan& plan, int path, int W, const DevWorld* worlds, const RowItem* items, int item_stride,
                   int ngroups, const float2* tw, cudaStream_t s);
void tc_row_release(TcPlan& plan);
// One GEMM through the same operand layouts and descriptors (diagnostic).
int tc_selftest(int path, int n, int k, const float* a, const float* b, float* d, std::string* err);

}  // namespace lenia
