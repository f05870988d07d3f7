// Tensor-core (tcgen05) DFT-as-GEMM column pass: LENIA_PATH_TF32 and LENIA_PATH_BF16X3.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "engine.cuh"

namespace lenia {

// Per-context device data of the tensor-core path: DFT matrices per column length.
struct TcPlan {
    int ready = 0;
    void* mats[16] = {};
    int sizes[16] = {};
    int nsizes = 0;
};

int tc_setup(TcPlan& plan, int path, std::string* err);
int tc_prepare_size(TcPlan& plan, int path, int H, std::string* err);
bool launch_col_tc(const TcPlan& plan, int path, int H, const DevWorld* worlds, const ColItem* items, int nitems,
                   cudaStream_t s);
void tc_release(TcPlan& plan);

}  // namespace lenia
