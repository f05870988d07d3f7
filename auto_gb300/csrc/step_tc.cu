// Tensor-core (tcgen05) DFT-as-GEMM column pass.
#include "step_tc.cuh"

namespace lenia {

int tc_setup(TcPlan& plan, int path, std::string* err) {
    (void)plan; (void)path;
    if (err) *err = "the tensor-core paths are not built in this library yet";
    return LENIA_EINVAL;
}
int tc_prepare_size(TcPlan& plan, int path, int H, std::string* err) {
    (void)plan; (void)path; (void)H; (void)err;
    return LENIA_EINVAL;
}
bool launch_col_tc(const TcPlan&, int, int, const DevWorld*, const ColItem*, int, cudaStream_t) { return false; }
void tc_release(TcPlan& plan) { plan.ready = 0; }

}  // namespace lenia
