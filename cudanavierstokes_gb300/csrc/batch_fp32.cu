// FP32-RHS instantiations of the batched persistent stage kernel.
#include "batch_launch.cuh"

namespace cns {
cudaError_t batch_occ_fp64(int S, int V, int* nb);
}

namespace cns {
void launch_batch_stage_fp32(int S, int V, dim3 grid, const BatchInst<float>* tab, const BatchCtl* ctl, int cur,
                             int stage, int quirk, unsigned* bar, int* err, unsigned long long* cnt, const MemberTable<float>& rt,
                             cudaStream_t s) {
    batch_launch_dispatch<float>(S, V, grid, tab, ctl, cur, stage, quirk, bar, err, cnt, rt, s);
}
void launch_batch_time_fp32(const BatchInst<float>* tab, const BatchCtl* ctl, cudaStream_t s) {
    batch_time_launch<float>(tab, ctl, s);
}
cudaError_t batch_occ_fp32(int S, int V, int* nb) { return batch_occ_dispatch<float>(S, V, nb); }

int batch_stage_occupancy(int fp32, int S, int V, int* blocks_per_sm) {
    *blocks_per_sm = 0;
    cudaError_t e = fp32 ? batch_occ_fp32(S, V, blocks_per_sm) : batch_occ_fp64(S, V, blocks_per_sm);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(CNS_ERR_CUDA, "occupancy query of the batch stage kernel failed");
    }
    return CNS_OK;
}
}  // namespace cns
