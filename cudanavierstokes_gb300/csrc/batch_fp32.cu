// FP32-RHS instantiations of the batched persistent stage kernel.
#include "batch_launch.cuh"

namespace cns {
cudaError_t batch_occ_fp64(int S, int V, int threads, int* nb);
}

namespace cns {
void launch_batch_stage_fp32(int S, int V, dim3 grid, dim3 block, const BatchInst<float>* tab, const BatchCtl* ctl,
                             int cur, int kind, double a, double b, int stage0, int quirk, unsigned* bar, int* err,
                             cudaStream_t s) {
    batch_launch_dispatch<float>(S, V, grid, block, tab, ctl, cur, kind, a, b, stage0, quirk, bar, err, s);
}
cudaError_t batch_occ_fp32(int S, int V, int threads, int* nb) { return batch_occ_dispatch<float>(S, V, threads, nb); }

int batch_stage_occupancy(int fp32, int S, int V, int threads, int* blocks_per_sm) {
    *blocks_per_sm = 0;
    cudaError_t e = fp32 ? batch_occ_fp32(S, V, threads, blocks_per_sm) : batch_occ_fp64(S, V, threads, blocks_per_sm);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(CNS_ERR_CUDA, "occupancy query of the batch stage kernel failed");
    }
    return CNS_OK;
}
}  // namespace cns
