// FP64 instantiations of the batched persistent stage kernel.
#include "batch_launch.cuh"

namespace cns {
void launch_batch_stage_fp64(int S, int V, dim3 grid, dim3 block, const BatchInst<double>* tab, const BatchCtl* ctl,
                             int cur, int kind, double a, double b, int stage0, int quirk, unsigned* bar, int* err,
                             cudaStream_t s) {
    batch_launch_dispatch<double>(S, V, grid, block, tab, ctl, cur, kind, a, b, stage0, quirk, bar, err, s);
}
cudaError_t batch_occ_fp64(int S, int V, int threads, int* nb) { return batch_occ_dispatch<double>(S, V, threads, nb); }
}  // namespace cns
