// FP64 instantiations of the batched persistent stage kernel.
#include "batch_launch.cuh"

namespace cns {
void launch_batch_stage_fp64(int S, int V, dim3 grid, const BatchInst<double>* tab, const BatchCtl* ctl, int cur,
                             int stage, int quirk, unsigned* bar, int* err, unsigned long long* cnt, const MemberTable<double>& rt,
                             cudaStream_t s) {
    batch_launch_dispatch<double>(S, V, grid, tab, ctl, cur, stage, quirk, bar, err, cnt, rt, s);
}
void launch_batch_time_fp64(const BatchInst<double>* tab, const BatchCtl* ctl, cudaStream_t s) {
    batch_time_launch<double>(tab, ctl, s);
}
cudaError_t batch_occ_fp64(int S, int V, int* nb) { return batch_occ_dispatch<double>(S, V, nb); }
}  // namespace cns
