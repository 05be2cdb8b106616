// batch_launch.cuh -- cooperative launch and occupancy query of the batched stage kernel.
#pragma once
#include "batch_kernel.cuh"

namespace cns {

template <typename R, int S, int V>
cudaError_t batch_launch_t(dim3 grid, const BatchInst<R>* tab, const BatchCtl* ctl, int cur, int stage, int quirk,
                           unsigned* bar, int* err, unsigned long long* cnt, const MemberTable<R>& rt, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(BATCH_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (sizeof(R) == 4 && rt.n > 0)
        return cudaLaunchKernelEx(&cfg, k_batch_stage<R, S, V, true>, tab, ctl, cur, stage, quirk, bar, err, cnt, rt);
    return cudaLaunchKernelEx(&cfg, k_batch_stage<R, S, V, false>, tab, ctl, cur, stage, quirk, bar, err, cnt, rt);
}

template <typename R>
cudaError_t batch_launch_dispatch(int S, int V, dim3 grid, const BatchInst<R>* tab, const BatchCtl* ctl, int cur,
                                  int stage, int quirk, unsigned* bar, int* err, unsigned long long* cnt, const MemberTable<R>& rt, cudaStream_t s) {
#define CNS_BL(SS, VV) \
    if (S == SS && V == VV) return batch_launch_t<R, SS, VV>(grid, tab, ctl, cur, stage, quirk, bar, err, cnt, rt, s);
    CNS_BL(1, 1) CNS_BL(2, 1) CNS_BL(2, 2) CNS_BL(3, 1) CNS_BL(3, 2) CNS_BL(3, 3)
    CNS_BL(4, 1) CNS_BL(4, 2) CNS_BL(4, 3) CNS_BL(4, 4)
#undef CNS_BL
    return cudaErrorInvalidValue;
}

template <typename R>
cudaError_t batch_time_launch(const BatchInst<R>* tab, const BatchCtl* ctl, cudaStream_t s) {
    k_batch_time<R><<<(CNS_BATCH_MAX + 127) / 128, 128, 0, s>>>(tab, ctl);
    return cudaGetLastError();
}

// resident blocks per SM: the smaller of the two RHS-phase variants
template <typename R, int S, int V>
cudaError_t batch_occ_t(int* nb) {
    int a = 0, b = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_batch_stage<R, S, V, false>, BATCH_THREADS, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_stage<R, S, V, true>, BATCH_THREADS, 0);
    *nb = a < b ? a : b;
    return e;
}

template <typename R>
cudaError_t batch_occ_dispatch(int S, int V, int* nb) {
#define CNS_BO(SS, VV)   \
    if (S == SS && V == VV) \
        return batch_occ_t<R, SS, VV>(nb);
    CNS_BO(1, 1) CNS_BO(2, 1) CNS_BO(2, 2) CNS_BO(3, 1) CNS_BO(3, 2) CNS_BO(3, 3)
    CNS_BO(4, 1) CNS_BO(4, 2) CNS_BO(4, 3) CNS_BO(4, 4)
#undef CNS_BO
    return cudaErrorInvalidValue;
}

}  // namespace cns
