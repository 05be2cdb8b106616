// batch_kernel.cuh -- one persistent, cooperative launch per Runge-Kutta stage that
// advances every instance of a batch (many simulations of different grid sizes and
// physical parameters sharing the stencil orders and the precision).
//
// The launch runs the four stage phases (ghost fill of the stencil inputs, velocity
// gradients / dilatation, dilatation ghosts, RHS + update + the new state's recovery) over
// the work units of all instances, with a grid barrier between phases. Work unit = a
// 32 x 4 tile of one x-y plane of one instance (point phases, the standalone RHS kernel's
// block) or 128 ghost cells (ghost phases); units of all instances are numbered
// consecutively (prefix offsets), so uneven grid sizes balance across the persistent
// blocks. The instance table (with each instance's stage updates prepared on the host),
// the instance count and the offsets live in device memory, so one captured graph serves
// any membership of the batch.
#pragma once
#include "../../include/cns.h"
#include "cns_common.cuh"
#include "cns_internal.h"
#include "kernels_point.cuh"
#include "kernels_rhs.cuh"

namespace cns {

constexpr int BATCH_THREADS = 128;   // 32 x 4 points or 128 ghost cells per work unit

template <typename R>
struct BatchInst {
    Geom g;
    Phys ph;
    CoefT<R> cf;
    double* scal;
    double* tlog;
    long long tcap;          // capacity of tlog
    RhsIn<R> in[2];          // stencil inputs (+ theta, gradients) of state buffer b
    Update<R> up[3][2];      // Wray stage s from state buffer b into 1 - b, with the new
                             // state's recovery (its derived fields of buffer 1 - b)
    int nbx, nby;            // units per plane: ceil(mx/32) x ceil(my/4)
};

struct BatchCtl {
    int n;                  // active instances
    int pad;
    long long unit_off[CNS_BATCH_MAX + 1];    // point-unit prefix offsets
    long long ghost_off[CNS_BATCH_MAX + 1];   // ghost-unit prefix offsets
};

// Grid barrier for a cooperative launch (all blocks co-resident). Spins a bounded number
// of times; on timeout it records an error and lets the block continue, so the kernel
// always terminates and the host reports CNS_ERR_TIMEOUT.
__device__ __forceinline__ void grid_barrier(unsigned* bar, unsigned nblocks, int* err,
                                             long long spin_limit = (1LL << 24)) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        if (atomicAdd(bar, 1u) == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*vgen == gen) {
                if (++spins > spin_limit) {
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

__device__ __forceinline__ int find_inst(const long long* off, int n, long long u) {
    int lo = 0, hi = n;   // off[lo] <= u < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= u) lo = mid; else hi = mid;
    }
    return lo;
}

// One instance's parameters of the RHS phase for one stage and parity
template <typename R>
struct StageParams {
    Geom g;
    CoefT<R> cf;
    RhsIn<R> in;
    Update<R> up;
    double* scal;
    int nbx, nby;
};

// block-cooperative copy of an instance's stage parameters into shared memory (whole words)
template <typename R>
__device__ __forceinline__ void stage_params_copy(StageParams<R>& sp, const BatchInst<R>& I, int cur, int stage) {
    const auto copy = [&](void* dst, const void* src, int bytes) {
        for (int w = threadIdx.x; w < bytes / 4; w += blockDim.x)
            static_cast<unsigned*>(dst)[w] = static_cast<const unsigned*>(src)[w];
    };
    static_assert(sizeof(Geom) % 4 == 0 && sizeof(CoefT<R>) % 4 == 0 && sizeof(RhsIn<R>) % 4 == 0 &&
                      sizeof(Update<R>) % 4 == 0,
                  "word copies");
    copy(&sp.g, &I.g, sizeof(Geom));
    copy(&sp.cf, &I.cf, sizeof(CoefT<R>));
    copy(&sp.in, &I.in[cur], sizeof(RhsIn<R>));
    copy(&sp.up, &I.up[stage][cur], sizeof(Update<R>));
    if (threadIdx.x == 0) {
        sp.scal = I.scal;
        sp.nbx = I.nbx;
        sp.nby = I.nby;
    }
}

// Stage 0 of a step: every instance's time advances by its dt (before the ghost fill,
// which reads the time in the boundary-layer wall perturbation)
template <typename R>
__global__ void k_batch_time(const BatchInst<R>* __restrict__ tab, const BatchCtl* __restrict__ ctl) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < ctl->n) advance_time(tab[q].scal, tab[q].tlog, tab[q].tcap);
}

// the (i, j, k) point of thread (tx, ty) in point unit lu of an instance
template <typename R>
__device__ __forceinline__ void unit_point(const BatchInst<R>& I, long long lu, int tx, int ty, int& i, int& j,
                                           int& k) {
    const long long pl = (long long)I.nbx * I.nby;
    k = (int)(lu / pl);
    const int r = (int)(lu - (long long)k * pl);
    const int by = r / I.nbx, bx = r - by * I.nbx;
    i = bx * 32 + tx;
    j = by * 4 + ty;
}

// FP32: 5 blocks of 128 per SM (96 registers): the instance parameters come from the table in
// global memory, not the constant bank, and at 7 blocks (72 registers) they spill 700 bytes a
// thread (measured 1,095 vs 1,498 Mpoint-steps/s on the 48-member ensemble). FP64: 4 blocks.
template <typename R, int S, int V>
__global__ void __launch_bounds__(BATCH_THREADS, sizeof(R) == 4 ? 5 : 4)
    k_batch_stage(const BatchInst<R>* __restrict__ tab, const BatchCtl* __restrict__ ctl, int cur, int stage,
                  int quirk, unsigned* bar, int* err) {
    const int n = ctl->n;
    if (n <= 0) return;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long npu = ctl->unit_off[n], ngu = ctl->ghost_off[n];
    const unsigned nb = gridDim.x;

    // phase 1: ghost cells of the stencil inputs of the current state
    for (long long u = blockIdx.x; u < ngu; u += gridDim.x) {
        const int q = find_inst(ctl->ghost_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long t = (u - ctl->ghost_off[q]) * BATCH_THREADS + threadIdx.x;
        if (t < ghost_count(I.g)) {
            const RhsIn<R>& in = I.in[cur];
            const StencilFields<R> f{(R*)in.r, (R*)in.u, (R*)in.v, (R*)in.w, (R*)in.t, (R*)in.p, (R*)in.h,
                                     (R*)in.m, (float4*)in.qa, (float4*)in.qb};
            ghost_state_cell<R>(I.g, I.ph, f, I.scal, (int)t);
        }
    }
    grid_barrier(bar, nb, err);
    // phase 2: dilatation from the packed records (FP32-RHS: the RHS forms the nine gradients
    // itself) or the nine velocity gradients and the dilatation
    for (long long u = blockIdx.x; u < npu; u += gridDim.x) {
        const int q = find_inst(ctl->unit_off, n, u);
        const BatchInst<R>& I = tab[q];
        int i, j, k;
        unit_point(I, u - ctl->unit_off[q], tx, ty, i, j, k);
        if (i < I.g.mx && j < I.g.my) {
            const RhsIn<R>& in = I.in[cur];
            if constexpr (sizeof(R) == 4) {
                dil_point_packed<V>(I.g, I.cf, in.qa, (float*)in.dil, i, j, k);
            } else {
                GradOut<R> go;
                for (int c = 0; c < 9; c++) go.g[c] = (R*)in.g[c];
                go.dil = (R*)in.dil;
                grad_point<R, V>(I.g, I.cf, in.u, in.v, in.w, go, i, j, k);
            }
        }
    }
    grid_barrier(bar, nb, err);
    // phase 3: dilatation ghosts
    for (long long u = blockIdx.x; u < ngu; u += gridDim.x) {
        const int q = find_inst(ctl->ghost_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long t = (u - ctl->ghost_off[q]) * BATCH_THREADS + threadIdx.x;
        if (t < ghost_count(I.g)) ghost_scalar_cell<R>(I.g, (R*)I.in[cur].dil, (int)t);
    }
    grid_barrier(bar, nb, err);
    // phase 4: RHS + stage update into the other state buffer + that state's recovery, every
    // neighbour from global memory (the standalone RHS kernel's point body). The unit's
    // instance parameters (geometry, coefficients, inputs, stage update) are staged in
    // shared memory when the instance changes: the point body reads them there instead of
    // through the table in global memory.
    __shared__ StageParams<R> sp;
    int qs = -1;
    for (long long u = blockIdx.x; u < npu; u += gridDim.x) {
        const int q = find_inst(ctl->unit_off, n, u);
        if (q != qs) {
            __syncthreads();   // the previous unit is done with sp
            stage_params_copy<R>(sp, tab[q], cur, stage);
            __syncthreads();
            qs = q;
        }
        int i, j, k;
        const long long lu = u - ctl->unit_off[q];
        {
            const long long pl = (long long)sp.nbx * sp.nby;
            k = (int)(lu / pl);
            const int r = (int)(lu - (long long)k * pl);
            const int by = r / sp.nbx, bx = r - by * sp.nbx;
            i = bx * 32 + tx;
            j = by * 4 + ty;
        }
        if (i < sp.g.mx && j < sp.g.my) rhs_point<R, S, V>(sp.g, sp.cf, sp.in, sp.up, sp.scal, quirk, i, j, k);
    }
}

}  // namespace cns
