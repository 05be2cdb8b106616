// batch_kernel.cuh -- one persistent, cooperative launch per Runge-Kutta stage that
// advances every instance of a batch (many simulations of different grid sizes and
// physical parameters sharing the stencil orders and the precision).
//
// The launch runs the five stage phases (state recovery, ghost fill, velocity
// gradients, dilatation ghosts, RHS + update) over the work units of all instances, with
// a grid barrier between phases. Work unit = a 32 x (blockDim/32) tile of one x-y plane
// of one instance (point phases) or blockDim ghost cells (ghost phases); units of all
// instances are numbered consecutively (prefix offsets), so uneven grid sizes balance
// across the persistent blocks. The instance table, the instance count and the offsets
// live in device memory, so one captured graph serves any membership of the batch.
#pragma once
#include "../../include/cns.h"
#include "cns_common.cuh"
#include "cns_internal.h"
#include "kernels_point.cuh"
#include "kernels_rhs.cuh"

namespace cns {

template <typename R>
struct BatchInst {
    Geom g;
    Phys ph;
    CoefT<R> cf;
    double* scal;
    double* tlog;
    long long tcap;     // capacity of tlog
    double* q[2][5];
    R* der[4];      // h, t, p, mu
    R* s32[4];      // FP32 stencil copies of rho, u, v, w (FP32-RHS mode) or nullptr
    R* dil;
    R* grad[9];
    R* rb[5];
    const double *spx, *spz, *rref, *uref, *vref, *wref, *eref;   // sponge (nullptr without)
    int nbx, nby;   // units per plane: ceil(mx/32) x ceil(my/rows)
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

template <typename R, int S, int V>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1) k_batch_stage(const BatchInst<R>* __restrict__ tab,
                                                     const BatchCtl* __restrict__ ctl, int cur, int kind, double a,
                                                     double b, int stage0, int quirk, unsigned* bar, int* err) {
    const int n = ctl->n;
    if (n <= 0) return;
    const int rows = blockDim.x >> 5;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long npu = ctl->unit_off[n], ngu = ctl->ghost_off[n];
    const unsigned nb = gridDim.x;

    // phase 1: state recovery (+ time advance at stage 0)
    for (long long u = blockIdx.x; u < npu; u += gridDim.x) {
        const int q = find_inst(ctl->unit_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long lu = u - ctl->unit_off[q];
        const int bx = (int)(lu % I.nbx), by = (int)((lu / I.nbx) % I.nby), k = (int)(lu / ((long long)I.nbx * I.nby));
        const int i = bx * 32 + tx, j = by * rows + ty;
        if (stage0 && lu == 0 && threadIdx.x == 0)
            advance_time(I.scal, I.tlog, I.tcap);
        if (i < I.g.mx && j < I.g.my) {
            DerivedOut<R> o{I.der[0], I.der[1], I.der[2], I.der[3], I.s32[0], I.s32[1], I.s32[2], I.s32[3]};
            state_point<R>(I.g, I.ph, StateIn{I.q[cur][0], I.q[cur][1], I.q[cur][2], I.q[cur][3], I.q[cur][4]}, o,
                           I.scal, i, j, k);
        }
    }
    grid_barrier(bar, nb, err);
    // phase 2: ghost fill of the stencil inputs
    for (long long u = blockIdx.x; u < ngu; u += gridDim.x) {
        const int q = find_inst(ctl->ghost_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long t = (u - ctl->ghost_off[q]) * blockDim.x + threadIdx.x;
        if (t < ghost_count(I.g)) {
            StencilFields<R> f;
            if (I.s32[0]) { f.r = I.s32[0]; f.u = I.s32[1]; f.v = I.s32[2]; f.w = I.s32[3]; }
            else {
                f.r = (R*)I.q[cur][0]; f.u = (R*)I.q[cur][1]; f.v = (R*)I.q[cur][2]; f.w = (R*)I.q[cur][3];
            }
            f.h = I.der[0]; f.t = I.der[1]; f.p = I.der[2]; f.m = I.der[3];
            ghost_state_cell<R>(I.g, I.ph, f, I.scal, (int)t);
        }
    }
    grid_barrier(bar, nb, err);
    // phase 3: velocity gradients and dilatation
    for (long long u = blockIdx.x; u < npu; u += gridDim.x) {
        const int q = find_inst(ctl->unit_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long lu = u - ctl->unit_off[q];
        const int bx = (int)(lu % I.nbx), by = (int)((lu / I.nbx) % I.nby), k = (int)(lu / ((long long)I.nbx * I.nby));
        const int i = bx * 32 + tx, j = by * rows + ty;
        if (i < I.g.mx && j < I.g.my) {
            const R* uu = I.s32[0] ? I.s32[1] : (const R*)I.q[cur][1];
            const R* vv = I.s32[0] ? I.s32[2] : (const R*)I.q[cur][2];
            const R* ww = I.s32[0] ? I.s32[3] : (const R*)I.q[cur][3];
            GradOut<R> go;
            for (int c = 0; c < 9; c++) go.g[c] = I.grad[c];
            go.dil = I.dil;
            grad_point<R, V, sizeof(R) == 4>(I.g, I.cf, uu, vv, ww, go, i, j, k);
        }
    }
    grid_barrier(bar, nb, err);
    // phase 4: dilatation ghosts
    for (long long u = blockIdx.x; u < ngu; u += gridDim.x) {
        const int q = find_inst(ctl->ghost_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long t = (u - ctl->ghost_off[q]) * blockDim.x + threadIdx.x;
        if (t < ghost_count(I.g)) ghost_scalar_cell<R>(I.g, I.dil, (int)t);
    }
    grid_barrier(bar, nb, err);
    // phase 5: RHS + stage update into the other state buffer. The unit's x-y neighbourhood
    // of the nine stencil fields is staged in shared memory, (32 + 2S) x (rows + 2S) per
    // field, filled with coalesced row loads; z neighbours come from global memory. (Tile
    // cells beyond the ghost layer, possible in the last unit of a row or column, are not
    // read from memory; no thread uses them.)
    constexpr int TX = 32 + 2 * S, FSMAX = TX * (8 + 2 * S);
    __shared__ R tile[TF_COUNT * FSMAX];
    const int FS = TX * (rows + 2 * S), nt = blockDim.x;
    for (long long u = blockIdx.x; u < npu; u += gridDim.x) {
        const int q = find_inst(ctl->unit_off, n, u);
        const BatchInst<R>& I = tab[q];
        const long long lu = u - ctl->unit_off[q];
        const int bx = (int)(lu % I.nbx), by = (int)((lu / I.nbx) % I.nby), k = (int)(lu / ((long long)I.nbx * I.nby));
        const int i0 = bx * 32, j0 = by * rows;
        RhsIn<R> in;
        if (I.s32[0]) { in.r = I.s32[0]; in.u = I.s32[1]; in.v = I.s32[2]; in.w = I.s32[3]; }
        else {
            in.r = (const R*)I.q[cur][0]; in.u = (const R*)I.q[cur][1];
            in.v = (const R*)I.q[cur][2]; in.w = (const R*)I.q[cur][3];
        }
        in.h = I.der[0]; in.t = I.der[1]; in.p = I.der[2]; in.m = I.der[3]; in.dil = I.dil;
        for (int c = 0; c < 9; c++) in.g[c] = I.grad[c];
        __syncthreads();   // the previous unit is done with the tile
        {
            const long long org = I.g.at(i0 - S, j0 - S, k);
            const int xlim = I.g.mx + 2 * S - i0, ylim = I.g.my + 2 * S - j0;
            const long long P = I.g.P;
            const R* src[TF_COUNT] = {in.u, in.v, in.w, in.r, in.h, in.p, in.t, in.m, in.dil};
#pragma unroll
            for (int f = 0; f < TF_COUNT; f++) {
                for (int e = threadIdx.x; e < FS; e += nt) {
                    const int yy = e / TX, xx = e - yy * TX;
                    tile[f * FS + e] = (xx < xlim && yy < ylim) ? ld(src[f], (int)(org + (long long)yy * P + xx)) : (R)0;
                }
            }
        }
        __syncthreads();
        const int i = i0 + tx, j = j0 + ty;
        if (i < I.g.mx && j < I.g.my) {
            Update<R> up;
            up.kind = kind; up.a = a; up.b = b; up.ca = (R)a; up.cb = (R)b; up.use_prev = a != 0.0;
            up.fuse = 0;   // this kernel recovers each stage's state in its own phase
            up.qin = StateIn{I.q[cur][0], I.q[cur][1], I.q[cur][2], I.q[cur][3], I.q[cur][4]};
            const int nx = 1 - cur;
            up.qout = StateOut{I.q[nx][0], I.q[nx][1], I.q[nx][2], I.q[nx][3], I.q[nx][4]};
            for (int c = 0; c < 5; c++) { up.rb[c] = I.rb[c]; up.k2[c] = nullptr; up.q0[c] = nullptr; }
            up.spx = I.spx; up.spz = I.spz; up.rref = I.rref; up.uref = I.uref; up.vref = I.vref;
            up.wref = I.wref; up.eref = I.eref;
            const R* ctr = tile + (ty + S) * TX + (tx + S);
            const NbTile<R> nbx{ctr, 1, FS}, nby{ctr, TX, FS};
            const int c = (int)I.g.at(i, j, k);
            const NbGlobal<R> nbz{&in, c, (int)I.g.PS};
            rhs_point_nb<R, S, V>(I.g, I.cf, in, up, I.scal, quirk, i, k, c, nbx, nby, nbz, ctr[TF_DIL * FS],
                                  ctr[TF_M * FS], ctr[TF_U * FS], ctr[TF_V * FS], ctr[TF_W * FS], ctr[TF_R * FS],
                                  ctr[TF_H * FS]);
        }
    }
}

}  // namespace cns
