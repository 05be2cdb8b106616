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

// FP32-RHS members' parameters as a kernel argument (constant bank): what the four phases'
// point bodies read of the member's geometry, inverse spacings, boundary constants, packed
// stencil inputs, Wray stage update and state recovery, for up to MEMBER_TABLE_MAX members. Read
// through shared memory instead, these parameters took registers and issue slots in
// every point (a one-member batch ran at 2,295 against 3,333 Mpoint-steps/s with them in
// the constant bank); larger batches take that path (n = 0 in the table).
constexpr int MEMBER_TABLE_MAX = 64;
constexpr int COL_NZ = 8;   // planes of a theta column unit (the table path's phase 2)

struct Member32 {
    long long base;
    int P, PS, mx, my, nbx, nby, nonuniform_x, use_prev, fuse, vexp_is_one;
    float inv[3], inv2[3], lam_mu, ca, cb, f_vexp, f_invRe;
    double cvInv, Rgas;
    const float* xp;
    const float* cvsx;
    const float4* qa;
    const float4* qb;
    const float* dil;
    long long fstride;    // elements between the fields of a state buffer / the RK register
    const double* qin;    // rho of the stage's input state; u, v, w, rhoE follow at fstride
    double* qout;         // the same of the output state
    float* rb;            // the RK register's first field
    const double *spx, *spz, *rref, *uref, *vref, *wref, *eref;
    float4* nqa;
    float4* nqb;
    double* scal;
    // the ghost and theta phases: ghost geometry, boundary constants, theta weights
    int G, mz, xbc, zbl, perturbed, pert_kc, pert_lp;
    double twall_top, twall_bot, hcoef, invRe, vexp, dy;
    double pert_amp1, pert_amp2, pert_omega1, pert_omega2, pert_lambda;
    float c1V[3][5];
};

template <typename R>
struct MemberTable {     // FP64 batches keep the device-table / shared-memory path
    int n;
};
template <>
struct MemberTable<float> {
    int n;                                     // members in the table; 0: use the shared-memory path
    long long unit_off[MEMBER_TABLE_MAX + 1];     // point-unit prefix offsets (as BatchCtl's)
    long long ghost_off[MEMBER_TABLE_MAX + 1];    // ghost-unit prefix offsets
    long long col_off[MEMBER_TABLE_MAX + 1];      // theta-column prefix offsets (32 x 4 x COL_NZ columns)
    Member32 m[MEMBER_TABLE_MAX];
};
// kernel arguments are limited to 32,764 bytes; the stage kernel's others take < 100
static_assert(sizeof(MemberTable<float>) <= 32600, "the member table must fit the kernel-argument space");

// a member's geometry and boundary constants for the ghost and theta phases
__device__ __forceinline__ Geom member_geom(const Member32& M) {
    Geom g{};
    g.mx = M.mx; g.my = M.my; g.mz = M.mz; g.G = M.G; g.P = M.P; g.PS = M.PS; g.base = M.base;
    g.xbc = M.xbc; g.zbl = M.zbl; g.nonuniform_x = M.nonuniform_x; g.dy = M.dy;
    return g;
}
__device__ __forceinline__ Phys member_phys(const Member32& M) {
    Phys ph{};
    ph.Rgas = M.Rgas; ph.invRe = M.invRe; ph.hcoef = M.hcoef; ph.vexp = M.vexp; ph.vexp_is_one = M.vexp_is_one;
    ph.twall_top = M.twall_top; ph.twall_bot = M.twall_bot; ph.perturbed = M.perturbed;
    ph.pert_kc = M.pert_kc; ph.pert_lp = M.pert_lp; ph.pert_amp1 = M.pert_amp1; ph.pert_amp2 = M.pert_amp2;
    ph.pert_omega1 = M.pert_omega1; ph.pert_omega2 = M.pert_omega2; ph.pert_lambda = M.pert_lambda;
    return ph;
}

// the RHS phase's point of member M: the standalone body (compile-time weights) on
// geometry, coefficients, inputs and stage update assembled from the table entry
template <int S, int V>
__device__ __forceinline__ void rhs_point_member(const Member32& M, int quirk, int i, int j, int k) {
    Geom g{};
    g.mx = M.mx; g.my = M.my; g.P = M.P; g.PS = M.PS; g.base = M.base; g.nonuniform_x = M.nonuniform_x;
    CoefT<float> cf{};
    for (int d = 0; d < 3; d++) { cf.inv[d] = M.inv[d]; cf.inv2[d] = M.inv2[d]; }
    cf.lam_mu = M.lam_mu; cf.xp = M.xp; cf.cvsx = M.cvsx;
    RhsIn<float> in{};
    in.qa = M.qa; in.qb = M.qb; in.dil = M.dil;
    Update<float> up{};
    up.kind = ST_LS; up.ca = M.ca; up.cb = M.cb; up.use_prev = M.use_prev;
    const long long fs = M.fstride;
    up.qin = StateIn{M.qin, M.qin + fs, M.qin + 2 * fs, M.qin + 3 * fs, M.qin + 4 * fs};
    up.qout = StateOut{M.qout, M.qout + fs, M.qout + 2 * fs, M.qout + 3 * fs, M.qout + 4 * fs};
    for (int q = 0; q < 5; q++) up.rb[q] = M.rb + q * fs;
    up.spx = M.spx; up.spz = M.spz; up.rref = M.rref; up.uref = M.uref; up.vref = M.vref; up.wref = M.wref;
    up.eref = M.eref;
    up.fuse = M.fuse; up.dnext.qa = M.nqa; up.dnext.qb = M.nqb;
    up.ph.cvInv = M.cvInv; up.ph.Rgas = M.Rgas; up.ph.vexp_is_one = M.vexp_is_one; up.ph.f_vexp = M.f_vexp;
    up.ph.f_invRe = M.f_invRe;
    rhs_point<float, S, V, true>(g, cf, in, up, M.scal, quirk, i, j, k);
}

// Dynamic in-order scheduling of a phase's units: blocks take the next unit from a device
// counter (one atomic per unit, issued while the block works on its current unit), so the
// units in flight stay a compact window in unit order, as the hardware dispatches the
// blocks of the standalone kernels, and faster blocks take more units. A block's units
// increase, so its instance is found by a forward scan from the previous one.
struct UnitQueue {
    long long u;
    int q, slot;
    __device__ __forceinline__ UnitQueue(unsigned long long* c, long long* s_next) : u(0), q(0), slot(0) {
        if (threadIdx.x == 0) s_next[0] = (long long)atomicAdd(c, 1ULL);
        __syncthreads();
        u = s_next[0];
    }
    // the instance of unit u (forward scan; units of one block only increase)
    __device__ __forceinline__ void locate(const long long* off) {
        while (u >= off[q + 1]) q++;
    }
};

// FP32: 7 blocks of 128 per SM (72 registers); the RHS phase uses the packed body with
// compile-time stencil weights, so a member's coefficients are six inverse spacings
// instead of tables; theta is computed by columns marching in z. FP64: 4 blocks.
//
// cnt[0..3]: the four phases' unit counters, zero at launch; each is reset by block 0 once
// no block can take from it any more (after the barrier that ends its phase; the RHS
// phase's counter at the start of the next launch, before its first barrier).
// TBL: every phase walks the members in an outer loop and reads their parameters from the
// kernel-argument table (FP32, up to MEMBER_TABLE_MAX members); otherwise the phases look
// members up per unit in the device table and the RHS phase stages them in shared memory.
// Two instantiations, so that neither path's registers constrain the other.
template <typename R, int S, int V, bool TBL>
__global__ void __launch_bounds__(BATCH_THREADS, sizeof(R) == 4 ? 7 : 4)
    k_batch_stage(const BatchInst<R>* __restrict__ tab, const BatchCtl* __restrict__ ctl, int cur, int stage,
                  int quirk, unsigned* bar, int* err, unsigned long long* cnt,
                  const __grid_constant__ MemberTable<R> rt) {
    const int n = ctl->n;
    if (n <= 0) return;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long npu = ctl->unit_off[n], ngu = ctl->ghost_off[n];
    const unsigned nb = gridDim.x;
    __shared__ long long s_next[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[3] = 0ULL;   // the previous launch's RHS counter

    // one pass over the units of a phase: body(u, q) for every unit taken by this block
    const auto sweep = [&](unsigned long long* c, const long long* off, long long total, auto&& body) {
        UnitQueue w(c, s_next);
        while (w.u < total) {
            long long mine = 0;
            if (threadIdx.x == 0) mine = (long long)atomicAdd(c, 1ULL);   // the next unit, in flight
            w.locate(off);
            body(w.u, w.q);
            w.slot ^= 1;
            if (threadIdx.x == 0) s_next[w.slot] = mine;
            __syncthreads();
            w.u = s_next[w.slot];
        }
    };

    if constexpr (sizeof(R) == 4 && TBL) {
        // members in outer loops: q is a loop counter, the same in every thread, and a
        // member's parameters come from the kernel-argument table
        const auto sweep_m = [&](unsigned long long* c, const long long* off, auto&& body) {
            UnitQueue w(c, s_next);
            for (int q = 0; q < rt.n; q++) {
                const Member32& M = rt.m[q];
                while (w.u < off[q + 1]) {
                    long long mine = 0;
                    if (threadIdx.x == 0) mine = (long long)atomicAdd(c, 1ULL);   // the next unit, in flight
                    body(M, w.u - off[q]);
                    w.slot ^= 1;
                    if (threadIdx.x == 0) s_next[w.slot] = mine;
                    __syncthreads();
                    w.u = s_next[w.slot];
                }
            }
        };
        const auto unit_ijk = [&](const Member32& M, long long lu, int& i, int& j, int& k) {
            const long long pl = (long long)M.nbx * M.nby;
            k = (int)(lu / pl);
            const int rr = (int)(lu - (long long)k * pl);
            const int by = rr / M.nbx, bx = rr - by * M.nbx;
            i = bx * 32 + tx;
            j = by * 4 + ty;
        };
        // phase 1: ghost cells of the stencil inputs of the current state
        sweep_m(cnt + 0, rt.ghost_off, [&](const Member32& M, long long lu) {
            const Geom g = member_geom(M);
            const long long t = lu * BATCH_THREADS + threadIdx.x;
            if (t < ghost_count(g))
                ghost_state_cell_packed(g, member_phys(M), (float4*)M.qa, (float4*)M.qb, M.scal, (int)t);
        });
        grid_barrier(bar, nb, err);
        if (blockIdx.x == 0 && threadIdx.x == 0) cnt[0] = 0ULL;
        // phase 2: dilatation from the packed records, by columns of 32 x 4 points marching
        // COL_NZ planes (the standalone z-marching body, halos in shared memory)
        {
            __shared__ float su[4][32 + 2 * V], sv[4 + 2 * V][32];
            sweep_m(cnt + 1, rt.col_off, [&](const Member32& M, long long lu) {
                const int nbz = (M.mz + COL_NZ - 1) / COL_NZ;
                const int bz = (int)(lu % nbz);
                const int r2 = (int)(lu / nbz);
                const int by = r2 / M.nbx, bx = r2 - by * M.nbx;
                CoefT<float> cf{};
                for (int d = 0; d < 3; d++)
                    for (int l = 0; l < 5; l++) cf.c1V[d][l] = M.c1V[d][l];
                cf.xp = M.xp;
                const int k0 = bz * COL_NZ;
                dil_column_packed<V, 4>(member_geom(M), cf, M.qa, (float*)M.dil, bx * 32, by * 4, k0,
                                        min(k0 + COL_NZ, M.mz), false, tx, ty, su, sv);
            });
        }
        grid_barrier(bar, nb, err);
        if (blockIdx.x == 0 && threadIdx.x == 0) cnt[1] = 0ULL;
        // phase 3: dilatation ghosts
        sweep_m(cnt + 2, rt.ghost_off, [&](const Member32& M, long long lu) {
            const Geom g = member_geom(M);
            const long long t = lu * BATCH_THREADS + threadIdx.x;
            if (t < ghost_count(g)) ghost_scalar_cell<float>(g, (float*)M.dil, (int)t);
        });
        grid_barrier(bar, nb, err);
        if (blockIdx.x == 0 && threadIdx.x == 0) cnt[2] = 0ULL;
        // phase 4: RHS + stage update + the new state's recovery (the standalone point body,
        // compile-time weights)
        sweep_m(cnt + 3, rt.unit_off, [&](const Member32& M, long long lu) {
            int i, j, k;
            unit_ijk(M, lu, i, j, k);
            if (i < M.mx && j < M.my) rhs_point_member<S, V>(M, quirk, i, j, k);
        });
    } else {
    // phase 1: ghost cells of the stencil inputs of the current state
    sweep(cnt + 0, ctl->ghost_off, ngu, [&](long long u, int q) {
        const BatchInst<R>& I = tab[q];
        const long long t = (u - ctl->ghost_off[q]) * BATCH_THREADS + threadIdx.x;
        if (t < ghost_count(I.g)) {
            const RhsIn<R>& in = I.in[cur];
            const StencilFields<R> f{(R*)in.r, (R*)in.u, (R*)in.v, (R*)in.w, (R*)in.t, (R*)in.p, (R*)in.h,
                                     (R*)in.m, (float4*)in.qa, (float4*)in.qb};
            ghost_state_cell<R>(I.g, I.ph, f, I.scal, (int)t);
        }
    });
    grid_barrier(bar, nb, err);
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[0] = 0ULL;
    // phase 2: dilatation from the packed records (FP32-RHS: the RHS forms the nine gradients
    // itself) or the nine velocity gradients and the dilatation
    sweep(cnt + 1, ctl->unit_off, npu, [&](long long u, int q) {
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
    });
    grid_barrier(bar, nb, err);
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[1] = 0ULL;
    // phase 3: dilatation ghosts
    sweep(cnt + 2, ctl->ghost_off, ngu, [&](long long u, int q) {
        const BatchInst<R>& I = tab[q];
        const long long t = (u - ctl->ghost_off[q]) * BATCH_THREADS + threadIdx.x;
        if (t < ghost_count(I.g)) ghost_scalar_cell<R>(I.g, (R*)I.in[cur].dil, (int)t);
    });
    grid_barrier(bar, nb, err);
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[2] = 0ULL;
    // phase 4: RHS + stage update into the other state buffer + that state's recovery, every
    // neighbour from global memory (the standalone RHS kernel's point body, compile-time
    // weights); the member's parameters are staged in shared memory when it changes
    __shared__ StageParams<R> sp;
    int qs = -1;
    sweep(cnt + 3, ctl->unit_off, npu, [&](long long u, int q) {
        if (q != qs) {
            __syncthreads();   // the previous unit is done with sp
            stage_params_copy<R>(sp, tab[q], cur, stage);
            __syncthreads();
            qs = q;
        }
        const long long lu = u - ctl->unit_off[q];
        const long long pl = (long long)sp.nbx * sp.nby;
        const int k = (int)(lu / pl);
        const int rr = (int)(lu - (long long)k * pl);
        const int by = rr / sp.nbx, bx = rr - by * sp.nbx;
        const int i = bx * 32 + tx, j = by * 4 + ty;
        if (i < sp.g.mx && j < sp.g.my) rhs_point<R, S, V, true>(sp.g, sp.cf, sp.in, sp.up, sp.scal, quirk, i, j, k);
    });
    }
}

}  // namespace cns
