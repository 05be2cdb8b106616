// kernels_common.cu -- state recovery, ghost fills, velocity gradients, reductions and
// layout conversion. The RHS/stage kernel lives in kernels_rhs.cuh.
#include "cns_common.cuh"
#include "cns_internal.h"

namespace cns {

// ---------------------------------------------------------------------------------
// State recovery (calcState, src/cuda_main.cu:218-242): T, p, H, mu, lambda from
// rho, u, v, w, rhoE. FP64 arithmetic; results stored as R. In FP32-RHS mode the
// stencil copies of rho, u, v, w are also written as FP32.
// Stage 0 of a step also advances the simulation time by dt (deviceAdvanceTime).
// ---------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128) k_state(Geom g, Phys ph, StateIn q, DerivedOut<R> o, double* scal,
                                               int advance_time, double* time_log) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (advance_time && i == 0 && j == 0 && k == 0) {
        double tn = scal[SC_TIME] + scal[SC_DT];
        scal[SC_TIME] = tn;
        if (time_log) *time_log = tn;
    }
    if (i >= g.mx || j >= g.my) return;
    const long long c = g.at(i, j, k);
    const double rr = q.r[c], uu = q.u[c], vv = q.v[c], ww = q.w[c], ee = q.e[c];
    const double inv = rcp_nr(rr);
    const double en = ee * inv - 0.5 * (uu * uu + vv * vv + ww * ww);
    const double T = ph.cvInv * en;
    const double pr = rr * ph.Rgas * T;
    const double hh = (ee + pr) * inv;
    o.t[c] = (R)T;
    o.p[c] = (R)pr;
    o.h[c] = (R)hh;
    if constexpr (sizeof(R) == 4) {
        // FP32-RHS mode: transport properties are RHS inputs, evaluated in FP32 from the
        // FP64 temperature
        const float Tf = (float)T;
        const float suth = ph.vexp_is_one ? Tf : powf(Tf, (float)ph.vexp);
        o.m[c] = suth * (float)ph.invRe;
        o.l[c] = suth * (float)ph.clam;
    } else {
        const double suth = ph.vexp_is_one ? T : pow(T, ph.vexp);
        o.m[c] = (R)(suth * ph.invRe);
        o.l[c] = (R)(suth * ph.clam);
    }
    if (o.r32) {
        o.r32[c] = (R)rr; o.u32[c] = (R)uu; o.v32[c] = (R)vv; o.w32[c] = (R)ww;
    }
    if (!(T > 0.0) || !(rr > 0.0)) scal[SC_NONFINITE] = 1.0;   // racy flag write, any writer is fine
}

// ---------------------------------------------------------------------------------
// Ghost fill for the stencil inputs rho, u, v, w, T, p, H, mu, lambda.
//   x: periodic | isothermal wall (BCxNumber1/3: p even, u v w odd, T = 2Tw - T,
//      mu, lambda, rho, H from the ghost p, T, u, v, w) | boundary layer (bottom: p, T
//      even, u v w odd, u perturbed; top: linear extrapolation; mu, lambda, rho, H derived)
//   y: periodic.   z: periodic | linear extrapolation about the end nodes.
// (src/boundary.h:38-188, src/boundary_condition_x.h:47-115, _y.h:19-58, _z.h:80-332)
// One thread per ghost cell of the six faces (no edges or corners are ever read).
// ---------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_ghost_state(Geom g, Phys ph, StencilFields<R> f, const double* scal) {
    const long long G = g.G;
    const long long nx = 2 * G * g.my * g.mz, ny = 2 * G * g.mx * g.mz, nz = 2 * G * g.mx * g.my;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    R* F[9] = {f.r, f.u, f.v, f.w, f.t, f.p, f.h, f.m, f.l};
    if (t < nx) {
        const int m = (int)(t % G) + 1; t /= G;
        const int side = (int)(t % 2); t /= 2;
        const int j = (int)(t % g.my);
        const int k = (int)(t / g.my);
        const int ig = side == 0 ? -m : g.mx - 1 + m;
        const long long cg = g.at(ig, j, k);
        if (g.xbc == XBC_PER) {
            const long long cs = g.at(side == 0 ? g.mx - m : m - 1, j, k);
#pragma unroll
            for (int q = 0; q < 9; q++) F[q][cg] = F[q][cs];
            return;
        }
        const int ip = side == 0 ? m - 1 : g.mx - m;
        const long long cp = g.at(ip, j, k);
        R ug, vg, wg, pg, Tg;
        if (g.xbc == XBC_WALL) {
            const double Tw = side == 0 ? ph.twall_bot : ph.twall_top;
            ug = -f.u[cp]; vg = -f.v[cp]; wg = -f.w[cp];
            pg = f.p[cp];
            Tg = (R)(2.0 * Tw) - f.t[cp];
        } else if (side == 0) {   // boundary layer, wall
            ug = -f.u[cp]; vg = -f.v[cp]; wg = -f.w[cp];
            pg = f.p[cp];
            Tg = f.t[cp];
            double pv;
            if (ph.perturbed && wall_perturbation(ph, g.dy, j, k, scal[SC_TIME], &pv)) ug = (R)pv;
        } else {                  // boundary layer, free stream: extrapolate through the last node
            const long long cl = g.at(g.mx - 1, j, k);
            const long long cm = g.at(g.mx - 1 - m, j, k);
            ug = (R)2.0 * f.u[cl] - f.u[cm];
            vg = (R)2.0 * f.v[cl] - f.v[cm];
            wg = (R)2.0 * f.w[cl] - f.w[cm];
            pg = (R)2.0 * f.p[cl] - f.p[cm];
            Tg = (R)2.0 * f.t[cl] - f.t[cm];
        }
        const R suth = ph.vexp_is_one ? Tg : cns_pow<R>(Tg, (R)ph.vexp);
        f.u[cg] = ug; f.v[cg] = vg; f.w[cg] = wg; f.p[cg] = pg; f.t[cg] = Tg;
        f.m[cg] = suth * (R)ph.invRe;
        f.l[cg] = suth * (R)ph.clam;
        f.h[cg] = Tg * (R)ph.hcoef + (R)0.5 * (ug * ug + vg * vg + wg * wg);
        f.r[cg] = pg / ((R)ph.Rgas * Tg);
        return;
    }
    t -= nx;
    if (t < ny) {
        const int m = (int)(t % G) + 1; t /= G;
        const int side = (int)(t % 2); t /= 2;
        const int i = (int)(t % g.mx);
        const int k = (int)(t / g.mx);
        const long long cg = g.at(i, side == 0 ? -m : g.my - 1 + m, k);
        const long long cs = g.at(i, side == 0 ? g.my - m : m - 1, k);
#pragma unroll
        for (int q = 0; q < 9; q++) F[q][cg] = F[q][cs];
        return;
    }
    t -= ny;
    if (t < nz) {
        const int m = (int)(t % G) + 1; t /= G;
        const int side = (int)(t % 2); t /= 2;
        const int i = (int)(t % g.mx);
        const int j = (int)(t / g.mx);
        const long long cg = g.at(i, j, side == 0 ? -m : g.mz - 1 + m);
        if (!g.zbl) {
            const long long cs = g.at(i, j, side == 0 ? g.mz - m : m - 1);
#pragma unroll
            for (int q = 0; q < 9; q++) F[q][cg] = F[q][cs];
        } else {
            const long long c0 = g.at(i, j, side == 0 ? 0 : g.mz - 1);
            const long long cm = g.at(i, j, side == 0 ? m : g.mz - 1 - m);
#pragma unroll
            for (int q = 0; q < 9; q++) F[q][cg] = (R)2.0 * F[q][c0] - F[q][cm];
        }
    }
}

// ---------------------------------------------------------------------------------
// Velocity gradients gij[0..8] = d(u,v,w)/d(x,y,z) at the viscous order and the
// dilatation (derVelX/Y/Z + calcDil, src/calc_stress.cu:20-63,87-96).
// ---------------------------------------------------------------------------------
template <typename R, int V>
__global__ void __launch_bounds__(128) k_grad(Geom g, CoefT<R> cf, const R* __restrict__ u, const R* __restrict__ v,
                                              const R* __restrict__ w, GradOut<R> o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.mx || j >= g.my) return;
    const long long c = g.at(i, j, k);
    const long long st[3] = {1, g.P, g.PS};
    const R* F[3] = {u, v, w};
    R out[9];
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const R* f = F[q];
            R s = cf.c1V[d][1] * (__ldg(f + c + st[d]) - __ldg(f + c - st[d]));
#pragma unroll
            for (int kk = 2; kk <= V; kk++)
                s = fma(cf.c1V[d][kk], __ldg(f + c + kk * st[d]) - __ldg(f + c - kk * st[d]), s);
            if (d == 0 && g.nonuniform_x) s *= cf.xp[i];
            out[3 * d + q] = s;
        }
    }
#pragma unroll
    for (int q = 0; q < 9; q++) o.g[q][c] = out[q];
    o.dil[c] = out[0] + out[4] + out[8];
}

// Dilatation ghosts (BCxNumber2 / BCyNumber1 / BCzNumber1): x periodic | wall: even |
// boundary layer: bottom even, top extrapolated; y periodic; z periodic | extrapolated.
template <typename R>
__global__ void __launch_bounds__(256) k_ghost_scalar(Geom g, R* f) {
    const long long G = g.G;
    const long long nx = 2 * G * g.my * g.mz, ny = 2 * G * g.mx * g.mz, nz = 2 * G * g.mx * g.my;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nx) {
        const int m = (int)(t % G) + 1; t /= G;
        const int side = (int)(t % 2); t /= 2;
        const int j = (int)(t % g.my);
        const int k = (int)(t / g.my);
        const long long cg = g.at(side == 0 ? -m : g.mx - 1 + m, j, k);
        if (g.xbc == XBC_PER) f[cg] = f[g.at(side == 0 ? g.mx - m : m - 1, j, k)];
        else if (g.xbc == XBC_WALL || side == 0) f[cg] = f[g.at(side == 0 ? m - 1 : g.mx - m, j, k)];
        else f[cg] = (R)2.0 * f[g.at(g.mx - 1, j, k)] - f[g.at(g.mx - 1 - m, j, k)];
        return;
    }
    t -= nx;
    if (t < ny) {
        const int m = (int)(t % G) + 1; t /= G;
        const int side = (int)(t % 2); t /= 2;
        const int i = (int)(t % g.mx);
        const int k = (int)(t / g.mx);
        f[g.at(i, side == 0 ? -m : g.my - 1 + m, k)] = f[g.at(i, side == 0 ? g.my - m : m - 1, k)];
        return;
    }
    t -= ny;
    if (t < nz) {
        const int m = (int)(t % G) + 1; t /= G;
        const int side = (int)(t % 2); t /= 2;
        const int i = (int)(t % g.mx);
        const int j = (int)(t / g.mx);
        const long long cg = g.at(i, j, side == 0 ? -m : g.mz - 1 + m);
        if (!g.zbl) f[cg] = f[g.at(i, j, side == 0 ? g.mz - m : m - 1)];
        else f[cg] = (R)2.0 * f[g.at(i, j, side == 0 ? 0 : g.mz - 1)] - f[g.at(i, j, side == 0 ? m : g.mz - 1 - m)];
    }
}

// ---------------------------------------------------------------------------------
// Reductions (deterministic two-pass: fixed partial slots, fixed summation order).
//   min dt (deviceCalcDt + minOfThreads, src/calc_stress.cu:140-160, cuda_math.cu:232-259)
//   sum rho dV, sum rho w dV, sum rhoE dV (integrateThreads, cuda_math.cu:143-171)
//   sum |u|^2 dV / V (AverageThreads, cuda_math.cu:173-201)
// partial layout: part[q*RED_BLOCKS + block], q = 0 dt-min, 1 rho, 2 rho w, 3 rhoE, 4 ke
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_partial(Geom g, Phys ph, StateIn q, const R* __restrict__ mu,
                                                                double* part, int want) {
    __shared__ double sh[5][RED_THREADS / 32];
    const long long n = (long long)g.mx * g.my * g.mz;
    double dtmin = 100000.0, s_r = 0.0, s_rw = 0.0, s_e = 0.0, s_k = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.mx);
        const long long jk = t / g.mx;
        const int j = (int)(jk % g.my);
        const int k = (int)(jk / g.my);
        const long long c = g.at(i, j, k);
        const double rr = q.r[c], uu = q.u[c], vv = q.v[c], ww = q.w[c], ee = q.e[c];
        const double wv = g.wvol[i];
        if (want & RED_DT) {
            double ien = ee / rr - 0.5 * (uu * uu + vv * vv + ww * ww);
            double sos = sqrt(ph.gam * (ph.gam - 1) * ien);
            double dx = g.dxv[i];
            double d2x = dx * dx;
            double m = (double)mu[c];
            double ci = fmax((fabs(uu) + sos) / dx, fmax((fabs(vv) + sos) * g.dy, (fabs(ww) + sos) * g.dz));
            double vi = fmax(m / d2x, fmax(m * g.d2y, m * g.d2z));
            dtmin = fmin(dtmin, ph.cfl / fmax(ci, vi));
        }
        if (want & RED_FORCE) { s_r += rr * wv; s_rw += rr * ww * wv; }
        if (want & RED_ENERGY) s_e += ee * wv;
        if (want & RED_KE) s_k += (uu * uu + vv * vv + ww * ww) * wv;
    }
    double vals[5] = {warp_min(dtmin), warp_sum(s_r), warp_sum(s_rw), warp_sum(s_e), warp_sum(s_k)};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int qq = 0; qq < 5; qq++) sh[qq][wid] = vals[qq];
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = sh[0][0], b = 0, c2 = 0, d = 0, e2 = 0;
        for (int w = 0; w < RED_THREADS / 32; w++) {
            a = fmin(a, sh[0][w]); b += sh[1][w]; c2 += sh[2][w]; d += sh[3][w]; e2 += sh[4][w];
        }
        part[0 * RED_BLOCKS + blockIdx.x] = a;
        part[1 * RED_BLOCKS + blockIdx.x] = b;
        part[2 * RED_BLOCKS + blockIdx.x] = c2;
        part[3 * RED_BLOCKS + blockIdx.x] = d;
        part[4 * RED_BLOCKS + blockIdx.x] = e2;
    }
}

// Final pass: one block. Writes dt (and dpdz with forcing, calcPressureGrad law
// src/calc_stress.cu:16-18) into the scalar block, and the bulk diagnostics into
// diag[0..1] when requested.
__global__ void __launch_bounds__(RED_THREADS) k_reduce_final(Phys ph, const double* part, int nblocks, int want,
                                                              double* scal, double* diag) {
    __shared__ double sh[5][RED_THREADS / 32];
    double a = 100000.0, b = 0, c = 0, d = 0, e = 0;
    for (int t = threadIdx.x; t < nblocks; t += blockDim.x) {
        a = fmin(a, part[0 * RED_BLOCKS + t]);
        b += part[1 * RED_BLOCKS + t];
        c += part[2 * RED_BLOCKS + t];
        d += part[3 * RED_BLOCKS + t];
        e += part[4 * RED_BLOCKS + t];
    }
    double vals[5] = {warp_min(a), warp_sum(b), warp_sum(c), warp_sum(d), warp_sum(e)};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int q = 0; q < 5; q++) sh[q][wid] = vals[q];
    __syncthreads();
    if (threadIdx.x != 0) return;
    a = sh[0][0]; b = c = d = e = 0;
    for (int w = 0; w < RED_THREADS / 32; w++) {
        a = fmin(a, sh[0][w]); b += sh[1][w]; c += sh[2][w]; d += sh[3][w]; e += sh[4][w];
    }
    if (want & RED_DT) {
        scal[SC_DT] = a;
        if (want & RED_FORCE) scal[SC_DPDZ] = 0.99 * scal[SC_DPDZ] - 0.5 * (c / b - 1);
    }
    if (diag) {
        if (want & RED_KE) { diag[0] = e / ph.Lx / ph.Ly / ph.Lz; diag[1] = __longlong_as_double(0x7ff8000000000000LL); }
        else if (want & RED_FORCE) { diag[0] = c / b; diag[1] = d; }
    }
}

// ---------------------------------------------------------------------------------
// Layout conversion between the padded device layout and contiguous [k][j][i] arrays.
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_unpack(Geom g, const double* __restrict__ src, T* __restrict__ dst) {
    const long long n = (long long)g.mx * g.my * g.mz;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.mx);
        const long long jk = t / g.mx;
        dst[g.at(i, (int)(jk % g.my), (int)(jk / g.my))] = (T)src[t];
    }
}
template <typename T>
__global__ void __launch_bounds__(256) k_pack(Geom g, const T* __restrict__ src, double* __restrict__ dst) {
    const long long n = (long long)g.mx * g.my * g.mz;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.mx);
        const long long jk = t / g.mx;
        dst[t] = (double)src[g.at(i, (int)(jk % g.my), (int)(jk / g.my))];
    }
}

// ---------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------
static inline dim3 point_grid(const Geom& g) { return dim3((g.mx + 31) / 32, (g.my + 3) / 4, g.mz); }
static inline dim3 point_block() { return dim3(32, 4, 1); }
static inline unsigned ghost_blocks(const Geom& g) {
    long long n = 2LL * g.G * ((long long)g.my * g.mz + (long long)g.mx * g.mz + (long long)g.mx * g.my);
    return (unsigned)((n + 255) / 256);
}

template <typename R>
void launch_state(const Geom& g, const Phys& ph, const StateIn& q, const DerivedOut<R>& o, double* scal,
                  int advance_time, double* time_log, cudaStream_t s) {
    k_state<R><<<point_grid(g), point_block(), 0, s>>>(g, ph, q, o, scal, advance_time, time_log);
}
template <typename R>
void launch_ghost_state(const Geom& g, const Phys& ph, const StencilFields<R>& f, const double* scal, cudaStream_t s) {
    k_ghost_state<R><<<ghost_blocks(g), 256, 0, s>>>(g, ph, f, scal);
}
template <typename R>
void launch_ghost_scalar(const Geom& g, R* f, cudaStream_t s) {
    k_ghost_scalar<R><<<ghost_blocks(g), 256, 0, s>>>(g, f);
}
template <typename R>
void launch_grad(int V, const Geom& g, const CoefT<R>& cf, const R* u, const R* v, const R* w, const GradOut<R>& o,
                 cudaStream_t s) {
    switch (V) {
    case 1: k_grad<R, 1><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o); break;
    case 2: k_grad<R, 2><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o); break;
    case 3: k_grad<R, 3><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o); break;
    default: k_grad<R, 4><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o); break;
    }
}
template <typename R>
int launch_reduce(const Geom& g, const Phys& ph, const StateIn& q, const R* mu, double* part, int want, double* scal,
                  double* diag, cudaStream_t s) {
    long long n = (long long)g.mx * g.my * g.mz;
    int nb = (int)((n + RED_THREADS - 1) / RED_THREADS);
    if (nb > RED_BLOCKS) nb = RED_BLOCKS;
    k_reduce_partial<R><<<nb, RED_THREADS, 0, s>>>(g, ph, q, mu, part, want);
    k_reduce_final<<<1, RED_THREADS, 0, s>>>(ph, part, nb, want, scal, diag);
    return 2;
}
template <typename T>
void launch_unpack(const Geom& g, const double* src, T* dst, cudaStream_t s) {
    k_unpack<T><<<1184, 256, 0, s>>>(g, src, dst);
}
template <typename T>
void launch_pack(const Geom& g, const T* src, double* dst, cudaStream_t s) {
    k_pack<T><<<1184, 256, 0, s>>>(g, src, dst);
}

#define CNS_INST(R)                                                                                               \
    template void launch_state<R>(const Geom&, const Phys&, const StateIn&, const DerivedOut<R>&, double*, int,   \
                                  double*, cudaStream_t);                                                        \
    template void launch_ghost_state<R>(const Geom&, const Phys&, const StencilFields<R>&, const double*,          \
                                        cudaStream_t);                                                           \
    template void launch_ghost_scalar<R>(const Geom&, R*, cudaStream_t);                                          \
    template void launch_grad<R>(int, const Geom&, const CoefT<R>&, const R*, const R*, const R*, const GradOut<R>&,  \
                                 cudaStream_t);                                                                  \
    template int launch_reduce<R>(const Geom&, const Phys&, const StateIn&, const R*, double*, int, double*,      \
                                  double*, cudaStream_t);                                                        \
    template void launch_unpack<R>(const Geom&, const double*, R*, cudaStream_t);                                 \
    template void launch_pack<R>(const Geom&, const R*, double*, cudaStream_t);
CNS_INST(double)
CNS_INST(float)

}  // namespace cns
