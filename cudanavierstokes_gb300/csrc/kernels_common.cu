// kernels_common.cu -- state recovery, ghost fills, velocity gradients, reductions and
// layout conversion. The RHS/stage kernel lives in kernels_rhs.cuh.
#include "cns_common.cuh"
#include "cns_internal.h"
#include "kernels_point.cuh"

namespace cns {

// Single-solver kernels: thin grids over the per-point bodies of kernels_point.cuh.
template <typename R>
__global__ void __launch_bounds__(128) k_state(Geom g, Phys ph, StateIn q, DerivedOut<R> o, double* scal,
                                               int adv, double* time_log, long long tcap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (adv && i == 0 && j == 0 && k == 0) advance_time(scal, time_log, tcap);
    if (i >= g.mx || j >= g.my) return;
    state_point<R>(g, ph, q, o, scal, i, j, k);
}

// the time advance of stage 0 of a step when the state recovery is fused into the RHS
__global__ void k_advance_time(double* scal, double* time_log, long long tcap) {
    if (threadIdx.x == 0 && blockIdx.x == 0) advance_time(scal, time_log, tcap);
}

template <typename R>
__global__ void __launch_bounds__(256) k_ghost_state(Geom g, Phys ph, StencilFields<R> f, const double* scal) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t < ghost_count(g)) ghost_state_cell<R>(g, ph, f, scal, t);
}

template <typename R, int V>
__global__ void __launch_bounds__(128) k_grad(Geom g, CoefT<R> cf, const R* __restrict__ u, const R* __restrict__ v,
                                              const R* __restrict__ w, GradOut<R> o, int own) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.mx || j >= g.my) return;
    grad_point<R, V, sizeof(R) == 4>(g, cf, u, v, w, o, i, j, (int)blockIdx.z, own != 0);
}

// FP32-RHS dilatation from the packed records (rho, u, v, w), marching in z: blocks of
// 32 x 8 threads, DIL_NZ (8) planes each (dil_column_packed, kernels_point.cuh).
constexpr int DIL_TX = 32, DIL_TY = 8, DIL_NZ = 8;

template <int V>
__global__ void __launch_bounds__(DIL_TX * DIL_TY) k_dil_march(Geom g, CoefT<float> cf, const float4* __restrict__ qa,
                                                               float* __restrict__ dil, int own) {
    __shared__ float su[DIL_TY][DIL_TX + 2 * V];   // u of the tile rows, x halo V on each side
    __shared__ float sv[DIL_TY + 2 * V][DIL_TX];   // v of the tile columns, y halo V on each side
    const int k0 = blockIdx.z * DIL_NZ;
    dil_column_packed<V, DIL_TY>(g, cf, qa, dil, blockIdx.x * DIL_TX, blockIdx.y * DIL_TY, k0,
                                 min(k0 + DIL_NZ, g.mz), own != 0, (int)threadIdx.x, (int)threadIdx.y, su, sv);
}

template <typename R>
__global__ void __launch_bounds__(256) k_ghost_scalar(Geom g, R* f) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t < ghost_count(g)) ghost_scalar_cell<R>(g, f, t);
}

// ---------------------------------------------------------------------------------
// Reductions (deterministic two-pass: fixed partial slots, fixed summation order).
//   min dt (deviceCalcDt + minOfThreads, src/calc_stress.cu:140-160, cuda_math.cu:232-259)
//   sum rho dV, sum rho w dV, sum rhoE dV (integrateThreads, cuda_math.cu:143-171)
//   sum |u|^2 dV / V (AverageThreads, cuda_math.cu:173-201)
// partial layout: part[q*RED_BLOCKS + block], q = 0 dt-min, 1 rho, 2 rho w, 3 rhoE,
// 4 |u|^2, 5 rho |u|^2
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
                                                                int mstride, double* part, int want) {
    __shared__ double sh[6][RED_THREADS / 32];
    const long long n = (long long)g.mx * g.my * g.mz;
    double dtmin = 100000.0, s_r = 0.0, s_rw = 0.0, s_e = 0.0, s_k = 0.0, s_rk = 0.0;
    // 32-bit index arithmetic: n is below the padded field size, itself below 2^31
    const unsigned mx = (unsigned)g.mx, my = (unsigned)g.my;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned tt = (unsigned)t, jk = tt / mx;
        const int i = (int)(tt - jk * mx);
        const int j = (int)(jk % my);
        const int k = (int)(jk / my);
        const long long c = g.at(i, j, k);
        const double rr = q.r[c], uu = q.u[c], vv = q.v[c], ww = q.w[c], ee = q.e[c];
        const double wv = g.wvol[i];
        if (want & RED_DT) {
            double ien = ee / rr - 0.5 * (uu * uu + vv * vv + ww * ww);
            double sos = sqrt(ph.gam * (ph.gam - 1) * ien);
            double dx = g.dxv[i];
            double d2x = dx * dx;
            double m = to_d<R>(mu[c * mstride]);
            double ci = fmax((fabs(uu) + sos) / dx, fmax((fabs(vv) + sos) * g.dy, (fabs(ww) + sos) * g.dz));
            double vi = fmax(m / d2x, fmax(m * g.d2y, m * g.d2z));
            dtmin = fmin(dtmin, ph.cfl / fmax(ci, vi));
        }
        if (want & RED_FORCE) { s_r += rr * wv; s_rw += rr * ww * wv; }
        if (want & RED_ENERGY) s_e += ee * wv;
        if (want & RED_KE) {
            const double q2 = (uu * uu + vv * vv + ww * ww) * wv;
            s_k += q2;
            s_rk += rr * q2;
        }
    }
    double vals[6] = {warp_min(dtmin), warp_sum(s_r), warp_sum(s_rw), warp_sum(s_e), warp_sum(s_k), warp_sum(s_rk)};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int qq = 0; qq < 6; qq++) sh[qq][wid] = vals[qq];
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = sh[0][0], b = 0, c2 = 0, d = 0, e2 = 0, f2 = 0;
        for (int w = 0; w < RED_THREADS / 32; w++) {
            a = fmin(a, sh[0][w]); b += sh[1][w]; c2 += sh[2][w]; d += sh[3][w]; e2 += sh[4][w]; f2 += sh[5][w];
        }
        part[0 * RED_BLOCKS + blockIdx.x] = a;
        part[1 * RED_BLOCKS + blockIdx.x] = b;
        part[2 * RED_BLOCKS + blockIdx.x] = c2;
        part[3 * RED_BLOCKS + blockIdx.x] = d;
        part[4 * RED_BLOCKS + blockIdx.x] = e2;
        part[5 * RED_BLOCKS + blockIdx.x] = f2;
    }
}

// Final pass: one block. Writes dt (and dpdz with forcing, calcPressureGrad law
// src/calc_stress.cu:16-18) into the scalar block, and the bulk diagnostics into
// diag[2 s], diag[2 s + 1] (s = the device step counter) when requested:
// unforced: <u.u> (the reference's kin) and <rho |u|^2>/2; forced: bulk velocity
// int(rho w)/int(rho) and int(rhoE) (calcBulk).
__global__ void __launch_bounds__(RED_THREADS) k_reduce_final(Phys ph, const double* part, int nblocks, int want,
                                                              double* scal, double* diag) {
    __shared__ double sh[6][RED_THREADS / 32];
    double a = 100000.0, b = 0, c = 0, d = 0, e = 0, f = 0;
    for (int t = threadIdx.x; t < nblocks; t += blockDim.x) {
        a = fmin(a, part[0 * RED_BLOCKS + t]);
        b += part[1 * RED_BLOCKS + t];
        c += part[2 * RED_BLOCKS + t];
        d += part[3 * RED_BLOCKS + t];
        e += part[4 * RED_BLOCKS + t];
        f += part[5 * RED_BLOCKS + t];
    }
    double vals[6] = {warp_min(a), warp_sum(b), warp_sum(c), warp_sum(d), warp_sum(e), warp_sum(f)};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int q = 0; q < 6; q++) sh[q][wid] = vals[q];
    __syncthreads();
    if (threadIdx.x != 0) return;
    a = sh[0][0]; b = c = d = e = f = 0;
    for (int w = 0; w < RED_THREADS / 32; w++) {
        a = fmin(a, sh[0][w]); b += sh[1][w]; c += sh[2][w]; d += sh[3][w]; e += sh[4][w]; f += sh[5][w];
    }
    if (want & RED_DT) {
        scal[SC_DT] = a;
        if (want & RED_FORCE) scal[SC_DPDZ] = 0.99 * scal[SC_DPDZ] - 0.5 * (c / b - 1);
    }
    if (diag) {
        double* dg = diag + 2 * (long long)scal[SC_STEP];
        const double vol = ph.Lx * ph.Ly * ph.Lz;
        if (want & RED_KE) { dg[0] = e / ph.Lx / ph.Ly / ph.Lz; dg[1] = 0.5 * f / vol; }
        else if (want & RED_FORCE) { dg[0] = c / b; dg[1] = d; }
    }
}

// ---------------------------------------------------------------------------------
// Layout conversion between the padded device layout and contiguous [k][j][i] arrays.
// ---------------------------------------------------------------------------------
template <typename T>
// (32-bit index arithmetic: the point count is below the padded field size, below 2^31)
__global__ void __launch_bounds__(256) k_unpack(Geom g, const double* __restrict__ src, T* __restrict__ dst) {
    const long long n = (long long)g.mx * g.my * g.mz;
    const unsigned mx = (unsigned)g.mx, my = (unsigned)g.my;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned tt = (unsigned)t, jk = tt / mx;
        dst[g.at((int)(tt - jk * mx), (int)(jk % my), (int)(jk / my))] = (T)src[t];
    }
}
template <typename T>
__global__ void __launch_bounds__(256) k_pack(Geom g, const T* __restrict__ src, double* __restrict__ dst) {
    const long long n = (long long)g.mx * g.my * g.mz;
    const unsigned mx = (unsigned)g.mx, my = (unsigned)g.my;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned tt = (unsigned)t, jk = tt / mx;
        const T x = src[g.at((int)(tt - jk * mx), (int)(jk % my), (int)(jk / my))];
        if constexpr (is_ff<T>) dst[t] = ff_to_d(x);
        else dst[t] = (double)x;
    }
}

// ---------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------
static inline dim3 point_grid(const Geom& g) { return dim3((g.mx + 31) / 32, (g.my + 3) / 4, g.mz); }
static inline dim3 point_block() { return dim3(32, 4, 1); }
static inline unsigned ghost_blocks(const Geom& g) { return (unsigned)((ghost_count(g) + 255) / 256); }

template <typename R>
void launch_state(const Geom& g, const Phys& ph, const StateIn& q, const DerivedOut<R>& o, double* scal,
                  int advance_time, double* time_log, long long tcap, cudaStream_t s) {
    k_state<R><<<point_grid(g), point_block(), 0, s>>>(g, ph, q, o, scal, advance_time, time_log, tcap);
}
void launch_advance_time(double* scal, double* time_log, long long tcap, cudaStream_t s) {
    k_advance_time<<<1, 32, 0, s>>>(scal, time_log, tcap);
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
                 int own, cudaStream_t s) {
    switch (V) {
    case 1: k_grad<R, 1><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o, own); break;
    case 2: k_grad<R, 2><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o, own); break;
    case 3: k_grad<R, 3><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o, own); break;
    default: k_grad<R, 4><<<point_grid(g), point_block(), 0, s>>>(g, cf, u, v, w, o, own); break;
    }
}
void launch_dil_packed(int V, const Geom& g, const CoefT<float>& cf, const float4* qa, float* dil, int own,
                       cudaStream_t s) {
    const dim3 grid((g.mx + DIL_TX - 1) / DIL_TX, (g.my + DIL_TY - 1) / DIL_TY, (g.mz + DIL_NZ - 1) / DIL_NZ);
    const dim3 block(DIL_TX, DIL_TY, 1);
    switch (V) {
    case 1: k_dil_march<1><<<grid, block, 0, s>>>(g, cf, qa, dil, own); break;
    case 2: k_dil_march<2><<<grid, block, 0, s>>>(g, cf, qa, dil, own); break;
    case 3: k_dil_march<3><<<grid, block, 0, s>>>(g, cf, qa, dil, own); break;
    default: k_dil_march<4><<<grid, block, 0, s>>>(g, cf, qa, dil, own); break;
    }
}
template <typename R>
int launch_reduce(const Geom& g, const Phys& ph, const StateIn& q, const R* mu, int mstride, double* part, int want,
                  double* scal, double* diag, cudaStream_t s) {
    long long n = (long long)g.mx * g.my * g.mz;
    int nb = (int)((n + RED_THREADS - 1) / RED_THREADS);
    if (nb > RED_BLOCKS) nb = RED_BLOCKS;
    k_reduce_partial<R><<<nb, RED_THREADS, 0, s>>>(g, ph, q, mu, mstride, part, want);
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
                                  double*, long long, cudaStream_t);                                                        \
    template void launch_ghost_state<R>(const Geom&, const Phys&, const StencilFields<R>&, const double*,          \
                                        cudaStream_t);                                                           \
    template void launch_ghost_scalar<R>(const Geom&, R*, cudaStream_t);                                          \
    template int launch_reduce<R>(const Geom&, const Phys&, const StateIn&, const R*, int, double*, int, double*, \
                                  double*, cudaStream_t);                                                        \
    template void launch_unpack<R>(const Geom&, const double*, R*, cudaStream_t);                                 \
    template void launch_pack<R>(const Geom&, const R*, double*, cudaStream_t);
CNS_INST(double)
CNS_INST(float)
template void launch_grad<double>(int, const Geom&, const CoefT<double>&, const double*, const double*, const double*,
                                  const GradOut<double>&, int, cudaStream_t);
// pair mode (FP32-pair RHS arithmetic): the stencil-input kernels and the RHS output
template void launch_state<ff>(const Geom&, const Phys&, const StateIn&, const DerivedOut<ff>&, double*, int, double*,
                               long long, cudaStream_t);
template void launch_ghost_state<ff>(const Geom&, const Phys&, const StencilFields<ff>&, const double*, cudaStream_t);
template void launch_ghost_scalar<ff>(const Geom&, ff*, cudaStream_t);
template int launch_reduce<ff>(const Geom&, const Phys&, const StateIn&, const ff*, int, double*, int, double*, double*,
                               cudaStream_t);
template void launch_pack<ff>(const Geom&, const ff*, double*, cudaStream_t);
template void launch_grad<ff>(int, const Geom&, const CoefT<ff>&, const ff*, const ff*, const ff*, const GradOut<ff>&,
                              int, cudaStream_t);

}  // namespace cns
