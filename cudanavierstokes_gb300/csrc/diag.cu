// diag.cu -- volume-averaged viscous dissipation and enstrophy of the current state:
//   eps = < tau_ij du_i/dx_j >,  tau_ij = mu (du_i/dx_j + du_j/dx_i - 2/3 delta_ij theta),
//   Omega = < |curl u|^2 >,
// averaged with the cell volumes over the box (the weights of the bulk integrals,
// src/calc_stress.cu:162-201). The gradients are those of derVelX/Y/Z at the viscous order
// (src/calc_stress.cu:20-63, with the velocity ghosts of src/boundary_condition_x.h:23-45
// and _z.h), mu that of calcState (src/cuda_main.cu:218-242). The reference has no such
// diagnostic (its dissipation is left to post-processing); for the Taylor-Green vortex eps
// is the kinetic-energy decay rate -dK/dt up to pressure-dilatation work. Computed in FP64
// from the FP64 state in both precision modes. Deterministic: per-block partials in fixed
// slots, summed in a fixed order.
#include <cuda_runtime.h>

#include "../../include/cns.h"
#include "cns_internal.h"
#include "kernels_point.cuh"
#include "solver_internal.h"

using namespace cns;

namespace {

constexpr int DG_THREADS = 128;   // 32 x 4 points of one plane per block
constexpr int DG_FINAL = 256;

// the velocity ghost layer of the FP64 state (in FP32-RHS mode the ghost kernel fills the
// FP32 stencil copies, not the state)
__global__ void __launch_bounds__(256) k_ghost_vel(Geom g, Phys ph, double* u, double* v, double* w,
                                                   const double* scal) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t < ghost_count(g)) ghost_vel_cell(g, ph, u, v, w, scal, t);
}

template <int V>
__global__ void __launch_bounds__(DG_THREADS) k_dissip(Geom g, Phys ph, CoefT<double> cf, StateIn q,
                                                       double* __restrict__ part) {
    const int i = blockIdx.x * 32 + (threadIdx.x & 31);
    const int j = blockIdx.y * 4 + (threadIdx.x >> 5);
    const int k = blockIdx.z;
    double phi = 0.0, ens = 0.0;
    if (i < g.mx && j < g.my) {
        const long long c = g.at(i, j, k);
        const long long st[3] = {1, g.P, g.PS};
        const double* F[3] = {q.u, q.v, q.w};
        double G[9];   // G[3 d + n] = d u_n / d x_d, as grad_point
#pragma unroll
        for (int d = 0; d < 3; d++) {
#pragma unroll
            for (int n = 0; n < 3; n++) {
                const double* f = F[n];
                double s = cf.c1V[d][1] * (f[c + st[d]] - f[c - st[d]]);
#pragma unroll
                for (int kk = 2; kk <= V; kk++) s = fma(cf.c1V[d][kk], f[c + kk * st[d]] - f[c - kk * st[d]], s);
                if (d == 0 && g.nonuniform_x) s *= cf.xp[i];
                G[3 * d + n] = s;
            }
        }
        const double rr = q.r[c], uu = q.u[c], vv = q.v[c], ww = q.w[c], ee = q.e[c];
        const double en = ee * rcp_nr(rr) - 0.5 * (uu * uu + vv * vv + ww * ww);
        const double T = ph.cvInv * en;
        const double mu = (ph.vexp_is_one ? T : pow_visc(T, ph.vexp)) * ph.invRe;
        const double th = G[0] + G[4] + G[8];
        double s = 0.0;
#pragma unroll
        for (int d = 0; d < 3; d++)
#pragma unroll
            for (int n = 0; n < 3; n++) {
                const double tau = G[3 * d + n] + G[3 * n + d] - (n == d ? (2.0 / 3.0) * th : 0.0);
                s = fma(tau, G[3 * d + n], s);
            }
        const double wx = G[5] - G[7], wy = G[6] - G[2], wz = G[1] - G[3];
        const double wv = g.wvol[i];
        phi = mu * s * wv;
        ens = (wx * wx + wy * wy + wz * wz) * wv;
    }
    __shared__ double sh[2][DG_THREADS];
    sh[0][threadIdx.x] = phi;
    sh[1][threadIdx.x] = ens;
    __syncthreads();
    for (int h = DG_THREADS / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + h];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        part[2 * b] = sh[0][0];
        part[2 * b + 1] = sh[1][0];
    }
}

// the block partials summed in a fixed order: thread t takes partials t, t + 256, ..., then a
// fixed tree; the means over the box volume
__global__ void __launch_bounds__(DG_FINAL) k_dissip_final(const double* __restrict__ part, long long nb, double vol,
                                                           double* __restrict__ out) {
    double a = 0.0, b = 0.0;
    for (long long t = threadIdx.x; t < nb; t += DG_FINAL) {
        a += part[2 * t];
        b += part[2 * t + 1];
    }
    __shared__ double sh[2][DG_FINAL];
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    __syncthreads();
    for (int h = DG_FINAL / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + h];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sh[0][0] / vol;
        out[1] = sh[1][0] / vol;
    }
}

int diag_error(cudaError_t e) {
    return cns::set_error(e == cudaErrorMemoryAllocation ? CNS_ERR_OOM : CNS_ERR_CUDA, cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int cns_dissipation(cns_solver* h, double* out) {
    if (!h || !out) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    if (!h->initialized) return cns::set_error(CNS_ERR_STATE, "no field has been copied in");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return diag_error(e);
    const Geom& g = h->geom;
    const int c = h->cur;
    const StateIn q{h->q[c][0], h->q[c][1], h->q[c][2], h->q[c][3], h->q[c][4]};
    const dim3 grid((g.mx + 31) / 32, (g.my + 3) / 4, g.mz);
    const long long nb = (long long)grid.x * grid.y * grid.z;
    double* buf = nullptr;   // partials, then the two means
    e = cudaMallocAsync(&buf, (2 * nb + 2) * sizeof(double), h->stream);
    if (e != cudaSuccess) return diag_error(e);
    const unsigned gb = (unsigned)((ghost_count(g) + 255) / 256);
    k_ghost_vel<<<gb, 256, 0, h->stream>>>(g, h->phys, h->q[c][1], h->q[c][2], h->q[c][3], h->scal);
    switch (h->p.stencil_visc) {
    case 1: k_dissip<1><<<grid, DG_THREADS, 0, h->stream>>>(g, h->phys, h->cf64, q, buf); break;
    case 2: k_dissip<2><<<grid, DG_THREADS, 0, h->stream>>>(g, h->phys, h->cf64, q, buf); break;
    case 3: k_dissip<3><<<grid, DG_THREADS, 0, h->stream>>>(g, h->phys, h->cf64, q, buf); break;
    default: k_dissip<4><<<grid, DG_THREADS, 0, h->stream>>>(g, h->phys, h->cf64, q, buf); break;
    }
    const double vol = h->phys.Lx * h->phys.Ly * h->phys.Lz;
    k_dissip_final<<<1, DG_FINAL, 0, h->stream>>>(buf, nb, vol, buf + 2 * nb);
    h->launches += 3;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf + 2 * nb, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(buf, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? CNS_OK : diag_error(e);
}

}  // extern "C"
