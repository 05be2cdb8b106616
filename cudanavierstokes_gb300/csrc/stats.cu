// stats.cu -- flow statistics of the current state on the device: the plane profiles over
// (y, z) of calcAvgChan and the wall friction Reynolds number of printRes
// (src/init.cpp:150-256), which the reference evaluates on the host after copying the
// fields back. Deterministic: fixed-order partial sums, no atomics.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/cns.h"
#include "cns_internal.h"
#include "solver_internal.h"

using namespace cns;

namespace {

constexpr int ST_THREADS = 128;   // x-indices per block
constexpr int ST_SLICES = 128;    // partial sums per x-index (row slices of the (y, z) plane)

// Per x-index sums over a slice of the (j, k) rows (coalesced along x): pass 0 sums rho,
// rho u, rho v, rho w, rhoE; pass 1 the squared deviations from the plane means.
__global__ void __launch_bounds__(ST_THREADS) k_plane_sum(Geom g, StateIn q, const double* __restrict__ mean,
                                                          double* __restrict__ part) {
    const int i = blockIdx.x * ST_THREADS + threadIdx.x;
    if (i >= g.mx) return;
    const long long rows = (long long)g.my * g.mz;
    double s[5] = {0, 0, 0, 0, 0};
    double m[5] = {0, 0, 0, 0, 0};
    if (mean)
        for (int f = 0; f < 5; f++) m[f] = mean[f * g.mx + i];
    for (long long rr = blockIdx.y; rr < rows; rr += gridDim.y) {
        const long long c = g.at(i, (int)(rr % g.my), (int)(rr / g.my));
        const double r = q.r[c], u = q.u[c], v = q.v[c], w = q.w[c], e = q.e[c];
        if (!mean) {
            s[0] += r; s[1] += r * u; s[2] += r * v; s[3] += r * w; s[4] += e;
        } else {
            s[0] += (r - m[0]) * (r - m[0]);
            s[1] += (u - m[1]) * (u - m[1]);
            s[2] += (v - m[2]) * (v - m[2]);
            s[3] += (w - m[3]) * (w - m[3]);
            s[4] += (e - m[4]) * (e - m[4]);
        }
    }
    for (int f = 0; f < 5; f++) part[((long long)f * gridDim.y + blockIdx.y) * g.mx + i] = s[f];
}

// Slices summed in order; pass 0 turns the sums into <rho>, <rho u>/<rho>, ..., <rhoE>,
// pass 1 into the mean squared deviations.
__global__ void k_plane_final(int mx, int slices, double n, int pass, const double* __restrict__ part,
                              double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mx) return;
    double s[5];
    for (int f = 0; f < 5; f++) {
        double a = 0.0;
        for (int b = 0; b < slices; b++) a += part[((long long)f * slices + b) * mx + i];
        s[f] = a / n;
    }
    if (pass == 0) {
        s[1] /= s[0]; s[2] /= s[0]; s[3] /= s[0];
    }
    for (int f = 0; f < 5; f++) out[f * mx + i] = s[f];
}

// u_tau rho_w / mu_w of each (j, k) wall column, block sums in a fixed tree order
__global__ void __launch_bounds__(256) k_friction(Geom g, const double* __restrict__ r, const double* __restrict__ w,
                                                  int S, double c1, double c2, double c3, double c4, double xp0,
                                                  double muw, double* __restrict__ part) {
    __shared__ double sh[256];
    const long long rows = (long long)g.my * g.mz;
    const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
    double val = 0.0;
    if (t < rows) {
        const int j = (int)(t % g.my), k = (int)(t / g.my);
        // the reference mirrors the first S interior values evenly about the wall, so the
        // k-th difference pairs w(i = k) with w(i = k - 1)
        const double co[4] = {c1, c2, c3, c4};
        double d = 0.0;
        for (int kk = 1; kk <= S; kk++) d += co[kk - 1] * (w[g.at(kk, j, k)] - w[g.at(kk - 1, j, k)]);
        d *= xp0;
        const double rw = r[g.at(0, j, k)];
        val = sqrt(muw * fabs(d) / rw) * rw / muw;
    }
    sh[threadIdx.x] = val;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_ordered(const double* __restrict__ part, int n, double scale, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < n; b++) s += part[b];
        *out = s * scale;
    }
}

int stats_error(cudaError_t e) {
    return cns::set_error(e == cudaErrorMemoryAllocation ? CNS_ERR_OOM : CNS_ERR_CUDA, cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int cns_plane_stats(cns_solver* h, double* out) {
    if (!h || !out) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    if (!h->initialized) return cns::set_error(CNS_ERR_STATE, "no field has been copied in");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return stats_error(e);
    const int mx = h->p.mx;
    double* buf = nullptr;   // partials, means, deviations
    const size_t np = (size_t)5 * ST_SLICES * mx;
    e = cudaMallocAsync(&buf, (np + 10 * (size_t)mx) * sizeof(double), h->stream);
    if (e != cudaSuccess) return stats_error(e);
    double* mean = buf + np;
    double* dev = mean + 5 * (size_t)mx;
    const StateIn q{h->q[h->cur][0], h->q[h->cur][1], h->q[h->cur][2], h->q[h->cur][3], h->q[h->cur][4]};
    const dim3 grid((mx + ST_THREADS - 1) / ST_THREADS, ST_SLICES);
    const double n = (double)h->p.my * h->p.mz;
    k_plane_sum<<<grid, ST_THREADS, 0, h->stream>>>(h->geom, q, nullptr, buf);
    k_plane_final<<<(mx + 127) / 128, 128, 0, h->stream>>>(mx, ST_SLICES, n, 0, buf, mean);
    k_plane_sum<<<grid, ST_THREADS, 0, h->stream>>>(h->geom, q, mean, buf);
    k_plane_final<<<(mx + 127) / 128, 128, 0, h->stream>>>(mx, ST_SLICES, n, 1, buf, dev);
    h->launches += 4;
    std::vector<double> hv(10 * (size_t)mx);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hv.data(), mean, hv.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                              h->stream);
    cudaFreeAsync(buf, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return stats_error(e);
    for (int i = 0; i < mx; i++) out[i] = h->hg.x[i];
    for (size_t c = 0; c < hv.size(); c++) out[(size_t)mx + c] = hv[c];
    return CNS_OK;
}

int cns_friction_reynolds(cns_solver* h, double* ret) {
    if (!h || !ret) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    if (!h->initialized) return cns::set_error(CNS_ERR_STATE, "no field has been copied in");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return stats_error(e);
    const int S = h->p.stencil_size;
    const long long rows = (long long)h->p.my * h->p.mz;
    const int nb = (int)((rows + 255) / 256);
    double* buf = nullptr;
    e = cudaMallocAsync(&buf, (nb + 1) * sizeof(double), h->stream);
    if (e != cudaSuccess) return stats_error(e);
    // first-derivative weights at the advective order with 1/dx (the reference's
    // coeffF / dx, src/init.cpp:229-234), the metric x'(0)^-1 and mu_w = T_w^viscexp / Re, T_w = 1
    const double* c1 = h->hg.c1S[0];
    const double muw = std::pow(1.0, h->p.viscexp) / h->p.Re;
    k_friction<<<nb, 256, 0, h->stream>>>(h->geom, h->q[h->cur][0], h->q[h->cur][3], S, c1[1], S > 1 ? c1[2] : 0.0,
                                          S > 2 ? c1[3] : 0.0, S > 3 ? c1[4] : 0.0, h->hg.xp[0], muw, buf);
    k_sum_ordered<<<1, 32, 0, h->stream>>>(buf, nb, 1.0 / (double)rows, buf + nb);
    h->launches += 2;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(ret, buf + nb, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(buf, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? CNS_OK : stats_error(e);
}

}  // extern "C"
