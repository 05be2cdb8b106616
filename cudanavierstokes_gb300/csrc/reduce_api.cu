// reduce_api.cu -- stateless device reductions of a caller-owned state: the CFL time step
// and the volume integrals behind the body-force controller and the bulk diagnostics
// (calcTimeStep / deviceCalcDt, calcPressureGrad, calcBulk: src/calc_stress.cu:98-201,
// hostReduceToMin / hostVolumeIntegral: src/cuda_math.cu:308-385).
//
// Two passes, deterministic: one block per z-plane writes five plane partials, then one
// block combines the planes in a fixed order.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/cns.h"
#include "cns_internal.h"

namespace {

constexpr int PLANE_THREADS = 256;

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double wmin(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// one block per plane k: part[q*mz + k], q = 0 min dt, 1 rho dV, 2 rho w dV, 3 rhoE dV, 4 |u|^2 dV
__global__ void __launch_bounds__(PLANE_THREADS) k_plane_reduce(int mx, int my, int mz, const double* __restrict__ r,
                                                                const double* __restrict__ u,
                                                                const double* __restrict__ v,
                                                                const double* __restrict__ w,
                                                                const double* __restrict__ e,
                                                                const double* __restrict__ mu,
                                                                const double* __restrict__ dxv, double dy, double dz,
                                                                double gam, double cfl, double* part) {
    __shared__ double sh[5][PLANE_THREADS / 32];
    const int k = blockIdx.x;
    const long long base = (long long)k * mx * my;
    const double dyinv = 1.0 / dy, dzinv = 1.0 / dz, vyz = dy * dz;
    double dtmin = 100000.0, sr = 0, srw = 0, se = 0, sk = 0;
    // 64-bit loop bound: the plane holds fewer than 2^31 points (checked on the host), so
    // t + blockDim.x cannot overflow
    const long long n = (long long)mx * my;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = (int)(t % mx);
        const long long c = base + t;
        const double rr = r[c], uu = u[c], vv = v[c], ww = w[c], ee = e[c];
        const double ien = ee / rr - 0.5 * (uu * uu + vv * vv + ww * ww);
        const double sos = sqrt(gam * (gam - 1) * ien);
        const double dx = dxv[i];
        const double m = mu[c];
        const double ci = fmax((fabs(uu) + sos) / dx, fmax((fabs(vv) + sos) * dyinv, (fabs(ww) + sos) * dzinv));
        const double vi = fmax(m / (dx * dx), fmax(m * dyinv * dyinv, m * dzinv * dzinv));
        dtmin = fmin(dtmin, cfl / fmax(ci, vi));
        const double wv = dx * vyz;
        sr += rr * wv;
        srw += rr * ww * wv;
        se += ee * wv;
        sk += (uu * uu + vv * vv + ww * ww) * wv;
    }
    const double vals[5] = {wmin(dtmin), wsum(sr), wsum(srw), wsum(se), wsum(sk)};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int q = 0; q < 5; q++) sh[q][wid] = vals[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = sh[0][0], b = 0, c = 0, d = 0, f = 0;
        for (int q = 0; q < PLANE_THREADS / 32; q++) {
            a = fmin(a, sh[0][q]); b += sh[1][q]; c += sh[2][q]; d += sh[3][q]; f += sh[4][q];
        }
        part[0 * mz + k] = a;
        part[1 * mz + k] = b;
        part[2 * mz + k] = c;
        part[3 * mz + k] = d;
        part[4 * mz + k] = f;
    }
}

// one block: combine the plane partials in plane order
__global__ void __launch_bounds__(32) k_plane_final(int mz, const double* __restrict__ part, double* out) {
    if (threadIdx.x != 0) return;
    double a = 100000.0, b = 0, c = 0, d = 0, f = 0;
    for (int k = 0; k < mz; k++) {
        a = fmin(a, part[0 * mz + k]);
        b += part[1 * mz + k];
        c += part[2 * mz + k];
        d += part[3 * mz + k];
        f += part[4 * mz + k];
    }
    out[0] = a; out[1] = b; out[2] = c; out[3] = d; out[4] = f;
}

}  // namespace

namespace cns {
// Argument check shared by the reduction entry points: a plane of fewer than 2^31 points,
// non-null pointers, positive spacings, gam > 1, cfl > 0. Records the message under `who`.
int check_reduce_args(const char* who, int mx, int my, int mz, const void* const* ptrs, int n, double dy, double dz,
                      double gam, double cfl) {
    char buf[200];
    if (mx < 1 || my < 1 || mz < 1 || (long long)mx * my >= (1LL << 31)) {
        snprintf(buf, sizeof buf, "%s: grid %d x %d x %d (every edge >= 1, mx*my < 2^31)", who, mx, my, mz);
        return set_error(CNS_ERR_INVALID, buf);
    }
    static const char* names[] = {"r", "u", "v", "w", "e", "mu", "dxv", "out"};
    for (int q = 0; q < n; q++)
        if (!ptrs[q]) {
            snprintf(buf, sizeof buf, "%s: %s is NULL", who, q < 8 ? names[q] : "pointer");
            return set_error(CNS_ERR_INVALID, buf);
        }
    if (!(dy > 0) || !(dz > 0) || !(gam > 1) || !(cfl > 0)) {
        snprintf(buf, sizeof buf, "%s: dy = %g, dz = %g, gam = %g, cfl = %g (need dy, dz, cfl > 0, gam > 1)", who,
                 dy, dz, gam, cfl);
        return set_error(CNS_ERR_INVALID, buf);
    }
    return CNS_OK;
}
}  // namespace cns

namespace cns {
// launch the two reduction passes with the given scratch (5*mz doubles)
int launch_plane_reduce(int mx, int my, int mz, const double* r, const double* u, const double* v, const double* w,
                        const double* e, const double* mu, const double* dxv, double dy, double dz, double gam,
                        double cfl, double* scratch, double* out, cudaStream_t s) {
    k_plane_reduce<<<mz, PLANE_THREADS, 0, s>>>(mx, my, mz, r, u, v, w, e, mu, dxv, dy, dz, gam, cfl, scratch);
    k_plane_final<<<1, 32, 0, s>>>(mz, scratch, out);
    return cudaGetLastError() == cudaSuccess ? CNS_OK : CNS_ERR_CUDA;
}
}  // namespace cns

extern "C" int cns_reduce_state(int mx, int my, int mz, const double* r, const double* u, const double* v,
                                const double* w, const double* e, const double* mu, const double* dxv, double dy,
                                double dz, double gam, double cfl, double* out, void* stream) {
    const void* ptrs[8] = {r, u, v, w, e, mu, dxv, out};
    if (int rc = cns::check_reduce_args("cns_reduce_state", mx, my, mz, ptrs, 8, dy, dz, gam, cfl)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    double* scratch = nullptr;
    const size_t bytes = 5 * (size_t)mz * sizeof(double);
    if (cudaError_t ce = cudaMalloc(&scratch, bytes); ce != cudaSuccess) {
        cudaGetLastError();
        char buf[200];
        snprintf(buf, sizeof buf, "cns_reduce_state: cudaMalloc of %zu bytes of plane partials failed: %s", bytes,
                 cudaGetErrorString(ce));
        return cns::set_error(CNS_ERR_OOM, buf);
    }
    int rc = cns::launch_plane_reduce(mx, my, mz, r, u, v, w, e, mu, dxv, dy, dz, gam, cfl, scratch, out, s);
    if (rc) cns::set_error(rc, "cns_reduce_state: kernel launch failed");
    if (cudaError_t ce = cudaStreamSynchronize(s); ce != cudaSuccess) {
        char buf[200];
        snprintf(buf, sizeof buf, "cns_reduce_state: %s", cudaGetErrorString(ce));
        rc = cns::set_error(CNS_ERR_CUDA, buf);
    }
    cudaFree(scratch);
    return rc;
}
