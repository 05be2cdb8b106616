// peak.cu -- FMA-throughput probe used to state the FP64 / FP32 pipe roofline next to the
// measured HBM bandwidth (the stencil path is bounded by the FP64 pipe, not by HBM).
#include <cuda_runtime.h>

#include "../../include/cns.h"
#include "cns_common.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T* out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int it = 0; it < iters; it++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-12345.0) out[blockIdx.x] = s;   // never true; keeps the chains live
}

template <typename T>
int probe(int device, int iters, double* tflops) {
    if (cudaSetDevice(device) != cudaSuccess) return CNS_ERR_CUDA;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    const int blocks = nsm * 8, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, blocks * sizeof(T)) != cudaSuccess) return CNS_ERR_OOM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_peak<T><<<blocks, threads>>>(out, iters / 10, (T)0.999999, (T)1e-7);   // warm-up
    cudaEventRecord(e0);
    k_fma_peak<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return CNS_ERR_CUDA;
    *tflops = 2.0 * 8.0 * (double)blocks * threads * (double)iters / (ms * 1e-3) / 1e12;
    return CNS_OK;
}

__global__ void __launch_bounds__(256) k_convert(const double* __restrict__ x, float* __restrict__ f_alu,
                                                 float* __restrict__ f_hw, const float* __restrict__ y,
                                                 double* __restrict__ d_alu, double* __restrict__ d_hw, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        f_alu[t] = cns::d2f(x[t]);
        f_hw[t] = __double2float_rn(x[t]);
        d_alu[t] = cns::f2d(y[t]);
        d_hw[t] = (double)y[t];
    }
}

__global__ void __launch_bounds__(256) k_pow(const double* __restrict__ x, double a, double* __restrict__ fast,
                                             double* __restrict__ lib, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        fast[t] = cns::pow_visc(x[t], a);
        lib[t] = pow(x[t], a);
    }
}

__global__ void __launch_bounds__(256) k_rcp(const double* __restrict__ x, double* __restrict__ fast,
                                             double* __restrict__ lib, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        fast[t] = cns::rcp_nr(x[t]);
        lib[t] = 1.0 / x[t];
    }
}

// pair arithmetic on (a, b, c): the scalar sum, product, fused multiply-add and compensated
// accumulation (a b + c), then the same through the packed two-lane forms with lane 0 on
// (a, b, c) and lane 1 on (b, c, a); every result as its two floats
__global__ void __launch_bounds__(256) k_pair(const double* __restrict__ a, const double* __restrict__ b,
                                              const double* __restrict__ c, float* __restrict__ out, long long n) {
    using cns::ff;
    using cns::ff2;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const ff pa = cns::d_to_ff(a[t]), pb = cns::d_to_ff(b[t]), pc = cns::d_to_ff(c[t]);
        cns::ffacc acc(pc);
        acc.add_prod(pa, pb);
        const ff2 x = cns::mk2(pa, pb), y = cns::mk2(pb, pc), z = cns::mk2(pc, pa);
        cns::ffacc2 acc2(z);
        acc2.add_prod(x, y);
        const ff2 s2 = x + y, m2 = x * y, f2 = fma(x, y, z), d2 = acc2.value();
        const ff r[15] = {pa, pb, pc, pa + pb, pa * pb, fma(pa, pb, pc), acc.value(),
                          cns::lane0(s2), cns::lane0(m2), cns::lane0(f2), cns::lane0(d2),
                          cns::lane1(s2), cns::lane1(m2), cns::lane1(f2), cns::lane1(d2)};
        for (int q = 0; q < 15; q++) {
            out[(t * 15 + q) * 2] = r[q].h;
            out[(t * 15 + q) * 2 + 1] = r[q].l;
        }
    }
}

}  // namespace

extern "C" int cns_selftest_pair(int device, const double* a, const double* b, const double* c, long long n,
                                 float* out) {
    if (!a || !b || !c || !out || n < 1 || n > (1LL << 24)) return CNS_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return CNS_ERR_CUDA;
    double* buf = nullptr;
    float* res = nullptr;
    const size_t nb = (size_t)n;
    if (cudaMalloc(&buf, nb * 3 * sizeof(double)) != cudaSuccess) return CNS_ERR_OOM;
    if (cudaMalloc(&res, nb * 30 * sizeof(float)) != cudaSuccess) {
        cudaFree(buf);
        return CNS_ERR_OOM;
    }
    cudaError_t e = cudaMemcpy(buf, a, nb * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(buf + nb, b, nb * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(buf + 2 * nb, c, nb * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_pair<<<512, 256>>>(buf, buf + nb, buf + 2 * nb, res, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, res, nb * 30 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    cudaFree(res);
    return e == cudaSuccess ? CNS_OK : CNS_ERR_CUDA;
}

extern "C" int cns_selftest_rcp(int device, const double* x, long long n, double* fast, double* lib) {
    if (!x || !fast || !lib || n < 1 || n > (1LL << 27)) return CNS_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return CNS_ERR_CUDA;
    double* buf = nullptr;
    const size_t nb = (size_t)n;
    if (cudaMalloc(&buf, nb * 3 * sizeof(double)) != cudaSuccess) return CNS_ERR_OOM;
    cudaError_t e = cudaMemcpy(buf, x, nb * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_rcp<<<1024, 256>>>(buf, buf + nb, buf + 2 * nb, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(fast, buf + nb, nb * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(lib, buf + 2 * nb, nb * 8, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e == cudaSuccess ? CNS_OK : CNS_ERR_CUDA;
}

extern "C" int cns_selftest_pow(int device, const double* x, long long n, double a, double* fast, double* lib) {
    if (!x || !fast || !lib || n < 1 || n > (1LL << 27)) return CNS_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return CNS_ERR_CUDA;
    double* buf = nullptr;
    const size_t nb = (size_t)n;
    if (cudaMalloc(&buf, nb * 3 * sizeof(double)) != cudaSuccess) return CNS_ERR_OOM;
    cudaError_t e = cudaMemcpy(buf, x, nb * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_pow<<<1024, 256>>>(buf, a, buf + nb, buf + 2 * nb, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(fast, buf + nb, nb * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(lib, buf + 2 * nb, nb * 8, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e == cudaSuccess ? CNS_OK : CNS_ERR_CUDA;
}

extern "C" int cns_selftest_convert(int device, const double* x, const float* y, long long n, float* f_alu,
                                    float* f_hw, double* d_alu, double* d_hw) {
    if (!x || !y || !f_alu || !f_hw || !d_alu || !d_hw || n < 1 || n > (1LL << 28)) return CNS_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return CNS_ERR_CUDA;
    char* buf = nullptr;
    const size_t nb = (size_t)n;
    if (cudaMalloc(&buf, nb * (8 + 4 + 4 + 4 + 8 + 8)) != cudaSuccess) return CNS_ERR_OOM;
    double* dx = (double*)buf;
    double* dda = dx + nb;
    double* ddh = dda + nb;
    float* dfa = (float*)(ddh + nb);
    float* dfh = dfa + nb;
    float* dy = dfh + nb;
    cudaError_t e = cudaMemcpy(dx, x, nb * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dy, y, nb * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_convert<<<1024, 256>>>(dx, dfa, dfh, dy, dda, ddh, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(f_alu, dfa, nb * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f_hw, dfh, nb * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d_alu, dda, nb * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d_hw, ddh, nb * 8, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e == cudaSuccess ? CNS_OK : CNS_ERR_CUDA;
}

extern "C" int cns_probe_fma_peak(int device, int fp64, int iters, double* tflops) {
    if (!tflops || iters < 10) return CNS_ERR_INVALID;
    return fp64 ? probe<double>(device, iters, tflops) : probe<float>(device, iters, tflops);
}
