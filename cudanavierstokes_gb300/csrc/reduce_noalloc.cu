// reduce_noalloc.cu -- cns_reduce_state_noalloc: the CFL time step and volume integrals
// of cns_reduce_state for callers that cannot allocate device memory.
//
// Who needs it: code running under a memory manager that owns every device allocation
// of the process (a host framework's caching allocator, or a solver service that divides
// a fixed HBM budget among its simulations and may not let a library take memory behind
// its back), and time-critical loops that must not call cudaMalloc/cudaFree, whose
// cudaFree waits for the whole device. They pass their own input and output buffers; the
// per-plane partial sums live in a fixed file-scope device array instead of a cudaMalloc'd
// scratch buffer.
//
// The scratch holds 5 doubles per z-plane for at most CNS_NOALLOC_MAX_PLANES planes
// (160 KiB). Every GPU that loads this library keeps that array for the life of the
// process. Every call shares it and it keeps the previous call's contents: each call
// writes all the partial slots it later reads, so nothing has to be cleared, but calls
// whose kernels overlap on the GPU (different streams, or different host threads, on the
// same device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/cns.h"
#include "cns_internal.h"

namespace cns {
int launch_plane_reduce(int mx, int my, int mz, const double* r, const double* u, const double* v, const double* w,
                        const double* e, const double* mu, const double* dxv, double dy, double dz, double gam,
                        double cfl, double* scratch, double* out, cudaStream_t s);
}

namespace {

static __device__ __align__(256) double g_plane_scratch[5 * CNS_NOALLOC_MAX_PLANES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double* g_scratch_addr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device. In host code the symbol
// g_plane_scratch is only a host-side stand-in, so the address is queried once per device
// with that device current and cached: the first call on a device does this set-up. The
// cached address belongs to the device's primary context; after cudaDeviceReset on that
// device the address is stale and later calls are invalid.
int scratch_address(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        cudaGetLastError();
        return cns::set_error(CNS_ERR_CUDA, "cns_reduce_state_noalloc: no current CUDA device");
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_plane_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            char buf[200];
            snprintf(buf, sizeof buf, "cns_reduce_state_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                     cudaGetErrorString(e));
            return cns::set_error(CNS_ERR_CUDA, buf);
        }
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return CNS_OK;
}

}  // namespace

extern "C" int cns_reduce_state_noalloc(int mx, int my, int mz, const double* r, const double* u, const double* v,
                                        const double* w, const double* e, const double* mu, const double* dxv,
                                        double dy, double dz, double gam, double cfl, double* out, void* stream) {
    if (mz > CNS_NOALLOC_MAX_PLANES) {
        char buf[200];
        snprintf(buf, sizeof buf, "cns_reduce_state_noalloc: mz = %d exceeds the fixed scratch of %d z-planes", mz,
                 CNS_NOALLOC_MAX_PLANES);
        return cns::set_error(CNS_ERR_INVALID, buf);
    }
    const void* ptrs[8] = {r, u, v, w, e, mu, dxv, out};
    if (int bad = cns::check_reduce_args("cns_reduce_state_noalloc", mx, my, mz, ptrs, 8, dy, dz, gam, cfl)) return bad;
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    rc = cns::launch_plane_reduce(mx, my, mz, r, u, v, w, e, mu, dxv, dy, dz, gam, cfl, scratch, out,
                                  (cudaStream_t)stream);
    if (rc) return cns::set_error(rc, "cns_reduce_state_noalloc: kernel launch failed");
    return CNS_OK;
}
