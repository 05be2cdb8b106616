// solver_internal.h -- the solver handle (internal; shared by solver.cu and batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/cns.h"
#include "cns_internal.h"
#include "grid.h"

namespace cns {
int set_error(int code, const char* msg);
}

struct cns_solver {
    using HostGrid = cns::HostGrid;
    using Geom = cns::Geom;
    using Phys = cns::Phys;
    template <typename R> using CoefT = cns::CoefT<R>;
    cns_params p{};
    int device = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    HostGrid hg;
    Geom geom{};
    Phys phys{};
    CoefT<double> cf64{};
    CoefT<float> cf32{};
    CoefT<cns::ff> cfp{};        // pair mode
    bool fp32 = false;
    bool pair = false;           // CNS_PREC_PAIR_RHS: RHS arithmetic in FP32 pairs (cns::ff)
    size_t rsz = 8;              // bytes of the RHS arithmetic type
    long long nalloc = 0;        // elements of one padded field
    std::vector<void*> allocs;
    int64_t bytes = 0;
    int64_t launches = 0;

    double* q[2][5] = {};        // state ping-pong (rho, u, v, w, rhoE)
    int cur = 0;
    // stencil inputs derived from the state buffer q[b], in der[b]: FP64 mode h, t, p, mu
    // (the state itself gives rho, u, v, w); FP32-RHS mode der[b][0] = the packed records
    // (rho, u, v, w) and der[b][1] = (T, p, H, mu), float4 each. The RHS kernel reads those of
    // q[cur] and writes those of the new state q[1 - cur] (fused state recovery). Pair mode:
    // der[b][0..3] = h, t, p, mu and der[b][4..7] = rho, u, v, w, all as pairs
    void* der[2][8] = {};
    bool der_ok[2] = {false, false};   // der[b] holds the recovery of q[b]
    int mu_buf = 0;                    // buffer of the latest state recovery in program order of
                                       // the reference (its mu sets the CFL time step)
    void* dil = nullptr;         // (R)
    void* grad[9] = {};          // (R)
    void* rb[5] = {};            // RHS register (R)
    void* k2[5] = {};            // classic RK3 k2 / RK4 accumulator (R)
    double* q0[5] = {};          // classic schemes: conserved state at the step start
    double* staging = nullptr;   // N doubles, host <-> device layout conversion
    double* scal = nullptr;      // device scalars (SC_*)
    double* part = nullptr;      // reduction partials 5 * RED_BLOCKS
    double* diag = nullptr;      // per-step bulk diagnostics (2 per step)
    double* tlog = nullptr;      // per-step time
    int diag_cap = 0;
    double *xp_d = nullptr, *cvsx_d = nullptr, *wvol_d = nullptr, *dxv_d = nullptr;
    float *xp_f = nullptr, *cvsx_f = nullptr;
    cns::ff *xp_p = nullptr, *cvsx_p = nullptr;
    double *spx = nullptr, *spz = nullptr, *rref = nullptr, *uref = nullptr, *vref = nullptr, *wref = nullptr,
           *eref = nullptr;
    bool has_sponge = false;
    bool initialized = false;
    // one captured time step per starting ping-pong parity (kernel arguments are
    // step-invariant: per-step log slots come from the device step counter)
    cudaGraphExec_t step_exec[2] = {nullptr, nullptr};
    int64_t step_kernels = 0;
    bool use_graphs = true;

    void drop_graphs() {
        for (int c = 0; c < 2; c++)
            if (step_exec[c]) { cudaGraphExecDestroy(step_exec[c]); step_exec[c] = nullptr; }
    }

    template <typename T>
    int alloc(T** ptr, size_t n) {
        void* p0 = nullptr;
        cudaError_t e = cudaMalloc(&p0, n * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cns::set_error(CNS_ERR_OOM, "cudaMalloc failed");
        }
        allocs.push_back(p0);
        bytes += (int64_t)(n * sizeof(T));
        *ptr = (T*)p0;
        return CNS_OK;
    }
    // nf fields of esz bytes in one allocation, field f at ptr[f] = base + f * nalloc elements
    // (a state buffer or an RK register as one block: kernels that take many fields can
    // address them from one base pointer and the field stride nalloc)
    int alloc_fields(void** ptr, int nf, size_t esz) {
        void* p0 = nullptr;
        cudaError_t e = cudaMalloc(&p0, (size_t)nalloc * esz * nf);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cns::set_error(CNS_ERR_OOM, "cudaMalloc of a field group failed");
        }
        allocs.push_back(p0);
        bytes += (int64_t)((size_t)nalloc * esz * nf);
        for (int f = 0; f < nf; f++) ptr[f] = (char*)p0 + (size_t)f * nalloc * esz;
        return CNS_OK;
    }
    int alloc_field(void** ptr, size_t esz) {
        void* p0 = nullptr;
        cudaError_t e = cudaMalloc(&p0, (size_t)nalloc * esz);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cns::set_error(CNS_ERR_OOM, "cudaMalloc of a field failed");
        }
        allocs.push_back(p0);
        bytes += (int64_t)((size_t)nalloc * esz);
        *ptr = p0;
        return CNS_OK;
    }
    ~cns_solver() {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        drop_graphs();
        for (void* a : allocs) cudaFree(a);
        if (own_stream) cudaStreamDestroy(own_stream);
        if (prev >= 0) cudaSetDevice(prev);
    }
};


namespace cns {
// parity swap: make buffer `want` the current state buffer (pointer swap, no copy)
inline void solver_set_parity(cns_solver* h, int want) {
    if (h->cur == want) return;
    for (int f = 0; f < 5; f++) {
        double* t = h->q[0][f];
        h->q[0][f] = h->q[1][f];
        h->q[1][f] = t;
    }
    for (int f = 0; f < 8; f++) {
        void* a = h->der[0][f]; h->der[0][f] = h->der[1][f]; h->der[1][f] = a;
    }
    const bool ok0 = h->der_ok[0];
    h->der_ok[0] = h->der_ok[1];
    h->der_ok[1] = ok0;
    h->mu_buf = 1 - h->mu_buf;
    h->cur = want;
    h->drop_graphs();
}
int solver_reduce(cns_solver* h, int want, double* diag);
// stencil inputs (+ theta, gradients) of state buffer b
template <typename R>
RhsIn<R> solver_rhs_in(cns_solver* h, int b);
// stage update of the given kind from state buffer c into 1 - c, with the fused recovery of
// the new state's derived fields
template <typename R>
Update<R> solver_stage_update(cns_solver* h, int kind, double a, double b, int c);
// recover the current state's derived fields unless they are current
int solver_ensure_state(cns_solver* h);
// one time step of the handle's scheme on h->stream (through its step graph when graphs
// are on), logging the time at the device step counter up to diag_cap entries
int solver_step(cns_solver* h);
}  // namespace cns
