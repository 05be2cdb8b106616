// cns_internal.h -- kernel argument bundles and host launchers (internal).
#pragma once
#include <cuda_runtime.h>
#include "cns_common.cuh"

namespace cns {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 1024;   // partial slots per reduced quantity
enum { RED_DT = 1, RED_FORCE = 2, RED_ENERGY = 4, RED_KE = 8 };

struct StateIn {
    const double *r, *u, *v, *w, *e;
};
struct StateOut {
    double *r, *u, *v, *w, *e;
};

// lambda = mu / (Pr Ec) at every point, ghosts included (wall and extrapolated ghosts
// are formed from the same T or linearly), so only mu is stored and the RHS applies
// the ratio once per point.
//
// FP64 mode: the stencil inputs rho, u, v, w are the state fields themselves and T, p, H,
// mu are four FP64 fields (h, t, p, m). FP32-RHS mode: the eight stencil inputs are packed
// per point into two 16-byte records, qa = (rho, u, v, w) and qb = (T, p, H, mu), so a
// neighbour costs two vector loads (and one address each) instead of eight scalar loads.
template <typename R>
struct DerivedOut {
    R *h, *t, *p, *m;   // FP64 mode
    R *r, *u, *v, *w;   // pair mode: the state's rho, u, v, w as pairs
    float4 *qa, *qb;    // FP32-RHS mode
};

// the eight ghosted stencil inputs
template <typename R>
struct StencilFields {
    R *r, *u, *v, *w, *t, *p, *h, *m;   // FP64 mode
    float4 *qa, *qb;                    // FP32-RHS mode (packed, see DerivedOut)
};

template <typename R>
struct GradOut {
    R* g[9];
    R* dil;
};

// RHS stage kernel inputs (FP64: separate fields and the nine velocity gradients; FP32-RHS:
// the packed records qa, qb and theta, the RHS kernel forms the gradients itself)
template <typename R>
struct RhsIn {
    const R *r, *u, *v, *w, *t, *p, *h, *m, *dil;
    const R* g[9];
    const float4 *qa, *qb;
};

// time-scheme stage kinds
enum StageKind {
    ST_RHS_ONLY = 0,   // write the RHS to rb, no update
    ST_LS = 1,         // Wray low storage: q += dt (a Rprev + b R), R stored in place of Rprev
    ST_C1 = 2,         // classic RK3 stage 1: q = q0 + R dt/2 (q0 saved from the current state)
    ST_C2 = 3,         // classic RK3 stage 2: q = q0 + (2R - k1) dt
    ST_C3 = 4,         // classic RK3 stage 3: q = q0 + dt (k1 + 4 k2 + R)/6
    ST_R4_1 = 5,       // RK4 stage 1: q0 saved, acc = R, q = q0 + dt/2 R
    ST_R4_2 = 6,       // RK4 stage 2: acc += 2R, q = q0 + dt/2 R
    ST_R4_3 = 7,       // RK4 stage 3: acc += 2R, q = q0 + dt R
    ST_R4_4 = 8        // RK4 stage 4: q = q0 + dt/6 (acc + R)
};

template <typename R>
struct Update {
    int kind;
    double a, b;            // low-storage coefficients
    R ca, cb;               // the same in R (no per-thread conversion)
    int use_prev;           // a != 0: the previous stage's RHS enters the combination
    StateIn qin;            // state at the stage start (point values only)
    StateOut qout;          // new state (interior)
    R* rb[5];               // RHS register (low storage: R_prev in, R out; classic: k1)
    R* k2[5];               // classic RK3 k2 / RK4 accumulator
    double* q0[5];          // classic schemes: conserved state at the step start
    // sponge (boundary layer): strengths and reference fields on the (x,z) plane
    const double *spx, *spz, *rref, *uref, *vref, *wref, *eref;
    // fused state recovery of the new state (calcState of the next stage): 0 = off
    int fuse;
    DerivedOut<R> dnext;
    Phys ph;
};

template <typename R>
void launch_state(const Geom& g, const Phys& ph, const StateIn& q, const DerivedOut<R>& o, double* scal,
                  int advance_time, double* time_log, long long tcap, cudaStream_t s);
void launch_advance_time(double* scal, double* time_log, long long tcap, cudaStream_t s);
template <typename R>
void launch_ghost_state(const Geom& g, const Phys& ph, const StencilFields<R>& f, const double* scal, cudaStream_t s);
template <typename R>
void launch_ghost_scalar(const Geom& g, R* f, cudaStream_t s);
template <typename R>
void launch_grad(int V, const Geom& g, const CoefT<R>& cf, const R* u, const R* v, const R* w, const GradOut<R>& o,
                 int own, cudaStream_t s);
// FP32-RHS dilatation (and its ghost images with own) from the packed records (rho, u, v, w)
void launch_dil_packed(int V, const Geom& g, const CoefT<float>& cf, const float4* qa, float* dil, int own,
                       cudaStream_t s);
// mu[c * mstride]: 1 for an FP64 field, 4 for the mu slot of the packed FP32 records
template <typename R>
int launch_reduce(const Geom& g, const Phys& ph, const StateIn& q, const R* mu, int mstride, double* part, int want,
                  double* scal, double* diag, cudaStream_t s);
template <typename T>
void launch_unpack(const Geom& g, const double* src, T* dst, cudaStream_t s);
template <typename T>
void launch_pack(const Geom& g, const T* src, double* dst, cudaStream_t s);

// record `msg` as the calling thread's cns_last_error() text and return `code`
int set_error(int code, const char* msg);

// argument check of the stateless reductions (records the message under `who`)
int check_reduce_args(const char* who, int mx, int my, int mz, const void* const* ptrs, int n, double dy, double dz,
                      double gam, double cfl);

// the RHS + stage kernel over the interior; returns the number of launches (band groups)
int launch_rhs_fp64(int S, int V, const Geom& g, const Phys& ph, const CoefT<double>& cf, const RhsIn<double>& in,
                    const Update<double>& up, double* scal, int quirk, cudaStream_t s);
int launch_rhs_fp32(int S, int V, const Geom& g, const Phys& ph, const CoefT<float>& cf, const RhsIn<float>& in,
                    const Update<float>& up, double* scal, int quirk, cudaStream_t s);
int launch_rhs_pair(int S, int V, const Geom& g, const Phys& ph, const CoefT<ff>& cf, const RhsIn<ff>& in,
                    const Update<ff>& up, double* scal, int quirk, cudaStream_t s);

}  // namespace cns
