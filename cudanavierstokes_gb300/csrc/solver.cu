// solver.cu -- solver handle, time-step orchestration and the C ABI (include/cns.h).
//
// One handle = one simulation resident on one GPU. A time step is
//   [every check_cfl / check_bulk steps: one fused two-pass reduction for dt, the body
//    force controller and the bulk diagnostics, all on the device]
//   k_advance_time, then per Runge-Kutta stage:
//     k_ghost_state -> k_grad (9 gradients + theta; FP32-RHS: k_dil_pair, theta only; both
//     write theta's ghost images on periodic and wall boundaries, the boundary layer adds
//     k_ghost_scalar) -> k_rhs (RHS of x, y, z + body force + sponge + update, and T, p, H,
//     mu of the new state for the next stage; on large planes one launch per group of
//     bands; k_state runs only after the state is set from outside)
// with no host round trip inside a run (the reference copies dt and dpdz through the
// host and MPI every check_cfl steps: src/cuda_main.cu:249-265).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/cns.h"
#include "cns_internal.h"
#include "grid.h"
#include "solver_internal.h"

using namespace cns;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? CNS_ERR_OOM : CNS_ERR_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                            \
    } while (0)

#define CKL()                                                                                        \
    do {                                                                                             \
        cudaError_t e_ = cudaGetLastError();                                                         \
        if (e_ != cudaSuccess)                                                                       \
            return fail(CNS_ERR_CUDA, "kernel launch: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                   \
    } while (0)

}  // namespace

namespace cns {
int set_error(int code, const char* msg) {
    g_err = msg ? msg : "";
    return code;
}
}  // namespace cns

namespace {

// ---- parameter validation ------------------------------------------------------------
int check_params(const cns_params* p) {
    if (!p) return fail(CNS_ERR_INVALID, "params is NULL");
    if (p->stencil_size < 1 || p->stencil_size > 4)
        return fail(CNS_ERR_INVALID, "stencil_size must be 1..4 (got %d)", p->stencil_size);
    if (p->stencil_visc < 1 || p->stencil_visc > p->stencil_size)
        return fail(CNS_ERR_INVALID, "stencil_visc must be 1..stencil_size (got %d)", p->stencil_visc);
    const int S = p->stencil_size;
    if (p->mx < 2 * S + 1 || p->my < 2 * S || p->mz < 2 * S + 1)
        return fail(CNS_ERR_INVALID, "grid %dx%dx%d too small for stencil half-width %d", p->mx, p->my, p->mz, S);
    if ((long long)p->mx * p->my * p->mz > (1LL << 34))
        return fail(CNS_ERR_INVALID, "grid too large");
    {
        // the stencil kernels address a padded field with 32-bit element offsets
        const long long G = S, P = ((16 + p->mx + G) + 15) / 16 * 16;
        if (P * (p->my + 2 * G) * (p->mz + 2 * G) >= (1LL << 31))
            return fail(CNS_ERR_INVALID, "grid %dx%dx%d too large: a padded field must hold fewer than 2^31 elements",
                        p->mx, p->my, p->mz);
    }
    if (!(p->Lx > 0) || !(p->Ly > 0) || !(p->Lz > 0)) return fail(CNS_ERR_INVALID, "domain lengths must be > 0");
    if (!(p->Re > 0) || !(p->Pr > 0) || !(p->Ma > 0) || !(p->gam > 1) || !(p->cfl > 0))
        return fail(CNS_ERR_INVALID, "Re, Pr, Ma, cfl must be > 0 and gam > 1");
    if (p->scheme < CNS_RK3_LOWSTORAGE || p->scheme > CNS_RK4_CLASSIC)
        return fail(CNS_ERR_INVALID, "unknown scheme %d", p->scheme);
    if (p->precision != CNS_PREC_FP64 && p->precision != CNS_PREC_FP32_RHS && p->precision != CNS_PREC_PAIR_RHS)
        return fail(CNS_ERR_INVALID, "unknown precision %d", p->precision);
    if (p->check_cfl < 1 || p->check_bulk < 1) return fail(CNS_ERR_INVALID, "check_cfl and check_bulk must be >= 1");
    if (p->boundary_layer && p->periodic_x)
        return fail(CNS_ERR_INVALID, "boundary_layer requires periodic_x = 0");
    if (p->nonuniform_x && p->stretch == 0.0) return fail(CNS_ERR_INVALID, "nonuniform_x needs stretch != 0");
    return CNS_OK;
}

template <typename R>
RhsIn<R> rhs_in(cns_solver* h, int c) {
    RhsIn<R> in{};
    if (h->fp32) {   // packed records (rho, u, v, w) and (T, p, H, mu)
        in.qa = (const float4*)h->der[c][0];
        in.qb = (const float4*)h->der[c][1];
    } else {
        if constexpr (is_ff<R>) {   // rho, u, v, w as pairs, written by the state recovery
            in.r = (const R*)h->der[c][4]; in.u = (const R*)h->der[c][5]; in.v = (const R*)h->der[c][6];
            in.w = (const R*)h->der[c][7];
        } else {
            in.r = (const R*)h->q[c][0]; in.u = (const R*)h->q[c][1]; in.v = (const R*)h->q[c][2];
            in.w = (const R*)h->q[c][3];
        }
        in.h = (const R*)h->der[c][0]; in.t = (const R*)h->der[c][1]; in.p = (const R*)h->der[c][2];
        in.m = (const R*)h->der[c][3];
        for (int q = 0; q < 9; q++) in.g[q] = (const R*)h->grad[q];
    }
    in.dil = (const R*)h->dil;
    return in;
}

StateIn state_in(cns_solver* h, int b) {
    return StateIn{h->q[b][0], h->q[b][1], h->q[b][2], h->q[b][3], h->q[b][4]};
}

// derived-field outputs of state buffer b
template <typename R>
DerivedOut<R> derived_out(cns_solver* h, int b) {
    DerivedOut<R> o{};
    if (h->fp32) {
        o.qa = (float4*)h->der[b][0];
        o.qb = (float4*)h->der[b][1];
    } else {
        o.h = (R*)h->der[b][0]; o.t = (R*)h->der[b][1]; o.p = (R*)h->der[b][2]; o.m = (R*)h->der[b][3];
        if constexpr (is_ff<R>) {
            o.r = (R*)h->der[b][4]; o.u = (R*)h->der[b][5]; o.v = (R*)h->der[b][6]; o.w = (R*)h->der[b][7];
        }
    }
    return o;
}

// calcState of the current state (when the RHS kernel has not recovered it already)
template <typename R>
int state_phase(cns_solver* h) {
    launch_state<R>(h->geom, h->phys, state_in(h, h->cur), derived_out<R>(h, h->cur), h->scal, 0, nullptr, 0,
                    h->stream);
    h->launches += 1;
    CKL();
    h->der_ok[h->cur] = true;
    h->mu_buf = h->cur;
    return CNS_OK;
}

// ghost cells of the stencil inputs of the current state
template <typename R>
int ghost_phase(cns_solver* h) {
    const int c = h->cur;
    const DerivedOut<R> o = derived_out<R>(h, c);
    StencilFields<R> f{};
    if (h->fp32) {
        f.qa = o.qa; f.qb = o.qb;
    } else if constexpr (is_ff<R>) {
        f.r = o.r; f.u = o.u; f.v = o.v; f.w = o.w;
        f.t = o.t; f.p = o.p; f.h = o.h; f.m = o.m;
    } else {
        f.r = (R*)h->q[c][0]; f.u = (R*)h->q[c][1]; f.v = (R*)h->q[c][2]; f.w = (R*)h->q[c][3];
        f.t = o.t; f.p = o.p; f.h = o.h; f.m = o.m;
    }
    launch_ghost_state<R>(h->geom, h->phys, f, h->scal, h->stream);
    h->launches += 1;
    CKL();
    return CNS_OK;
}

template <typename R>
int grad_phase(cns_solver* h) {
    // every dilatation ghost is a copy of one interior value unless the boundary layer
    // extrapolates: then the gradient kernel writes them itself
    const bool own = h->geom.xbc != XBC_BL && !h->geom.zbl;
    if constexpr (std::is_same<R, float>::value) {   // FP32-RHS: theta alone, from the packed records
        launch_dil_packed(h->p.stencil_visc, h->geom, h->cf32, (const float4*)h->der[h->cur][0], (float*)h->dil,
                          own ? 1 : 0, h->stream);
    } else {
        GradOut<R> o;
        for (int q = 0; q < 9; q++) o.g[q] = (R*)h->grad[q];
        o.dil = (R*)h->dil;
        const RhsIn<R> in = rhs_in<R>(h, h->cur);
        if constexpr (is_ff<R>)
            launch_grad<R>(h->p.stencil_visc, h->geom, h->cfp, in.u, in.v, in.w, o, own ? 1 : 0, h->stream);
        else
            launch_grad<R>(h->p.stencil_visc, h->geom, h->cf64, in.u, in.v, in.w, o, own ? 1 : 0, h->stream);
    }
    h->launches += 1;
    if (!own) {
        launch_ghost_scalar<R>(h->geom, (R*)h->dil, h->stream);
        h->launches += 1;
    }
    CKL();
    return CNS_OK;
}

// the stage update from state buffer c into 1 - c; with fuse, the RHS kernel also recovers
// the new state's derived fields (the next stage's calcState)
template <typename R>
Update<R> stage_update(cns_solver* h, int kind, double a, double b, int c, bool fuse) {
    Update<R> up{};
    up.kind = kind;
    up.a = a;
    up.b = b;
    up.ca = R(a);
    up.cb = R(b);
    up.use_prev = a != 0.0;
    up.qin = state_in(h, c);
    const int nb = 1 - c;
    up.qout = StateOut{h->q[nb][0], h->q[nb][1], h->q[nb][2], h->q[nb][3], h->q[nb][4]};
    for (int q = 0; q < 5; q++) {
        up.rb[q] = (R*)h->rb[q];
        up.k2[q] = (R*)h->k2[q];
        up.q0[q] = h->q0[q];
    }
    if (h->has_sponge) {
        up.spx = h->spx; up.spz = h->spz; up.rref = h->rref; up.uref = h->uref; up.vref = h->vref;
        up.wref = h->wref; up.eref = h->eref;
    }
    if (fuse) {
        up.fuse = 1;
        up.dnext = derived_out<R>(h, nb);
        up.ph = h->phys;
    }
    return up;
}

template <typename R>
int rhs_phase(cns_solver* h, int kind, double a, double b) {
    const Update<R> up = stage_update<R>(h, kind, a, b, h->cur, kind != ST_RHS_ONLY);
    const int nb = 1 - h->cur;
    const int quirk = h->p.quirk_dissipation_y != 0;
    int nl;
    if constexpr (std::is_same<R, float>::value)
        nl = launch_rhs_fp32(h->p.stencil_size, h->p.stencil_visc, h->geom, h->phys, h->cf32, rhs_in<float>(h, h->cur),
                             up, h->scal, quirk, h->stream);
    else if constexpr (is_ff<R>)
        nl = launch_rhs_pair(h->p.stencil_size, h->p.stencil_visc, h->geom, h->phys, h->cfp, rhs_in<ff>(h, h->cur),
                             up, h->scal, quirk, h->stream);
    else
        nl = launch_rhs_fp64(h->p.stencil_size, h->p.stencil_visc, h->geom, h->phys, h->cf64,
                             rhs_in<double>(h, h->cur), up, h->scal, quirk, h->stream);
    h->launches += nl;
    CKL();
    if (kind != ST_RHS_ONLY) {
        // in the reference's program order the latest state recovery before the next
        // step's time-step reduction is that of this stage's input state
        h->mu_buf = h->cur;
        h->der_ok[nb] = true;
        h->cur = nb;
    }
    return CNS_OK;
}

int state_any(cns_solver* h) {
    return h->fp32 ? state_phase<float>(h) : h->pair ? state_phase<ff>(h) : state_phase<double>(h);
}
int ghost_any(cns_solver* h) {
    return h->fp32 ? ghost_phase<float>(h) : h->pair ? ghost_phase<ff>(h) : ghost_phase<double>(h);
}
// the derived fields of the current state, recovered unless the last stage did it
int ensure_state(cns_solver* h) { return h->der_ok[h->cur] ? CNS_OK : state_any(h); }
int grad_any(cns_solver* h) {
    return h->fp32 ? grad_phase<float>(h) : h->pair ? grad_phase<ff>(h) : grad_phase<double>(h);
}
int rhs_any(cns_solver* h, int kind, double a, double b) {
    return h->fp32 ? rhs_phase<float>(h, kind, a, b)
                   : h->pair ? rhs_phase<ff>(h, kind, a, b) : rhs_phase<double>(h, kind, a, b);
}

}  // namespace

namespace cns {
template <typename R>
RhsIn<R> solver_rhs_in(cns_solver* h, int b) { return rhs_in<R>(h, b); }
template <typename R>
Update<R> solver_stage_update(cns_solver* h, int kind, double a, double b, int c) {
    return stage_update<R>(h, kind, a, b, c, true);
}
template RhsIn<float> solver_rhs_in<float>(cns_solver*, int);
template RhsIn<double> solver_rhs_in<double>(cns_solver*, int);
template Update<float> solver_stage_update<float>(cns_solver*, int, double, double, int);
template Update<double> solver_stage_update<double>(cns_solver*, int, double, double, int);
int solver_ensure_state(cns_solver* h) { return ensure_state(h); }
}  // namespace cns

int cns::solver_reduce(cns_solver* h, int want, double* diag) {
    if (h->fp32)   // mu is the fourth value of the packed record (T, p, H, mu)
        launch_reduce<float>(h->geom, h->phys, state_in(h, h->cur), (const float*)h->der[h->mu_buf][1] + 3, 4, h->part,
                             want, h->scal, diag, h->stream);
    else if (h->pair)
        launch_reduce<ff>(h->geom, h->phys, state_in(h, h->cur), (const ff*)h->der[h->mu_buf][3], 1, h->part, want,
                          h->scal, diag, h->stream);
    else launch_reduce<double>(h->geom, h->phys, state_in(h, h->cur), (const double*)h->der[h->mu_buf][3], 1, h->part,
                               want, h->scal, diag, h->stream);
    h->launches += 2;
    CKL();
    return CNS_OK;
}

namespace {

const double WRAY_A[3] = {0., -17. / 60., -5. / 12.};   // src/cuda_main.cu:10-11
const double WRAY_B[3] = {8. / 15., 5. / 12., 3. / 4.};

// one full time step (stages of the selected scheme)
int step_stages(cns_solver* h, double* time_log) {
    int rc;
    const int sch = h->p.scheme;
    const int nst = sch == CNS_RK4_CLASSIC ? 4 : 3;
    // the state recovery of each stage's input comes from the previous stage's RHS kernel
    // (ensure_state before the first step)
    for (int s = 0; s < nst; s++) {
        if (s == 0) {
            launch_advance_time(h->scal, time_log, h->diag_cap, h->stream);
            h->launches += 1;
        }
        if ((rc = ghost_any(h))) return rc;
        if ((rc = grad_any(h))) return rc;
        int kind;
        double a = 0, b = 0;
        if (sch == CNS_RK3_LOWSTORAGE) { kind = ST_LS; a = WRAY_A[s]; b = WRAY_B[s]; }
        else if (sch == CNS_RK3_CLASSIC) kind = s == 0 ? ST_C1 : s == 1 ? ST_C2 : ST_C3;
        else kind = ST_R4_1 + s;
        if ((rc = rhs_any(h, kind, a, b))) return rc;
    }
    return CNS_OK;
}

// one time step through the captured graph of the current parity (captured on first use)
int step_graph(cns_solver* h) {
    const int c = h->cur;
    const int nst = h->p.scheme == CNS_RK4_CLASSIC ? 4 : 3;
    if (!h->step_exec[c]) {
        const int64_t l0 = h->launches;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = step_stages(h, h->tlog);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
        h->cur = c;
        h->step_kernels = h->launches - l0;
        h->launches = l0;
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CK(e);
        e = cudaGraphInstantiate(&h->step_exec[c], graph, 0);
        cudaGraphDestroy(graph);
        CK(e);
    }
    CK(cudaGraphLaunch(h->step_exec[c], h->stream));
    h->launches += h->step_kernels;
    h->cur = c ^ (nst & 1);
    return CNS_OK;
}

}  // namespace

int cns::solver_step(cns_solver* h) {
    const int rc = ensure_state(h);
    if (rc) return rc;
    return h->use_graphs ? step_graph(h) : step_stages(h, h->tlog);
}

namespace {

int upload_grid_tables(cns_solver* h) {
    const int mx = h->p.mx, V = h->p.stencil_visc;
    const HostGrid& g = h->hg;
    int rc;
    if ((rc = h->alloc(&h->xp_d, mx)) || (rc = h->alloc(&h->wvol_d, mx)) || (rc = h->alloc(&h->dxv_d, mx)) ||
        (rc = h->alloc(&h->cvsx_d, (size_t)mx * (2 * V + 1))) || (rc = h->alloc(&h->xp_f, mx)) ||
        (rc = h->alloc(&h->cvsx_f, (size_t)mx * (2 * V + 1))) || (rc = h->alloc(&h->xp_p, mx)) ||
        (rc = h->alloc(&h->cvsx_p, (size_t)mx * (2 * V + 1))))
        return rc;
    std::vector<float> xpf(g.xp.begin(), g.xp.end()), cvf(g.cvsx.begin(), g.cvsx.end());
    std::vector<ff> xpp, cvp;
    for (double v : g.xp) xpp.push_back(ff(v));
    for (double v : g.cvsx) cvp.push_back(ff(v));
    CK(cudaMemcpy(h->xp_p, xpp.data(), mx * sizeof(ff), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->cvsx_p, cvp.data(), cvp.size() * sizeof(ff), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->xp_d, g.xp.data(), mx * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->wvol_d, g.wvol.data(), mx * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->dxv_d, g.dxv.data(), mx * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->cvsx_d, g.cvsx.data(), g.cvsx.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->xp_f, xpf.data(), mx * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->cvsx_f, cvf.data(), cvf.size() * sizeof(float), cudaMemcpyHostToDevice));
    return CNS_OK;
}

int sync_and_check(cns_solver* h) {
    CK(cudaStreamSynchronize(h->stream));
    double sc[SC_COUNT];
    CK(cudaMemcpy(sc, h->scal, sizeof sc, cudaMemcpyDeviceToHost));
    if (sc[SC_NONFINITE] != 0.0) return fail(CNS_ERR_NONFINITE, "non-positive or non-finite density/temperature");
    return CNS_OK;
}

}  // namespace

// =========================================================================================
// C ABI
// =========================================================================================
extern "C" {

const char* cns_last_error(void) { return g_err.c_str(); }

const char* cns_version(void) { return "cns-gb300 0.1 (sm_103a)"; }

void cns_default_params(cns_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->mx = p->my = p->mz = 64;
    p->Lx = p->Ly = p->Lz = 2.0 * M_PI;
    p->stencil_size = p->stencil_visc = 4;
    p->Re = 1600.0; p->Pr = 0.71; p->Ma = 0.1; p->gam = 1.4; p->viscexp = 1.0;
    p->cfl = 0.5;
    p->scheme = CNS_RK3_LOWSTORAGE;
    p->periodic_x = 1;
    p->stretch = 5.0;
    p->twall_top = p->twall_bot = 1.0;
    p->check_cfl = 100;
    p->check_bulk = 100;
    p->quirk_dissipation_y = 1;
    p->precision = CNS_PREC_FP64;
    p->ndivz = 1;
    p->dpdz_init = 0.00372;
    p->sp_top_str = 1.0; p->sp_top_len = 1.0; p->sp_top_exp = 2.0;
    p->sp_inl_str = 0.5; p->sp_inl_len = 20.0; p->sp_inl_exp = 2.0;
    p->sp_out_str = 0.5; p->sp_out_len = 20.0; p->sp_out_exp = 2.0;
    p->pert_kc = 110; p->pert_lp = 40;
    p->pert_amp1 = 2e-4; p->pert_amp2 = 3e-5; p->pert_omega1_per_re = 121.e-6; p->pert_omega2 = 10.0;
}

int cns_check_params(const cns_params* p) {
    g_err.clear();
    return check_params(p);
}

int cns_create(const cns_params* pin, int device, cns_solver** out) {
    g_err.clear();
    if (!out) return fail(CNS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int rc = check_params(pin);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CNS_ERR_CUDA, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) return fail(CNS_ERR_INVALID, "device %d out of range (%d devices)", device, ndev);
    CK(cudaSetDevice(device));

    cns_solver* h = new cns_solver();
    h->p = *pin;
    h->device = device;
    h->fp32 = pin->precision == CNS_PREC_FP32_RHS;
    h->pair = pin->precision == CNS_PREC_PAIR_RHS;
    h->rsz = h->fp32 ? 4 : 8;   // FP64 and pairs: 8 bytes
    const cns_params& p = h->p;
    const int S = p.stencil_size, G = S;
    build_grid(p, h->hg);

    // padded layout: 16-element left pad so interior rows start 128 B (FP64) / 64 B (FP32) aligned
    Geom& g = h->geom;
    g.mx = p.mx; g.my = p.my; g.mz = p.mz; g.G = G;
    const long long XL = 16;
    g.P = ((XL + p.mx + G) + 15) / 16 * 16;
    g.PS = g.P * (p.my + 2LL * G);
    g.base = (long long)G * g.PS + (long long)G * g.P + XL;
    h->nalloc = g.PS * (p.mz + 2LL * G);
    g.xbc = p.periodic_x ? XBC_PER : (p.boundary_layer ? XBC_BL : XBC_WALL);
    g.zbl = p.boundary_layer ? 1 : 0;
    g.nonuniform_x = p.nonuniform_x ? 1 : 0;
    g.dx = h->hg.dx; g.dy = h->hg.dy; g.dz = h->hg.dz; g.d2x = h->hg.d2x; g.d2y = h->hg.d2y; g.d2z = h->hg.d2z;

    Phys& ph = h->phys;
    ph.gam = p.gam;
    ph.Ec = ((p.gam - 1.0) * p.Ma) * p.Ma;      // (gam - 1.f)*Ma*Ma   (globals.h:47)
    ph.Rgas = 1.0 / ((p.gam * p.Ma) * p.Ma);    // 1.f/(gam*Ma*Ma)    (globals.h:48)
    ph.Re = p.Re; ph.Pr = p.Pr; ph.vexp = p.viscexp;
    ph.invRe = 1.0 / p.Re;
    ph.clam = 1.0 / p.Re / p.Pr / ph.Ec;
    ph.cvInv = (p.gam - 1.0) / ph.Rgas;
    ph.hcoef = ph.Rgas * p.gam / (p.gam - 1.0);
    ph.twall_top = p.twall_top; ph.twall_bot = p.twall_bot;
    ph.cfl = p.cfl; ph.Lx = p.Lx; ph.Ly = p.Ly; ph.Lz = p.Lz;
    ph.vexp_is_one = p.viscexp == 1.0;
    ph.quirk = p.quirk_dissipation_y;
    ph.perturbed = p.perturbed;
    ph.pert_kc = p.pert_kc; ph.pert_lp = p.pert_lp;
    ph.pert_amp1 = p.pert_amp1; ph.pert_amp2 = p.pert_amp2;
    ph.pert_omega1 = p.Re * p.pert_omega1_per_re; ph.pert_omega2 = p.pert_omega2;
    ph.pert_lambda = p.Ly / (2.0 * M_PI);
    ph.f_Rgas = (float)ph.Rgas; ph.f_cvInv = (float)ph.cvInv; ph.f_invRe = (float)ph.invRe;
    ph.f_vexp = (float)ph.vexp;

    for (int d = 0; d < 3; d++)
        for (int k = 0; k < 5; k++) {
            h->cf64.c1S[d][k] = h->hg.c1S[d][k]; h->cf64.c1V[d][k] = h->hg.c1V[d][k]; h->cf64.c2V[d][k] = h->hg.c2V[d][k];
            h->cf32.c1S[d][k] = (float)h->hg.c1S[d][k]; h->cf32.c1V[d][k] = (float)h->hg.c1V[d][k];
            h->cf32.c2V[d][k] = (float)h->hg.c2V[d][k];
            h->cf64.fq[d][k] = h->hg.fq[d][k]; h->cf64.fc[d][k] = h->hg.fc[d][k];
            h->cf32.fq[d][k] = (float)h->hg.fq[d][k]; h->cf32.fc[d][k] = (float)h->hg.fc[d][k];
        }
    // lambda = mu / (Pr Ec)  (calcState, src/cuda_main.cu:218-242)
    h->cf64.lam_mu = 1.0 / (p.Pr * ph.Ec);
    h->cf32.lam_mu = (float)h->cf64.lam_mu;
    const double inv[3] = {h->hg.dx, h->hg.dy, h->hg.dz}, inv2[3] = {h->hg.d2x, h->hg.d2y, h->hg.d2z};
    for (int d = 0; d < 3; d++) {
        h->cf64.inv[d] = inv[d]; h->cf64.inv2[d] = inv2[d];
        h->cf32.inv[d] = (float)inv[d]; h->cf32.inv2[d] = (float)inv2[d];
    }
    {   // the pair mode's tables: each FP64 coefficient as its nearest pair
        CoefT<ff>& cp = h->cfp;
        const CoefT<double>& cd = h->cf64;
        for (int d = 0; d < 3; d++) {
            for (int k = 0; k < 5; k++) {
                cp.c1S[d][k] = ff(cd.c1S[d][k]); cp.c1V[d][k] = ff(cd.c1V[d][k]); cp.c2V[d][k] = ff(cd.c2V[d][k]);
                cp.fq[d][k] = ff(cd.fq[d][k]); cp.fc[d][k] = ff(cd.fc[d][k]);
            }
            cp.inv[d] = ff(cd.inv[d]); cp.inv2[d] = ff(cd.inv2[d]);
        }
        cp.lam_mu = ff(cd.lam_mu);
    }

    CK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;

    const size_t rs = h->rsz;
    const size_t N = (size_t)p.mx * p.my * p.mz;
    for (int b = 0; b < 2 && !rc; b++)
        rc = h->alloc_fields((void**)h->q[b], 5, 8);   // rho, u, v, w, rhoE of buffer b in one block
    for (int b = 0; b < 2; b++) {
        if (h->fp32)   // packed FP32 records (rho, u, v, w) and (T, p, H, mu)
            for (int f = 0; f < 2 && !rc; f++) rc = h->alloc_field(&h->der[b][f], sizeof(float4));
        else           // h, t, p, mu (pair mode: and rho, u, v, w)
            for (int f = 0; f < (h->pair ? 8 : 4) && !rc; f++) rc = h->alloc_field(&h->der[b][f], rs);
    }
    if (!rc) rc = h->alloc_field(&h->dil, rs);
    if (!h->fp32)   // FP32-RHS: the RHS kernel forms the velocity gradients itself
        for (int f = 0; f < 9 && !rc; f++) rc = h->alloc_field(&h->grad[f], rs);
    if (!rc) rc = h->alloc_fields(h->rb, 5, rs);
    if (!rc && p.scheme != CNS_RK3_LOWSTORAGE) {
        for (int f = 0; f < 5 && !rc; f++) rc = h->alloc_field(&h->k2[f], rs);
        for (int f = 0; f < 5 && !rc; f++) rc = h->alloc_field((void**)&h->q0[f], 8);
    }
    if (!rc) rc = h->alloc(&h->staging, N);
    if (!rc) rc = h->alloc(&h->scal, SC_COUNT);
    if (!rc) rc = h->alloc(&h->part, 6 * RED_BLOCKS);
    if (!rc) rc = upload_grid_tables(h);
    if (rc) { delete h; return rc; }
    h->cf64.xp = h->xp_d; h->cf64.cvsx = h->cvsx_d;
    h->cf32.xp = h->xp_f; h->cf32.cvsx = h->cvsx_f;
    h->cfp.xp = h->xp_p; h->cfp.cvsx = h->cvsx_p;
    g.xp = h->xp_d; g.cvsx = h->cvsx_d; g.wvol = h->wvol_d; g.dxv = h->dxv_d;

    // zero every field once so ghost corners and unused padding hold finite values
    for (int b = 0; b < 2; b++)
        for (int f = 0; f < 5; f++) CK(cudaMemsetAsync(h->q[b][f], 0, (size_t)h->nalloc * 8, h->stream));
    for (int f = 0; f < 5; f++) CK(cudaMemsetAsync(h->rb[f], 0, (size_t)h->nalloc * rs, h->stream));
    double sc[SC_COUNT] = {0};
    sc[SC_DPDZ] = p.forcing ? p.dpdz_init : 0.0;   // cuda_utils.cu:68-70
    CK(cudaMemcpyAsync(h->scal, sc, sizeof sc, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *out = h;
    return CNS_OK;
}

int cns_destroy(cns_solver* h) {
    delete h;
    return CNS_OK;
}

int cns_set_stream(cns_solver* h, void* stream) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return CNS_OK;
}

int cns_get_grid(cns_solver* h, double* x, double* xp, double* xpp, double* y, double* z) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    const HostGrid& g = h->hg;
    if (x) std::memcpy(x, g.x.data(), g.x.size() * 8);
    if (xp) std::memcpy(xp, g.xp.data(), g.xp.size() * 8);
    if (xpp) std::memcpy(xpp, g.xpp.data(), g.xpp.size() * 8);
    if (y) std::memcpy(y, g.y.data(), g.y.size() * 8);
    if (z) std::memcpy(z, g.z.data(), g.z.size() * 8);
    return CNS_OK;
}

int cns_host_grid(const cns_params* p, double* x, double* xp, double* xpp, double* y, double* z) {
    g_err.clear();
    int rc = check_params(p);
    if (rc) return rc;
    HostGrid g;
    build_grid(*p, g);
    if (x) std::memcpy(x, g.x.data(), g.x.size() * 8);
    if (xp) std::memcpy(xp, g.xp.data(), g.xp.size() * 8);
    if (xpp) std::memcpy(xpp, g.xpp.data(), g.xpp.size() * 8);
    if (y) std::memcpy(y, g.y.data(), g.y.size() * 8);
    if (z) std::memcpy(z, g.z.data(), g.z.size() * 8);
    return CNS_OK;
}

int cns_set_sponge(cns_solver* h, const double* sx, const double* sz, const double* rr, const double* ur,
                   const double* wr, const double* er) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    if (!sx || !sz || !rr || !ur || !wr || !er) return fail(CNS_ERR_INVALID, "sponge arrays must not be NULL");
    const int mx = h->p.mx, mz = h->p.mz;
    const size_t n2 = (size_t)mx * mz;
    CK(cudaSetDevice(h->device));
    int rc;
    if (!h->spx) {
        if ((rc = h->alloc(&h->spx, mx)) || (rc = h->alloc(&h->spz, mz)) || (rc = h->alloc(&h->rref, n2)) ||
            (rc = h->alloc(&h->uref, n2)) || (rc = h->alloc(&h->vref, n2)) || (rc = h->alloc(&h->wref, n2)) ||
            (rc = h->alloc(&h->eref, n2)))
            return rc;
    }
    // momentum references rho*u, 0, rho*w (copySpongeToDevice, src/sponge.cu:57-61)
    std::vector<double> um(n2), vm(n2, 0.0), wm(n2);
    for (size_t g = 0; g < n2; g++) { um[g] = ur[g] * rr[g]; wm[g] = wr[g] * rr[g]; }
    CK(cudaMemcpy(h->spx, sx, mx * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->spz, sz, mz * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->rref, rr, n2 * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->uref, um.data(), n2 * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->vref, vm.data(), n2 * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->wref, wm.data(), n2 * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->eref, er, n2 * 8, cudaMemcpyHostToDevice));
    h->has_sponge = h->p.boundary_layer != 0;
    h->drop_graphs();
    return CNS_OK;
}

int cns_set_sponge_profiles(cns_solver* h, int n, const double* xin, const double* rin, const double* uin,
                            const double* win, const double* ein, int init_fields) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    if (n < 3 || !xin || !rin || !uin || !win) return fail(CNS_ERR_INVALID, "profile needs >= 3 points");
    (void)ein;   // the reference re-derives rhoE from rho, u, w and a uniform pressure
    for (int i = 1; i < n; i++)
        if (!(xin[i] > xin[i - 1])) return fail(CNS_ERR_INVALID, "profile x must increase strictly");
    const cns_params& p = h->p;
    const HostGrid& g = h->hg;
    const int mx = p.mx, mz = p.mz;
    std::vector<double> r2(n), u2(n), w2(n);
    spline_second(xin, rin, n, r2.data());
    spline_second(xin, uin, n, u2.data());
    spline_second(xin, win, n, w2.data());
    std::vector<double> spx(mx), spz(mz), rr((size_t)mx * mz), ur((size_t)mx * mz), wr((size_t)mx * mz),
        er((size_t)mx * mz);
    sponge_strengths(p, g, spx.data(), spz.data());
    const double Rgas = h->phys.Rgas;
    for (int k = 0; k < mz; k++)
        for (int i = 0; i < mx; i++) {
            const size_t q = (size_t)i + (size_t)k * mx;
            const double scale = pow(1 + g.z[k] / p.Re, 0.5);   // src/sponge.cu:162
            rr[q] = spline_eval(xin, rin, r2.data(), n, g.x[i] / scale);
            ur[q] = spline_eval(xin, uin, u2.data(), n, g.x[i] / scale) / (scale * p.Re);
            wr[q] = spline_eval(xin, win, w2.data(), n, g.x[i] / scale);
            er[q] = Rgas / (p.gam - 1.0) + rr[q] * 0.5 * (ur[q] * ur[q] + wr[q] * wr[q]);
        }
    int rc = cns_set_sponge(h, spx.data(), spz.data(), rr.data(), ur.data(), wr.data(), er.data());
    if (rc || !init_fields) return rc;
    const size_t N = (size_t)mx * p.my * mz;
    std::vector<double> R(N), U(N), Vv(N, 0.0), W(N), E(N);
    for (int k = 0; k < mz; k++)
        for (int j = 0; j < p.my; j++)
            for (int i = 0; i < mx; i++) {
                const size_t q = (size_t)i + (size_t)k * mx, c = (size_t)i + (size_t)j * mx + (size_t)k * mx * p.my;
                R[c] = rr[q]; U[c] = ur[q]; W[c] = wr[q]; E[c] = er[q];
            }
    return cns_copy_field(h, 0, R.data(), U.data(), Vv.data(), W.data(), E.data());
}

int cns_copy_field(cns_solver* h, int direction, double* r, double* u, double* v, double* w, double* e) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    double* host[5] = {r, u, v, w, e};
    for (int f = 0; f < 5; f++)
        if (!host[f]) return fail(CNS_ERR_INVALID, "field pointer %d is NULL", f);
    CK(cudaSetDevice(h->device));
    const size_t N = (size_t)h->p.mx * h->p.my * h->p.mz;
    if (direction == 0) {
        for (int f = 0; f < 5; f++) {
            CK(cudaMemcpyAsync(h->staging, host[f], N * 8, cudaMemcpyHostToDevice, h->stream));
            launch_unpack<double>(h->geom, h->staging, h->q[h->cur][f], h->stream);
            h->launches++;
        }
        CKL();
        h->der_ok[0] = h->der_ok[1] = false;
        int rc = state_any(h);   // calcState (copyField(0), src/cuda_utils.cu:331-332)
        if (rc) return rc;
        h->initialized = true;
        return sync_and_check(h);
    } else if (direction == 1) {
        if (!h->initialized) return fail(CNS_ERR_STATE, "no field has been copied in");
        for (int f = 0; f < 5; f++) {
            launch_pack<double>(h->geom, h->q[h->cur][f], h->staging, h->stream);
            h->launches++;
            CK(cudaMemcpyAsync(host[f], h->staging, N * 8, cudaMemcpyDeviceToHost, h->stream));
        }
        CKL();
        CK(cudaStreamSynchronize(h->stream));
        return CNS_OK;
    }
    return fail(CNS_ERR_INVALID, "direction must be 0 (host to device) or 1 (device to host)");
}

int cns_run(cns_solver* h, int nsteps, double* par1, double* par2, double* time) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    if (nsteps < 0) return fail(CNS_ERR_INVALID, "nsteps < 0");
    if (!h->initialized) return fail(CNS_ERR_STATE, "cns_copy_field(0) (or sponge init) must precede cns_run");
    if (nsteps == 0) return CNS_OK;
    CK(cudaSetDevice(h->device));
    int rc;
    if (h->diag_cap < nsteps) {
        // grow the per-step log buffers (allocation stays with the handle; captured step
        // graphs refer to the old buffers and are dropped)
        double *d = nullptr, *t = nullptr;
        const int cap = nsteps < 1024 ? 1024 : nsteps;
        if ((rc = h->alloc(&d, 2 * (size_t)cap)) || (rc = h->alloc(&t, (size_t)cap))) return rc;
        h->diag = d; h->tlog = t; h->diag_cap = cap;
        h->drop_graphs();
    }
    CK(cudaMemsetAsync(h->scal + SC_STEP, 0, sizeof(double), h->stream));   // step counter of this run
    if ((rc = ensure_state(h))) return rc;   // outside any captured step graph
    const int forcing = h->p.forcing != 0;
    for (int s = 0; s < nsteps; s++) {
        int want = 0;
        double* dg = nullptr;
        if (s % h->p.check_cfl == 0) want |= RED_DT | (forcing ? RED_FORCE : 0);
        if (s % h->p.check_bulk == 0) {
            want |= forcing ? (RED_FORCE | RED_ENERGY) : RED_KE;
            dg = h->diag;
        }
        if (want && (rc = cns::solver_reduce(h, want, dg))) return rc;
        rc = h->use_graphs ? step_graph(h) : step_stages(h, h->tlog);
        if (rc) return rc;
    }
    rc = sync_and_check(h);
    if (rc) return rc;
    if (par1 || par2) {
        std::vector<double> d(2 * (size_t)nsteps);
        CK(cudaMemcpy(d.data(), h->diag, d.size() * 8, cudaMemcpyDeviceToHost));
        for (int s = 0; s < nsteps; s++) {
            const bool has = s % h->p.check_bulk == 0;
            if (par1) par1[s] = has ? d[2 * s] : NAN;
            if (par2) par2[s] = has ? d[2 * s + 1] : NAN;
        }
    }
    if (time) CK(cudaMemcpy(time, h->tlog, (size_t)nsteps * 8, cudaMemcpyDeviceToHost));
    return CNS_OK;
}

int cns_set_graphs(cns_solver* h, int enable) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    h->use_graphs = enable != 0;
    if (!h->use_graphs) h->drop_graphs();
    return CNS_OK;
}

int cns_calc_rhs(cns_solver* h, double* rr, double* ru, double* rv, double* rw, double* re) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    if (!h->initialized) return fail(CNS_ERR_STATE, "no field has been copied in");
    double* out[5] = {rr, ru, rv, rw, re};
    CK(cudaSetDevice(h->device));
    int rc;
    if ((rc = state_any(h)) || (rc = ghost_any(h)) || (rc = grad_any(h)) || (rc = rhs_any(h, ST_RHS_ONLY, 0, 0)))
        return rc;
    const size_t N = (size_t)h->p.mx * h->p.my * h->p.mz;
    for (int f = 0; f < 5; f++) {
        if (h->fp32) launch_pack<float>(h->geom, (const float*)h->rb[f], h->staging, h->stream);
        else if (h->pair) launch_pack<ff>(h->geom, (const ff*)h->rb[f], h->staging, h->stream);
        else launch_pack<double>(h->geom, (const double*)h->rb[f], h->staging, h->stream);
        h->launches++;
        if (out[f]) CK(cudaMemcpyAsync(out[f], h->staging, N * 8, cudaMemcpyDeviceToHost, h->stream));
    }
    CKL();
    CK(cudaStreamSynchronize(h->stream));
    return CNS_OK;
}

int cns_get_scalars(cns_solver* h, double* dt, double* dpdz, double* time) {
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    CK(cudaSetDevice(h->device));
    double sc[SC_COUNT];
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(sc, h->scal, sizeof sc, cudaMemcpyDeviceToHost));
    if (dt) *dt = sc[SC_DT];
    if (dpdz) *dpdz = sc[SC_DPDZ];
    if (time) *time = sc[SC_TIME];
    return CNS_OK;
}

int cns_set_scalars(cns_solver* h, double dt, double dpdz, double time, int64_t step) {
    (void)step;
    if (!h) return fail(CNS_ERR_INVALID, "handle is NULL");
    CK(cudaSetDevice(h->device));
    double sc[SC_COUNT];
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(sc, h->scal, sizeof sc, cudaMemcpyDeviceToHost));
    sc[SC_DT] = dt; sc[SC_DPDZ] = dpdz; sc[SC_TIME] = time;
    CK(cudaMemcpy(h->scal, sc, sizeof sc, cudaMemcpyHostToDevice));
    return CNS_OK;
}

int cns_time_phases(cns_solver* h, int nstages, double* ms) {
    if (!h || !ms || nstages < 1) return fail(CNS_ERR_INVALID, "bad arguments");
    if (!h->initialized) return fail(CNS_ERR_STATE, "no field has been copied in");
    CK(cudaSetDevice(h->device));
    cudaEvent_t ev[4];
    for (int i = 0; i < 4; i++) CK(cudaEventCreate(&ev[i]));
    double acc[3] = {0, 0, 0};
    int rc = ensure_state(h);
    for (int s = 0; s < nstages && !rc; s++) {
        const int st = s % 3;
        CK(cudaEventRecord(ev[0], h->stream));
        if ((rc = ghost_any(h))) break;
        CK(cudaEventRecord(ev[1], h->stream));
        if ((rc = grad_any(h))) break;
        CK(cudaEventRecord(ev[2], h->stream));
        if ((rc = rhs_any(h, ST_LS, WRAY_A[st], WRAY_B[st]))) break;
        CK(cudaEventRecord(ev[3], h->stream));
        CK(cudaEventSynchronize(ev[3]));
        for (int i = 0; i < 3; i++) {
            float t = 0.f;
            CK(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
            acc[i] += t;
        }
    }
    for (int i = 0; i < 4; i++) cudaEventDestroy(ev[i]);
    if (rc) return rc;
    for (int i = 0; i < 3; i++) ms[i] = acc[i] / nstages;
    return CNS_OK;
}

int64_t cns_kernel_launches(const cns_solver* h) { return h ? h->launches : 0; }

int64_t cns_device_bytes(const cns_solver* h) { return h ? h->bytes : 0; }

}  // extern "C"
