// kernels_point.cuh -- per-point / per-ghost-cell bodies of the stage phases, shared by
// the single-solver kernels (kernels_common.cu) and the batched persistent stage kernel
// (batch.cu).
#pragma once
#include "cns_common.cuh"
#include "cns_internal.h"

namespace cns {

// ---------------------------------------------------------------------------------
// State recovery (calcState, src/cuda_main.cu:218-242): T, p, H, mu from rho, u, v, w,
// rhoE in FP64; stored as R (lambda = mu / (Pr Ec) is applied in the RHS). In FP32-RHS
// mode the packed records qa = (rho, u, v, w) and qb = (T, p, H, mu) are written as FP32
// roundings and mu is evaluated in FP32 from the FP64 T rounded to FP32.
// ---------------------------------------------------------------------------------
// T, p, H, mu (and the FP32 copies) of one point from its FP64 state and 1/rho; the state
// kernel and the fused epilogue of the RHS kernel share it
template <typename R>
__device__ __forceinline__ void state_store(const Phys& ph, const DerivedOut<R>& o, double* scal, long long c,
                                            double rr, double inv, double uu, double vv, double ww, double ee) {
    if constexpr (sizeof(R) == 4) {
        // FP32-RHS: the same recovery with R T shared by p = rho (R T) and H = E/rho + R T
        // (= (rhoE + p)/rho), one FP64 operation fewer on the pipe this mode is short of
        const double er = ee * inv;
        const double T = ph.cvInv * fma(-0.5, uu * uu + vv * vv + ww * ww, er);
        const double RT = ph.Rgas * T;
        const double pr = rr * RT;
        const double hh = er + RT;
        const float Tf = d2f(T);
        const float suth = ph.vexp_is_one ? Tf : powf(Tf, ph.f_vexp);
        const float rf = d2f(rr);
        o.qa[c] = make_float4(rf, d2f(uu), d2f(vv), d2f(ww));
        o.qb[c] = make_float4(Tf, d2f(pr), d2f(hh), suth * ph.f_invRe);
        // the positivity test on the FP32 roundings keeps it off the FP64 pipe
        if (!(Tf > 0.f) || !(rf > 0.f)) scal[SC_NONFINITE] = 1.0;   // racy flag write, any writer is fine
    } else {
        // R T shared by p = rho (R T) and H = E/rho + R T (= (rhoE + p)/rho); the positivity
        // test on the bit patterns (integer units)
        const double er = ee * inv;
        const double T = ph.cvInv * fma(-0.5, uu * uu + vv * vv + ww * ww, er);
        const double RT = ph.Rgas * T;
        const double pr = rr * RT;
        const double hh = er + RT;
        const double suth = ph.vexp_is_one ? T : pow_visc(T, ph.vexp);
        if constexpr (is_ff<R>) {   // the pair mode's stencil inputs include rho, u, v, w
            o.r[c] = d_to_ff(rr);
            o.u[c] = d_to_ff(uu);
            o.v[c] = d_to_ff(vv);
            o.w[c] = d_to_ff(ww);
        }
        o.t[c] = to_r<R>(T);
        o.p[c] = to_r<R>(pr);
        o.h[c] = to_r<R>(hh);
        o.m[c] = to_r<R>(suth * ph.invRe);
        if (!positive_bits(T) || !positive_bits(rr)) scal[SC_NONFINITE] = 1.0;   // racy flag write, any writer is fine
    }
}

template <typename R>
__device__ __forceinline__ void state_point(const Geom& g, const Phys& ph, const StateIn& q, const DerivedOut<R>& o,
                                            double* scal, int i, int j, int k) {
    const long long c = g.at(i, j, k);
    const double rr = q.r[c], uu = q.u[c], vv = q.v[c], ww = q.w[c], ee = q.e[c];
    state_store<R>(ph, o, scal, c, rr, rcp_nr(rr), uu, vv, ww, ee);
}

// Stage 0 of a step advances the simulation time by dt (deviceAdvanceTime) and, with a
// time log of capacity tcap, stores the new time at the device step counter and advances
// the counter (a full log is left as it is).
__device__ __forceinline__ void advance_time(double* scal, double* time_log, long long tcap) {
    const double tn = scal[SC_TIME] + scal[SC_DT];
    scal[SC_TIME] = tn;
    if (time_log) {
        const long long st = (long long)scal[SC_STEP];
        if (st < tcap) {
            time_log[st] = tn;
            scal[SC_STEP] = (double)(st + 1);
        }
    }
}

__host__ __device__ __forceinline__ long long ghost_count(const Geom& g) {
    const long long G = g.G;
    return 2 * G * ((long long)g.my * g.mz + (long long)g.mx * g.mz + (long long)g.mx * g.my);
}

// Ghost cell numbering shared by the state and dilatation fills: x faces first (m, the
// distance from the face, fastest, then side, j, k), then the y faces and the z faces with i
// fastest (then m, side and k or j), so that a warp's loads and stores on the y and z faces
// are row segments. 32-bit arithmetic: the ghost count is below the padded field size,
// itself below 2^31.
struct GhostCell {
    int face;       // 0 x, 1 y, 2 z
    int m;          // 1..G, distance of the ghost from the boundary node
    int side;       // 0 low, 1 high
    int i, j, k;    // the two in-face indices (the face's own index is unused)
};

__device__ __forceinline__ GhostCell ghost_cell_of(const Geom& g, int t) {
    const unsigned G = (unsigned)g.G, mx = (unsigned)g.mx, my = (unsigned)g.my;
    const unsigned nx = 2u * G * my * (unsigned)g.mz, ny = 2u * G * mx * (unsigned)g.mz;
    unsigned u = (unsigned)t;
    GhostCell c;
    c.i = c.j = c.k = 0;
    if (u < nx) {
        c.face = 0;
        c.m = (int)(u % G) + 1; u /= G;
        c.side = (int)(u & 1u); u >>= 1;
        c.j = (int)(u % my);
        c.k = (int)(u / my);
        return c;
    }
    u -= nx;
    const bool yf = u < ny;
    if (!yf) u -= ny;
    c.face = yf ? 1 : 2;
    c.i = (int)(u % mx); u /= mx;
    c.m = (int)(u % G) + 1; u /= G;
    c.side = (int)(u & 1u); u >>= 1;
    if (yf) c.k = (int)u;
    else c.j = (int)u;
    return c;
}

// ---------------------------------------------------------------------------------
// Ghost cell t of the stencil inputs rho, u, v, w, T, p, H, mu.
//   x: periodic | isothermal wall (BCxNumber1/3: p even, u v w odd, T = 2Tw - T,
//      mu, rho, H from the ghost p, T, u, v, w) | boundary layer (bottom: p, T
//      even, u v w odd, u perturbed; top: linear extrapolation; mu, rho, H derived)
//   y: periodic.   z: periodic | linear extrapolation about the end nodes.
// (src/boundary.h:38-188, src/boundary_condition_x.h:47-115, _y.h:19-58, _z.h:80-332)
// Only the six faces are filled (no stencil reads an edge or a corner). All loads of a cell
// are issued before its stores (the eight fields may alias as far as the compiler knows).
// ---------------------------------------------------------------------------------
// FP32-RHS mode: the same images on the packed records qa = (rho, u, v, w), qb = (T, p, H,
// mu), in the same FP32 arithmetic as the FP64-mode cell below with R = float
__device__ __forceinline__ void ghost_state_cell_packed(const Geom& g, const Phys& ph, float4* __restrict__ qa,
                                                        float4* __restrict__ qb, const double* scal, int t) {
    const GhostCell gc = ghost_cell_of(g, t);
    const int m = gc.m, side = gc.side;
    long long cg, cs;
    if (gc.face == 0) {
        const int j = gc.j, k = gc.k;
        cg = g.at(side == 0 ? -m : g.mx - 1 + m, j, k);
        if (g.xbc != XBC_PER) {
            const long long cp = g.at(side == 0 ? m - 1 : g.mx - m, j, k);
            float ug, vg, wg, pg, Tg;
            if (g.xbc == XBC_WALL) {
                const double Tw = side == 0 ? ph.twall_bot : ph.twall_top;
                const float4 a = qa[cp], b = qb[cp];
                ug = -a.y; vg = -a.z; wg = -a.w;
                pg = b.y;
                Tg = (float)(2.0 * Tw) - b.x;
            } else if (side == 0) {   // boundary layer, wall
                const float4 a = qa[cp], b = qb[cp];
                ug = -a.y; vg = -a.z; wg = -a.w;
                pg = b.y;
                Tg = b.x;
                double pv;
                if (ph.perturbed && wall_perturbation(ph, g.dy, j, k, scal[SC_TIME], &pv)) ug = d2f(pv);
            } else {                  // boundary layer, free stream: extrapolate through the last node
                const long long cl = g.at(g.mx - 1, j, k);
                const long long cm = g.at(g.mx - 1 - m, j, k);
                const float4 al = qa[cl], am = qa[cm], bl = qb[cl], bm = qb[cm];
                ug = 2.0f * al.y - am.y;
                vg = 2.0f * al.z - am.z;
                wg = 2.0f * al.w - am.w;
                pg = 2.0f * bl.y - bm.y;
                Tg = 2.0f * bl.x - bm.x;
            }
            const float suth = ph.vexp_is_one ? Tg : powf(Tg, (float)ph.vexp);
            const float hg = Tg * (float)ph.hcoef + 0.5f * (ug * ug + vg * vg + wg * wg);
            qa[cg] = make_float4(pg / ((float)ph.Rgas * Tg), ug, vg, wg);
            qb[cg] = make_float4(Tg, pg, hg, suth * (float)ph.invRe);
            return;
        }
        cs = g.at(side == 0 ? g.mx - m : m - 1, j, k);
    } else if (gc.face == 1) {
        cg = g.at(gc.i, side == 0 ? -m : g.my - 1 + m, gc.k);
        cs = g.at(gc.i, side == 0 ? g.my - m : m - 1, gc.k);
    } else {
        cg = g.at(gc.i, gc.j, side == 0 ? -m : g.mz - 1 + m);
        if (g.zbl) {
            const long long c0 = g.at(gc.i, gc.j, side == 0 ? 0 : g.mz - 1);
            const long long cm = g.at(gc.i, gc.j, side == 0 ? m : g.mz - 1 - m);
            const float4 a0 = qa[c0], am = qa[cm], b0 = qb[c0], bm = qb[cm];
            qa[cg] = make_float4(2.0f * a0.x - am.x, 2.0f * a0.y - am.y, 2.0f * a0.z - am.z, 2.0f * a0.w - am.w);
            qb[cg] = make_float4(2.0f * b0.x - bm.x, 2.0f * b0.y - bm.y, 2.0f * b0.z - bm.z, 2.0f * b0.w - bm.w);
            return;
        }
        cs = g.at(gc.i, gc.j, side == 0 ? g.mz - m : m - 1);
    }
    const float4 a = qa[cs], b = qb[cs];
    qa[cg] = a;
    qb[cg] = b;
}

template <typename R>
__device__ __forceinline__ void ghost_state_cell(const Geom& g, const Phys& ph, const StencilFields<R>& f,
                                                 const double* scal, int t) {
    if constexpr (sizeof(R) == 4) {
        ghost_state_cell_packed(g, ph, f.qa, f.qb, scal, t);
        return;
    }
    R* F[8] = {f.r, f.u, f.v, f.w, f.t, f.p, f.h, f.m};
    const GhostCell gc = ghost_cell_of(g, t);
    const int m = gc.m, side = gc.side;
    long long cg, cs;
    if (gc.face == 0) {
        const int j = gc.j, k = gc.k;
        cg = g.at(side == 0 ? -m : g.mx - 1 + m, j, k);
        if (g.xbc != XBC_PER) {
            // in FP64 (the pair mode converts the interior values and the results)
            const long long cp = g.at(side == 0 ? m - 1 : g.mx - m, j, k);
            const auto rd = [&](const R* a, long long e) { return to_d<R>(a[e]); };
            double ug, vg, wg, pg, Tg;
            if (g.xbc == XBC_WALL) {
                const double Tw = side == 0 ? ph.twall_bot : ph.twall_top;
                ug = -rd(f.u, cp); vg = -rd(f.v, cp); wg = -rd(f.w, cp);
                pg = rd(f.p, cp);
                Tg = 2.0 * Tw - rd(f.t, cp);
            } else if (side == 0) {   // boundary layer, wall
                ug = -rd(f.u, cp); vg = -rd(f.v, cp); wg = -rd(f.w, cp);
                pg = rd(f.p, cp);
                Tg = rd(f.t, cp);
                double pv;
                if (ph.perturbed && wall_perturbation(ph, g.dy, j, k, scal[SC_TIME], &pv)) ug = pv;
            } else {                  // boundary layer, free stream: extrapolate through the last node
                const long long cl = g.at(g.mx - 1, j, k);
                const long long cm = g.at(g.mx - 1 - m, j, k);
                ug = 2.0 * rd(f.u, cl) - rd(f.u, cm);
                vg = 2.0 * rd(f.v, cl) - rd(f.v, cm);
                wg = 2.0 * rd(f.w, cl) - rd(f.w, cm);
                pg = 2.0 * rd(f.p, cl) - rd(f.p, cm);
                Tg = 2.0 * rd(f.t, cl) - rd(f.t, cm);
            }
            const double suth = ph.vexp_is_one ? Tg : cns_pow<double>(Tg, ph.vexp);
            f.u[cg] = to_r<R>(ug); f.v[cg] = to_r<R>(vg); f.w[cg] = to_r<R>(wg); f.p[cg] = to_r<R>(pg);
            f.t[cg] = to_r<R>(Tg);
            f.m[cg] = to_r<R>(suth * ph.invRe);
            f.h[cg] = to_r<R>(Tg * ph.hcoef + 0.5 * (ug * ug + vg * vg + wg * wg));
            f.r[cg] = to_r<R>(pg / (ph.Rgas * Tg));
            return;
        }
        cs = g.at(side == 0 ? g.mx - m : m - 1, j, k);
    } else if (gc.face == 1) {
        cg = g.at(gc.i, side == 0 ? -m : g.my - 1 + m, gc.k);
        cs = g.at(gc.i, side == 0 ? g.my - m : m - 1, gc.k);
    } else {
        cg = g.at(gc.i, gc.j, side == 0 ? -m : g.mz - 1 + m);
        if (g.zbl) {
            const long long c0 = g.at(gc.i, gc.j, side == 0 ? 0 : g.mz - 1);
            const long long cm = g.at(gc.i, gc.j, side == 0 ? m : g.mz - 1 - m);
            R a[8], b[8];
#pragma unroll
            for (int q = 0; q < 8; q++) { a[q] = F[q][c0]; b[q] = F[q][cm]; }
#pragma unroll
            for (int q = 0; q < 8; q++) F[q][cg] = (R)2.0 * a[q] - b[q];
            return;
        }
        cs = g.at(gc.i, gc.j, side == 0 ? g.mz - m : m - 1);
    }
    R v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = F[q][cs];
#pragma unroll
    for (int q = 0; q < 8; q++) F[q][cg] = v[q];
}

// Ghost images of the dilatation at interior point (i, j, k), element c, written by the point
// itself where every dilatation ghost is a copy of one interior value (x periodic or wall:
// even mirror; y, z periodic), which makes the dilatation ghost fill unnecessary
template <typename R>
__device__ __forceinline__ void dil_ghost_owner(const Geom& g, R* __restrict__ f, long long c, int i, int j, int k,
                                                R val) {
    const int G = g.G;
    if (g.xbc == XBC_PER) {
        if (i < G) f[c + g.mx] = val;
        if (i >= g.mx - G) f[c - g.mx] = val;
    } else {   // wall: the ghost at -1 - i (bottom) or 2 mx - 1 - i (top) mirrors i
        if (i < G) f[c - 1 - 2 * i] = val;
        if (i >= g.mx - G) f[c + 2 * (g.mx - i) - 1] = val;
    }
    const long long ly = (long long)g.my * g.P, lz = (long long)g.mz * g.PS;
    if (j < G) f[c + ly] = val;
    if (j >= g.my - G) f[c - ly] = val;
    if (k < G) f[c + lz] = val;
    if (k >= g.mz - G) f[c - lz] = val;
}

// Ghost cell t of the velocity alone (the u, v, w part of ghost_state_cell, for FP64
// velocity fields whose other stencil inputs are not needed: the dissipation diagnostic)
__device__ __forceinline__ void ghost_vel_cell(const Geom& g, const Phys& ph, double* u, double* v, double* w,
                                               const double* scal, int t) {
    double* F[3] = {u, v, w};
    const GhostCell gc = ghost_cell_of(g, t);
    const int m = gc.m, side = gc.side;
    long long cg, cs;
    if (gc.face == 0) {
        const int j = gc.j, k = gc.k;
        cg = g.at(side == 0 ? -m : g.mx - 1 + m, j, k);
        if (g.xbc != XBC_PER) {
            double ug, vg, wg;
            if (g.xbc == XBC_WALL || side == 0) {   // wall or boundary-layer wall: odd
                const long long cp = g.at(side == 0 ? m - 1 : g.mx - m, j, k);
                ug = -u[cp]; vg = -v[cp]; wg = -w[cp];
                double pv;
                if (g.xbc == XBC_BL && ph.perturbed && wall_perturbation(ph, g.dy, j, k, scal[SC_TIME], &pv)) ug = pv;
            } else {                                // boundary-layer free stream: extrapolated
                const long long cl = g.at(g.mx - 1, j, k);
                const long long cm = g.at(g.mx - 1 - m, j, k);
                ug = 2.0 * u[cl] - u[cm];
                vg = 2.0 * v[cl] - v[cm];
                wg = 2.0 * w[cl] - w[cm];
            }
            u[cg] = ug; v[cg] = vg; w[cg] = wg;
            return;
        }
        cs = g.at(side == 0 ? g.mx - m : m - 1, j, k);
    } else if (gc.face == 1) {
        cg = g.at(gc.i, side == 0 ? -m : g.my - 1 + m, gc.k);
        cs = g.at(gc.i, side == 0 ? g.my - m : m - 1, gc.k);
    } else {
        cg = g.at(gc.i, gc.j, side == 0 ? -m : g.mz - 1 + m);
        if (g.zbl) {
            const long long c0 = g.at(gc.i, gc.j, side == 0 ? 0 : g.mz - 1);
            const long long cm = g.at(gc.i, gc.j, side == 0 ? m : g.mz - 1 - m);
            double a[3], b[3];
#pragma unroll
            for (int q = 0; q < 3; q++) { a[q] = F[q][c0]; b[q] = F[q][cm]; }
#pragma unroll
            for (int q = 0; q < 3; q++) F[q][cg] = 2.0 * a[q] - b[q];
            return;
        }
        cs = g.at(gc.i, gc.j, side == 0 ? g.mz - m : m - 1);
    }
    double val[3];
#pragma unroll
    for (int q = 0; q < 3; q++) val[q] = F[q][cs];
#pragma unroll
    for (int q = 0; q < 3; q++) F[q][cg] = val[q];
}

// ---------------------------------------------------------------------------------
// Velocity gradients gij[0..8] = d(u,v,w)/d(x,y,z) at the viscous order and the
// dilatation (derVelX/Y/Z + calcDil, src/calc_stress.cu:20-63,87-96).
// ---------------------------------------------------------------------------------
// DIL_ONLY: only the three diagonal gradients and theta (the FP32-RHS kernel forms the nine
// gradients itself from the velocity stencils it loads, and needs theta at its neighbours).
// own: also write the dilatation's ghost images (dil_ghost_owner; periodic and wall x,
// periodic z only).
template <typename R, int V, bool DIL_ONLY = false>
__device__ __forceinline__ void grad_point(const Geom& g, const CoefT<R>& cf, const R* __restrict__ u,
                                           const R* __restrict__ v, const R* __restrict__ w, const GradOut<R>& o,
                                           int i, int j, int k, bool own = false) {
    const long long c = g.at(i, j, k);
    const long long st[3] = {1, g.P, g.PS};
    const R* F[3] = {u, v, w};
    R out[9];
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
            if (DIL_ONLY && q != d) continue;
            const R* f = F[q];
            R s = cf.c1V[d][1] * (__ldg(f + c + st[d]) - __ldg(f + c - st[d]));
#pragma unroll
            for (int kk = 2; kk <= V; kk++)
                s = fma(cf.c1V[d][kk], __ldg(f + c + kk * st[d]) - __ldg(f + c - kk * st[d]), s);
            if (d == 0 && g.nonuniform_x) s *= cf.xp[i];
            out[3 * d + q] = s;
        }
    }
    if constexpr (!DIL_ONLY) {
#pragma unroll
        for (int q = 0; q < 9; q++) o.g[q][c] = out[q];
    }
    const R th = out[0] + out[4] + out[8];
    o.dil[c] = th;
    if (own) dil_ghost_owner<R>(g, o.dil, c, i, j, k, th);
}

// FP32-RHS dilatation from the packed records qa = (rho, u, v, w): the diagonal gradients
// du/dx, dv/dy, dw/dz at the viscous order (grad_point's DIL_ONLY arithmetic) and theta.
template <int V>
__device__ __forceinline__ void dil_point_packed(const Geom& g, const CoefT<float>& cf,
                                                 const float4* __restrict__ qa, float* __restrict__ dil, int i, int j,
                                                 int k, bool own = false) {
    const int c = (int)g.at(i, j, k);
    const int P = (int)g.P, PS = (int)g.PS;
    float sx = cf.c1V[0][1] * (__ldg(qa + c + 1).y - __ldg(qa + c - 1).y);
    float sy = cf.c1V[1][1] * (__ldg(qa + c + P).z - __ldg(qa + c - P).z);
    float sz = cf.c1V[2][1] * (__ldg(qa + c + PS).w - __ldg(qa + c - PS).w);
#pragma unroll
    for (int kk = 2; kk <= V; kk++) {
        sx = fma(cf.c1V[0][kk], __ldg(qa + c + kk).y - __ldg(qa + c - kk).y, sx);
        sy = fma(cf.c1V[1][kk], __ldg(qa + c + kk * P).z - __ldg(qa + c - kk * P).z, sy);
        sz = fma(cf.c1V[2][kk], __ldg(qa + c + kk * PS).w - __ldg(qa + c - kk * PS).w, sz);
    }
    if (g.nonuniform_x) sx *= cf.xp[i];
    const float th = sx + sy + sz;
    dil[c] = th;
    if (own) dil_ghost_owner<float>(g, dil, c, i, j, k, th);
}

// FP32-RHS dilatation of a column of points from the packed records (rho, u, v, w): the
// threads (tx, ty), tx < 32, ty < TY, own the x-y tile [i0, i0 + 32) x [j0, j0 + TY) and march
// the planes [k0, k1). Per plane every thread loads its own record once (u into the x-halo
// row tile su, v into the y-halo column tile sv in shared memory) and the record V planes
// ahead, whose w enters a register ring holding w at k - V .. k + V; threads at the tile
// edges also load the x and y halos; the next plane's loads are issued before the current
// plane is computed. About 2 + 2V/TY + 2V/32 record loads per point instead of the 6V of a
// point-per-thread stencil (each record is 16 bytes of which one value is used); the
// arithmetic per point is grad_point's (DIL_ONLY): the same sums in the same order. Tile
// slots outside [-V, mx + V) x [-V, my + V) are never read by an interior point and are not
// loaded; every loaded slot lies in the ghosted allocation (G = S >= V). All threads of the
// block call it (it synchronises the block).
template <int V, int TY>
__device__ __forceinline__ void dil_column_packed(const Geom& g, const CoefT<float>& cf, const float4* __restrict__ qa,
                                                  float* __restrict__ dil, int i0, int j0, int k0, int k1, bool own,
                                                  int tx, int ty, float (*su)[32 + 2 * V], float (*sv)[32]) {
    static_assert(V <= TY, "the y halo rows are loaded by the first and last V tile rows");
    const int i = i0 + tx, j = j0 + ty;
    const bool inside = i < g.mx && j < g.my;
    const bool ghosted = i < g.mx + V && j < g.my + V;   // own slot of the tiles is read by someone
    const int P = (int)g.P, PS = (int)g.PS;
    const int c0 = (int)g.at(i, j, 0);   // element of (i, j, 0); plane k adds k * PS
    float xp = 1.0f;
    if (g.nonuniform_x && inside) xp = cf.xp[i];
    // w at planes k - V .. k + V (ring[V] = the current plane)
    float ring[2 * V + 1];
#pragma unroll
    for (int l = 0; l < 2 * V; l++) ring[l] = inside ? __ldg(qa + c0 + (k0 - V + l) * PS).w : 0.0f;
    // the loads of plane k: w at k + V, the own record's u and v, the x and y halos
    float nw = 0.f, nu = 0.f, nv = 0.f, hxl = 0.f, hxr = 0.f, hyl = 0.f, hyr = 0.f;
    const auto fetch = [&](int k) {
        const int ck = c0 + k * PS;
        nw = inside ? __ldg(qa + ck + V * PS).w : 0.0f;
        if (ghosted) {
            const float4 rec = __ldg(qa + ck);
            nu = rec.y;
            nv = rec.z;
        }
        if (tx < V && j < g.my) hxl = __ldg(qa + ck - V).y;                           // x = i - V >= -V
        if (tx >= 32 - V && i < g.mx && j < g.my) hxr = __ldg(qa + ck + V).y;          // x = i + V < mx + V
        if (ty < V && i < g.mx) hyl = __ldg(qa + ck - V * P).z;                       // y = j - V >= -V
        if (ty >= TY - V && j < g.my && i < g.mx) hyr = __ldg(qa + ck + V * P).z;      // y = j + V < my + V
    };
    if (k0 < k1) fetch(k0);
    for (int k = k0; k < k1; k++) {
        const float cw = nw, cu = nu, cv = nv, cxl = hxl, cxr = hxr, cyl = hyl, cyr = hyr;
        if (k + 1 < k1) fetch(k + 1);
        ring[2 * V] = cw;
        const int ck = c0 + k * PS;
        __syncthreads();   // the previous plane's tiles are no longer read
        su[ty][tx + V] = cu;
        sv[ty + V][tx] = cv;
        if (tx < V) su[ty][tx] = cxl;
        if (tx >= 32 - V) su[ty][tx + 2 * V] = cxr;
        if (ty < V) sv[ty][tx] = cyl;
        if (ty >= TY - V) sv[ty + 2 * V][tx] = cyr;
        __syncthreads();
        if (inside) {
            float sx = cf.c1V[0][1] * (su[ty][tx + V + 1] - su[ty][tx + V - 1]);
            float sy = cf.c1V[1][1] * (sv[ty + V + 1][tx] - sv[ty + V - 1][tx]);
            float sz = cf.c1V[2][1] * (ring[V + 1] - ring[V - 1]);
#pragma unroll
            for (int kk = 2; kk <= V; kk++) {
                sx = fma(cf.c1V[0][kk], su[ty][tx + V + kk] - su[ty][tx + V - kk], sx);
                sy = fma(cf.c1V[1][kk], sv[ty + V + kk][tx] - sv[ty + V - kk][tx], sy);
                sz = fma(cf.c1V[2][kk], ring[V + kk] - ring[V - kk], sz);
            }
            if (g.nonuniform_x) sx *= xp;
            const float th = sx + sy + sz;
            dil[ck] = th;
            if (own) dil_ghost_owner<float>(g, dil, ck, i, j, k, th);
        }
#pragma unroll
        for (int l = 0; l < 2 * V; l++) ring[l] = ring[l + 1];
    }
}

// Dilatation ghost cell t (BCxNumber2 / BCyNumber1 / BCzNumber1): x periodic | wall:
// even | boundary layer: bottom even, top extrapolated; y periodic; z periodic | extrapolated.
template <typename R>
__device__ __forceinline__ void ghost_scalar_cell(const Geom& g, R* f, int t) {
    const GhostCell gc = ghost_cell_of(g, t);
    const int m = gc.m, side = gc.side;
    if (gc.face == 0) {
        const int j = gc.j, k = gc.k;
        const long long cg = g.at(side == 0 ? -m : g.mx - 1 + m, j, k);
        if (g.xbc == XBC_PER) f[cg] = f[g.at(side == 0 ? g.mx - m : m - 1, j, k)];
        else if (g.xbc == XBC_WALL || side == 0) f[cg] = f[g.at(side == 0 ? m - 1 : g.mx - m, j, k)];
        else f[cg] = (R)2.0 * f[g.at(g.mx - 1, j, k)] - f[g.at(g.mx - 1 - m, j, k)];
    } else if (gc.face == 1) {
        f[g.at(gc.i, side == 0 ? -m : g.my - 1 + m, gc.k)] = f[g.at(gc.i, side == 0 ? g.my - m : m - 1, gc.k)];
    } else {
        const int i = gc.i, j = gc.j;
        const long long cg = g.at(i, j, side == 0 ? -m : g.mz - 1 + m);
        if (!g.zbl) f[cg] = f[g.at(i, j, side == 0 ? g.mz - m : m - 1)];
        else f[cg] = (R)2.0 * f[g.at(i, j, side == 0 ? 0 : g.mz - 1)] - f[g.at(i, j, side == 0 ? m : g.mz - 1 - m)];
    }
}

}  // namespace cns
