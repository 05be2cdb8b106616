// kernels_rhs.cuh -- the RHS + Runge-Kutta stage kernel (one thread per grid point).
//
// Per point it forms the x, y and z contributions of deviceRHSX/Y/Z
// (src/cuda_rhs.cu:9-396), the body force, the sponge (src/sponge.cu:31-41) and then
// the stage update of the selected time scheme (sumLowStorageRK3 + deviceMul/deviceDiv,
// src/cuda_main.cu:109-186,244-247; eulerSum*/rk3final*, src/cuda_main.cu:188-216),
// writing the new state to the other state buffer. All neighbour reads hit the ghosted
// layout, so there is no boundary branching.
//
// The split-form convective derivative is evaluated in its telescoped form. The
// reference accumulates the two interface fluxes F_{i+1/2}, F_{i-1/2} over every
// (l, m) pair of the Kennedy-Gruber sum (src/cuda_derivs.h:30-155) and differences
// them; all pairs except (i-l, i) and (i, i+l) cancel exactly, so
//   d(f g h)/dx |_i = c/dx * sum_l a_l [ P(i-l, i) - P(i, i+l) ],
//   P(a, b) = (f_a + f_b)(g_a + g_b)(h_a + h_b),  a_l = -coeffF[S-l],  c = 1/2 (two
//   factors) or 1/4 (three factors),
// which is the same value with 2 instead of l(l+1) pair products per l. The product
// (rho_a+rho_b)(g_a+g_b) is shared by the mass flux and the four cubic fluxes.
#pragma once
#include "cns_common.cuh"
#include "cns_internal.h"
#include "kernels_point.cuh"

namespace cns {

template <typename R>
__device__ __forceinline__ R ld(const R* __restrict__ p, int o) { return __ldg(p + o); }

// Neighbours of the centre point along one direction, in global memory at a stride.
//
// Element offsets are 32-bit: every padded field holds fewer than 2^31 elements (checked
// when a solver is created), and 64-bit offset arithmetic costs two integer instructions
// per neighbour address.
template <typename R>
struct NbGlobal {
    const RhsIn<R>* in;
    int c, st;
    __device__ __forceinline__ R u(int l) const { return ld(in->u, c + l * st); }
    __device__ __forceinline__ R v(int l) const { return ld(in->v, c + l * st); }
    __device__ __forceinline__ R w(int l) const { return ld(in->w, c + l * st); }
    __device__ __forceinline__ R r(int l) const { return ld(in->r, c + l * st); }
    __device__ __forceinline__ R h(int l) const { return ld(in->h, c + l * st); }
    __device__ __forceinline__ R p(int l) const { return ld(in->p, c + l * st); }
    __device__ __forceinline__ R t(int l) const { return ld(in->t, c + l * st); }
    __device__ __forceinline__ R m(int l) const { return ld(in->m, c + l * st); }
    __device__ __forceinline__ R dil(int l) const { return ld(in->dil, c + l * st); }
};

// first derivative sum_k co[k] (f_k - f_-k) and second derivative co[0] f_0 +
// sum_k co[k] (f_k + f_-k) of the values get(l), l = -K..K
template <typename R, int K, class Get>
__device__ __forceinline__ R d1(const Get& get, const R* co) {
    R s = co[1] * (get(1) - get(-1));
#pragma unroll
    for (int k = 2; k <= K; k++) s = fma(co[k], get(k) - get(-k), s);
    return s;
}

template <typename R, int K, class Get>
__device__ __forceinline__ R d2u(const Get& get, const R* co) {
    R s = co[0] * get(0);
#pragma unroll
    for (int k = 1; k <= K; k++) s = fma(co[k], get(k) + get(-k), s);
    return s;
}

// non-uniform x second derivative with the per-point table (derDevSharedV2x, nonUniformX)
template <typename R, int V, class Get>
__device__ __forceinline__ R d2x_nu(const Get& get, const R* __restrict__ cvsx, int mx, int i) {
    R s = (R)0;
#pragma unroll
    for (int it = 0; it < 2 * V + 1; it++) s = fma(__ldg(cvsx + it * mx + i), get(it - V), s);
    return s;
}

// f(a[k]) for k = 0, 1, 2 of a register array, with k a literal after inlining or uniform
// at run time: branches, no indexed (local-memory) access
template <typename T, int N, class F>
__device__ __forceinline__ void at3(T (&a)[N], int k, F f) {
    if (k == 0) f(a[0]); else if (k == 1) f(a[1]); else f(a[2]);
}

// FP64 body: contribution of direction DIR (deviceRHSX/Y/Z) on the separate stencil fields.
// Terms that every direction multiplies by the same centre value are summed over the
// directions first and multiplied once per point (rhs_point_nb): the second derivatives of
// u, v, w, T in L[] (times mu), the viscous momentum terms grad mu . s + mu/3 grad theta in
// W[] (the energy equation's work u_i W_i), the conduction in cond (times lambda/mu), and
// the mass flux, whose half carries the centre value of the four cubic fluxes. The stress
// row tau_{DIR,c}/mu comes from rhs_point_nb, which forms the symmetric tensor once. The
// direction is an argument: called with a literal it folds like a template parameter; the
// pair type calls it in a loop that is not unrolled (rhs_point_nb).
// (The FP32-RHS mode has its own body on the packed records, rhs_dir_packed below.)
template <typename R, int S, int V, bool MAYBE_X, class NB>
__device__ __forceinline__ void rhs_direction(const Geom& g, const CoefT<R>& cf, const NB& nb, int i, const int DIR,
                                              const R (&tau)[3], R m3, R u0, R v0, R w0, R r0, R (&acc)[5],
                                              R (&W)[3], R (&L)[4], R& cond) {
    const bool nux = MAYBE_X && DIR == 0 && g.nonuniform_x;   // MAYBE_X false: y or z (folds)
    const R xpi = nux ? cf.xp[i] : (R)1;
    const R* c1V = cf.c1V[DIR];
    const R* c1S = cf.c1S[DIR];
    const R* c2V = cf.c2V[DIR];

    // velocity stencils, loaded once for the viscous second derivatives and the fluxes
    R us[2 * S + 1], vs[2 * S + 1], ws[2 * S + 1];
    us[S] = u0; vs[S] = v0; ws[S] = w0;
#pragma unroll
    for (int l = 1; l <= S; l++) {
        us[S + l] = nb.u(l); us[S - l] = nb.u(-l);
        vs[S + l] = nb.v(l); vs[S - l] = nb.v(-l);
        ws[S + l] = nb.w(l); ws[S - l] = nb.w(-l);
    }
    // d mu/dx s_{DIR,c}; the second derivatives d2 u_c/dx2 continue the sums L[]
    const auto gm = [&](int l) { return nb.m(l); };
    const auto gt = [&](int l) { return nb.t(l); };
    const auto gd = [&](int l) { return nb.dil(l); };
    const auto gp = [&](int l) { return nb.p(l); };
    const R dmu = d1<R, V>(gm, c1V) * xpi;
    if (nux) {
#pragma unroll
        for (int it = 0; it < 2 * V + 1; it++) {
            const R cw = __ldg(cf.cvsx + it * g.mx + i);
            L[0] = fma(cw, us[S + it - V], L[0]);
            L[1] = fma(cw, vs[S + it - V], L[1]);
            L[2] = fma(cw, ws[S + it - V], L[2]);
            L[3] = fma(cw, nb.t(it - V), L[3]);
        }
    } else {
        L[0] = fma(c2V[0], us[S], L[0]);
        L[1] = fma(c2V[0], vs[S], L[1]);
        L[2] = fma(c2V[0], ws[S], L[2]);
        L[3] = fma(c2V[0], nb.t(0), L[3]);
#pragma unroll
        for (int k = 1; k <= V; k++) {
            L[0] = fma(c2V[k], us[S + k] + us[S - k], L[0]);
            L[1] = fma(c2V[k], vs[S + k] + vs[S - k], L[1]);
            L[2] = fma(c2V[k], ws[S + k] + ws[S - k], L[2]);
            L[3] = fma(c2V[k], nb.t(k) + nb.t(-k), L[3]);
        }
    }
    W[0] = fma(tau[0], dmu, W[0]);
    W[1] = fma(tau[1], dmu, W[1]);
    W[2] = fma(tau[2], dmu, W[2]);
    // heat conduction lambda d2T + dlambda dT = (lambda/mu) (mu d2T + dmu dT); mu d2T and
    // the ratio are applied once per point
    const R dt = d1<R, V>(gt, c1V) * xpi;
    cond = fma(dt, dmu, cond);
    // mu/3 d(theta) on the DIR momentum (and its work), pressure gradient
    const R dth = d1<R, V>(gd, c1V) * xpi;
    const R dp = d1<R, S>(gp, c1S) * xpi;
    at3(W, MAYBE_X ? DIR : (DIR == 1 ? 1 : 2), [&](R& w) { w = fma(m3, dth, w); });

    // split-form convective derivatives, telescoped (see file comment); with a uniform
    // spacing the flux weights already carry 1/2 or 1/4 and 1/dx, so they accumulate
    // straight into the RHS. With Q-(l) = (rho_{-l}+rho_0)(g_{-l}+g_0) and
    // Q+(l) = (rho_0+rho_l)(g_0+g_l), the cubic flux of phi is
    //   sum_l a_l [Q-(phi_{-l}+phi_0) - Q+(phi_0+phi_l)]
    //     = sum_l [(a_l Q-) phi_{-l} - (a_l Q+) phi_l]  +  phi_0 sum_l a_l (Q- - Q+),
    // and the last sum is half the mass flux, so the products a_l Q+- are shared by the four
    // cubic fluxes. The phi_0 terms of all directions are added from the summed mass flux
    // once per point.
    // The mass flux weights are twice the cubic ones (fq = 0.5 c1S, fc = 0.25 c1S: exactly
    // 2 fc), so the mass flux is 2 sum_l (a_l Q- - a_l Q+); a_l Q+- = (a_l rho_0 + a_l rho_+-)
    // (g_+- + g_0) with a_l rho_0 shared by the two: 17 operations per l.
    const R un = (MAYBE_X && DIR == 0) ? u0 : (DIR == 1 ? v0 : w0);
    R sd = (R)0, fu = nux ? (R)0 : acc[1], fv = nux ? (R)0 : acc[2], fw = nux ? (R)0 : acc[3],
      fe = nux ? (R)0 : acc[4];
    const R* fcb = cf.fc[DIR];
#pragma unroll
    for (int l = 1; l <= S; l++) {
        const R rm = nb.r(-l), rp = nb.r(l);
        const R um = us[S - l], up = us[S + l];
        const R vm = vs[S - l], vp = vs[S + l];
        const R wm = ws[S - l], wp = ws[S + l];
        const R hm = nb.h(-l), hp = nb.h(l);
        const R gm = (MAYBE_X && DIR == 0) ? um : (DIR == 1 ? vm : wm);
        const R gp = (MAYBE_X && DIR == 0) ? up : (DIR == 1 ? vp : wp);
        const R ar0 = fcb[l] * r0;
        const R am = fma(fcb[l], rm, ar0) * (gm + un);
        const R ap = fma(fcb[l], rp, ar0) * (un + gp);
        sd += am - ap;
        fu = fma(am, um, fma(-ap, up, fu));
        fv = fma(am, vm, fma(-ap, vp, fv));
        fw = fma(am, wm, fma(-ap, wp, fw));
        fe = fma(am, hm, fma(-ap, hp, fe));
    }
    const R fr = nux ? sd + sd : fma((R)2, sd, acc[0]);
    if (nux) {
        acc[0] = fma(xpi, fr, acc[0]);
        acc[1] = fma(xpi, fu, acc[1]);
        acc[2] = fma(xpi, fv, acc[2]);
        acc[3] = fma(xpi, fw, acc[3]);
        acc[4] = fma(xpi, fe, acc[4]);
    } else {
        acc[0] = fr; acc[1] = fu; acc[2] = fv; acc[3] = fw; acc[4] = fe;
    }
    if (MAYBE_X && DIR == 0) acc[1] -= dp; else if (DIR == 1) acc[2] -= dp; else acc[3] -= dp;
}

// Pair-type body of one direction: the sums of rhs_direction in one pass over the offsets
// l = 1..S that is not unrolled (the pair arithmetic is ~15 instructions per operation, and
// the unrolled body does not fit the instruction caches). At each l it loads the neighbours
// on either side and feeds every sum that needs them; each sum keeps rhs_direction's terms
// and order (centre term, then l ascending; the stretched-x second derivative adds the pair
// (-l, l) per l) in an accumulator whose tail is normalised once at the end, two sums at a
// time through the packed FP32x2 forms (ffacc2, ff.cuh).
template <int S, int V, bool MAYBE_X>
__device__ __forceinline__ void rhs_dir_pair(const Geom& g, const CoefT<ff>& cf, const NbGlobal<ff>& nb, int i,
                                             const int DIR, const ff (&tau)[3], ff m3, ff u0, ff v0, ff w0, ff r0,
                                             ff (&acc)[5], ff (&W)[3], ff (&L)[4], ff& cond) {
    const bool nux = MAYBE_X && DIR == 0 && g.nonuniform_x;
    const ff t0 = nb.t(0);
    {   // centre terms of the second derivatives
        const ff cw = nux ? __ldg(cf.cvsx + V * g.mx + i) : cf.c2V[DIR][0];
        const ff2 cw2 = mk2(cw, cw);
        const ff2 luv = fma(cw2, mk2(u0, v0), mk2(L[0], L[1])), lwt = fma(cw2, mk2(w0, t0), mk2(L[2], L[3]));
        L[0] = lane0(luv); L[1] = lane1(luv); L[2] = lane0(lwt); L[3] = lane1(lwt);
    }
    const ff un = (MAYBE_X && DIR == 0) ? u0 : (DIR == 1 ? v0 : w0);
    const ff zero(0);
    const ff2 zero2 = mk2(zero, zero), un2 = mk2(un, un);
    // lanes: (p, theta), (mu, T), (L_u, L_v), (L_w, L_T), (F_u, F_v), (F_w, F_e), and the mass
    // flux as (sum a_l Q-, -sum a_l Q+)
    ffacc2 Dpth(zero2), Dmt(zero2), Luv(mk2(L[0], L[1])), Lwt(mk2(L[2], L[3])), Sd(zero2);
    ffacc2 Fuv(nux ? zero2 : mk2(acc[1], acc[2])), Fwe(nux ? zero2 : mk2(acc[3], acc[4]));
#pragma unroll 1
    for (int l = 1; l <= S; l++) {
        const ff um = nb.u(-l), up = nb.u(l), vm = nb.v(-l), vp = nb.v(l), wm = nb.w(-l), wp = nb.w(l);
        // theta's weight is zero beyond the viscous half-width (its ghosts hold finite values)
        Dpth.add_prod(mk2(cf.c1S[DIR][l], l <= V ? cf.c1V[DIR][l] : zero),
                      mk2(nb.p(l), nb.dil(l)) - mk2(nb.p(-l), nb.dil(-l)));
        if (l <= V) {
            const ff c1 = cf.c1V[DIR][l];
            const ff tm = nb.t(-l), tp = nb.t(l);
            Dmt.add_prod(mk2(c1, c1), mk2(nb.m(l), tp) - mk2(nb.m(-l), tm));
            if (nux) {
                const ff cm = __ldg(cf.cvsx + (V - l) * g.mx + i), cp = __ldg(cf.cvsx + (V + l) * g.mx + i);
                const ff2 cm2 = mk2(cm, cm), cp2 = mk2(cp, cp);
                Luv.add_prod(cm2, mk2(um, vm)); Luv.add_prod(cp2, mk2(up, vp));
                Lwt.add_prod(cm2, mk2(wm, tm)); Lwt.add_prod(cp2, mk2(wp, tp));
            } else {
                const ff c2 = cf.c2V[DIR][l];
                const ff2 c22 = mk2(c2, c2);
                Luv.add_prod(c22, mk2(up, vp) + mk2(um, vm));
                Lwt.add_prod(c22, mk2(wp, tp) + mk2(wm, tm));
            }
        }
        // telescoped split-form fluxes (rhs_direction): lanes (a_l Q-, a_l Q+)
        const ff gm = (MAYBE_X && DIR == 0) ? um : (DIR == 1 ? vm : wm);
        const ff gp = (MAYBE_X && DIR == 0) ? up : (DIR == 1 ? vp : wp);
        const ff fc = cf.fc[DIR][l];
        const ff ar0 = fc * r0;
        const ff2 q = fma(mk2(fc, fc), mk2(nb.r(-l), nb.r(l)), mk2(ar0, ar0)) * (mk2(gm, gp) + un2);
        const float2 sgn = make_float2(1.0f, -1.0f);   // (a_l Q-, -a_l Q+), exact
        const ff2 qs = ff2{__fmul2_rn(q.h, sgn), __fmul2_rn(q.l, sgn)};
        Sd.add(qs);
        const ff2 am2 = mk2(lane0(qs), lane0(qs)), ap2 = mk2(lane1(qs), lane1(qs));
        Fuv.add_prod(am2, mk2(um, vm)); Fuv.add_prod(ap2, mk2(up, vp));
        Fwe.add_prod(am2, mk2(wm, nb.h(-l))); Fwe.add_prod(ap2, mk2(wp, nb.h(l)));
    }
    const ff2 luv = Luv.value(), lwt = Lwt.value(), pth = Dpth.value(), mt = Dmt.value();
    const ff2 s2 = Sd.value(), fuv = Fuv.value(), fwe = Fwe.value();
    L[0] = lane0(luv); L[1] = lane1(luv); L[2] = lane0(lwt); L[3] = lane1(lwt);
    ff dmu = lane0(mt), dt = lane1(mt), dth = lane1(pth), dp = lane0(pth);
    const ff sd = lane0(s2) + lane1(s2);
    if (nux) {
        const ff xpi = cf.xp[i];
        const ff2 x2 = mk2(xpi, xpi), a = mt * x2, b = pth * x2;
        dmu = lane0(a); dt = lane1(a); dp = lane0(b); dth = lane1(b);
    }
    {   // W_q += tau_q dmu, cond += dT dmu (two packed multiply-adds)
        const ff2 d2 = mk2(dmu, dmu);
        const ff2 w01 = fma(mk2(tau[0], tau[1]), d2, mk2(W[0], W[1])), w2c = fma(mk2(tau[2], dt), d2, mk2(W[2], cond));
        W[0] = lane0(w01); W[1] = lane1(w01); W[2] = lane0(w2c); cond = lane1(w2c);
    }
    at3(W, MAYBE_X ? DIR : (DIR == 1 ? 1 : 2), [&](ff& w) { w = fma(m3, dth, w); });
    const ff fr = nux ? sd + sd : fma(ff(2), sd, acc[0]);
    if (nux) {
        const ff xpi = cf.xp[i];
        const ff2 x2 = mk2(xpi, xpi);
        const ff2 a01 = fma(x2, mk2(fr, lane0(fuv)), mk2(acc[0], acc[1]));
        const ff2 a23 = fma(x2, mk2(lane1(fuv), lane0(fwe)), mk2(acc[2], acc[3]));
        acc[0] = lane0(a01); acc[1] = lane1(a01); acc[2] = lane0(a23); acc[3] = lane1(a23);
        acc[4] = fma(xpi, lane1(fwe), acc[4]);
    } else {
        acc[0] = fr; acc[1] = lane0(fuv); acc[2] = lane1(fuv); acc[3] = lane0(fwe); acc[4] = lane1(fwe);
    }
    if (MAYBE_X && DIR == 0) acc[1] -= dp; else if (DIR == 1) acc[2] -= dp; else acc[3] -= dp;
}

// Body force, sponge, stage update and the new state's recovery of the point at element
// c, given its RHS accumulators acc (convective, pressure and viscous terms) and centre
// values u0, v0, w0, r0 in the arithmetic type R
template <typename R>
__device__ __forceinline__ void stage_tail(const Geom& g, const Update<R>& up, double* __restrict__ scal, int i, int k,
                                           int c, R (&acc)[5], R u0, R v0, R w0, R r0) {
    // ---- body force and sponge (RHS terms, arithmetic type R) ----
    const R dpdz = to_r<R>(scal[SC_DPDZ]);
    acc[3] += dpdz;
    acc[4] = fma(dpdz, w0, acc[4]);
    const double rr = up.qin.r[c], uu = up.qin.u[c], vv = up.qin.v[c], ww = up.qin.w[c], ee = up.qin.e[c];
    if (up.spx) {
        const R sg = to_r<R>(up.spx[i] + up.spz[k]);
        const long long i2 = (long long)i + (long long)k * g.mx;
        if constexpr (sizeof(R) == 8) {   // FP64 (and the pair type: the term in FP64, then split)
            const double sgd = up.spx[i] + up.spz[k];
            acc[0] += to_r<R>(sgd * (up.rref[i2] - rr));
            acc[1] += to_r<R>(sgd * (up.uref[i2] - rr * uu));
            acc[2] += to_r<R>(sgd * (up.vref[i2] - rr * vv));
            acc[3] += to_r<R>(sgd * (up.wref[i2] - rr * ww));
            acc[4] += to_r<R>(sgd * (up.eref[i2] - ee));
        } else {
            acc[0] += sg * (to_r<R>(up.rref[i2]) - r0);
            acc[1] += sg * (to_r<R>(up.uref[i2]) - r0 * u0);
            acc[2] += sg * (to_r<R>(up.vref[i2]) - r0 * v0);
            acc[3] += sg * (to_r<R>(up.wref[i2]) - r0 * w0);
            acc[4] += sg * (to_r<R>(up.eref[i2]) - to_r<R>(ee));
        }
    }
    if (up.kind == ST_RHS_ONLY) {
#pragma unroll
        for (int q = 0; q < 5; q++) up.rb[q][c] = acc[q];
        return;
    }
    // ---- stage update: the RHS combination in R, the accumulation into the state in FP64 ----
    // The register arrays are read in full before any of them is written: the compiler
    // cannot prove that rb[q] and rb[q+1] (or k2) do not overlap, so interleaved
    // load/store pairs would serialise five memory round trips at the end of every thread.
    const double dt = scal[SC_DT];
    double qn[5];
    if (up.kind == ST_LS) {
        const double q0[5] = {rr, uu * rr, vv * rr, ww * rr, ee};
        const R a = up.ca, b = up.cb;
        R prev[5] = {0, 0, 0, 0, 0};
        if (up.use_prev) {
#pragma unroll
            for (int q = 0; q < 5; q++) prev[q] = up.rb[q][c];
        }
        if constexpr (sizeof(R) == 8) {
            // q0 + dt (a prev + b acc) with dt a, dt b formed once: two operations per field
            const double dta = dt * up.a, dtb = dt * up.b;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                qn[q] = fma(dtb, to_d<R>(acc[q]), up.use_prev ? fma(dta, to_d<R>(prev[q]), q0[q]) : q0[q]);
                up.rb[q][c] = acc[q];
            }
        } else {
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const R x = up.use_prev ? fma(a, prev[q], b * acc[q]) : b * acc[q];
                qn[q] = fma(dt, to_d<R>(x), q0[q]);
                up.rb[q][c] = acc[q];
            }
        }
    } else if (up.kind == ST_C1 || up.kind == ST_R4_1) {
        const double q0[5] = {rr, rr * uu, rr * vv, rr * ww, ee};
#pragma unroll
        for (int q = 0; q < 5; q++) {
            up.q0[q][c] = q0[q];
            const double Rd = to_d<R>(acc[q]);
            if (up.kind == ST_C1) { qn[q] = q0[q] + Rd * dt / 2.0; up.rb[q][c] = acc[q]; }
            else { qn[q] = q0[q] + 0.5 * dt * Rd; up.k2[q][c] = acc[q]; }
        }
    } else {
        double q0[5];
        R k1[5] = {0, 0, 0, 0, 0}, kk[5] = {0, 0, 0, 0, 0};
        const bool use_k1 = up.kind == ST_C2 || up.kind == ST_C3, use_k2 = up.kind != ST_C2;
#pragma unroll
        for (int q = 0; q < 5; q++) {
            q0[q] = up.q0[q][c];
            if (use_k1) k1[q] = up.rb[q][c];
            if (use_k2) kk[q] = up.k2[q][c];
        }
#pragma unroll
        for (int q = 0; q < 5; q++) {
            const double Rd = to_d<R>(acc[q]);
            switch (up.kind) {
            case ST_C2: qn[q] = q0[q] + (2 * Rd - to_d<R>(k1[q])) * dt; up.k2[q][c] = acc[q]; break;
            case ST_C3: qn[q] = q0[q] + dt * (to_d<R>(k1[q]) + 4 * to_d<R>(kk[q]) + Rd) / 6.; break;
            case ST_R4_2: up.k2[q][c] = to_r<R>(to_d<R>(kk[q]) + 2.0 * Rd); qn[q] = q0[q] + 0.5 * dt * Rd; break;
            case ST_R4_3: up.k2[q][c] = to_r<R>(to_d<R>(kk[q]) + 2.0 * Rd); qn[q] = q0[q] + dt * Rd; break;
            default: qn[q] = q0[q] + dt / 6.0 * (to_d<R>(kk[q]) + Rd); break;
            }
        }
    }
    const double inv = rcp_nr(qn[0]);
    const double un = qn[1] * inv, vn = qn[2] * inv, wn = qn[3] * inv;
    up.qout.r[c] = qn[0];
    up.qout.u[c] = un;
    up.qout.v[c] = vn;
    up.qout.w[c] = wn;
    up.qout.e[c] = qn[4];
    // the next stage's state recovery from the values in registers (bit for bit the state
    // kernel's result on the stored state)
    if (up.fuse) state_store<R>(up.ph, up.dnext, scal, c, qn[0], inv, un, vn, wn, qn[4]);
}

// FP64 RHS + stage update of one interior point (i, ., k) at element c, with the neighbours
// along x, y, z from the accessors nx, ny, nz and the centre values given
template <typename R, int S, int V, class NX, class NY, class NZ>
__device__ __forceinline__ void rhs_point_nb(const Geom& g, const CoefT<R>& cf, const RhsIn<R>& in,
                                             const Update<R>& up, double* __restrict__ scal, int quirk, int i,
                                             int k, int c, const NX& nx, const NY& ny, const NZ& nz, R th0,
                                             R m0, R u0, R v0, R w0, R r0, R h0) {
    R Gr[9];   // the gradient kernel's fields, Gr[3 a + b] = d u_b / d x_a
#pragma unroll
    for (int q = 0; q < 9; q++) Gr[q] = ld(in.g[q], c);
    // the stress tensor tau / mu (uXtmp, vXtmp, wXtmp of deviceRHSX and its y/z twins) and
    // the viscous dissipation tau_ab d u_b / d x_a / mu; an off-diagonal pair contributes
    // tau_ab (d u_b/d x_a + d u_a/d x_b) = tau_ab^2, except y-z with the quirk
    // (cuda_rhs.cu:175: tau_yz dv/dz in the y sum as in the z sum)
    const R th23 = (R)(2. / 3.) * th0;
    const R t00 = fma((R)2, Gr[0], -th23), t11 = fma((R)2, Gr[4], -th23), t22 = fma((R)2, Gr[8], -th23);
    const R t01 = Gr[1] + Gr[3], t02 = Gr[2] + Gr[6], t12 = Gr[5] + Gr[7];
    const R q12 = quirk ? Gr[7] + Gr[7] : t12;
    const R diss = fma(t00, Gr[0], fma(t11, Gr[4], fma(t22, Gr[8], fma(t01, t01, fma(t02, t02, t12 * q12)))));
    const R tx[3] = {t00, t01, t02}, ty[3] = {t01, t11, t12}, tz[3] = {t02, t12, t22};
    const R m3 = m0 * (R)(1.0 / 3.0);
    R acc[5] = {0, 0, 0, 0, 0};
    R W[3] = {0, 0, 0};
    R L[4] = {0, 0, 0, 0};
    R cond = 0;
    if constexpr (is_ff<R> && std::is_same<NX, NbGlobal<R>>::value && std::is_same<NY, NX>::value &&
                  std::is_same<NZ, NX>::value) {
        // the pair arithmetic is ~15 instructions per operation: x (with the stretched-grid
        // terms) and one copy of the y / z body walked twice, each a loop over the offsets
        // (rhs_dir_pair), keep the kernel's code within the instruction caches
        rhs_dir_pair<S, V, true>(g, cf, nx, i, 0, tx, m3, u0, v0, w0, r0, acc, W, L, cond);
#pragma unroll 1
        for (int d = 1; d < 3; d++) {
            const R td[3] = {d == 1 ? t01 : t02, d == 1 ? t11 : t12, d == 1 ? t12 : t22};
            NX nb = ny;   // the accessors differ in their stride only
            nb.st = d == 1 ? ny.st : nz.st;
            rhs_dir_pair<S, V, false>(g, cf, nb, i, d, td, m3, u0, v0, w0, r0, acc, W, L, cond);
        }
    } else {
        rhs_direction<R, S, V, true>(g, cf, nx, i, 0, tx, m3, u0, v0, w0, r0, acc, W, L, cond);
        rhs_direction<R, S, V, false>(g, cf, ny, i, 1, ty, m3, u0, v0, w0, r0, acc, W, L, cond);
        rhs_direction<R, S, V, false>(g, cf, nz, i, 2, tz, m3, u0, v0, w0, r0, acc, W, L, cond);
    }
    // the centre values of the cubic fluxes: phi_0 times half the mass flux
    const R half = (R)0.5 * acc[0];
    acc[1] = fma(u0, half, acc[1]);
    acc[2] = fma(v0, half, acc[2]);
    acc[3] = fma(w0, half, acc[3]);
    acc[4] = fma(h0, half, acc[4]);
#pragma unroll
    for (int q = 0; q < 3; q++) W[q] = fma(m0, L[q], W[q]);
    cond = fma(m0, L[3], cond);
    acc[1] += W[0];
    acc[2] += W[1];
    acc[3] += W[2];
    acc[4] += fma(m0, diss, cf.lam_mu * cond) + fma(u0, W[0], fma(v0, W[1], w0 * W[2]));

    stage_tail<R>(g, up, scal, i, k, c, acc, u0, v0, w0, r0);
}

// ---------------------------------------------------------------------------------
// FP32-RHS point body on the packed stencil records qa = (rho, u, v, w), qb = (T, p, H, mu)
// and theta. One pass per direction walks the offsets l = 1..S once: at each l it loads
// the two records on either side (four 16-byte loads) and theta (for l <= V) and feeds
// every sum that needs them -- the first derivatives of u, v, w, mu, T, theta at the
// viscous order and of p at the advective order, the second derivatives of u, v, w, T, and
// the telescoped split-form fluxes -- so no stencil is held in registers. Each sum is
// accumulated in the order of the FP64-mode body (centre term, then l ascending) with the
// same expressions; the non-uniform x second derivative adds the pair (l, -l) per l.
// ---------------------------------------------------------------------------------
//
// CW (compile-time weights): the sums use the central-difference weights as immediates and
// are scaled by the direction's inverse spacing (or its square) afterwards; the flux sums
// carry neither 1/2, 1/4 nor 1/dx, which the final combination applies. The batched stage
// kernel uses this form: its members' coefficients would otherwise come through shared
// memory and occupy registers. The standalone kernel reads the premultiplied tables from
// its launch parameters (constant bank operands).
template <int S, int V, int DIR, bool CW>
__device__ __forceinline__ void rhs_dir_packed(const Geom& g, const CoefT<float>& cf, const RhsIn<float>& in, int c,
                                               int st, int i, float (&Gr)[9], float m0, float m3, float u0, float v0,
                                               float w0, float r0, float h0, float T0, float (&acc)[5],
                                               float (&W)[3], float& cond, float& dmu_dir) {
    static_assert(V <= S, "the viscous half-width never exceeds the advective one");
    const bool nux = (DIR == 0) && g.nonuniform_x;
    const float xpi = nux ? cf.xp[i] : 1.0f;
    const float* c1V = cf.c1V[DIR];
    const float* c1S = cf.c1S[DIR];
    const float* c2V = cf.c2V[DIR];
    const float* fq = cf.fq[DIR];
    const float* fcb = cf.fc[DIR];
    const auto w1V = [&](int l) { if constexpr (CW) return fd1(V, l); else return c1V[l]; };
    const auto w1S = [&](int l) { if constexpr (CW) return fd1(S, l); else return c1S[l]; };
    const auto w2V = [&](int l) { if constexpr (CW) return fd2(V, l); else return c2V[l]; };
    const auto wq = [&](int l) { if constexpr (CW) return fd1(S, l); else return fq[l]; };
    const auto wc = [&](int l) { if constexpr (CW) return fd1(S, l); else return fcb[l]; };
    const float un = DIR == 0 ? u0 : (DIR == 1 ? v0 : w0);

    float gu = 0.f, gv = 0.f, gw = 0.f, dmu = 0.f, dT = 0.f, dth = 0.f, dp = 0.f;
    float d2uu, d2vv, d2ww, d2tt;
    if (nux) {
        const float cw = __ldg(cf.cvsx + V * g.mx + i);
        d2uu = cw * u0; d2vv = cw * v0; d2ww = cw * w0; d2tt = cw * T0;
    } else {
        d2uu = w2V(0) * u0; d2vv = w2V(0) * v0; d2ww = w2V(0) * w0; d2tt = w2V(0) * T0;
    }
    float sq = 0.f, fu = (nux || CW) ? 0.f : acc[1], fv = (nux || CW) ? 0.f : acc[2],
          fw = (nux || CW) ? 0.f : acc[3], fe = (nux || CW) ? 0.f : acc[4];
#pragma unroll
    for (int l = 1; l <= S; l++) {
        const float4 Ap = __ldg(in.qa + c + l * st), Am = __ldg(in.qa + c - l * st);
        const float4 Bp = __ldg(in.qb + c + l * st), Bm = __ldg(in.qb + c - l * st);
        if (l <= V) {
            const float thp = __ldg(in.dil + c + l * st), thm = __ldg(in.dil + c - l * st);
            if (l == 1) {
                gu = w1V(1) * (Ap.y - Am.y); gv = w1V(1) * (Ap.z - Am.z); gw = w1V(1) * (Ap.w - Am.w);
                dmu = w1V(1) * (Bp.w - Bm.w); dT = w1V(1) * (Bp.x - Bm.x); dth = w1V(1) * (thp - thm);
            } else {
                gu = fma(w1V(l), Ap.y - Am.y, gu); gv = fma(w1V(l), Ap.z - Am.z, gv);
                gw = fma(w1V(l), Ap.w - Am.w, gw);
                dmu = fma(w1V(l), Bp.w - Bm.w, dmu); dT = fma(w1V(l), Bp.x - Bm.x, dT);
                dth = fma(w1V(l), thp - thm, dth);
            }
            if (nux) {
                const float cp = __ldg(cf.cvsx + (V + l) * g.mx + i), cm = __ldg(cf.cvsx + (V - l) * g.mx + i);
                d2uu = fma(cp, Ap.y, fma(cm, Am.y, d2uu));
                d2vv = fma(cp, Ap.z, fma(cm, Am.z, d2vv));
                d2ww = fma(cp, Ap.w, fma(cm, Am.w, d2ww));
                d2tt = fma(cp, Bp.x, fma(cm, Bm.x, d2tt));
            } else {
                d2uu = fma(w2V(l), Ap.y + Am.y, d2uu);
                d2vv = fma(w2V(l), Ap.z + Am.z, d2vv);
                d2ww = fma(w2V(l), Ap.w + Am.w, d2ww);
                d2tt = fma(w2V(l), Bp.x + Bm.x, d2tt);
            }
        }
        dp = l == 1 ? w1S(1) * (Bp.y - Bm.y) : fma(w1S(l), Bp.y - Bm.y, dp);
        // telescoped split-form fluxes (rhs_direction: a_l Q+- shared by the cubic fluxes)
        const float gm = DIR == 0 ? Am.y : (DIR == 1 ? Am.z : Am.w);
        const float gp = DIR == 0 ? Ap.y : (DIR == 1 ? Ap.z : Ap.w);
        const float Qm = (Am.x + r0) * (gm + un);
        const float Qp = (r0 + Ap.x) * (un + gp);
        sq = fma(wq(l), Qm - Qp, sq);
        const float am = wc(l) * Qm, ap = wc(l) * Qp;
        fu = fma(am, Am.y, fma(-ap, Ap.y, fu));
        fv = fma(am, Am.z, fma(-ap, Ap.z, fv));
        fw = fma(am, Am.w, fma(-ap, Ap.w, fw));
        fe = fma(am, Bm.z, fma(-ap, Bp.z, fe));
    }
    // first derivatives: x' on a non-uniform x; with CW also the inverse spacing
    const float s1 = CW ? cf.inv[DIR] * xpi : xpi;
    if (nux || CW) { gu *= s1; gv *= s1; gw *= s1; }
    Gr[3 * DIR + 0] = gu; Gr[3 * DIR + 1] = gv; Gr[3 * DIR + 2] = gw;
    if (CW && !nux) {
        const float s2 = cf.inv2[DIR];
        d2uu *= s2; d2vv *= s2; d2ww *= s2; d2tt *= s2;
    }
    dmu *= s1;
    dmu_dir = dmu;
    W[0] = fma(d2uu, m0, W[0]);
    W[1] = fma(d2vv, m0, W[1]);
    W[2] = fma(d2ww, m0, W[2]);
    // heat conduction (lambda / mu)(mu d2T + dmu dT), the ratio applied once per point
    dT *= s1;
    cond = fma(d2tt, m0, cond);
    cond = fma(dT, dmu, cond);
    dth *= s1;
    dp *= s1;
    W[DIR] = fma(m3, dth, W[DIR]);
    if constexpr (CW) {
        // fluxes: mass c/dx * sq with c = 1/2, the cubic ones c/dx (f + phi_0 sq) with c = 1/4
        const float q2 = 0.5f * s1, q4 = 0.25f * s1;
        acc[0] = fma(q2, sq, acc[0]);
        acc[1] = fma(q4, fma(u0, sq, fu), acc[1]);
        acc[2] = fma(q4, fma(v0, sq, fv), acc[2]);
        acc[3] = fma(q4, fma(w0, sq, fw), acc[3]);
        acc[4] = fma(q4, fma(h0, sq, fe), acc[4]);
    } else {
        const float half = 0.5f * sq;
        fu = fma(u0, half, fu);
        fv = fma(v0, half, fv);
        fw = fma(w0, half, fw);
        fe = fma(h0, half, fe);
        const float fr = nux ? sq : acc[0] + sq;
        if (nux) {
            acc[0] = fma(xpi, fr, acc[0]);
            acc[1] = fma(xpi, fu, acc[1]);
            acc[2] = fma(xpi, fv, acc[2]);
            acc[3] = fma(xpi, fw, acc[3]);
            acc[4] = fma(xpi, fe, acc[4]);
        } else {
            acc[0] = fr; acc[1] = fu; acc[2] = fv; acc[3] = fw; acc[4] = fe;
        }
    }
    acc[1 + DIR] -= dp;
}

template <int S, int V, bool CW>
__device__ __forceinline__ void rhs_point_packed(const Geom& g, const CoefT<float>& cf, const RhsIn<float>& in,
                                                 const Update<float>& up, double* __restrict__ scal, int quirk, int i,
                                                 int j, int k) {
    const int c = (int)g.at(i, j, k);
    const float4 A0 = __ldg(in.qa + c), B0 = __ldg(in.qb + c);
    const float th0 = __ldg(in.dil + c);
    const float r0 = A0.x, u0 = A0.y, v0 = A0.z, w0 = A0.w;
    const float T0 = B0.x, h0 = B0.z, m0 = B0.w;
    const float m3 = m0 * (float)(1.0 / 3.0);
    float Gr[9];
    float acc[5] = {0, 0, 0, 0, 0};
    float W[3] = {0, 0, 0};
    float diss = 0, cond = 0;
    float dmu[3];
    rhs_dir_packed<S, V, 0, CW>(g, cf, in, c, 1, i, Gr, m0, m3, u0, v0, w0, r0, h0, T0, acc, W, cond, dmu[0]);
    rhs_dir_packed<S, V, 1, CW>(g, cf, in, c, (int)g.P, i, Gr, m0, m3, u0, v0, w0, r0, h0, T0, acc, W, cond, dmu[1]);
    rhs_dir_packed<S, V, 2, CW>(g, cf, in, c, (int)g.PS, i, Gr, m0, m3, u0, v0, w0, r0, h0, T0, acc, W, cond,
                                dmu[2]);
    // stress rows, dissipation and grad(mu) . s of every direction, now that all nine
    // gradients are known (y: tau_yz dv/dz with the quirk, src/cuda_rhs.cu:175)
#pragma unroll
    for (int d = 0; d < 3; d++) {
        float tau[3];
#pragma unroll
        for (int q = 0; q < 3; q++)
            tau[q] = (q == d) ? 2.0f * Gr[3 * d + q] - (float)(2. / 3.) * th0 : Gr[3 * d + q] + Gr[3 * q + d];
        const float dw = (d == 1 && quirk) ? Gr[7] : Gr[3 * d + 2];
        diss = fma(tau[0], Gr[3 * d + 0], diss);
        diss = fma(tau[1], Gr[3 * d + 1], diss);
        diss = fma(tau[2], dw, diss);
        W[0] = fma(tau[0], dmu[d], W[0]);
        W[1] = fma(tau[1], dmu[d], W[1]);
        W[2] = fma(tau[2], dmu[d], W[2]);
    }
    acc[1] += W[0];
    acc[2] += W[1];
    acc[3] += W[2];
    acc[4] += fma(m0, diss, cf.lam_mu * cond) + fma(u0, W[0], fma(v0, W[1], w0 * W[2]));
    stage_tail<float>(g, up, scal, i, k, c, acc, u0, v0, w0, r0);
}

// RHS + stage update of one interior point (i, j, k), every neighbour from global memory
// (CW: the FP32 body with compile-time weights, see rhs_dir_packed)
template <typename R, int S, int V, bool CW = false>
__device__ __forceinline__ void rhs_point(const Geom& g, const CoefT<R>& cf, const RhsIn<R>& in, const Update<R>& up,
                                          double* __restrict__ scal, int quirk, int i, int j, int k) {
    if constexpr (sizeof(R) == 4) {
        rhs_point_packed<S, V, CW>(g, cf, in, up, scal, quirk, i, j, k);
    } else {
        const int c = (int)g.at(i, j, k);
        const R th0 = ld(in.dil, c), m0 = ld(in.m, c);
        const R u0 = ld(in.u, c), v0 = ld(in.v, c), w0 = ld(in.w, c), r0 = ld(in.r, c), h0 = ld(in.h, c);
        const NbGlobal<R> nx{&in, c, 1}, ny{&in, c, (int)g.P}, nz{&in, c, (int)g.PS};
        rhs_point_nb<R, S, V>(g, cf, in, up, scal, quirk, i, k, c, nx, ny, nz, th0, m0, u0, v0, w0, r0, h0);
    }
}

// FP32: 7 blocks of 128 per SM (72 registers) measured fastest (6: 80 registers, +13 %
// time; 5: 96 registers, and stages that read the RK register ran 3.5x slower); FP64: the
// FP64 pipe bounds the kernel at 3 to 5 blocks alike; pairs: 4 blocks (122 registers)
// 856 Mpoint-steps/s on the channel against 815 with 5 (96 registers)
//
// One launch covers the 4-row bands [band0, band0 + gridDim.y) of every plane; blocks are
// dispatched x fastest, then bands, then planes. On large planes the bands are split into
// groups launched one after another, so the planes a z stencil spans stay in L2 while a
// group's blocks sweep them (one launch over whole planes would cycle ~2S planes of the
// inputs through L2 between their uses).
template <typename R, int S, int V>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 7 : 4) k_rhs(Geom g, const __grid_constant__ CoefT<R> cf,
                                                                                   const __grid_constant__ RhsIn<R> in, Update<R> up,
                                             double* __restrict__ scal, int quirk, int band0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = (band0 + (int)blockIdx.y) * blockDim.y + threadIdx.y;
    if (i >= g.mx || j >= g.my) return;
    rhs_point<R, S, V>(g, cf, in, up, scal, quirk, i, j, (int)blockIdx.z);
}

// Bands per launch: all of them while 3 S planes of a band group at 72 B per point (the
// stencil inputs of the FP64 kernel; twice the FP32 kernel's, whose other traffic streams
// through L2 alongside) fit in half of L2, else the largest group that does (at least 8
// bands). Measured on a 512^3 channel, FP32 RHS step: one launch 45.1 ms, groups of 75
// bands 38.6, 37 bands 36.9, 18 bands 36.9, 9 bands 37.3 ms; on 256^3 one launch (this
// rule) 4.64 ms, groups of 37 bands 4.69, 18 bands 4.74 ms; the FP64 step is the same
// either way (FP64-pipe bound).
inline int rhs_band_group(const Geom& g) {
    const int nby = (g.my + 3) / 4;
    const size_t budget = (size_t)64 << 20, per_band = (size_t)3 * g.G * g.mx * 4 * 72;
    const size_t fit = budget / per_band;
    if (fit >= (size_t)nby) return nby;
    return fit < 8 ? 8 : (int)fit;
}

template <typename R>
int launch_rhs_t(int S, int V, const Geom& g, const CoefT<R>& cf, const RhsIn<R>& in, const Update<R>& up,
                 double* scal, int quirk, cudaStream_t s) {
    const int nby = (g.my + 3) / 4, group = rhs_band_group(g);
    int n = 0;
    for (int b0 = 0; b0 < nby; b0 += group, n++) {
        dim3 grid((g.mx + 31) / 32, (unsigned)(nby - b0 < group ? nby - b0 : group), g.mz), block(32, 4, 1);
#define CNS_RHS_CASE(SS, VV) \
    if (S == SS && V == VV) { k_rhs<R, SS, VV><<<grid, block, 0, s>>>(g, cf, in, up, scal, quirk, b0); continue; }
        CNS_RHS_CASE(1, 1)
        CNS_RHS_CASE(2, 1) CNS_RHS_CASE(2, 2)
        CNS_RHS_CASE(3, 1) CNS_RHS_CASE(3, 2) CNS_RHS_CASE(3, 3)
        CNS_RHS_CASE(4, 1) CNS_RHS_CASE(4, 2) CNS_RHS_CASE(4, 3) CNS_RHS_CASE(4, 4)
#undef CNS_RHS_CASE
        return n;   // no instantiation for these orders
    }
    return n;
}

}  // namespace cns
