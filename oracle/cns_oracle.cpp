/*
 * cns_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the CudaNavierStokes time-advance path (state recovery,
 * velocity gradients, dilatation, split-form RHS in x/y/z with boundary conditions,
 * sponge, body force, CFL dt, bulk diagnostics, Wray low-storage RK3 and classic RK3),
 * plus a textbook classic RK4 that has no reference counterpart (rk4Step).
 * It is the parity reference for the GPU library and the timed CPU baseline. It follows
 * the reference kernels line by line, including their arithmetic order, the
 * double-interface flux loops and the y viscous-dissipation quirk, and processes
 * padded lines exactly as the reference's shared-memory pencils do.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
 * library, and only as the test oracle / CPU baseline. The product (cudanavierstokes_gb300)
 * never links or calls it.
 *
 * Reference files followed (paths inside the CudaNavierStokes project):
 *   src/globals.h:69-95           stencil coefficient tables
 *   src/init.cpp:32-92,258-277    grid, derivGrid
 *   src/cuda_utils.cu:49-139      inverse spacings, cell widths, x second-derivative table
 *   src/cuda_main.cu:218-247      calcState, sumLowStorageRK3
 *   src/cuda_main.cu:44-186       runSimulation / runSimulationLowStorage
 *   src/cuda_main.cu:188-216      eulerSum*, rk3final*
 *   src/calc_stress.cu:20-63      derVelX/Y/Z, :87-96 calcDil
 *   src/calc_stress.cu:98-201     calcPressureGrad, calcTimeStep/deviceCalcDt, calcBulk
 *   src/cuda_rhs.cu:9-396         deviceRHSX/Y/Z
 *   src/cuda_derivs.h:30-386      flux and derivative operators
 *   src/boundary.h, src/boundary_condition_{x,y,z}.h   ghost fills
 *   src/perturbation.h:25-53      wall blowing/suction
 *   src/sponge.cu:31-41,83-177    addSponge, calculateSponge
 */
#include "../include/cns.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline double MAXD(double a, double b) { return a >= b ? a : b; }   // main.h:12
inline double MIND(double a, double b) { return a <= b ? a : b; }   // main.h:13

/* src/globals.h:69-95: central first (F) and second (S) derivative coefficients */
void fd_coeffs(int n, std::vector<double>& F, std::vector<double>& Sc) {
    switch (n) {
    case 1: F = {-1.0 / 2.0};                         Sc = {1.0, -2.0}; break;
    case 2: F = {1.0 / 12.0, -2.0 / 3.0};             Sc = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0}; break;
    case 3: F = {-1.0 / 60.0, 3.0 / 20.0, -3.0 / 4.0}; Sc = {1.0 / 90.0, -3.0 / 20.0, 3.0 / 2.0, -49.0 / 18.0}; break;
    default: F = {1.0 / 280.0, -4.0 / 105.0, 1.0 / 5.0, -4.0 / 5.0};
             Sc = {-1.0 / 560.0, 8.0 / 315.0, -1.0 / 5.0, 8.0 / 5.0, -205.0 / 72.0}; break;
    }
}

enum { XPER = 0, XWALL = 1, XBL = 2 };

struct Oracle {
    cns_params p;
    int mx, my, mz, S, V;
    size_t N;
    double Ec, Rgas;
    double dxr;                       /* init.cpp dx (uniform computational spacing) */
    double d_dx, d_dy, d_dz, d_d2x, d_d2y, d_d2z;   /* cuda_utils.cu:61-90 */
    std::vector<double> x, xp, xpp, y, z, dxv;
    std::vector<double> cF, cS, cVF, cVS, cVSx;
    std::vector<double> r, u, v, w, e, h, t, pr, m, l, dil;
    std::vector<double> g[9];
    std::vector<double> R1[5], R2[5], R3[5], O[5];
    double dt = 0.0, dpdz = 0.0, time = 0.0;
    bool sponge = false;
    std::vector<double> spx, spz, rref, uref, vref, wref, eref;
    int xbc;

    size_t id(int i, int j, int k) const { return (size_t)i + (size_t)j * mx + (size_t)k * mx * my; }
};

/* ---------------- grid: src/init.cpp:32-92, 258-277 ---------------- */
void derivGrid(const Oracle& o, double* d2f, double* df, const double* f, double dx) {
    const int S = o.S, n = o.mx;
    std::vector<double> fb(n + 2 * S);
    for (int i = S; i < n + S; i++) fb[i] = f[i - S];
    for (int i = 0; i < S; i++) {
        fb[i] = -fb[2 * S - i - 1];
        fb[n + S + i] = 2 * o.p.Lx - fb[n + S - i - 1];
    }
    for (int i = 0; i < n; i++) {
        df[i] = 0.0;
        d2f[i] = o.cS[S] * fb[i + S] / dx / dx;
        for (int it = 0; it < S; it++) {
            df[i] += o.cF[it] * (fb[i + it] - fb[i + S * 2 - it]) / dx;
            d2f[i] += o.cS[it] * (fb[i + it] + fb[i + S * 2 - it]) / dx / dx;
        }
    }
}

void build_grid(Oracle& o) {
    const cns_params& p = o.p;
    const int mx = o.mx;
    o.x.assign(mx, 0.0); o.xp.assign(mx, 0.0); o.xpp.assign(mx, 0.0);
    o.y.assign(o.my, 0.0); o.z.assign(o.mz, 0.0);
    double dx = p.Lx * (1.0) / (mx);
    std::vector<double> xn(mx + 1);
    int denom = mx;
    double denom2 = 2.0;
    if (p.boundary_layer) { denom *= 2; denom2 /= 2; }
    for (int i = 0; i < mx + 1; i++)
        xn[i] = tanh(p.stretch * ((i * 1.0) / denom - 0.5)) / tanh(p.stretch * 0.5);
    for (int i = 0; i < mx; i++) o.x[i] = p.Lx * (1.0 + (xn[i] + xn[i + 1]) / 2.0) / denom2;
    derivGrid(o, o.xpp.data(), o.xp.data(), o.x.data(), dx);
    for (int i = 0; i < mx; i++) o.xp[i] = 1.0 / o.xp[i];
    if (!p.nonuniform_x) {
        for (int i = 0; i < mx; i++) o.x[i] = p.Lx * (0.5 + i * 1.0) / (mx);
        dx = o.x[1] - o.x[0];
    }
    for (int j = 0; j < o.my; j++) o.y[j] = p.Ly * (0.5 + j * 1.0) / (o.my);
    for (int k = 0; k < o.mz; k++) o.z[k] = p.Lz * (0.5 + k * 1.0) / (o.mz);
    o.dxr = dx;

    /* setGPUParameters, src/cuda_utils.cu:61-139 */
    o.d_dx = 1.0 / dx;
    o.d_dy = 1.0 / (o.y[1] - o.y[0]);
    o.d_dz = 1.0 / (o.z[1] - o.z[0]);
    o.dxv.assign(mx, 0.0);
    o.dxv[0] = (o.x[1] + o.x[0]) / 2.0;
    for (int i = 1; i < mx - 1; i++) o.dxv[i] = (o.x[i + 1] - o.x[i - 1]) / 2.0;
    o.dxv[mx - 1] = p.Lx - (o.x[mx - 1] + o.x[mx - 2]) / 2.0;
    o.d_d2x = o.d_dx * o.d_dx;
    o.d_d2y = o.d_dy * o.d_dy;
    o.d_d2z = o.d_dz * o.d_dz;
    const int V = o.V;
    o.cVSx.assign((size_t)mx * (2 * V + 1), 0.0);
    for (int it = 0; it < V; it++)
        for (int i = 0; i < mx; i++)
            o.cVSx[i + it * mx] = (o.cVS[it] * (o.xp[i] * o.xp[i]) * o.d_d2x -
                                   o.cVF[it] * o.xpp[i] * (o.xp[i] * o.xp[i] * o.xp[i]) * o.d_dx);
    for (int i = 0; i < mx; i++) o.cVSx[i + V * mx] = o.cVS[V] * (o.xp[i] * o.xp[i]) * o.d_d2x;
    for (int it = V + 1; it < 2 * V + 1; it++)
        for (int i = 0; i < mx; i++)
            o.cVSx[i + it * mx] = (o.cVS[2 * V - it] * (o.xp[i] * o.xp[i]) * o.d_d2x +
                                   o.cVF[2 * V - it] * o.xpp[i] * (o.xp[i] * o.xp[i] * o.xp[i]) * o.d_dx);
}

/* ---------------- calcState: src/cuda_main.cu:218-242 ---------------- */
void calcState(Oracle& o) {
    const double gam = o.p.gam, Rgas = o.Rgas, Re = o.p.Re, Pr = o.p.Pr, Ec = o.Ec, vexp = o.p.viscexp;
    const double cvInv = (gam - 1.0) / Rgas;
    const long long N = (long long)o.N;
#pragma omp parallel for schedule(static)
    for (long long gl = 0; gl < N; gl++) {
        double invrho = 1.0 / o.r[gl];
        double en = o.e[gl] * invrho - 0.5 * (o.u[gl] * o.u[gl] + o.v[gl] * o.v[gl] + o.w[gl] * o.w[gl]);
        o.t[gl] = cvInv * en;
        o.pr[gl] = o.r[gl] * Rgas * o.t[gl];
        o.h[gl] = (o.e[gl] + o.pr[gl]) * invrho;
        double suth = pow(o.t[gl], vexp);
        o.m[gl] = suth / Re;
        o.l[gl] = suth / Re / Pr / Ec;
    }
}

/* ---------------- shared-memory pencil operators: src/cuda_derivs.h ---------------- */
/* padded line f[0 .. n+2S), interior at [S, S+n); si = interior index + S */
struct Ops {
    const Oracle* o;
    int dir;           /* 0 x, 1 y, 2 z */
    double d, d2;      /* inverse spacing, squared */
    bool nux;          /* non-uniform x */

    double D1S(const double* f, int si) const {       /* derDevShared1{x,y,z} */
        const int S = o->S;
        double df = 0.0;
        if (dir == 0) {
            for (int it = 0; it < S; it++) df += o->cF[it] * (f[si + it - S] - f[si + S - it]);
            df = df * d;
            if (nux) df = df * o->xp[si - S];
        } else {
            for (int it = 0; it < S; it++) df += o->cF[it] * (f[si + it - S] - f[si + S - it]) * d;
        }
        return df;
    }
    double D1V(const double* f, int si) const {       /* derDevSharedV1{x,y,z} */
        const int V = o->V, S = o->S;
        double df = 0.0;
        if (dir == 0) {
            for (int it = 0; it < V; it++) df += o->cVF[it] * (f[si + it - V] - f[si + V - it]);
            df = df * d;
            if (nux) df = df * o->xp[si - S];
        } else {
            for (int it = 0; it < V; it++) df += o->cVF[it] * (f[si + it - V] - f[si + V - it]) * d;
        }
        return df;
    }
    double D2V(const double* f, int si) const {       /* derDevSharedV2{x,y,z} */
        const int V = o->V, S = o->S;
        double d2f;
        if (dir == 0 && nux) {
            d2f = 0.0;
            for (int it = 0; it < 2 * V + 1; it++) d2f += o->cVSx[it * o->mx + (si - S)] * f[si + it - V];
        } else {
            d2f = o->cVS[V] * f[si] * d2;
            for (int it = 0; it < V; it++) d2f += o->cVS[it] * (f[si + it - V] + f[si + V - it]) * d2;
        }
        return d2f;
    }
    double quad(const double* f, const double* g, int si) const {   /* fluxQuadShared* */
        const int S = o->S;
        double flxp = 0.0, flxm = 0.0;
        for (int lt = 1; lt < S + 1; lt++)
            for (int mt = 0; mt < lt; mt++) {
                flxp -= o->cF[S - lt] * (f[si - mt] + f[si - mt + lt]) * (g[si - mt] + g[si - mt + lt]);
                flxm -= o->cF[S - lt] * (f[si - mt - 1] + f[si - mt + lt - 1]) * (g[si - mt - 1] + g[si - mt + lt - 1]);
            }
        double df = 0.5 * d * (flxm - flxp);
        if (dir == 0 && nux) df = df * o->xp[si - S];
        return df;
    }
    double cube(const double* f, const double* g, const double* hh, int si) const {  /* fluxCubeShared* */
        const int S = o->S;
        double flxp = 0.0, flxm = 0.0;
        for (int lt = 1; lt < S + 1; lt++)
            for (int mt = 0; mt < lt; mt++) {
                flxp -= o->cF[S - lt] * (f[si - mt] + f[si - mt + lt]) * (g[si - mt] + g[si - mt + lt]) *
                        (hh[si - mt] + hh[si - mt + lt]);
                flxm -= o->cF[S - lt] * (f[si - mt - 1] + f[si - mt + lt - 1]) * (g[si - mt - 1] + g[si - mt + lt - 1]) *
                        (hh[si - mt - 1] + hh[si - mt + lt - 1]);
            }
        double df = 0.25 * d * (flxm - flxp);
        if (dir == 0 && nux) df = df * o->xp[si - S];
        return df;
    }
};

/* ---------------- ghost fills on padded lines: src/boundary.h ---------------- */
inline void perB(double* f, int n, int S) {                    /* perBC{x,y,z} */
    for (int t = 0; t < S; t++) { f[t] = f[t + n]; f[n + S + t] = f[S + t]; }
}
inline void wallVel(double* f, int n, int S) {                 /* wallBCxVel */
    for (int t = 0; t < S; t++) { f[t] = -f[2 * S - 1 - t]; f[n + S + t] = -f[n + S - 1 - t]; }
}
inline void wallMir(double* f, int n, int S) {                 /* wallBCxMir */
    for (int t = 0; t < S; t++) { f[t] = f[2 * S - 1 - t]; f[n + S + t] = f[n + S - 1 - t]; }
}
inline void wallExt(double* f, int n, int S, double Bt, double Bb) {   /* wallBCxExt */
    for (int t = 0; t < S; t++) { f[t] = 2.0 * Bb - f[2 * S - 1 - t]; f[n + S + t] = 2.0 * Bt - f[n + S - 1 - t]; }
}
inline void topExt(double* f, int n, int S) {                  /* topBCxExt / topBCzExt */
    for (int t = 0; t < S; t++) f[n + S + t] = 2.0 * f[n + S - 1] - f[n + S - 2 - t];
}
inline void botExtVal(double* f, int S, double Bb) {           /* botBCxExt */
    for (int t = 0; t < S; t++) f[t] = 2.0 * Bb - f[2 * S - 1 - t];
}
inline void botMir(double* f, int S) {                         /* botBCxMir */
    for (int t = 0; t < S; t++) f[t] = f[2 * S - 1 - t];
}
inline void botExtNode(double* f, int S) {                     /* botBCzExt */
    for (int t = 0; t < S; t++) f[t] = 2.0 * f[S] - f[2 * S - t];
}

/* PerturbUvel, src/perturbation.h:25-53: sets every bottom ghost of u in the k window */
void perturbU(const Oracle& o, double* su, int j, int k) {
    const cns_params& p = o.p;
    int kC = p.pert_kc, LP = p.pert_lp;
    int kSt = kC - LP / 2, kEn = kC + LP / 2;
    int ktot = k;
    if (ktot >= kSt && ktot <= kEn) {
        int alpha, beta, kappa;
        if (ktot < kC) { kappa = 1; alpha = ktot - kSt; beta = kC - kSt; }
        else { kappa = -1; alpha = kEn - ktot; beta = kEn - kC; }
        double ksi = alpha * 1.0 / beta;
        double gg = (15.1875 * ksi * ksi * ksi * ksi * ksi) - (35.4375 * ksi * ksi * ksi * ksi) + (20.25 * ksi * ksi * ksi);
        double y_glob = (j) / o.d_dy;
        double lambda = p.Ly / (2.0 * M_PI);
        double omega1 = p.Re * p.pert_omega1_per_re;
        double val = p.pert_amp1 * kappa * gg * sin(omega1 * o.time) +
                     p.pert_amp2 * kappa * gg * sin(p.pert_omega2 * o.time) * cos(y_glob / lambda);
        for (int t = 0; t < o.S; t++) su[t] = val;
    }
}

/* mlBoundPT / rhBoundPT, src/boundary.h:121-148 */
void mlBound(const Oracle& o, double* sm, double* sl, const double* st, int n) {
    const int S = o.S;
    for (int t = 0; t < S; t++) {
        for (int side = 0; side < 2; side++) {
            int g = side == 0 ? t : n + S + t;
            double suth = pow(st[g], o.p.viscexp);
            sm[g] = suth / o.p.Re;
            sl[g] = suth / o.p.Re / o.p.Pr / o.Ec;
        }
    }
}
void rhBound(const Oracle& o, double* sr, double* sh, const double* sp, const double* st, const double* su,
             const double* sv, const double* sw, int n) {
    const int S = o.S;
    const double Rgas = o.Rgas, gam = o.p.gam;
    for (int t = 0; t < S; t++) {
        for (int side = 0; side < 2; side++) {
            int g = side == 0 ? t : n + S + t;
            sh[g] = st[g] * Rgas * gam / (gam - 1.0) + 0.5 * (su[g] * su[g] + sv[g] * sv[g] + sw[g] * sw[g]);
            sr[g] = sp[g] / (Rgas * st[g]);
        }
    }
}

/* BCxderVel, src/boundary_condition_x.h:23-45 */
void bcx_vel(const Oracle& o, double* su, double* sv, double* sw, int j, int k) {
    const int n = o.mx, S = o.S;
    if (o.xbc == XPER) { perB(su, n, S); perB(sv, n, S); perB(sw, n, S); }
    else if (o.xbc == XBL) {
        topExt(su, n, S); topExt(sv, n, S); topExt(sw, n, S);
        botExtVal(su, S, 0.0); botExtVal(sv, S, 0.0); botExtVal(sw, S, 0.0);
        if (o.p.perturbed) perturbU(o, su, j, k);
    } else { wallVel(su, n, S); wallVel(sv, n, S); wallVel(sw, n, S); }
}

/* z ghost fill for any field: periodic or (boundary layer) node extrapolation,
 * BCzderVel / BCzNumber1-4 with nDivZ == 1, src/boundary_condition_z.h */
inline void bcz(const Oracle& o, double* f) {
    if (o.p.boundary_layer) { topExt(f, o.mz, o.S); botExtNode(f, o.S); }
    else perB(f, o.mz, o.S);
}

/* ---------------- derVelX/Y/Z + calcDil: src/calc_stress.cu:20-63, 87-96 ---------------- */
void derVel(Oracle& o) {
    const int mx = o.mx, my = o.my, mz = o.mz, S = o.S;
    Ops ox{&o, 0, o.d_dx, o.d_d2x, o.p.nonuniform_x != 0};
    Ops oy{&o, 1, o.d_dy, o.d_d2y, false};
    Ops oz{&o, 2, o.d_dz, o.d_d2z, false};
#pragma omp parallel
    {
        int L = std::max(mx, std::max(my, mz)) + 2 * S;
        std::vector<double> bu(L), bv(L), bw(L);
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < mz; k++)
            for (int j = 0; j < my; j++) {
                for (int i = 0; i < mx; i++) { size_t g = o.id(i, j, k); bu[i + S] = o.u[g]; bv[i + S] = o.v[g]; bw[i + S] = o.w[g]; }
                bcx_vel(o, bu.data(), bv.data(), bw.data(), j, k);
                for (int i = 0; i < mx; i++) {
                    size_t g = o.id(i, j, k);
                    o.g[0][g] = ox.D1V(bu.data(), i + S);
                    o.g[1][g] = ox.D1V(bv.data(), i + S);
                    o.g[2][g] = ox.D1V(bw.data(), i + S);
                }
            }
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < mz; k++)
            for (int i = 0; i < mx; i++) {
                for (int j = 0; j < my; j++) { size_t g = o.id(i, j, k); bu[j + S] = o.u[g]; bv[j + S] = o.v[g]; bw[j + S] = o.w[g]; }
                perB(bu.data(), my, S); perB(bv.data(), my, S); perB(bw.data(), my, S);
                for (int j = 0; j < my; j++) {
                    size_t g = o.id(i, j, k);
                    o.g[3][g] = oy.D1V(bu.data(), j + S);
                    o.g[4][g] = oy.D1V(bv.data(), j + S);
                    o.g[5][g] = oy.D1V(bw.data(), j + S);
                }
            }
#pragma omp for collapse(2) schedule(static)
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++) {
                for (int k = 0; k < mz; k++) { size_t g = o.id(i, j, k); bu[k + S] = o.u[g]; bv[k + S] = o.v[g]; bw[k + S] = o.w[g]; }
                bcz(o, bu.data()); bcz(o, bv.data()); bcz(o, bw.data());
                for (int k = 0; k < mz; k++) {
                    size_t g = o.id(i, j, k);
                    o.g[6][g] = oz.D1V(bu.data(), k + S);
                    o.g[7][g] = oz.D1V(bv.data(), k + S);
                    o.g[8][g] = oz.D1V(bw.data(), k + S);
                }
            }
    }
    const long long N = (long long)o.N;
#pragma omp parallel for schedule(static)
    for (long long gl = 0; gl < N; gl++) o.dil[gl] = o.g[0][gl] + o.g[4][gl] + o.g[8][gl];
}

/* ---------------- deviceRHSX/Y/Z: src/cuda_rhs.cu:9-396 ---------------- */
void rhs(Oracle& o, std::vector<double>* R) {
    const int mx = o.mx, my = o.my, mz = o.mz, S = o.S;
    const double dpdz = o.dpdz;
    Ops ox{&o, 0, o.d_dx, o.d_d2x, o.p.nonuniform_x != 0};
    Ops oy{&o, 1, o.d_dy, o.d_d2y, false};
    Ops oz{&o, 2, o.d_dz, o.d_d2z, false};
#pragma omp parallel
    {
        int L = std::max(mx, std::max(my, mz)) + 2 * S;
        std::vector<double> su(L), sv(L), sw(L), st(L), sp(L), s1(L), s2(L);
        /* ---- X (cuda_rhs.cu:9-128), writes ---- */
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < mz; k++)
            for (int j = 0; j < my; j++) {
                for (int i = 0; i < mx; i++) {
                    size_t g = o.id(i, j, k);
                    su[i + S] = o.u[g]; sv[i + S] = o.v[g]; sw[i + S] = o.w[g]; st[i + S] = o.t[g];
                    sp[i + S] = o.pr[g]; s1[i + S] = o.m[g]; s2[i + S] = o.l[g];
                }
                /* BCxNumber1 (boundary_condition_x.h:47-85) */
                if (o.xbc == XPER) {
                    perB(su.data(), mx, S); perB(sv.data(), mx, S); perB(sw.data(), mx, S); perB(st.data(), mx, S);
                    perB(sp.data(), mx, S); perB(s1.data(), mx, S); perB(s2.data(), mx, S);
                } else if (o.xbc == XBL) {
                    topExt(su.data(), mx, S); topExt(sv.data(), mx, S); topExt(sw.data(), mx, S);
                    topExt(sp.data(), mx, S); topExt(st.data(), mx, S);
                    botMir(sp.data(), S); botMir(st.data(), S);
                    botExtVal(su.data(), S, 0.0); botExtVal(sv.data(), S, 0.0); botExtVal(sw.data(), S, 0.0);
                    if (o.p.perturbed) perturbU(o, su.data(), j, k);
                    mlBound(o, s1.data(), s2.data(), st.data(), mx);
                } else {
                    wallMir(sp.data(), mx, S);
                    wallVel(su.data(), mx, S); wallVel(sv.data(), mx, S); wallVel(sw.data(), mx, S);
                    wallExt(st.data(), mx, S, o.p.twall_top, o.p.twall_bot);
                    mlBound(o, s1.data(), s2.data(), st.data(), mx);
                }
                for (int i = 0; i < mx; i++) {
                    size_t g = o.id(i, j, k);
                    int si = i + S;
                    double dudx = o.g[0][g], dvdx = o.g[1][g], dwdx = o.g[2][g], dudy = o.g[3][g], dudz = o.g[6][g];
                    double uX = (2 * dudx - 2. / 3. * o.dil[g]);
                    double vX = (dvdx + dudy);
                    double wX = (dwdx + dudz);
                    double eX = s1[si] * (uX * dudx + vX * dvdx + wX * dwdx);
                    double wrk2 = ox.D1V(s1.data(), si);
                    uX *= wrk2; vX *= wrk2; wX *= wrk2;
                    double wrk1 = ox.D2V(su.data(), si); uX = uX + wrk1 * s1[si];
                    wrk1 = ox.D2V(sv.data(), si); vX = vX + wrk1 * s1[si];
                    wrk1 = ox.D2V(sw.data(), si); wX = wX + wrk1 * s1[si];
                    eX = eX + su[si] * uX + sv[si] * vX + sw[si] * wX;
                    wrk1 = ox.D2V(st.data(), si);
                    eX = eX + wrk1 * s2[si];
                    wrk2 = ox.D1V(s2.data(), si);
                    wrk1 = ox.D1V(st.data(), si);
                    eX = eX + wrk1 * wrk2;
                    R[0][g] = uX; R[1][g] = vX; R[2][g] = wX; R[3][g] = eX;   /* staged, see below */
                }
                /* pressure and dilatation derivatives: s_prop2 <- dil, BCxNumber2 */
                for (int i = 0; i < mx; i++) s2[i + S] = o.dil[o.id(i, j, k)];
                if (o.xbc == XPER) perB(s2.data(), mx, S);
                else if (o.xbc == XBL) { topExt(s2.data(), mx, S); botMir(s2.data(), S); }
                else wallMir(s2.data(), mx, S);
                for (int i = 0; i < mx; i++) {
                    size_t g = o.id(i, j, k);
                    int si = i + S;
                    double wrk2 = ox.D1V(s2.data(), si);
                    double wrk1 = ox.D1S(sp.data(), si);
                    R[0][g] = R[0][g] + s1[si] * wrk2 / 3.0 - wrk1;
                    R[3][g] = R[3][g] + s1[si] * wrk2 / 3.0 * su[si];
                }
                /* fluxes: s_prop1 <- r, s_prop2 <- h, BCxNumber3 */
                for (int i = 0; i < mx; i++) { size_t g = o.id(i, j, k); s1[i + S] = o.r[g]; s2[i + S] = o.h[g]; }
                if (o.xbc == XPER) { perB(s1.data(), mx, S); perB(s2.data(), mx, S); }
                else rhBound(o, s1.data(), s2.data(), sp.data(), st.data(), su.data(), sv.data(), sw.data(), mx);
                for (int i = 0; i < mx; i++) {
                    size_t g = o.id(i, j, k);
                    int si = i + S;
                    double rX = ox.quad(s1.data(), su.data(), si);
                    double uX = R[0][g] + ox.cube(s1.data(), su.data(), su.data(), si);
                    double vX = R[1][g] + ox.cube(s1.data(), su.data(), sv.data(), si);
                    double wX = R[2][g] + ox.cube(s1.data(), su.data(), sw.data(), si);
                    double eX = R[3][g] + ox.cube(s1.data(), su.data(), s2.data(), si);
                    R[0][g] = rX; R[1][g] = uX; R[2][g] = vX; R[3][g] = wX; R[4][g] = eX;
                }
            }
        /* ---- Y (cuda_rhs.cu:130-262), += ---- */
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < mz; k++)
            for (int i = 0; i < mx; i++) {
                for (int j = 0; j < my; j++) {
                    size_t g = o.id(i, j, k);
                    su[j + S] = o.u[g]; sv[j + S] = o.v[g]; sw[j + S] = o.w[g]; s1[j + S] = o.m[g]; s2[j + S] = o.dil[g];
                    sp[j + S] = o.pr[g]; st[j + S] = o.t[g];
                }
                perB(su.data(), my, S); perB(sv.data(), my, S); perB(sw.data(), my, S);
                perB(s1.data(), my, S); perB(s2.data(), my, S); perB(sp.data(), my, S); perB(st.data(), my, S);
                for (int j = 0; j < my; j++) {
                    size_t g = o.id(i, j, k);
                    int si = j + S;
                    double dvdx = o.g[1][g], dudy = o.g[3][g], dvdy = o.g[4][g], dwdy = o.g[5][g], dvdz = o.g[7][g];
                    double uY = (dudy + dvdx);
                    double vY = (2 * dvdy - 2. / 3. * s2[si]);
                    double wY = (dwdy + dvdz);
                    double eY = s1[si] * (uY * dudy + vY * dvdy + wY * (o.p.quirk_dissipation_y ? dvdz : dwdy));
                    double wrk2 = oy.D1V(s1.data(), si);
                    uY *= wrk2; vY *= wrk2; wY *= wrk2;
                    double wrk1 = oy.D2V(su.data(), si); uY = uY + wrk1 * s1[si];
                    wrk1 = oy.D2V(sv.data(), si); vY = vY + wrk1 * s1[si];
                    wrk1 = oy.D2V(sw.data(), si); wY = wY + wrk1 * s1[si];
                    eY = eY + su[si] * uY + sv[si] * vY + sw[si] * wY;
                    wrk2 = oy.D1V(s2.data(), si);
                    vY = vY + s1[si] * wrk2 / 3.0;
                    eY = eY + s1[si] * wrk2 / 3.0 * sv[si];
                    wrk1 = oy.D1S(sp.data(), si);
                    vY = vY - wrk1;
                    /* staged in the output slots of the fluxes below */
                    o.O[0][g] = uY; o.O[1][g] = vY; o.O[2][g] = wY; o.O[3][g] = eY;
                }
                /* fourier terms: s_prop <- lam, s_dil <- t (BCyNumber3) */
                for (int j = 0; j < my; j++) { size_t g = o.id(i, j, k); s1[j + S] = o.l[g]; s2[j + S] = o.t[g]; }
                perB(s1.data(), my, S); perB(s2.data(), my, S);
                for (int j = 0; j < my; j++) {
                    size_t g = o.id(i, j, k);
                    int si = j + S;
                    double wrk1 = oy.D2V(s2.data(), si);
                    double eY = o.O[3][g] + wrk1 * s1[si];
                    double wrk2 = oy.D1V(s1.data(), si);
                    wrk1 = oy.D1V(s2.data(), si);
                    o.O[3][g] = eY + wrk1 * wrk2;
                }
                /* fluxes: s_prop <- r, s_dil <- h */
                for (int j = 0; j < my; j++) { size_t g = o.id(i, j, k); s1[j + S] = o.r[g]; s2[j + S] = o.h[g]; }
                perB(s1.data(), my, S); perB(s2.data(), my, S);
                for (int j = 0; j < my; j++) {
                    size_t g = o.id(i, j, k);
                    int si = j + S;
                    double rY = oy.quad(s1.data(), sv.data(), si);
                    double uY = o.O[0][g] + oy.cube(s1.data(), sv.data(), su.data(), si);
                    double vY = o.O[1][g] + oy.cube(s1.data(), sv.data(), sv.data(), si);
                    double wY = o.O[2][g] + oy.cube(s1.data(), sv.data(), sw.data(), si);
                    double eY = o.O[3][g] + oy.cube(s1.data(), sv.data(), s2.data(), si);
                    R[0][g] += rY; R[1][g] += uY; R[2][g] += vY; R[3][g] += wY; R[4][g] += eY;
                }
            }
        /* ---- Z (cuda_rhs.cu:264-396), += with body force ---- */
#pragma omp for collapse(2) schedule(static)
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++) {
                for (int k = 0; k < mz; k++) {
                    size_t g = o.id(i, j, k);
                    su[k + S] = o.u[g]; sv[k + S] = o.v[g]; sw[k + S] = o.w[g]; s1[k + S] = o.m[g]; s2[k + S] = o.dil[g];
                    sp[k + S] = o.pr[g];
                }
                bcz(o, su.data()); bcz(o, sv.data()); bcz(o, sw.data()); bcz(o, s1.data()); bcz(o, s2.data());
                bcz(o, sp.data());
                for (int k = 0; k < mz; k++) {
                    size_t g = o.id(i, j, k);
                    int si = k + S;
                    double dwdx = o.g[2][g], dwdy = o.g[5][g], dudz = o.g[6][g], dvdz = o.g[7][g], dwdz = o.g[8][g];
                    double uZ = (dudz + dwdx);
                    double vZ = (dvdz + dwdy);
                    double wZ = (2 * dwdz - 2. / 3. * s2[si]);
                    double eZ = s1[si] * (uZ * dudz + vZ * dvdz + wZ * dwdz);
                    double wrk2 = oz.D1V(s1.data(), si);
                    uZ *= wrk2; vZ *= wrk2; wZ *= wrk2;
                    double wrk1 = oz.D2V(su.data(), si); uZ = uZ + wrk1 * s1[si];
                    wrk1 = oz.D2V(sv.data(), si); vZ = vZ + wrk1 * s1[si];
                    wrk1 = oz.D2V(sw.data(), si); wZ = wZ + wrk1 * s1[si];
                    eZ = eZ + su[si] * uZ + sv[si] * vZ + sw[si] * wZ;
                    wrk2 = oz.D1V(s2.data(), si);
                    wZ = wZ + s1[si] * wrk2 / 3.0;
                    eZ = eZ + s1[si] * wrk2 / 3.0 * sw[si];
                    wrk1 = oz.D1S(sp.data(), si);
                    wZ = wZ - wrk1;
                    o.O[0][g] = uZ; o.O[1][g] = vZ; o.O[2][g] = wZ; o.O[3][g] = eZ;
                }
                for (int k = 0; k < mz; k++) { size_t g = o.id(i, j, k); s1[k + S] = o.l[g]; s2[k + S] = o.t[g]; }
                bcz(o, s1.data()); bcz(o, s2.data());
                for (int k = 0; k < mz; k++) {
                    size_t g = o.id(i, j, k);
                    int si = k + S;
                    double wrk1 = oz.D2V(s2.data(), si);
                    double eZ = o.O[3][g] + wrk1 * s1[si];
                    double wrk2 = oz.D1V(s1.data(), si);
                    wrk1 = oz.D1V(s2.data(), si);
                    o.O[3][g] = eZ + wrk1 * wrk2;
                }
                for (int k = 0; k < mz; k++) { size_t g = o.id(i, j, k); s1[k + S] = o.r[g]; s2[k + S] = o.h[g]; }
                bcz(o, s1.data()); bcz(o, s2.data());
                for (int k = 0; k < mz; k++) {
                    size_t g = o.id(i, j, k);
                    int si = k + S;
                    double rZ = oz.quad(s1.data(), sw.data(), si);
                    double uZ = o.O[0][g] + oz.cube(s1.data(), sw.data(), su.data(), si);
                    double vZ = o.O[1][g] + oz.cube(s1.data(), sw.data(), sv.data(), si);
                    double wZ = o.O[2][g] + oz.cube(s1.data(), sw.data(), sw.data(), si);
                    double eZ = o.O[3][g] + oz.cube(s1.data(), sw.data(), s2.data(), si);
                    R[0][g] += rZ; R[1][g] += uZ; R[2][g] += vZ;
                    R[3][g] += wZ + dpdz;
                    R[4][g] += eZ + dpdz * sw[si];
                }
            }
    }
    /* addSponge, src/sponge.cu:31-41 */
    if (o.p.boundary_layer && o.sponge) {
        const long long N = (long long)o.N;
#pragma omp parallel for schedule(static)
        for (long long gl = 0; gl < N; gl++) {
            int i = (int)(gl % mx);
            int k = (int)(gl / ((long long)mx * my));
            size_t i2 = (size_t)i + (size_t)k * mx;
            double s = (o.spx[i] + o.spz[k]);
            R[0][gl] += s * (o.rref[i2] - o.r[gl]);
            R[1][gl] += s * (o.uref[i2] - o.r[gl] * o.u[gl]);
            R[2][gl] += s * (o.vref[i2] - o.r[gl] * o.v[gl]);
            R[3][gl] += s * (o.wref[i2] - o.r[gl] * o.w[gl]);
            R[4][gl] += s * (o.eref[i2] - o.e[gl]);
        }
    }
}

/* calcRHS, src/cuda_main.cu:15-42 */
void calcRHS(Oracle& o, std::vector<double>* R) {
    calcState(o);
    derVel(o);
    rhs(o, R);
}

/* calcTimeStep + deviceCalcDt + minOfThreads, src/calc_stress.cu:122-160, cuda_math.cu:232-259 */
void calcTimeStep(Oracle& o) {
    const double gam = o.p.gam, CFL = o.p.cfl;
    const int mx = o.mx;
    const long long N = (long long)o.N;
    double best = 100000;
#pragma omp parallel for schedule(static) reduction(min : best)
    for (long long gl = 0; gl < N; gl++) {
        double ien = o.e[gl] / o.r[gl] - 0.5 * (o.u[gl] * o.u[gl] + o.v[gl] * o.v[gl] + o.w[gl] * o.w[gl]);
        double sos = pow(gam * (gam - 1) * ien, 0.5);
        double dx = o.dxv[gl % mx];
        double d2x = dx * dx;
        double dtConvInv = MAXD((fabs(o.u[gl]) + sos) / dx, MAXD((fabs(o.v[gl]) + sos) * o.d_dy, (fabs(o.w[gl]) + sos) * o.d_dz));
        double dtViscInv = MAXD(o.m[gl] / d2x, MAXD(o.m[gl] * o.d_d2y, o.m[gl] * o.d_d2z));
        double val = CFL / MAXD(dtConvInv, dtViscInv);
        best = MIND(best, val);
    }
    o.dt = best;
}

/* volume integral, integrateThreads (src/cuda_math.cu:143-171): sum f*dxv[i]/d_dy/d_dz */
double volInt(const Oracle& o, const std::vector<double>& f, const std::vector<double>* f2) {
    const int mx = o.mx;
    const long long N = (long long)o.N;
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (long long gl = 0; gl < N; gl++) {
        double val = f2 ? f[gl] * (*f2)[gl] : f[gl];
        s += val * o.dxv[gl % mx] / o.d_dy / o.d_dz;
    }
    return s;
}

/* calcPressureGrad, src/calc_stress.cu:98-120, law at :16-18 */
void calcPressureGrad(Oracle& o) {
    double prev = o.dpdz;
    double rbulk = volInt(o, o.r, nullptr);
    double rw = volInt(o, o.r, &o.w);
    o.dpdz = 0.99 * prev - 0.5 * (rw / rbulk - 1);
}

/* calcBulk, src/calc_stress.cu:162-201 */
void calcBulk(Oracle& o, double* par1, double* par2) {
    const int mx = o.mx;
    const long long N = (long long)o.N;
    if (o.p.forcing) {
        double rbulk = volInt(o, o.r, nullptr);
        double rw = volInt(o, o.r, &o.w);
        *par1 = rw / rbulk;
        *par2 = volInt(o, o.e, nullptr);
    } else {
        double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
        for (long long gl = 0; gl < N; gl++) {
            double a = o.u[gl] * o.u[gl] + o.v[gl] * o.v[gl] + o.w[gl] * o.w[gl];
            s += a * o.dxv[gl % mx] / o.d_dy / o.d_dz / o.p.Lx / o.p.Ly / o.p.Lz;
        }
        *par1 = s;
        *par2 = NAN;
    }
}

const double ALPHA[3] = {0., -17. / 60., -5. / 12.};   /* src/cuda_main.cu:10-11 */
const double BETA[3] = {8. / 15., 5. / 12., 3. / 4.};

/* momentum conversion + sumLowStorageRK3 + division (src/cuda_main.cu:127-139, :244-247) */
void lowStorageUpdate(Oracle& o, const std::vector<double>* A, const std::vector<double>* B, int step) {
    const long long N = (long long)o.N;
    const double dt = o.dt, a = ALPHA[step], b = BETA[step];
#pragma omp parallel for schedule(static)
    for (long long gl = 0; gl < N; gl++) {
        double ru = o.u[gl] * o.r[gl], rv = o.v[gl] * o.r[gl], rw = o.w[gl] * o.r[gl];
        double rn = o.r[gl] + dt * (a * A[0][gl] + b * B[0][gl]);
        ru = ru + dt * (a * A[1][gl] + b * B[1][gl]);
        rv = rv + dt * (a * A[2][gl] + b * B[2][gl]);
        rw = rw + dt * (a * A[3][gl] + b * B[3][gl]);
        o.e[gl] = o.e[gl] + dt * (a * A[4][gl] + b * B[4][gl]);
        o.r[gl] = rn;
        o.u[gl] = ru / rn; o.v[gl] = rv / rn; o.w[gl] = rw / rn;
    }
}

/* Classic four-stage Runge-Kutta on the conserved variables. NO REFERENCE COUNTERPART:
 * the reference's README.md:26 names "rk4", but src/ implements only the two RK3 schemes,
 * so this is a restatement of the textbook method (Kutta 1901), not of reference code:
 *   k1 = R(q0), q1 = q0 + dt/2 k1;  k2 = R(q1), q2 = q0 + dt/2 k2;
 *   k3 = R(q2), q3 = q0 + dt k3;    k4 = R(q3), q  = q0 + dt/6 (k1 + 2 k2 + 2 k3 + k4),
 * with the weighted sum accumulated as K = k1, K += 2 k2, K += 2 k3 as the stages arrive,
 * and the velocities of each stage state recovered as momentum / rho (the RK3 schemes'
 * deviceMul / deviceDiv convention, src/cuda_main.cu:127-139). */
void rk4Step(Oracle& o) {
    const long long N = (long long)o.N;
    const double dt = o.dt;
    std::vector<double> Q0[5], K[5];
    for (int f = 0; f < 5; f++) { Q0[f].resize(N); K[f].resize(N); }
#pragma omp parallel for schedule(static)
    for (long long gl = 0; gl < N; gl++) {
        Q0[0][gl] = o.r[gl];
        Q0[1][gl] = o.r[gl] * o.u[gl]; Q0[2][gl] = o.r[gl] * o.v[gl]; Q0[3][gl] = o.r[gl] * o.w[gl];
        Q0[4][gl] = o.e[gl];
    }
    auto set_state = [&](long long gl, const double* q) {
        o.r[gl] = q[0]; o.e[gl] = q[4];
        o.u[gl] = q[1] / q[0]; o.v[gl] = q[2] / q[0]; o.w[gl] = q[3] / q[0];
    };
    for (int st = 0; st < 4; st++) {
        calcRHS(o, o.R1);
#pragma omp parallel for schedule(static)
        for (long long gl = 0; gl < N; gl++) {
            double q[5];
            for (int f = 0; f < 5; f++) {
                const double k = o.R1[f][gl];
                if (st == 0) { K[f][gl] = k; q[f] = Q0[f][gl] + 0.5 * dt * k; }
                else if (st == 1) { K[f][gl] = K[f][gl] + 2.0 * k; q[f] = Q0[f][gl] + 0.5 * dt * k; }
                else if (st == 2) { K[f][gl] = K[f][gl] + 2.0 * k; q[f] = Q0[f][gl] + dt * k; }
                else q[f] = Q0[f][gl] + dt / 6.0 * (K[f][gl] + k);
            }
            set_state(gl, q);
        }
    }
}

int run(Oracle& o, int nsteps, double* par1, double* par2, double* timearr, double* dtlog, double* dpdzlog) {
    const long long N = (long long)o.N;
    for (int istep = 0; istep < nsteps; istep++) {
        if (istep % o.p.check_cfl == 0) {
            calcTimeStep(o);
            if (o.p.forcing) calcPressureGrad(o);
        }
        o.time += o.dt;
        if (timearr) timearr[istep] = o.time;
        if (dtlog) dtlog[istep] = o.dt;
        if (dpdzlog) dpdzlog[istep] = o.dpdz;
        double b1 = NAN, b2 = NAN;
        if (istep % o.p.check_bulk == 0) calcBulk(o, &b1, &b2);
        if (par1) par1[istep] = b1;
        if (par2) par2[istep] = b2;

        if (o.p.scheme == CNS_RK3_LOWSTORAGE) {
            calcRHS(o, o.R1); lowStorageUpdate(o, o.R1, o.R1, 0);
            calcRHS(o, o.R2); lowStorageUpdate(o, o.R1, o.R2, 1);
            calcRHS(o, o.R1); lowStorageUpdate(o, o.R2, o.R1, 2);
        } else if (o.p.scheme == CNS_RK4_CLASSIC) {
            rk4Step(o);
        } else {
            /* runSimulation, src/cuda_main.cu:44-107 */
            const double dt = o.dt;
#pragma omp parallel for schedule(static)
            for (long long gl = 0; gl < N; gl++) {
                o.O[1][gl] = o.r[gl] * o.u[gl]; o.O[2][gl] = o.r[gl] * o.v[gl]; o.O[3][gl] = o.r[gl] * o.w[gl];
                o.O[0][gl] = o.r[gl]; o.O[4][gl] = o.e[gl];
            }
            /* the RHS staging slots O[0..3] are reused by rhs(); keep the stage-0 copy apart */
            std::vector<double> Q0[5];
            for (int f = 0; f < 5; f++) Q0[f] = o.O[f];
            calcRHS(o, o.R1);
#pragma omp parallel for schedule(static)
            for (long long gl = 0; gl < N; gl++) {
                o.r[gl] = (Q0[0][gl] + o.R1[0][gl] * (dt) / 2.0);
                o.e[gl] = (Q0[4][gl] + o.R1[4][gl] * (dt) / 2.0);
                o.u[gl] = (Q0[1][gl] + o.R1[1][gl] * (dt) / 2.0) / o.r[gl];
                o.v[gl] = (Q0[2][gl] + o.R1[2][gl] * (dt) / 2.0) / o.r[gl];
                o.w[gl] = (Q0[3][gl] + o.R1[3][gl] * (dt) / 2.0) / o.r[gl];
            }
            calcRHS(o, o.R2);
#pragma omp parallel for schedule(static)
            for (long long gl = 0; gl < N; gl++) {
                o.r[gl] = Q0[0][gl] + (2 * o.R2[0][gl] - o.R1[0][gl]) * (dt);
                o.e[gl] = Q0[4][gl] + (2 * o.R2[4][gl] - o.R1[4][gl]) * (dt);
                o.u[gl] = (Q0[1][gl] + (2 * o.R2[1][gl] - o.R1[1][gl]) * (dt)) / o.r[gl];
                o.v[gl] = (Q0[2][gl] + (2 * o.R2[2][gl] - o.R1[2][gl]) * (dt)) / o.r[gl];
                o.w[gl] = (Q0[3][gl] + (2 * o.R2[3][gl] - o.R1[3][gl]) * (dt)) / o.r[gl];
            }
            calcRHS(o, o.R3);
#pragma omp parallel for schedule(static)
            for (long long gl = 0; gl < N; gl++) {
                o.r[gl] = Q0[0][gl] + (dt) * (o.R1[0][gl] + 4 * o.R2[0][gl] + o.R3[0][gl]) / 6.;
                o.e[gl] = Q0[4][gl] + (dt) * (o.R1[4][gl] + 4 * o.R2[4][gl] + o.R3[4][gl]) / 6.;
                o.u[gl] = (Q0[1][gl] + (dt) * (o.R1[1][gl] + 4 * o.R2[1][gl] + o.R3[1][gl]) / 6.) / o.r[gl];
                o.v[gl] = (Q0[2][gl] + (dt) * (o.R1[2][gl] + 4 * o.R2[2][gl] + o.R3[2][gl]) / 6.) / o.r[gl];
                o.w[gl] = (Q0[3][gl] + (dt) * (o.R1[3][gl] + 4 * o.R2[3][gl] + o.R3[3][gl]) / 6.) / o.r[gl];
            }
        }
    }
    /* leave derived fields consistent with the final state (calcState of the next RHS) */
    return 0;
}

/* natural cubic spline through (xa[i], ya[i]), i = 0..n-1 (tridiagonal solve), and its
 * evaluation by bisection; the interpolation calculateSponge uses (src/sponge.cu:156-177) */
void spline_second(const double* xa, const double* ya, int n, double* y2) {
    std::vector<double> uu(n, 0.0);
    y2[0] = uu[0] = 0.0;
    for (int i = 1; i < n - 1; i++) {
        double sig = (xa[i] - xa[i - 1]) / (xa[i + 1] - xa[i - 1]);
        double pp = sig * y2[i - 1] + 2.0;
        y2[i] = (sig - 1.0) / pp;
        uu[i] = (ya[i + 1] - ya[i]) / (xa[i + 1] - xa[i]) - (ya[i] - ya[i - 1]) / (xa[i] - xa[i - 1]);
        uu[i] = (6.0 * uu[i] / (xa[i + 1] - xa[i - 1]) - sig * uu[i - 1]) / pp;
    }
    y2[n - 1] = 0.0;
    for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + uu[k];
}
double spline_eval(const double* xa, const double* ya, const double* y2, int n, double xv) {
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int k = (hi + lo) >> 1;
        if (xa[k] > xv) hi = k; else lo = k;
    }
    double hh = xa[hi] - xa[lo];
    double a = (xa[hi] - xv) / hh, b = (xv - xa[lo]) / hh;
    return a * ya[lo] + b * ya[hi] + ((a * a * a - a) * y2[lo] + (b * b * b - b) * y2[hi]) * (hh * hh) / 6.0;
}

thread_local char g_err[256] = "";

/* ---------------- src/init.cpp:150-208 calcAvgChan: plane profiles over (y, z) ----------------
 * out[q * mx + i], q = 0..10: x, <rho>, <rho u>/<rho>, <rho v>/<rho>, <rho w>/<rho>, <rhoE>,
 * then the plane means of (rho - <rho>)^2, (u - ~u)^2, (v - ~v)^2, (w - ~w)^2, (rhoE - <rhoE>)^2
 * (the columns of the reference's prof.txt), each term divided by my*mz before summation. */
void plane_stats(const Oracle& o, double* out) {
    const int mx = o.mx, my = o.my, mz = o.mz;
    for (int i = 0; i < mx; i++) {
        double rm = 0, um = 0, vm = 0, wm = 0, em = 0;
        for (int k = 0; k < mz; k++)
            for (int j = 0; j < my; j++) {
                const size_t c = o.id(i, j, k);
                rm += o.r[c] / my / mz;
                um += o.r[c] * o.u[c] / my / mz;
                vm += o.r[c] * o.v[c] / my / mz;
                wm += o.r[c] * o.w[c] / my / mz;
                em += o.e[c] / my / mz;
            }
        um /= rm; vm /= rm; wm /= rm;
        double rf = 0, uf = 0, vf = 0, wf = 0, ef = 0;
        for (int k = 0; k < mz; k++)
            for (int j = 0; j < my; j++) {
                const size_t c = o.id(i, j, k);
                rf += (o.r[c] - rm) * (o.r[c] - rm) / my / mz;
                uf += (o.u[c] - um) * (o.u[c] - um) / my / mz;
                vf += (o.v[c] - vm) * (o.v[c] - vm) / my / mz;
                wf += (o.w[c] - wm) * (o.w[c] - wm) / my / mz;
                ef += (o.e[c] - em) * (o.e[c] - em) / my / mz;
            }
        const double col[11] = {o.x[i], rm, um, vm, wm, em, rf, uf, vf, wf, ef};
        for (int q = 0; q < 11; q++) out[(size_t)q * mx + i] = col[q];
    }
}

/* ---------------- src/init.cpp:210-256 printRes: friction Reynolds number at x = 0 ----------------
 * Re_tau = < u_tau rho_w / mu_w > over (y, z), u_tau = sqrt(mu_w |dw/dx| / rho_w), mu_w = 1/Re
 * (T_w = 1), dw/dx at the first point from the interior values mirrored evenly about the
 * wall, at the advective order, times x'(0)^-1 (xp[0]). */
double friction_reynolds(const Oracle& o) {
    const int S = o.S;
    double Ret = 0.0;
    for (int k = 0; k < o.mz; k++)
        for (int j = 0; j < o.my; j++) {
            const double temw = 1.0;
            const double suth = pow(temw, o.p.viscexp);
            const double muw = suth / o.p.Re;
            double ub[9];
            for (int i = S; i < S * 2 + 1; i++) ub[i] = o.w[o.id(i - S, j, k)];
            for (int i = 0; i < S; i++) ub[i] = o.w[o.id(S - i - 1, j, k)];
            double dudx = 0;
            for (int i = 0; i < S; i++) dudx += o.cF[i] * (ub[i] - ub[S * 2 - i]) / o.dxr;
            dudx *= o.xp[0];
            const double rw = o.r[o.id(0, j, k)];
            const double ut = sqrt(muw * fabs(dudx) / rw);
            Ret += ut * rw / muw;
        }
    return Ret / o.my / o.mz;
}

}  // namespace

/* Volume-averaged viscous dissipation <tau_ij du_i/dx_j> and enstrophy <|curl u|^2> of the
 * current state: the restatement of the library's diagnostic (which the reference leaves
 * to post-processing) on the reference's own pieces: gradients of derVel
 * (src/calc_stress.cu:20-63), mu of calcState (src/cuda_main.cu:218-242), cell weights of
 * the bulk integrals (src/calc_stress.cu:162-201). */
void dissipation(Oracle& o, double* out) {
    calcState(o);
    derVel(o);
    const int mx = o.mx;
    const long long N = (long long)o.N;
    double sp = 0.0, se = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : sp, se)
    for (long long gl = 0; gl < N; gl++) {
        double G[9];
        for (int q = 0; q < 9; q++) G[q] = o.g[q][gl];   /* G[3 d + n] = d u_n / d x_d */
        const double th = o.dil[gl];
        double s = 0.0;
        for (int d = 0; d < 3; d++)
            for (int n = 0; n < 3; n++) {
                double tau = G[3 * d + n] + G[3 * n + d] - (n == d ? 2.0 / 3.0 * th : 0.0);
                s += tau * G[3 * d + n];
            }
        const double wx = G[5] - G[7], wy = G[6] - G[2], wz = G[1] - G[3];
        const double wv = o.dxv[gl % mx] / o.d_dy / o.d_dz;
        sp += o.m[gl] * s * wv;
        se += (wx * wx + wy * wy + wz * wz) * wv;
    }
    const double vol = o.p.Lx * o.p.Ly * o.p.Lz;
    out[0] = sp / vol;
    out[1] = se / vol;
}

extern "C" {

const char* cnso_last_error(void) { return g_err; }

void cnso_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int cnso_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void* cnso_create(const cns_params* p) {
    if (!p) return nullptr;
    if (p->stencil_size < 1 || p->stencil_size > 4 || p->stencil_visc < 1 || p->stencil_visc > p->stencil_size ||
        p->mx < 2 * p->stencil_size || p->my < 2 * p->stencil_size || p->mz < 2 * p->stencil_size ||
        p->check_cfl < 1 || p->check_bulk < 1) {
        snprintf(g_err, sizeof g_err, "invalid parameters");
        return nullptr;
    }
    Oracle* o = new Oracle();
    o->p = *p;
    o->mx = p->mx; o->my = p->my; o->mz = p->mz; o->S = p->stencil_size; o->V = p->stencil_visc;
    o->N = (size_t)p->mx * p->my * p->mz;
    o->Ec = ((p->gam - 1.f) * p->Ma * p->Ma);      /* globals.h:47 */
    o->Rgas = (1.f / (p->gam * p->Ma * p->Ma));    /* globals.h:48 */
    fd_coeffs(o->S, o->cF, o->cS);
    fd_coeffs(o->V, o->cVF, o->cVS);
    o->xbc = p->periodic_x ? XPER : (p->boundary_layer ? XBL : XWALL);
    build_grid(*o);
    size_t N = o->N;
    for (auto* f : {&o->r, &o->u, &o->v, &o->w, &o->e, &o->h, &o->t, &o->pr, &o->m, &o->l, &o->dil}) f->assign(N, 0.0);
    for (int i = 0; i < 9; i++) o->g[i].assign(N, 0.0);
    for (int i = 0; i < 5; i++) { o->R1[i].assign(N, 0.0); o->R2[i].assign(N, 0.0); o->O[i].assign(N, 0.0); }
    if (p->scheme != CNS_RK3_LOWSTORAGE)
        for (int i = 0; i < 5; i++) o->R3[i].assign(N, 0.0);
    o->dpdz = p->forcing ? p->dpdz_init : 0.0;     /* cuda_utils.cu:68-70 */
    return o;
}

void cnso_destroy(void* h) { delete (Oracle*)h; }

int cnso_get_grid(void* h, double* x, double* xp, double* xpp, double* y, double* z, double* dxv) {
    Oracle* o = (Oracle*)h;
    if (x) std::memcpy(x, o->x.data(), sizeof(double) * o->mx);
    if (xp) std::memcpy(xp, o->xp.data(), sizeof(double) * o->mx);
    if (xpp) std::memcpy(xpp, o->xpp.data(), sizeof(double) * o->mx);
    if (y) std::memcpy(y, o->y.data(), sizeof(double) * o->my);
    if (z) std::memcpy(z, o->z.data(), sizeof(double) * o->mz);
    if (dxv) std::memcpy(dxv, o->dxv.data(), sizeof(double) * o->mx);
    return 0;
}

/* copyField(0) + calcState (src/cuda_utils.cu:299-333) */
int cnso_set_state(void* h, const double* r, const double* u, const double* v, const double* w, const double* e) {
    Oracle* o = (Oracle*)h;
    size_t nb = sizeof(double) * o->N;
    std::memcpy(o->r.data(), r, nb); std::memcpy(o->u.data(), u, nb); std::memcpy(o->v.data(), v, nb);
    std::memcpy(o->w.data(), w, nb); std::memcpy(o->e.data(), e, nb);
    calcState(*o);
    return 0;
}

int cnso_get_state(void* h, double* r, double* u, double* v, double* w, double* e) {
    Oracle* o = (Oracle*)h;
    size_t nb = sizeof(double) * o->N;
    if (r) std::memcpy(r, o->r.data(), nb);
    if (u) std::memcpy(u, o->u.data(), nb);
    if (v) std::memcpy(v, o->v.data(), nb);
    if (w) std::memcpy(w, o->w.data(), nb);
    if (e) std::memcpy(e, o->e.data(), nb);
    return 0;
}

/* derived fields of the last calcState: h, t, p, mu, lam */
int cnso_get_derived(void* h, double* hh, double* t, double* p, double* m, double* l) {
    Oracle* o = (Oracle*)h;
    size_t nb = sizeof(double) * o->N;
    if (hh) std::memcpy(hh, o->h.data(), nb);
    if (t) std::memcpy(t, o->t.data(), nb);
    if (p) std::memcpy(p, o->pr.data(), nb);
    if (m) std::memcpy(m, o->m.data(), nb);
    if (l) std::memcpy(l, o->l.data(), nb);
    return 0;
}

/* velocity gradients gij[0..8] and dilatation of the current state */
int cnso_gradients(void* h, double* gout /* 9*N */, double* dil) {
    Oracle* o = (Oracle*)h;
    derVel(*o);
    for (int i = 0; i < 9; i++)
        if (gout) std::memcpy(gout + (size_t)i * o->N, o->g[i].data(), sizeof(double) * o->N);
    if (dil) std::memcpy(dil, o->dil.data(), sizeof(double) * o->N);
    return 0;
}

int cnso_set_sponge(void* h, const double* spx, const double* spz, const double* rref, const double* uref,
                    const double* wref, const double* eref) {
    Oracle* o = (Oracle*)h;
    const int mx = o->mx, mz = o->mz;
    size_t n2 = (size_t)mx * mz;
    o->spx.assign(spx, spx + mx);
    o->spz.assign(spz, spz + mz);
    o->rref.assign(rref, rref + n2);
    o->uref.resize(n2); o->vref.assign(n2, 0.0); o->wref.resize(n2);
    o->eref.assign(eref, eref + n2);
    for (size_t g = 0; g < n2; g++) {              /* copySpongeToDevice, sponge.cu:57-61 */
        o->uref[g] = uref[g] * rref[g];
        o->wref[g] = wref[g] * rref[g];
    }
    o->sponge = true;
    return 0;
}

/* sponge strengths (src/sponge.cu:115-129) */
int cnso_sponge_strengths(void* h, double* spx, double* spz) {
    Oracle* o = (Oracle*)h;
    const cns_params& p = o->p;
    for (int i = 0; i < o->mx; i++) {
        spx[i] = 0.0;
        if ((p.sp_top_len > 0.0) && (o->x[i] >= p.Lx - p.sp_top_len))
            spx[i] = p.sp_top_str * pow((o->x[i] - (p.Lx - p.sp_top_len)) / p.sp_top_len, p.sp_top_exp);
    }
    for (int k = 0; k < o->mz; k++) {
        spz[k] = 0.0;
        double fz = o->z[k];
        if ((p.sp_inl_len > 0.0) && (fz <= p.sp_inl_len))
            spz[k] = p.sp_inl_str * pow((p.sp_inl_len - fz) / p.sp_inl_len, p.sp_inl_exp);
        if ((p.sp_out_len > 0.0) && (fz >= (p.Lz - p.sp_out_len)))
            spz[k] = p.sp_out_str * pow((fz - (p.Lz - p.sp_out_len)) / p.sp_out_len, p.sp_out_exp);
    }
    return 0;
}

/* reference fields from a 1D profile (src/sponge.cu:156-169), spline on the n given points */
int cnso_sponge_refs(void* h, int n, const double* xin, const double* rin, const double* uin, const double* win,
                     const double* ein, double* rref, double* uref, double* wref, double* eref) {
    Oracle* o = (Oracle*)h;
    const cns_params& p = o->p;
    std::vector<double> r2(n), u2(n), w2(n), e2(n);
    spline_second(xin, rin, n, r2.data());
    spline_second(xin, uin, n, u2.data());
    spline_second(xin, win, n, w2.data());
    spline_second(xin, ein, n, e2.data());
    for (int k = 0; k < o->mz; k++)
        for (int i = 0; i < o->mx; i++) {
            size_t g = (size_t)i + (size_t)k * o->mx;
            double scale = pow(1 + o->z[k] / p.Re, 0.5);
            rref[g] = spline_eval(xin, rin, r2.data(), n, o->x[i] / scale);
            uref[g] = spline_eval(xin, uin, u2.data(), n, o->x[i] / scale);
            uref[g] /= (scale * p.Re);
            wref[g] = spline_eval(xin, win, w2.data(), n, o->x[i] / scale);
            double pconst = o->Rgas;
            eref[g] = pconst / (p.gam - 1.0) + rref[g] * 0.5 * (uref[g] * uref[g] + wref[g] * wref[g]);
        }
    return 0;
}

/* one calcRHS on the current state */
int cnso_rhs(void* h, double* rr, double* ru, double* rv, double* rw, double* re) {
    Oracle* o = (Oracle*)h;
    calcRHS(*o, o->R1);
    size_t nb = sizeof(double) * o->N;
    std::memcpy(rr, o->R1[0].data(), nb); std::memcpy(ru, o->R1[1].data(), nb);
    std::memcpy(rv, o->R1[2].data(), nb); std::memcpy(rw, o->R1[3].data(), nb);
    std::memcpy(re, o->R1[4].data(), nb);
    return 0;
}

int cnso_calc_dt(void* h, double* dt) {
    Oracle* o = (Oracle*)h;
    calcTimeStep(*o);
    *dt = o->dt;
    return 0;
}

int cnso_bulk(void* h, double* par1, double* par2) {
    Oracle* o = (Oracle*)h;
    calcBulk(*o, par1, par2);
    return 0;
}

int cnso_run(void* h, int nsteps, double* par1, double* par2, double* timearr, double* dtlog, double* dpdzlog) {
    Oracle* o = (Oracle*)h;
    return run(*o, nsteps, par1, par2, timearr, dtlog, dpdzlog);
}

int cnso_get_scalars(void* h, double* dt, double* dpdz, double* time) {
    Oracle* o = (Oracle*)h;
    if (dt) *dt = o->dt;
    if (dpdz) *dpdz = o->dpdz;
    if (time) *time = o->time;
    return 0;
}

int cnso_set_scalars(void* h, double dt, double dpdz, double time) {
    Oracle* o = (Oracle*)h;
    o->dt = dt; o->dpdz = dpdz; o->time = time;
    return 0;
}

int cnso_plane_stats(void* h, double* out) {
    plane_stats(*(Oracle*)h, out);
    return 0;
}

int cnso_dissipation(void* h, double* out) {
    dissipation(*(Oracle*)h, out);
    return 0;
}

int cnso_friction_reynolds(void* h, double* ret) {
    *ret = friction_reynolds(*(Oracle*)h);
    return 0;
}

}  // extern "C"
