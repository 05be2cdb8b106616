// grid.cpp -- host-side grid, metric and coefficient construction, sponge set-up.
//
// initGrid / derivGrid (src/init.cpp:32-92, 258-277), the inverse spacings, cell widths
// and non-uniform x second-derivative table of setGPUParameters (src/cuda_utils.cu:60-139),
// and calculateSponge's strengths and profile interpolation (src/sponge.cu:115-169).
#include "grid.h"

#include <cmath>

namespace cns {

void fd_coeffs(int n, double F[4], double Sc[5]) {
    // central first / second derivative weights of order 2n (src/globals.h:69-95)
    static const double f1[1] = {-1.0 / 2.0}, s1[2] = {1.0, -2.0};
    static const double f2[2] = {1.0 / 12.0, -2.0 / 3.0}, s2[3] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0};
    static const double f3[3] = {-1.0 / 60.0, 3.0 / 20.0, -3.0 / 4.0},
                        s3[4] = {1.0 / 90.0, -3.0 / 20.0, 3.0 / 2.0, -49.0 / 18.0};
    static const double f4[4] = {1.0 / 280.0, -4.0 / 105.0, 1.0 / 5.0, -4.0 / 5.0},
                        s4[5] = {-1.0 / 560.0, 8.0 / 315.0, -1.0 / 5.0, 8.0 / 5.0, -205.0 / 72.0};
    const double* f = n == 1 ? f1 : n == 2 ? f2 : n == 3 ? f3 : f4;
    const double* s = n == 1 ? s1 : n == 2 ? s2 : n == 3 ? s3 : s4;
    for (int i = 0; i < n; i++) F[i] = f[i];
    for (int i = 0; i <= n; i++) Sc[i] = s[i];
}

static void deriv_grid(const cns_params& p, int S, const double* cF, const double* cS, double* d2f, double* df,
                       const double* f, double dx) {
    const int n = p.mx;
    std::vector<double> fb(n + 2 * S);
    for (int i = S; i < n + S; i++) fb[i] = f[i - S];
    for (int i = 0; i < S; i++) {
        fb[i] = -fb[2 * S - i - 1];                       // odd image about x = 0
        fb[n + S + i] = 2 * p.Lx - fb[n + S - i - 1];     // odd image about x = Lx
    }
    for (int i = 0; i < n; i++) {
        df[i] = 0.0;
        d2f[i] = cS[S] * fb[i + S] / dx / dx;
        for (int it = 0; it < S; it++) {
            df[i] += cF[it] * (fb[i + it] - fb[i + S * 2 - it]) / dx;
            d2f[i] += cS[it] * (fb[i + it] + fb[i + S * 2 - it]) / dx / dx;
        }
    }
}

int build_grid(const cns_params& p, HostGrid& g) {
    const int mx = p.mx, S = p.stencil_size, V = p.stencil_visc;
    double cF[4], cS[5], cVF[4], cVS[5];
    fd_coeffs(S, cF, cS);
    fd_coeffs(V, cVF, cVS);
    g.x.assign(mx, 0.0); g.xp.assign(mx, 0.0); g.xpp.assign(mx, 0.0);
    g.y.assign(p.my, 0.0); g.z.assign(p.mz, 0.0);

    // tanh-stretched cell-centred x; the boundary layer uses the lower half of the
    // symmetric channel mapping (src/init.cpp:36-55)
    double dx = p.Lx * (1.0) / (mx);
    std::vector<double> xn(mx + 1);
    int denom = mx;
    double denom2 = 2.0;
    if (p.boundary_layer) { denom *= 2; denom2 /= 2; }
    for (int i = 0; i < mx + 1; i++) xn[i] = tanh(p.stretch * ((i * 1.0) / denom - 0.5)) / tanh(p.stretch * 0.5);
    for (int i = 0; i < mx; i++) g.x[i] = p.Lx * (1.0 + (xn[i] + xn[i + 1]) / 2.0) / denom2;
    deriv_grid(p, S, cF, cS, g.xpp.data(), g.xp.data(), g.x.data(), dx);
    for (int i = 0; i < mx; i++) g.xp[i] = 1.0 / g.xp[i];
    if (!p.nonuniform_x) {   // uniform override keeps the stretched xp/xpp (src/init.cpp:57-63)
        for (int i = 0; i < mx; i++) g.x[i] = p.Lx * (0.5 + i * 1.0) / (mx);
        dx = g.x[1] - g.x[0];
    }
    for (int j = 0; j < p.my; j++) g.y[j] = p.Ly * (0.5 + j * 1.0) / (p.my);
    for (int k = 0; k < p.mz; k++) g.z[k] = p.Lz * (0.5 + k * 1.0) / (p.mz);

    // setGPUParameters (src/cuda_utils.cu:60-139)
    g.dx = 1.0 / dx;
    g.dy = 1.0 / (g.y[1] - g.y[0]);
    g.dz = 1.0 / (g.z[1] - g.z[0]);
    g.d2x = g.dx * g.dx;
    g.d2y = g.dy * g.dy;
    g.d2z = g.dz * g.dz;
    g.dxv.assign(mx, 0.0);
    g.dxv[0] = (g.x[1] + g.x[0]) / 2.0;
    for (int i = 1; i < mx - 1; i++) g.dxv[i] = (g.x[i + 1] - g.x[i - 1]) / 2.0;
    g.dxv[mx - 1] = p.Lx - (g.x[mx - 1] + g.x[mx - 2]) / 2.0;
    g.wvol.assign(mx, 0.0);
    for (int i = 0; i < mx; i++) g.wvol[i] = g.dxv[i] / g.dy / g.dz;
    g.cvsx.assign((size_t)mx * (2 * V + 1), 0.0);
    for (int it = 0; it < V; it++)
        for (int i = 0; i < mx; i++)
            g.cvsx[i + it * mx] = (cVS[it] * (g.xp[i] * g.xp[i]) * g.d2x -
                                   cVF[it] * g.xpp[i] * (g.xp[i] * g.xp[i] * g.xp[i]) * g.dx);
    for (int i = 0; i < mx; i++) g.cvsx[i + V * mx] = cVS[V] * (g.xp[i] * g.xp[i]) * g.d2x;
    for (int it = V + 1; it < 2 * V + 1; it++)
        for (int i = 0; i < mx; i++)
            g.cvsx[i + it * mx] = (cVS[2 * V - it] * (g.xp[i] * g.xp[i]) * g.d2x +
                                   cVF[2 * V - it] * g.xpp[i] * (g.xp[i] * g.xp[i] * g.xp[i]) * g.dx);
    for (int d = 0; d < 3; d++) {
        const double inv = d == 0 ? g.dx : d == 1 ? g.dy : g.dz;
        const double inv2 = d == 0 ? g.d2x : d == 1 ? g.d2y : g.d2z;
        for (int k = 0; k < 5; k++) g.c1S[d][k] = g.c1V[d][k] = g.c2V[d][k] = g.fq[d][k] = g.fc[d][k] = 0.0;
        for (int k = 1; k <= S; k++) {
            g.c1S[d][k] = -cF[S - k] * inv;
            g.fq[d][k] = 0.5 * g.c1S[d][k];
            g.fc[d][k] = 0.25 * g.c1S[d][k];
        }
        for (int k = 1; k <= V; k++) g.c1V[d][k] = -cVF[V - k] * inv;
        for (int k = 0; k <= V; k++) g.c2V[d][k] = cVS[V - k] * inv2;
    }
    return 0;
}

void sponge_strengths(const cns_params& p, const HostGrid& g, double* spx, double* spz) {
    for (int i = 0; i < p.mx; i++) {
        spx[i] = 0.0;
        if ((p.sp_top_len > 0.0) && (g.x[i] >= p.Lx - p.sp_top_len))
            spx[i] = p.sp_top_str * pow((g.x[i] - (p.Lx - p.sp_top_len)) / p.sp_top_len, p.sp_top_exp);
    }
    for (int k = 0; k < p.mz; k++) {
        spz[k] = 0.0;
        const double fz = g.z[k];
        if ((p.sp_inl_len > 0.0) && (fz <= p.sp_inl_len))
            spz[k] = p.sp_inl_str * pow((p.sp_inl_len - fz) / p.sp_inl_len, p.sp_inl_exp);
        if ((p.sp_out_len > 0.0) && (fz >= (p.Lz - p.sp_out_len)))
            spz[k] = p.sp_out_str * pow((fz - (p.Lz - p.sp_out_len)) / p.sp_out_len, p.sp_out_exp);
    }
}

// Natural cubic spline: second derivatives by the tridiagonal sweep, evaluation by
// bisection on the bracketing interval.
void spline_second(const double* xa, const double* ya, int n, double* y2) {
    std::vector<double> uu(n, 0.0);
    y2[0] = uu[0] = 0.0;
    for (int i = 1; i < n - 1; i++) {
        const double sig = (xa[i] - xa[i - 1]) / (xa[i + 1] - xa[i - 1]);
        const double pp = sig * y2[i - 1] + 2.0;
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
        const int k = (hi + lo) >> 1;
        if (xa[k] > xv) hi = k; else lo = k;
    }
    const double h = xa[hi] - xa[lo];
    const double a = (xa[hi] - xv) / h, b = (xv - xa[lo]) / h;
    return a * ya[lo] + b * ya[hi] + ((a * a * a - a) * y2[lo] + (b * b * b - b) * y2[hi]) * (h * h) / 6.0;
}

}  // namespace cns
