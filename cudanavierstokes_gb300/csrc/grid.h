// grid.h -- host-side grid and coefficient tables (internal).
#pragma once
#include <vector>
#include "../../include/cns.h"

namespace cns {

struct HostGrid {
    std::vector<double> x, xp, xpp, y, z, dxv, wvol, cvsx;
    double dx, dy, dz, d2x, d2y, d2z;   // inverse spacings (d_dx ... of the reference)
    double c1S[3][5], c1V[3][5], c2V[3][5], fq[3][5], fc[3][5];
};

void fd_coeffs(int n, double F[4], double Sc[5]);
int build_grid(const cns_params& p, HostGrid& g);
void sponge_strengths(const cns_params& p, const HostGrid& g, double* spx, double* spz);
void spline_second(const double* xa, const double* ya, int n, double* y2);
double spline_eval(const double* xa, const double* ya, const double* y2, int n, double xv);

}  // namespace cns
