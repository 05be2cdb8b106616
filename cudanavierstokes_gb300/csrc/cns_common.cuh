// cns_common.cuh -- device-side layout, constants and helpers shared by all kernels.
//
// HBM layout: every field is an FP64 (or FP32, for the FP32-RHS stencil inputs) 3D
// array with a ghost layer of width G = S (the advective half-width) on all six faces,
// x fastest. Ghost cells hold the reference's boundary images (periodic copies,
// wall mirrors, isothermal-wall temperature, extrapolation), filled once per stage by
// the ghost kernels, so the stencil kernels index neighbours with plain strides and
// no boundary branches. This replaces the reference's per-pencil shared-memory
// ghost fills (src/boundary.h, src/boundary_condition_{x,y,z}.h) and its MPI halos.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ff.cuh"
#include "pow_tables.h"

namespace cns {

enum XBC { XBC_PER = 0, XBC_WALL = 1, XBC_BL = 2 };

// indices into the device scalar block
enum { SC_DT = 0, SC_DPDZ = 1, SC_TIME = 2, SC_NONFINITE = 3, SC_STEP = 4, SC_COUNT = 8 };

struct Geom {
    int mx, my, mz, G;
    long long P;      // row pitch (elements)
    long long PS;     // plane stride (elements)
    long long base;   // element offset of interior point (0,0,0)
    int xbc;          // XBC_*
    int zbl;          // 1: z ends extrapolated (boundary layer), 0: periodic
    int nonuniform_x;
    const double* xp;     // [mx] 1/x'(xi)
    const double* cvsx;   // [(2V+1)*mx] non-uniform x second-derivative weights, index it*mx+i
    const double* wvol;   // [mx] cell volume dxv[i]/d_dy/d_dz
    const double* dxv;    // [mx] cell widths
    double dx, dy, dz, d2x, d2y, d2z;   // inverse spacings and their squares

    __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
        return base + (long long)k * PS + (long long)j * P + i;
    }
};

struct Phys {
    double gam, Rgas, Re, Pr, Ec, vexp;
    double invRe, clam, cvInv, hcoef;   // 1/Re, 1/(Re Pr Ec), (gam-1)/Rgas, Rgas*gam/(gam-1)
    double twall_top, twall_bot, cfl, Lx, Ly, Lz;
    int vexp_is_one, quirk, perturbed;
    int pert_kc, pert_lp;
    double pert_amp1, pert_amp2, pert_omega1, pert_omega2, pert_lambda;
    // FP32 copies for the FP32-RHS state kernel (converted once on the host)
    float f_Rgas, f_cvInv, f_invRe, f_vexp;
};

// Stencil coefficients premultiplied by the inverse grid spacing of each direction,
// in the arithmetic type R of the kernel that uses them.
//   c1S[d][k]: first derivative at the advective order 2S,  D f = sum_k c1S[k] (f_{+k} - f_{-k})
//   c1V[d][k]: first derivative at the viscous order 2V
//   c2V[d][k]: second derivative at order 2V (uniform), D2 f = c2V[0] f_0 + sum_k c2V[k](f_{+k}+f_{-k})
// from the central tables of src/globals.h:69-95 (c1[k] = -coeffF[K-k], c2[k] = coeffS[K-k]).
// xp / cvsx are the non-uniform x metric tables in type R.
template <typename R>
struct CoefT {
    R c1S[3][5];
    R c1V[3][5];
    R c2V[3][5];
    R fq[3][5];      // 0.5  * c1S: split-form quadratic flux (rho u) weights
    R fc[3][5];      // 0.25 * c1S: split-form cubic flux (rho u phi) weights
    R lam_mu;        // lambda / mu = 1 / (Pr Ec)
    R inv[3];        // inverse grid spacing of each direction (d_dx, d_dy, d_dz)
    R inv2[3];       // their squares
    const R* xp;     // [mx]
    const R* cvsx;   // [(2V+1)*mx], index it*mx + i
};

// Central-difference weights of half-width K as compile-time constants (the same tables,
// src/globals.h:69-95: fd1(K, k) = -coeffF[K-k], fd2(K, k) = coeffS[K-k]), for point bodies
// that scale the weighted sums by the inverse spacings instead of reading premultiplied
// tables. Standard central (Fornberg) weights of order 2K.
__host__ __device__ constexpr float fd1(int K, int k) {
    return K == 1 ? (k == 1 ? 1.0f / 2.0f : 0.0f)
         : K == 2 ? (k == 1 ? 2.0f / 3.0f : k == 2 ? -1.0f / 12.0f : 0.0f)
         : K == 3 ? (k == 1 ? 3.0f / 4.0f : k == 2 ? -3.0f / 20.0f : k == 3 ? 1.0f / 60.0f : 0.0f)
         : (k == 1 ? 4.0f / 5.0f : k == 2 ? -1.0f / 5.0f : k == 3 ? 4.0f / 105.0f : k == 4 ? -1.0f / 280.0f : 0.0f);
}
__host__ __device__ constexpr float fd2(int K, int k) {
    return K == 1 ? (k == 0 ? -2.0f : k == 1 ? 1.0f : 0.0f)
         : K == 2 ? (k == 0 ? -5.0f / 2.0f : k == 1 ? 4.0f / 3.0f : k == 2 ? -1.0f / 12.0f : 0.0f)
         : K == 3 ? (k == 0 ? -49.0f / 18.0f : k == 1 ? 3.0f / 2.0f : k == 2 ? -3.0f / 20.0f : k == 3 ? 1.0f / 90.0f
                                                                                                   : 0.0f)
         : (k == 0 ? -205.0f / 72.0f : k == 1 ? 8.0f / 5.0f : k == 2 ? -1.0f / 5.0f : k == 3 ? 8.0f / 315.0f
                                                                                    : k == 4 ? -1.0f / 560.0f : 0.0f);
}

// perturbation of the bottom-wall u ghosts (src/perturbation.h:25-53)
__device__ __forceinline__ bool wall_perturbation(const Phys& ph, double dy_inv, int j, int k, double time,
                                                  double* val) {
    int kSt = ph.pert_kc - ph.pert_lp / 2, kEn = ph.pert_kc + ph.pert_lp / 2;
    if (k < kSt || k > kEn) return false;
    int alpha, beta, kappa;
    if (k < ph.pert_kc) { kappa = 1; alpha = k - kSt; beta = ph.pert_kc - kSt; }
    else { kappa = -1; alpha = kEn - k; beta = kEn - ph.pert_kc; }
    double ksi = alpha * 1.0 / beta;
    double g = (15.1875 * ksi * ksi * ksi * ksi * ksi) - (35.4375 * ksi * ksi * ksi * ksi) + (20.25 * ksi * ksi * ksi);
    double y_glob = j / dy_inv;
    *val = ph.pert_amp1 * kappa * g * sin(ph.pert_omega1 * time) +
           ph.pert_amp2 * kappa * g * sin(ph.pert_omega2 * time) * cos(y_glob / ph.pert_lambda);
    return true;
}

// FP64 <-> FP32 conversions on the integer ALUs. The hardware conversions issue on the
// FP64 pipe, which on this part runs at 1/64 of the FP32 rate and bounds the FP32-RHS
// kernels, so they are done with bit operations on the IEEE 754 binary64 / binary32
// layouts (sign | exponent | fraction; biases 1023 and 127), without branches:
//   double -> float: the result keeps the 8 low exponent bits with bit 7 flipped
//     (e - 896 = e ^ 0x80 mod 256 for 897 <= e <= 1150) and the 23 leading fraction bits,
//     rounded half to even on the 29 discarded bits; the carry of the rounding runs into
//     the exponent (and to infinity at the top of the range), as the format intends;
//   float -> double: exact, exponent + 896 and the fraction shifted by 29.
// Results equal __double2float_rn and (double)f bit for bit, except that a result or an
// input in the binary32 subnormal range (below 2^-126 in magnitude) becomes a signed zero
// and every NaN becomes the quiet NaN of its sign.
__device__ __forceinline__ float d2f(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned ah = hi & 0x7fffffffu;
    unsigned body = (__funnelshift_l(lo, hi, 3) & 0x7fffffffu) ^ 0x40000000u;
    body += ((lo & 0x1fffffffu) + (body & 1u) + 0x0fffffffu) >> 29;
    body = ah < 0x38100000u ? 0u : body;                                    // |x| < 2^-126
    body = ah >= 0x47f00000u ? 0x7f800000u : body;                          // |x| >= 2^128, inf
    body = (ah > 0x7ff00000u || (ah == 0x7ff00000u && lo != 0u)) ? 0x7fc00000u : body;   // NaN
    return __uint_as_float((hi & 0x80000000u) | body);
}

__device__ __forceinline__ double f2d(float f) {
    const unsigned b = __float_as_uint(f), a = b & 0x7fffffffu;
    const bool tiny = a < 0x00800000u, special = a >= 0x7f800000u;
    unsigned hi = (a >> 3) + 0x38000000u, lo = a << 29;
    hi = tiny ? 0u : (special ? ((a >> 3) | 0x7ff00000u) : hi);
    lo = tiny ? 0u : lo;
    return __hiloint2double((int)((b & 0x80000000u) | hi), (int)lo);
}

// conversions between FP64 and the arithmetic type R of a kernel
template <typename R>
__device__ __forceinline__ R to_r(double x) {
    if constexpr (sizeof(R) == 4) return d2f(x);
    else if constexpr (is_ff<R>) return d_to_ff(x);
    else return x;
}
template <typename R>
__device__ __forceinline__ double to_d(R x) {
    if constexpr (sizeof(R) == 4) return f2d(x);
    else if constexpr (is_ff<R>) return ff_to_d(x);
    else return x;
}

// Reciprocal of a double from an FP32 seed r0 (|e| <= ~2^-23 with e = 1 - x r0):
// 1/x = r0 / (1 - e) = r0 (1 + e + e^2 + ...), taken to e^2 (cubic convergence, truncation
// ~2^-69, below the final rounding) in three fused multiply-adds, cheaper than the IEEE
// division on the FP64 pipe. The seed needs x and 1/x to be FP32 normals, so magnitudes
// outside [2^-125, 2^125) (and zero, infinity, NaN) take the IEEE division; densities never
// do. A GPU self test (cns_selftest_rcp) bounds it at one ulp of 1.0 / x.
__device__ __forceinline__ double rcp_nr(double x) {
    const unsigned ah = (unsigned)__double2hiint(x) & 0x7fffffffu;
    if (ah - 0x38200000u >= 0x47c00000u - 0x38200000u) return 1.0 / x;   // |x| outside [2^-125, 2^125)
    const double r = f2d(__frcp_rn(d2f(x)));
    const double e = fma(-x, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

// x > 0 (NaN excluded) from the IEEE bit pattern, on the integer units: the patterns of
// +denormals .. +infinity are the signed 64-bit integers in (0, 0x7ff0000000000000]
__device__ __forceinline__ bool positive_bits(double x) {
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7ff0000000000000LL;
}

// x^a in FP64 for the viscosity law mu ~ T^a, as exp(a ln x) with 64-entry tables
// (pow_tables.h, generated with 60-digit arithmetic by gen_pow_tables.py):
//   ln x = k ln2 - ln r_i + ln(1 + d),  x = 2^k m,  m in [1, 2),  i = the top 6 fraction
//     bits of m,  r_i ~ 1/c_i for the subinterval centre c_i = 1 + (i + 1/2)/64,
//     d = m r_i - 1 (one rounding, |d| < 2^-7),  ln(1 + d) by its series to d^8
//     (truncation below 2^-66), ln2 and -ln r_i as double-doubles;
//   exp y = 2^(j/64) exp(r),  j = nearest(64 y / ln2),  r = y - j ln2/64 with ln2/64 split
//     in a 41-bit head (j ln2_hi exact) and a tail (Cody & Waite's reduction), |r| <= 0.0055,
//     exp(r) - 1 = r + r^2 (1/2 + r/6 + ... + r^4/720) (truncation below 2^-65), 2^(i/64)
//     as a double-double.
// About 28 FP64 operations and five table loads (L1-resident) against ~120 for the library
// pow, which runs on the FP64 pipe. The error of exp(y) is that of y, about |y| ulp, so it
// serves |a ln x| < 1 (T^0.7 for 0.24 < T < 4.2, the temperatures of these flows), within a
// few ulp of pow (a GPU test bounds it); other arguments take pow itself.
__device__ __forceinline__ double pow_visc(double x, double a) {
    const double INV_LN2_64 = 92.33248261689366, SHIFT = 6755399441055744.0;   // 64/ln2, 1.5 * 2^52
    if (!(x > 1e-300 && x < 1e300)) return pow(x, a);
    const unsigned hx = (unsigned)__double2hiint(x);
    const int k = (int)(hx >> 20) - 1023;
    const int i = (int)((hx >> 14) & 63u);                 // top 6 bits of the fraction
    const double m = __hiloint2double((int)((hx & 0x000fffffu) | 0x3ff00000u), __double2loint(x));
    const double d = fma(m, __ldg(&kPowRcp[i]), -1.0);
    double q = -1.0 / 8.0;                                 // ln(1 + d) = d + d^2 q(d)
    q = fma(q, d, 1.0 / 7.0); q = fma(q, d, -1.0 / 6.0); q = fma(q, d, 1.0 / 5.0);
    q = fma(q, d, -1.0 / 4.0); q = fma(q, d, 1.0 / 3.0); q = fma(q, d, -0.5);
    const double l1p = fma(d * d, q, d);
    // k as a double through the 2^52 + 2^31 bias (no conversion instruction)
    const double kd = __hiloint2double(0x43300000, (int)((unsigned)k + 0x80000000u)) -
                      __hiloint2double(0x43300000, (int)0x80000000u);
    const double hi = fma(kd, POW_LN2_HI, __ldg(&kPowLnHi[i]));
    const double lo = fma(kd, POW_LN2_LO, __ldg(&kPowLnLo[i]));
    const double y = a * (hi + (lo + l1p));
    if (!(fabs(y) < 1.0)) return pow(x, a);
    const double t = fma(y, INV_LN2_64, SHIFT);
    const int j = __double2loint(t);
    const double jd = t - SHIFT;
    double r = fma(-jd, POW_LN2_64_HI, y);
    r = fma(-jd, POW_LN2_64_LO, r);
    double p = 1.0 / 720.0;                                // exp(r) - 1 = r + r^2 p(r)
    p = fma(p, r, 1.0 / 120.0); p = fma(p, r, 1.0 / 24.0); p = fma(p, r, 1.0 / 6.0); p = fma(p, r, 0.5);
    const double em1 = fma(r * r, p, r);
    const int ti = j & 63, e = j >> 6;                     // j = 64 e + ti, e = floor(j / 64)
    const double th = __ldg(&kPowExpHi[ti]);
    const double res = th + fma(th, em1, __ldg(&kPowExpLo[ti]));
    return __hiloint2double(__double2hiint(res) + (int)((unsigned)e << 20), __double2loint(res));
}

template <typename R> __device__ __forceinline__ R cns_pow(R a, R b);
template <> __device__ __forceinline__ double cns_pow<double>(double a, double b) { return pow_visc(a, b); }
template <> __device__ __forceinline__ float cns_pow<float>(float a, float b) { return powf(a, b); }

}  // namespace cns
