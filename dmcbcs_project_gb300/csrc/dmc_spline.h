// Opt-in up-down Jastrow spline (no counterpart in the reference, whose
// Jastrow is the zero-energy two-body solution of coshpot.f90:14-143).
//
//   u_s(r) = sum_{k=0}^{15} t_k phi_k(r),   r in [0, L/2],   h = L / 34,
//   phi_0(r) = B(r/h),   phi_k(r) = B(r/h - k) + B(r/h + k)  (k >= 1),
//
// B the centred cubic B-spline on [-2, 2].  Every phi_k is even in r (so
// u_s'(0) = 0, no cusp) and vanishes with its first two derivatives at
// r = 17 h = L/2, where the reference's pair tables end.  u_s is added to
// the reference's up-down Jastrow table (u, u', u'' on the table grid), so
// with all t_k = 0 the wavefunction is the reference's.  The knots t_k are
// the 16 Jastrow parameters of the adjoint gradients.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define DMC_HD __host__ __device__
#else
#define DMC_HD
#endif

namespace dmc {

constexpr int kJastrowKnots = 16;
constexpr double kJastrowCells = 34.0;   // h = L / kJastrowCells

// B(t), B'(t), B''(t) of the centred cubic B-spline
DMC_HD inline void bspline3(double t, double& f, double& fp, double& fpp)
{
    const double a = fabs(t);
    if (a >= 2.0) {
        f = fp = fpp = 0.0;
        return;
    }
    const double sg = t < 0.0 ? -1.0 : 1.0;
    if (a < 1.0) {
        f = 2.0 / 3.0 - a * a + 0.5 * a * a * a;
        fp = sg * (-2.0 * a + 1.5 * a * a);
        fpp = -2.0 + 3.0 * a;
    } else {
        const double q = 2.0 - a;
        f = q * q * q / 6.0;
        fp = -sg * 0.5 * q * q;
        fpp = q;
    }
}

// phi_k(r) and its first two r-derivatives, knot spacing h
DMC_HD inline void jastrow_knot_basis(int k, double r, double h, double& f, double& fp, double& fpp)
{
    const double t = r / h;
    bspline3(t - k, f, fp, fpp);
    if (k > 0) {
        double f2, p2, q2;
        bspline3(t + k, f2, p2, q2);
        f += f2;
        fp += p2;
        fpp += q2;
    }
    fp /= h;
    fpp /= h * h;
}

}  // namespace dmc
