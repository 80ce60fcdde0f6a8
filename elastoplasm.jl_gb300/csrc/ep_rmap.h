// ep_rmap.h -- principal-space form of the 2d finite-strain Drucker-Prager
// return (elast.jl:51-54, DP.jl:33-66) used by the learned return map.
//
// In plane strain the 2d return acts on the Voigt stress (xx, yy, xy) through
// P = (s_xx + s_yy) / 2 and tau_II only, so it commutes with rotations: in the
// principal frame of the trial log strain the shear stays zero and the map is a
// function of the two principal strains.  Everything is scaled by the current
// cohesion c: strains by s = c / (2G), stresses by c.  The map is positively
// homogeneous in (strain, c), so the scaled form depends on the scaled strains,
// tan(phi) and lambda / (2G) only.
//
// Features of a trial point (RM_NX floats):
//   x0, x1, x2  principal trial strains / s, x0 >= x1, x2 = 0 (plane strain)
//   x3          c / RM_CREF
//   x4, x5      tan(phi), tan(psi) (psi = 0, DP.jl:37)
//   x6          phi_n = f_s / c >= 0, the scaled overstress of the trial stress
// The network output y (RM_NY floats, 3 used) is the plastic correction per unit
// overstress:  returned strains / s = x[0..2] + phi_n * y.  In the shear region
// of the exact map y = (-1, 1, 0); near the apex it is not constant.
#pragma once

#include "ep_scalar.h"

namespace ep {

constexpr int RM_NX = 8;
constexpr int RM_NY = 4;
constexpr double RM_CREF = 2.0e4;
constexpr double RM_PHI_MIN = 1.0e-6;   // below: the point is returned by the exact map

// scaled plane-strain stress (xx, yy) of scaled principal strains (e1, e2); l2g = lambda / (2G)
EP_HD void rm_stress(double e1, double e2, double l2g, double* t) {
    const double tr = e1 + e2;
    t[0] = l2g * tr + e1;
    t[1] = l2g * tr + e2;
}

// scaled principal strains of a scaled principal stress (inverse of rm_stress)
EP_HD void rm_strain(double t1, double t2, double l2g, double* e) {
    const double tr = (t1 + t2) / (1.0 + 2.0 * l2g);
    e[0] = t1 - l2g * tr;
    e[1] = t2 - l2g * tr;
}

// scaled overstress f_s / c of a scaled Voigt stress (DP.jl:40-46 with c = 1)
EP_HD double rm_overstress(double t0, double t1, double t2, double tphi) {
    const double P = (t0 + t1) / 2.0;
    const double d0 = t0 - P, d1 = t1 - P;
    const double tII = sqrt(0.5 * (d0 * d0 + d1 * d1) + t2 * t2);
    const double den = sqrt(9.0 + (12.0 * tphi) * tphi);
    return tII + ((3.0 * tphi) / den) * P - 3.0 / den;
}

// exact label of one feature row (FP64): returns 0 when the row is not a
// plastic trial (the map leaves it unchanged or phi_n is below RM_PHI_MIN)
EP_HD int rm_label(const float* x, double l2g, float* y) {
    const double e1 = x[0], e2 = x[1], tphi = x[4];
    double t[3];
    rm_stress(e1, e2, l2g, t);
    t[2] = 0.0;
    const double phin = rm_overstress(t[0], t[1], 0.0, tphi);
    double ep1 = 0.0;
    // the reference's return with c0 = 1, no softening, K = G = 1 (only its stress is used)
    const double dl = dp_return<3>(t, 0.0, 1.0, 0.0, tphi, 0.0, 1.0, 0.0, 1.0, 1.0, &ep1);
    y[0] = y[1] = y[2] = y[3] = 0.f;
    if (dl == 0.0 || !(phin > RM_PHI_MIN)) return 0;
    double e[2];
    rm_strain(t[0], t[1], l2g, e);
    y[0] = (float)((e[0] - e1) / phin);
    y[1] = (float)((e[1] - e2) / phin);
    return 1;
}

}  // namespace ep
