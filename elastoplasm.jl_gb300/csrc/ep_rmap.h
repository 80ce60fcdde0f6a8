// ep_rmap.h -- principal-space form of the finite-strain Drucker-Prager
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
// The 3d return (outer cone, DP.jl:19-21) acts on P = tr(s) / 3 and tau_II = sqrt(J2)
// in the same way: with an isotropic stiffness it is coaxial with the trial log strain
// and a function of the three principal strains.
//
// Features of a trial point (RM_NX floats):
//   x0, x1, x2  principal trial strains / s, x0 >= x1 >= x2 (x2 = 0 in plane strain)
//   x3          c / RM_CREF
//   x4, x5      tan(phi), tan(psi) (psi = 0, DP.jl:37)
//   x6          phi_n = f_s / c >= 0, the scaled overstress of the trial stress
//   x7          0: the 2d plane-strain map, 1: the 3d map (not a network input)
// The network output y (RM_NY floats, 3 used) is the plastic correction per unit
// overstress:  returned strains / s = x[0..2] + phi_n * y (2d), or + phi_n * (y0 e_m +
// y1 q + y2 r) in the trial's frame (3d, rm_frame3).  In the shear region of the exact
// map y = (-1, 1, 0) (2d) and (0, -sqrt2, 0) (3d); near the apex it is not constant.
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

// 3d: scaled principal stress of scaled principal strains, its inverse, the overstress
// f_s / c of the outer cone (DP.jl:19-21, 40-46; sin and cos of phi from tan phi)
EP_HD void rm_stress3(const double* e, double l2g, double* t) {
    const double tr = e[0] + e[1] + e[2];
    for (int i = 0; i < 3; ++i) t[i] = l2g * tr + e[i];
}

EP_HD void rm_strain3(const double* t, double l2g, double* e) {
    const double tr = (t[0] + t[1] + t[2]) / (1.0 + 3.0 * l2g);
    for (int i = 0; i < 3; ++i) e[i] = t[i] - l2g * tr;
}

EP_HD void rm_sincos(double tphi, double* sphi, double* cphi) {
    const double r = 1.0 / sqrt(1.0 + tphi * tphi);
    *sphi = tphi * r;
    *cphi = r;
}

EP_HD double rm_overstress3(const double* t, double tphi) {
    double sphi, cphi;
    rm_sincos(tphi, &sphi, &cphi);
    const double P = (t[0] + t[1] + t[2]) / 3.0;
    const double d0 = t[0] - P, d1 = t[1] - P, d2 = t[2] - P;
    const double tII = sqrt(0.5 * (d0 * d0 + d1 * d1 + d2 * d2));
    const DPParam m = dp_param3(sphi, cphi, 1.0);
    return tII + m.eta * P - m.xi;
}

// 3d output frame of a trial: e_m = (1,1,1)/sqrt3, q = the unit trial deviator of x[0..2]
// ((1,-1,0)/sqrt2 for a hydrostatic trial), r = e_m x q.  A 3d row's target is the correction in
// this frame, (y.e_m, y.q, y.r): constant (0, -sqrt2, 0) in the shear region of the exact map
// (the return shrinks the deviator radially), which BF16 activations represent well.
template <typename T>
EP_HD void rm_frame3(T x0, T x1, T x2, T* em, T* q, T* r) {
    const T is3 = (T)0.57735026918962576, is2 = (T)0.70710678118654752;
    const T xm = (x0 + x1 + x2) / (T)3;
    T d[3] = {x0 - xm, x1 - xm, x2 - xm};
    const T n = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (n > (T)0) {
        for (int i = 0; i < 3; ++i) q[i] = d[i] / n;
    } else {
        q[0] = is2; q[1] = -is2; q[2] = (T)0;
    }
    em[0] = em[1] = em[2] = is3;
    r[0] = em[1] * q[2] - em[2] * q[1];
    r[1] = em[2] * q[0] - em[0] * q[2];
    r[2] = em[0] * q[1] - em[1] * q[0];
}

// exact label of one 3d feature row
EP_HD int rm_label3(const float* x, double l2g, float* y) {
    const double e[3] = {x[0], x[1], x[2]}, tphi = x[4];
    double t[6], sphi, cphi;
    rm_stress3(e, l2g, t);
    t[3] = t[4] = t[5] = 0.0;
    const double phin = rm_overstress3(t, tphi);
    rm_sincos(tphi, &sphi, &cphi);
    double ep1 = 0.0;
    const double dl = dp_return<6>(t, 0.0, 1.0, 0.0, tphi, sphi, cphi, 0.0, 1.0, 1.0, &ep1);
    y[0] = y[1] = y[2] = y[3] = 0.f;
    if (dl == 0.0 || !(phin > RM_PHI_MIN)) return 0;
    double r[3], c[3], fm[3], fq[3], fr[3];
    rm_strain3(t, l2g, r);
    for (int i = 0; i < 3; ++i) c[i] = (r[i] - e[i]) / phin;
    rm_frame3<double>(e[0], e[1], e[2], fm, fq, fr);
    y[0] = (float)(c[0] * fm[0] + c[1] * fm[1] + c[2] * fm[2]);
    y[1] = (float)(c[0] * fq[0] + c[1] * fq[1] + c[2] * fq[2]);
    y[2] = (float)(c[0] * fr[0] + c[1] * fr[1] + c[2] * fr[2]);
    return 1;
}

// exact label of one feature row (FP64): returns 0 when the row is not a
// plastic trial (the map leaves it unchanged or phi_n is below RM_PHI_MIN)
EP_HD int rm_label(const float* x, double l2g, float* y) {
    if (x[7] > 0.5f) return rm_label3(x, l2g, y);
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
