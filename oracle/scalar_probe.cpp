// scalar_probe.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the library's per-point arithmetic (elastoplasm.jl_gb300/csrc/ep_scalar.h, the code
// under test, compiled for the host with -ffp-contract=off exactly as the FP64 device step and
// the C++ oracle compile it) over arrays of inputs, so that tests/test_pointmath.py can hold it
// to the independent numpy restatement oracle/pointmath.py.  Arrays are point-major: point p's
// k values at [p*k .. p*k+k); matrices are column-major D x D per point.
#include <stdint.h>

#include "../elastoplasm.jl_gb300/csrc/ep_scalar.h"

using namespace ep;

extern "C" {

void probe_bspline(int64_t n, const double* xi, const double* xn, double xB0, double xB1, double dx, double* f,
                   double* df, int32_t* cls) {
    for (int64_t p = 0; p < n; ++p) {
        cls[p] = bspline_class(xn[p], xB0, xB1, dx);
        bspline(cls[p], xi[p], dx, &f[p], &df[p]);
    }
}

void probe_gimp(int64_t n, const double* dxp, double h, const double* lp, double* f, double* df) {
    for (int64_t p = 0; p < n; ++p) gimp(dxp[p], h, lp[p], &f[p], &df[p]);
}

void probe_hat(int64_t n, const double* dxp, double h, double* f, double* df) {
    for (int64_t p = 0; p < n; ++p) hat(dxp[p], h, &f[p], &df[p]);
}

// s: nstr per point, in-out; dlam, ep1 per point (ep1 in-out)
void probe_dp(int64_t n, int32_t nstr, double* s, const double* ep2, const double* c0, const double* cr,
              const double* tphi, const double* sphi, const double* cphi, double Hp, double Kc, double Gc,
              double* ep1, double* dlam) {
    for (int64_t p = 0; p < n; ++p) {
        if (nstr == 3)
            dlam[p] = dp_return<3>(s + 3 * p, ep2[p], c0[p], cr[p], tphi[p], sphi[p], cphi[p], Hp, Kc, Gc, &ep1[p]);
        else
            dlam[p] = dp_return<6>(s + 6 * p, ep2[p], c0[p], cr[p], tphi[p], sphi[p], cphi[p], Hp, Kc, Gc, &ep1[p]);
    }
}

void probe_j2(int64_t n, int32_t nstr, double* s, const double* ep2, const double* c0, const double* cr, double Hp,
              const double* Del, double* ep1, int32_t* yielded) {
    for (int64_t p = 0; p < n; ++p) {
        if (nstr == 3) yielded[p] = j2_return<3>(s + 3 * p, ep2[p], c0[p], cr[p], Hp, Del, &ep1[p]);
        else yielded[p] = j2_return<6>(s + 6 * p, ep2[p], c0[p], cr[p], Hp, Del, &ep1[p]);
    }
}

// 2d: s (3 per point) in-out; ep1 out; status per point (1 yielded, 0 elastic, -1 not converged)
void probe_mc(int64_t n, double* s, const double* ep2, const double* c0, const double* cr, const double* sphi,
              const double* cphi, double Hp, const double* Del, double* ep1, int32_t* status) {
    double LU[9];
    int piv[3];
    for (int i = 0; i < 9; ++i) LU[i] = Del[i];
    lu_factor<3>(LU, piv);
    for (int64_t p = 0; p < n; ++p)
        status[p] = mc_return(s + 3 * p, ep2[p], c0[p], cr[p], sphi[p], cphi[p], Hp, Del, LU, piv, &ep1[p]);
}

// s (nstr per point) and epV in-out; ep1 out; status per point (1 yielded, 0 elastic)
void probe_camc(int64_t n, int32_t nstr, double* s, const double* ep2, double* epV, double Kc, const double* Del,
                double* ep1, int32_t* status) {
    for (int64_t p = 0; p < n; ++p) {
        if (nstr == 3) status[p] = camc_return<3>(s + 3 * p, ep2[p], &epV[p], Kc, Del, &ep1[p]);
        else status[p] = camc_return<6>(s + 6 * p, ep2[p], &epV[p], Kc, Del, &ep1[p]);
    }
}

// b in-out (D*D per point); eps (D*D), tau (nstr) out
void probe_finite_elast(int64_t n, int32_t D, const double* dF, double* b, const double* Del, double* eps,
                        double* tau) {
    for (int64_t p = 0; p < n; ++p) {
        if (D == 2) finite_elast<2>(dF + 4 * p, b + 4 * p, eps + 4 * p, tau + 3 * p, Del);
        else finite_elast<3>(dF + 9 * p, b + 9 * p, eps + 9 * p, tau + 6 * p, Del);
    }
}

void probe_finite_rebuild_b(int64_t n, int32_t D, const double* tau, const double* Del, double* eps, double* b) {
    const int NS = D == 2 ? 3 : 6;
    double LU[36];
    int piv[6];
    for (int i = 0; i < NS * NS; ++i) LU[i] = Del[i];
    if (D == 2) lu_factor<3>(LU, piv);
    else lu_factor<6>(LU, piv);
    for (int64_t p = 0; p < n; ++p) {
        if (D == 2) finite_rebuild_b<2>(tau + 3 * p, LU, piv, eps + 4 * p, b + 4 * p);
        else finite_rebuild_b<3>(tau + 6 * p, LU, piv, eps + 9 * p, b + 9 * p);
    }
}

void probe_infinitesimal_elast(int64_t n, int32_t D, const double* dF, double* sig, const double* Del, double* eps,
                               double* w, double* sJ) {
    for (int64_t p = 0; p < n; ++p) {
        if (D == 2) infinitesimal_elast<2>(dF + 4 * p, sig + 3 * p, eps + 4 * p, w + 4 * p, sJ + 4 * p, Del, 0);
        else infinitesimal_elast<3>(dF + 9 * p, sig + 6 * p, eps + 9 * p, w + 9 * p, sJ + 9 * p, Del, 0);
    }
}

void probe_exp_log(int64_t n, const double* x, double* ex, double* lx) {
    for (int64_t p = 0; p < n; ++p) {
        ex[p] = ep_exp(x[p]);
        lx[p] = x[p] > 0.0 ? ep_log(x[p]) : 0.0;
    }
}

// eigenvalues (D) and column-major eigenvectors (D*D) of symmetric column-major matrices
void probe_eig(int64_t n, int32_t D, const double* A, double* lam, double* V) {
    for (int64_t p = 0; p < n; ++p) {
        if (D == 2) eig_sym<2>(A + 4 * p, lam + 2 * p, V + 4 * p);
        else eig_sym<3>(A + 9 * p, lam + 3 * p, V + 9 * p);
    }
}

void probe_det(int64_t n, int32_t D, const double* A, double* det) {
    for (int64_t p = 0; p < n; ++p) det[p] = D == 2 ? det_lu<2>(A + 4 * p) : det_lu<3>(A + 9 * p);
}

}  // extern "C"
