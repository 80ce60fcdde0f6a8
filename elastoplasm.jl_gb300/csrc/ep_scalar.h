// ep_scalar.h -- per-point and per-node arithmetic of the MPM step, compiled
// identically for the host (gcc, -ffp-contract=off) and the device (nvcc,
// -fmad=false in the FP64 kernels).  Every function uses only +, -, *, /,
// sqrt, fabs, frexp, ldexp and rint, which are correctly rounded / exact on
// both sides, so the FP64 device step reproduces a host computation bit for
// bit when it adds in the same order.
//
// The expressions follow the Julia source of ElastoPlasm term by term
// (left-to-right association, x^2 = x*x, x^3 = (x*x)*x, no fused multiply-add):
//   B-spline pieces       workflow/shpfun/basis/bsmpm.jl:1-78
//   GIMP                  workflow/shpfun/basis/gimpm.jl:1-14
//   linear                workflow/shpfun/basis/smpm.jl:1-10
//   grid update           workflow/mapsto/solve.jl:14-40
//   finite elasticity     workflow/elastoplast/elast/elast.jl:14-56
//   infinitesimal elast.  workflow/elastoplast/elast/elast.jl:69-80
//   Drucker-Prager        workflow/elastoplast/plast/retmap/DP.jl:1-100
//   J2                    workflow/elastoplast/plast/retmap/J2.jl:1-76 (restated, see j2_return)
//
// Third-party arithmetic the reference calls through Julia's LinearAlgebra and
// Base (eigen via LAPACK, det/`\` via LU, log/exp) is restated here from the
// published methods named at each function.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define EP_HD __host__ __device__ __forceinline__
#else
#define EP_HD static inline
#endif

namespace ep {

// ---------------------------------------------------------------------------
// exp and log.  exp: Cody & Waite argument reduction x = k ln2 + r with a
// two-part ln2 (hi has 32 significant bits so k*hi is exact), then the Taylor
// series of e^r to degree 13 (|r| <= ln2/2, truncation < 2^-56) in Horner form.
// log: x = 2^e m with m in (sqrt(2)/2, sqrt(2)], s = (m-1)/(m+1),
// log m = 2 atanh(s) = 2s + 2s^3 (1/3 + s^2/5 + ...), 11 odd terms (|s|<0.172).
// Both are within a few ulp of the correctly rounded result (tested).
// ---------------------------------------------------------------------------
EP_HD double ep_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    const double ln2_hi = 0x1.62e42fee00000p-1;
    const double ln2_lo = 0x1.a39ef35793c76p-33;
    const double inv_ln2 = 0x1.71547652b82fep+0;
    double k = rint(x * inv_ln2);
    double r = (x - k * ln2_hi) - k * ln2_lo;
    double p = 0x1.6124613a86d09p-33;            // 1/13!
    p = p * r + 0x1.1eed8eff8d898p-29;           // 1/12!
    p = p * r + 0x1.ae64567f544e4p-26;           // 1/11!
    p = p * r + 0x1.27e4fb7789f5cp-22;           // 1/10!
    p = p * r + 0x1.71de3a556c734p-19;           // 1/9!
    p = p * r + 0x1.a01a01a01a01ap-16;           // 1/8!
    p = p * r + 0x1.a01a01a01a01ap-13;           // 1/7!
    p = p * r + 0x1.6c16c16c16c17p-10;           // 1/6!
    p = p * r + 0x1.1111111111111p-7;            // 1/5!
    p = p * r + 0x1.5555555555555p-5;            // 1/4!
    p = p * r + 0x1.5555555555555p-3;            // 1/3!
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int ki = (int)k;
    if (ki > 1023) return ldexp(ldexp(p, ki - 1000), 1000);
    if (ki < -1021) return ldexp(ldexp(p, ki + 1000), -1000);
    return ldexp(p, ki);
}

EP_HD double ep_log(double x) {
    if (x != x) return x;
    if (x < 0.0) return NAN;
    if (x == 0.0) return -INFINITY;
    if (x == INFINITY) return x;
    int e;
    double m = frexp(x, &e);                   // x = m 2^e, m in [0.5, 1)
    if (m < 0x1.6a09e667f3bcdp-1) {            // below sqrt(2)/2: m in [1, sqrt 2) after doubling
        m = m * 2.0;
        e = e - 1;
    }
    double f = m - 1.0;                        // exact (Sterbenz)
    double s = f / (2.0 + f);
    double z = s * s;
    double q = 0x1.642c8590b2164p-5;           // 1/23
    q = q * z + 0x1.8618618618618p-5;          // 1/21
    q = q * z + 0x1.af286bca1af28p-5;          // 1/19
    q = q * z + 0x1.e1e1e1e1e1e1ep-5;          // 1/17
    q = q * z + 0x1.1111111111111p-4;          // 1/15
    q = q * z + 0x1.3b13b13b13b14p-4;          // 1/13
    q = q * z + 0x1.745d1745d1746p-4;          // 1/11
    q = q * z + 0x1.c71c71c71c71cp-4;          // 1/9
    q = q * z + 0x1.2492492492492p-3;          // 1/7
    q = q * z + 0x1.999999999999ap-3;          // 1/5
    q = q * z + 0x1.5555555555555p-2;          // 1/3
    double logm = 2.0 * s + (2.0 * s) * (z * q);
    const double ln2_hi = 0x1.62e42fee00000p-1;
    const double ln2_lo = 0x1.a39ef35793c76p-33;
    double de = (double)e;
    return de * ln2_hi + (logm + de * ln2_lo);
}

// x^y for x > 0 through exp(y log x); used for ΔJ^(1/dim) in 3d (volumetric.jl:34).
EP_HD double ep_pow(double x, double y) { return ep_exp(y * ep_log(x)); }

// Julia `sign` for Float64: sign(±0) = ±0, NaN -> NaN.
EP_HD double jsign(double x) {
    if (x > 0.0) return 1.0;
    if (x < 0.0) return -1.0;
    return x;
}

// Julia `fld(a, h)` for Float64: the floor of the exact quotient, computed as
// round((a - mod(a, h)) / h) with an exact fmod (Base: div(x, y, RoundDown)).
EP_HD double jfld(double a, double h) {
    double r = fmod(a, h);
    if (r != 0.0 && ((r < 0.0) != (h < 0.0))) r = r + h;
    return rint((a - r) / h);
}

// ---------------------------------------------------------------------------
// Julia's generic 2-norm of a short vector (LinearAlgebra.generic_norm2, used
// for length < 32 instead of BLAS nrm2): plain sum of squares unless the
// squares under/overflow, then scaled by max|x_i|.  solve.jl:29.
// ---------------------------------------------------------------------------
template <int N>
EP_HD double jnorm(const double* x) {
    double mx = 0.0;
    for (int i = 0; i < N; ++i) {
        double a = fabs(x[i]);
        if (a > mx || a != a) mx = a;
    }
    if (mx == 0.0 || mx == INFINITY || mx != mx) return mx;
    double mm = mx * mx;
    if ((double)N * mm < INFINITY && mm != 0.0) {
        double s = x[0] * x[0];
        for (int i = 1; i < N; ++i) s = s + x[i] * x[i];
        return sqrt(s);
    }
    double s = 0.0;
    for (int i = 0; i < N; ++i) {
        double y = x[i] / mx;
        s = s + y * y;
    }
    return mx * sqrt(s);
}

// ---------------------------------------------------------------------------
// Small dense LU with partial pivoting (first maximal |a_ik| wins, rows
// swapped, multipliers scaled by the reciprocal pivot), i.e. the arithmetic of
// LAPACK getrf as called by LinearAlgebra.det and `\` (deform.jl:17-18,
// DP.jl:64).  A is column-major n x n, overwritten by L\U; piv holds the row
// chosen at each step.  Returns 0 when a zero pivot is met.
// ---------------------------------------------------------------------------
template <int N>
EP_HD int lu_factor(double* A, int* piv) {
    int ok = 1;
    for (int k = 0; k < N; ++k) {
        int p = k;
        double amax = fabs(A[k + N * k]);
        for (int i = k + 1; i < N; ++i) {
            double a = fabs(A[i + N * k]);
            if (a > amax) { amax = a; p = i; }
        }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < N; ++j) {
                double t = A[k + N * j];
                A[k + N * j] = A[p + N * j];
                A[p + N * j] = t;
            }
        double akk = A[k + N * k];
        if (akk == 0.0) { ok = 0; continue; }
        double r = 1.0 / akk;
        for (int i = k + 1; i < N; ++i) A[i + N * k] = A[i + N * k] * r;
        for (int j = k + 1; j < N; ++j)
            for (int i = k + 1; i < N; ++i) A[i + N * j] = A[i + N * j] - A[i + N * k] * A[k + N * j];
    }
    return ok;
}

// det(A) = prod(diag(U)) * (-1)^(#row swaps), 0 for a singular factorisation.
template <int N>
EP_HD double det_lu(const double* Ain) {
    double A[N * N];
    int piv[N];
    for (int i = 0; i < N * N; ++i) A[i] = Ain[i];
    if (!lu_factor<N>(A, piv)) return 0.0;
    double P = 1.0;
    int c = 0;
    for (int i = 0; i < N; ++i) {
        P = P * A[i + N * i];
        if (piv[i] != i) c++;
    }
    return (c & 1) ? P * -1.0 : P * 1.0;
}

// x = A \ b with the factors of lu_factor: row swaps, unit-lower forward
// substitution, then upper back substitution column by column (reference BLAS trsv order).
template <int N>
EP_HD void lu_solve(const double* LU, const int* piv, const double* b, double* x) {
    for (int i = 0; i < N; ++i) x[i] = b[i];
    for (int k = 0; k < N; ++k)
        if (piv[k] != k) { double t = x[k]; x[k] = x[piv[k]]; x[piv[k]] = t; }
    for (int j = 0; j < N; ++j) {
        double xj = x[j];
        if (xj != 0.0)
            for (int i = j + 1; i < N; ++i) x[i] = x[i] - xj * LU[i + N * j];
    }
    for (int j = N - 1; j >= 0; --j) {
        if (x[j] != 0.0) {
            x[j] = x[j] / LU[j + N * j];
            double xj = x[j];
            for (int i = 0; i < j; ++i) x[i] = x[i] - xj * LU[i + N * j];
        }
    }
}

// APIC (p2n.jl:208-280, shpfun/misc.jl:15-28, mapsto/Bij.jl:14-26), column-major N x N:
//   Dᵢⱼ = N_k (δ δᵀ) of the LAST existing stencil node k (Dij_nd assigns instead of adding);
//   C = Bᵢⱼ D⁻¹ with D⁻¹ = inv(D) when |det D| > 1e-12, else the identity (p2n.jl:221-225);
//   the momentum of node k gets N ms (v + C δ_k); Bᵢⱼ = Σ_k N_k (v_k δ_kᵀ) after G2P.
// The rank-one D has det D = 0 up to rounding, so the identity branch is the one taken unless
// N² δx² δz² approaches 1e-12 / 2.2e-16 (node distances of several metres).
template <int N>
EP_HD void apic_bdinv(const double* B, const double* Dm, double* C) {
    double Di[N * N];
    if (fabs(det_lu<N>(Dm)) > 1.0e-12) {
        double LU[N * N];
        int piv[N];
        for (int i = 0; i < N * N; ++i) LU[i] = Dm[i];
        lu_factor<N>(LU, piv);
        for (int j = 0; j < N; ++j) {
            double e[N];
            for (int i = 0; i < N; ++i) e[i] = (i == j) ? 1.0 : 0.0;
            lu_solve<N>(LU, piv, e, &Di[N * j]);
        }
    } else {
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) Di[i + N * j] = (i == j) ? 1.0 : 0.0;
    }
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            double s = B[i] * Di[N * j];
            for (int k = 1; k < N; ++k) s = s + B[i + N * k] * Di[k + N * j];
            C[i + N * j] = s;
        }
}

// (C δ)_i summed left to right
template <int N>
EP_HD double apic_row(const double* C, int i, const double* dl) {
    double s = C[i] * dl[0];
    for (int k = 1; k < N; ++k) s = s + C[i + N * k] * dl[k];
    return s;
}

// ---------------------------------------------------------------------------
// Symmetric eigen-decomposition by Jacobi rotations (Golub & Van Loan,
// "Matrix Computations", Alg. 8.5.1 sym.Schur2 and cyclic Jacobi 8.5.3).
// Only +,-,*,/,sqrt, so host and device agree bit for bit.  The reference
// calls LAPACK through `eigen(b, sortby=nothing)` (elast.jl:51, DP.jl:65) and
// only ever uses V diag(f(λ)) V', which does not depend on eigenvalue order.
// ---------------------------------------------------------------------------
EP_HD void jacobi_t(double app, double aqq, double apq, double* c, double* s) {
    double tau = (aqq - app) / (2.0 * apq);
    double t;
    if (fabs(tau) > 1.0e150) t = 0.5 / tau;
    else t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
    *c = 1.0 / sqrt(1.0 + t * t);
    *s = t * (*c);
}

// A = [[a, b], [b, d]]: eigenvalues lam[0..1], eigenvectors as the columns of V (column-major).
EP_HD void eig_sym2(double a, double b, double d, double* lam, double* V) {
    if (b == 0.0) {
        lam[0] = a; lam[1] = d;
        V[0] = 1.0; V[1] = 0.0; V[2] = 0.0; V[3] = 1.0;
        return;
    }
    double c, s;
    jacobi_t(a, d, b, &c, &s);
    double t = s / c;
    lam[0] = a - t * b;
    lam[1] = d + t * b;
    V[0] = c;  V[1] = -s;   // column 0
    V[2] = s;  V[3] = c;    // column 1
}

// Symmetric 3x3 (column-major input, only the upper triangle read).
EP_HD void eig_sym3(const double* Ain, double* lam, double* V) {
    double A[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = (i <= j) ? Ain[i + 3 * j] : Ain[j + 3 * i];
    double W[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
    const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
    for (int sweep = 0; sweep < 32; ++sweep) {
        int rotated = 0;
        for (int k = 0; k < 3; ++k) {
            int p = P[k], q = Q[k];
            double apq = A[p][q];
            if (apq == 0.0) continue;
            if (fabs(apq) <= 1.0e-18 * (fabs(A[p][p]) + fabs(A[q][q]))) {
                A[p][q] = 0.0; A[q][p] = 0.0;
                continue;
            }
            rotated = 1;
            double c, s;
            jacobi_t(A[p][p], A[q][q], apq, &c, &s);
            double t = s / c;
            double app = A[p][p] - t * apq;
            double aqq = A[q][q] + t * apq;
            A[p][p] = app; A[q][q] = aqq; A[p][q] = 0.0; A[q][p] = 0.0;
            int r = 3 - p - q;
            double arp = A[r][p], arq = A[r][q];
            double nrp = c * arp - s * arq;
            double nrq = s * arp + c * arq;
            A[r][p] = nrp; A[p][r] = nrp; A[r][q] = nrq; A[q][r] = nrq;
            for (int i = 0; i < 3; ++i) {
                double wp = W[i][p], wq = W[i][q];
                W[i][p] = c * wp - s * wq;
                W[i][q] = s * wp + c * wq;
            }
        }
        if (!rotated) break;
    }
    for (int i = 0; i < 3; ++i) {
        lam[i] = A[i][i];
        for (int j = 0; j < 3; ++j) V[i + 3 * j] = W[i][j];
    }
}

// R = V diag(f) V' in the operation order of Julia's matmul2x2!/matmul3x3!
// for `n*diagm(f)*n'` (left product first; the exact zeros of diagm dropped).
template <int D>
EP_HD void vdvt(const double* V, const double* f, double* R) {
    double M[D * D];
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) M[i + D * j] = V[i + D * j] * f[j];
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
            double s = M[i] * V[j];
            for (int k = 1; k < D; ++k) s = s + M[i + D * k] * V[j + D * k];
            R[i + D * j] = s;
        }
}

// C = A*B for D x D column-major (Julia matmul2x2!/matmul3x3!: A11*B11 + A12*B21 + A13*B31).
template <int D>
EP_HD void matmul(const double* A, const double* B, double* C) {
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
            double s = A[i] * B[D * j];
            for (int k = 1; k < D; ++k) s = s + A[i + D * k] * B[k + D * j];
            C[i + D * j] = s;
        }
}

// C = A*B' (B transposed).
template <int D>
EP_HD void matmul_bt(const double* A, const double* B, double* C) {
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
            double s = A[i] * B[j];
            for (int k = 1; k < D; ++k) s = s + A[i + D * k] * B[j + D * k];
            C[i + D * j] = s;
        }
}

// C = A'*B (A transposed).
template <int D>
EP_HD void matmul_at(const double* A, const double* B, double* C) {
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
            double s = A[D * i] * B[D * j];
            for (int k = 1; k < D; ++k) s = s + A[k + D * i] * B[k + D * j];
            C[i + D * j] = s;
        }
}

// Symmetric eigen of a D x D tensor given as a full column-major matrix; the
// off-diagonal pairs are averaged (the reference's LAPACK call sees the
// rounding asymmetry of ΔF*b*ΔF'; the symmetric part is the tensor meant).
template <int D>
EP_HD void eig_sym(const double* A, double* lam, double* V) {
    if (D == 2) {
        eig_sym2(A[0], 0.5 * (A[2] + A[1]), A[3], lam, V);
    } else {
        double S[9];
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) S[i + 3 * j] = (i == j) ? A[i + 3 * j] : 0.5 * (A[i + 3 * j] + A[j + 3 * i]);
        eig_sym3(S, lam, V);
    }
}

// ---------------------------------------------------------------------------
// Voigt conversions (elast.jl:14-32, `mutate`): 2d (xx, yy, xy), 3d (xx, yy, zz, yz, xz, xy).
// ---------------------------------------------------------------------------
template <int D>
EP_HD void voigt_from_tensor(const double* T, double chi, double* v) {
    if (D == 2) {
        v[0] = T[0]; v[1] = T[3]; v[2] = chi * T[2];          // ϵ[1,1], ϵ[2,2], Χ ϵ[1,2]
    } else {
        v[0] = T[0]; v[1] = T[4]; v[2] = T[8];
        v[3] = chi * T[7];                                    // Χ ϵ[2,3]
        v[4] = chi * T[6];                                    // Χ ϵ[1,3]
        v[5] = chi * T[3];                                    // Χ ϵ[1,2]
    }
}

template <int D>
EP_HD void tensor_from_voigt(const double* v, double chi, double* T) {
    if (D == 2) {
        double o = chi * v[2];
        T[0] = v[0]; T[1] = o; T[2] = o; T[3] = v[1];
    } else {
        double xy = chi * v[5], xz = chi * v[4], yz = chi * v[3];
        T[0] = v[0]; T[1] = xy; T[2] = xz;
        T[3] = xy;   T[4] = v[1]; T[5] = yz;
        T[6] = xz;   T[7] = yz;   T[8] = v[2];
    }
}

// y = Del*x (row dot products in column order).
template <int S>
EP_HD void matvec(const double* Del, const double* x, double* y) {
    for (int i = 0; i < S; ++i) {
        double s = Del[i] * x[0];
        for (int j = 1; j < S; ++j) s = s + Del[i + S * j] * x[j];
        y[i] = s;
    }
}

// ---------------------------------------------------------------------------
// Shape functions.
// ---------------------------------------------------------------------------
// Node classes of the cubic B-spline basis (bsmpm.jl:63-76), decided by exact
// comparison of the node coordinate with the boundary table xB and h.
enum { BS_T1 = 0, BS_T2 = 1, BS_T3 = 2, BS_T4 = 3, BS_INVALID = 4 };

EP_HD int bspline_class(double xn, double xB0, double xB1, double dx) {
    if (xn == xB0) return BS_T1;
    if (xn == (xB0 + dx)) return BS_T2;
    if ((xB0 + dx) < xn && xn < (xB1 - dx)) return BS_T3;
    if (xn == (xB1 - dx)) return BS_T4;
    if (xn == xB1) return BS_T1;
    return BS_INVALID;
}

EP_HD void bs_t1(double x, double* f, double* df) {
    double F = 0.0, G = 0.0;
    if (-2.0 <= x && x <= -1.0) {
        F = (1.0 / 6.0) * ((x * x) * x) + x * x + 2.0 * x + (4.0 / 3.0);
        G = (3.0 / 6.0) * (x * x) + 2.0 * x + 2.0;
    } else if (-1.0 <= x && x <= 0.0) {
        F = (-1.0 / 6.0) * ((x * x) * x) + x + 1.0;
        G = (-3.0 / 6.0) * (x * x) + 1.0;
    } else if (0.0 <= x && x <= 1.0) {
        F = (1.0 / 6.0) * ((x * x) * x) - x + 1.0;
        G = (3.0 / 6.0) * (x * x) - 1.0;
    } else if (1.0 <= x && x <= 2.0) {
        F = (-1.0 / 6.0) * ((x * x) * x) + x * x - 2.0 * x + (4.0 / 3.0);
        G = (-3.0 / 6.0) * (x * x) + 2.0 * x - 2.0;
    }
    *f = F; *df = G;
}

EP_HD void bs_t2(double x, double* f, double* df) {
    double F = 0.0, G = 0.0;
    if (-1.0 <= x && x <= 0.0) {
        F = (-1.0 / 3.0) * ((x * x) * x) - (x * x) + (2.0 / 3.0);
        G = (-3.0 / 3.0) * (x * x) - 2.0 * x;
    } else if (0.0 <= x && x <= 1.0) {
        F = (1.0 / 2.0) * ((x * x) * x) - (x * x) + (2.0 / 3.0);
        G = (3.0 / 2.0) * (x * x) - 2.0 * x;
    } else if (1.0 <= x && x <= 2.0) {
        F = (-1.0 / 6.0) * ((x * x) * x) + x * x - 2.0 * x + (4.0 / 3.0);
        G = (-3.0 / 6.0) * (x * x) + 2.0 * x - 2.0;
    }
    *f = F; *df = G;
}

EP_HD void bs_t3(double x, double* f, double* df) {
    double F = 0.0, G = 0.0;
    if (-2.0 <= x && x <= -1.0) {
        F = (1.0 / 6.0) * ((x * x) * x) + x * x + 2.0 * x + (4.0 / 3.0);
        G = (3.0 / 6.0) * (x * x) + 2.0 * x + 2.0;
    } else if (-1.0 <= x && x <= 0.0) {
        F = (-1.0 / 2.0) * ((x * x) * x) - x * x + (2.0 / 3.0);
        G = (-3.0 / 2.0) * (x * x) - 2.0 * x;
    } else if (0.0 <= x && x <= 1.0) {
        F = (1.0 / 2.0) * ((x * x) * x) - (x * x) + (2.0 / 3.0);
        G = (3.0 / 2.0) * (x * x) - 2.0 * x;
    } else if (1.0 <= x && x <= 2.0) {
        F = (-1.0 / 6.0) * ((x * x) * x) + x * x - 2.0 * x + (4.0 / 3.0);
        G = (-3.0 / 6.0) * (x * x) + 2.0 * x - 2.0;
    }
    *f = F; *df = G;
}

EP_HD void bs_t4(double x, double* f, double* df) {
    double F = 0.0, G = 0.0;
    if (-2.0 <= x && x <= -1.0) {
        F = (1.0 / 6.0) * ((x * x) * x) + x * x + 2.0 * x + (4.0 / 3.0);
        G = (3.0 / 6.0) * (x * x) + 2.0 * x + 2.0;
    } else if (-1.0 <= x && x <= 0.0) {
        F = (-1.0 / 2.0) * ((x * x) * x) - x * x + (2.0 / 3.0);
        G = (-3.0 / 2.0) * (x * x) - 2.0 * x;
    } else if (0.0 <= x && x <= 1.0) {
        F = (1.0 / 3.0) * ((x * x) * x) - x * x + (2.0 / 3.0);
        G = (3.0 / 3.0) * (x * x) - 2.0 * x;
    }
    *f = F; *df = G;
}

// ϕ∂ϕ(ξ, xn, xB, Δx) (bsmpm.jl:63-78): value and derivative divided by Δx.
EP_HD void bspline(int cls, double xi, double dx, double* f, double* df) {
    double F = 0.0, G = 0.0;
    switch (cls) {
        case BS_T1: bs_t1(xi, &F, &G); break;
        case BS_T2: bs_t2(xi, &F, &G); break;
        case BS_T3: bs_t3(xi, &F, &G); break;
        case BS_T4: bs_t4(xi, &F, &G); break;
        default: break;
    }
    *f = F; *df = G / dx;
}

// S∂S(δx, h, lp): GIMP (gimpm.jl:1-14).
EP_HD void gimp(double dxp, double h, double lp, double* f, double* df) {
    double S = 0.0, G = 0.0;
    double a = fabs(dxp);
    if (a < lp) {
        S = 1.0 - ((4.0 * (dxp * dxp) + (2.0 * lp) * (2.0 * lp)) / ((8.0 * h) * lp));
        G = -((8.0 * dxp) / ((8.0 * h) * lp));
    } else if ((a >= lp) && (a <= (h - lp))) {
        S = 1.0 - (a / h);
        G = jsign(dxp) * (-1.0 / h);
    } else if ((a >= (h - lp)) && (a < (h + lp))) {
        double r = (h + lp) - a;
        S = (r * r) / ((4.0 * h) * lp);
        G = (-jsign(dxp) * r) / ((2.0 * h) * lp);
    }
    *f = S; *df = G;
}

// N∂N(δx, h): linear hat (smpm.jl:1-10).
EP_HD void hat(double dxp, double h, double* f, double* df) {
    if (-h < dxp && dxp <= 0.0) { *f = 1.0 + dxp / h; *df = 1.0 / h; }
    else if (0.0 < dxp && dxp <= h) { *f = 1.0 - dxp / h; *df = -1.0 / h; }
    else { *f = 0.0; *df = 0.0; }
}

// ---------------------------------------------------------------------------
// Material parameters of a point for the return maps (DP.jl:13-24): t = tan ϕ
// in 2d; s, c = sin ϕ, cos ϕ in 3d (computed once on the host with libm).
// ---------------------------------------------------------------------------
struct DPParam { double eta, etaB, xi; };

EP_HD DPParam dp_param2(double tphi, double coh) {
    DPParam r;
    double den = sqrt(9.0 + (12.0 * tphi) * tphi);
    r.eta = (3.0 * tphi) / den;
    r.etaB = (3.0 * 0.0) / sqrt(9.0 + (12.0 * 0.0) * 0.0);      // ψ = 0 (DP.jl:37)
    r.xi = (3.0 * coh) / den;
    return r;
}

EP_HD DPParam dp_param3(double sphi, double cphi, double coh) {
    DPParam r;
    const double sq3 = 0x1.bb67ae8584caap+0;                   // sqrt(3.0), correctly rounded
    r.eta = (6.0 * sphi) / (sq3 * (3.0 + sphi));
    r.etaB = (6.0 * 0.0) / (sq3 * (3.0 + 0.0));
    r.xi = ((6.0 * coh) * cphi) / (sq3 * (3.0 + sphi));
    return r;
}

// Closed-form Drucker-Prager return on Voigt stress s[NS] (DP.jl:33-62 and 69-98).
// Returns Δλ (0 when elastic) and adds to *ep1 (ϵpII[1,p]).
template <int NS>
EP_HD double dp_return(double* s, double ep2, double c0, double cr, double tphi, double sphi, double cphi,
                       double Hp, double Kc, double Gc, double* ep1) {
    double coh = c0 + Hp * ep2;
    if (coh < cr) coh = cr;
    const int D = (NS == 3) ? 2 : 3;
    double P, tauII, t0[NS];
    if (NS == 3) {
        P = (s[0] + s[1]) / 2.0;
        t0[0] = s[0] - P; t0[1] = s[1] - P; t0[2] = s[2] - 0.0;
        tauII = sqrt(0.5 * (t0[0] * t0[0] + t0[1] * t0[1]) + t0[2] * t0[2]);
    } else {
        P = (s[0] + s[1] + s[2]) / 3.0;
        for (int i = 0; i < 3; ++i) t0[i] = s[i] - P;
        for (int i = 3; i < 6; ++i) t0[i] = s[i] - 0.0;
        tauII = sqrt(0.5 * (t0[0] * t0[0] + t0[1] * t0[1] + t0[2] * t0[2]) + t0[3] * t0[3] + t0[4] * t0[4] + t0[5] * t0[5]);
    }
    DPParam m = (NS == 3) ? dp_param2(tphi, coh) : dp_param3(sphi, cphi, coh);
    double eta = m.eta, etaB = m.etaB, xi = m.xi;
    double sm = xi / eta;
    double tP = xi - eta * (xi / eta);
    double fs = tauII + eta * P - xi;
    double sq = sqrt(1.0 + eta * eta);
    double hh = tauII - tP - sq * (P - sm);
    double dlam = 0.0;
    if ((fs > 0.0 && P < sm) || (hh > 0.0 && P >= sm)) {
        double dl = fs / (Gc + (Kc * eta) * etaB);
        double Pn = P - (Kc * etaB) * dl;
        double tn = xi - eta * (P - (Kc * etaB) * dl);
        dlam = dl;
        double r = tn / tauII;
        for (int i = 0; i < NS; ++i) s[i] = t0[i] * r + (i < D ? Pn : 0.0);
        *ep1 = *ep1 + dl * sqrt((1.0 / 3.0) + (2.0 / 9.0) * (etaB * etaB));
    }
    if (hh <= 0.0 && P >= sm) {
        double dl = (P - sm) / Kc;
        double Pn = sm - P;
        dlam = dl;
        double r = 0.0 / tauII;
        for (int i = 0; i < NS; ++i) s[i] = t0[i] * r + (i < D ? Pn : 0.0);
        const double sq2 = 0x1.6a09e667f3bcdp+0;                  // sqrt(2.0)
        *ep1 = *ep1 + (sq2 * dl) / 3.0;
    }
    return dlam;
}

// J2 yield function (J2.jl:1-20): f = sqrt(2 J2) - κ and the flow direction n.
// In 2d the mean stress ignores σzz, as in the reference (J2.jl:3-4).
template <int NS>
EP_HD double j2_yield(const double* s, double kappa, double* n) {
    double P, J2, x[NS];
    if (NS == 3) {
        P = (s[0] + s[1]) / 2.0;
        x[0] = s[0] - P; x[1] = s[1] - P; x[2] = s[2] - 0.0;
        J2 = 0.5 * (x[0] * x[0] + x[1] * x[1] + 2.0 * (x[2] * x[2]));
    } else {
        P = (s[0] + s[1] + s[2]) / 3.0;
        for (int i = 0; i < 3; ++i) x[i] = s[i] - P;
        for (int i = 3; i < 6; ++i) x[i] = s[i] - 0.0;
        J2 = 0.5 * (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + 2.0 * (x[3] * x[3]) + 2.0 * (x[4] * x[4]) + 2.0 * (x[5] * x[5]));
    }
    double xn = sqrt(2.0 * J2);
    for (int i = 0; i < NS; ++i) n[i] = x[i] / xn;
    return xn - kappa;
}

// J2 cutting-plane return (J2.jl:21-76) with the reference's intended fields:
// cohesion from the point's c0/cr, γ written to ϵpII[1,p] (the reference writes
// ϵpII[p,1], J2.jl:40,70), at most 19 iterations, ftol = 1e-9.  Returns 1 when
// the point yielded.  Δλ is left untouched, as in the reference.
template <int NS>
EP_HD int j2_return(double* s, double ep2, double c0, double cr, double Hp, const double* Del, double* ep1) {
    double kappa = c0 + Hp * ep2;
    if (!(kappa >= cr)) kappa = (kappa != kappa) ? kappa : cr;    // max(cr, ·)
    double n[NS];
    double f = j2_yield<NS>(s, kappa, n);
    if (!(f > 0.0)) return 0;
    double g0 = ep2;
    int it = 1;
    while (fabs(f) > 1.0e-9 && it < 20) {
        double row[NS];
        for (int j = 0; j < NS; ++j) {
            double a = n[0] * Del[NS * j];
            for (int i = 1; i < NS; ++i) a = a + n[i] * Del[i + NS * j];
            row[j] = a;
        }
        double den = row[0] * n[0];
        for (int j = 1; j < NS; ++j) den = den + row[j] * n[j];
        double dl = f / den;
        for (int i = 0; i < NS; ++i) {
            double a = (dl * Del[i]) * n[0];
            for (int j = 1; j < NS; ++j) a = a + (dl * Del[i + NS * j]) * n[j];
            s[i] = s[i] - a;
        }
        g0 = g0 + dl;
        kappa = c0 + Hp * g0;
        if (!(kappa >= cr)) kappa = (kappa != kappa) ? kappa : cr;
        f = j2_yield<NS>(s, kappa, n);
        it = it + 1;
    }
    *ep1 = g0;
    return 1;
}

// ---------------------------------------------------------------------------
// Mohr-Coulomb return, 2d plane strain (plast/retmap/MCRetMap.jl:1-54).  The reference's function is
// commented out of its dispatcher (plast.jl:14-15) and reads fields the Point no longer has (mpts.ϕ,
// mpts.c₀ at :11-12 and mpts.c0 at :33); it is restated with the Solid's fields and otherwise as
// written: ψ = 0.5° (:3), H = cos ϕ Hp (:11), c = max(c₀ + Hp ϵII, cᵣ) with ϵII the softening input
// ϵpII[2,p] plus the plastic strain of this return (:12-13, :32-34), the yield function on the
// in-plane Mohr circle f = τII + σm sin ϕ − c cos ϕ (:14-15), and the non-associated cutting plane
// Δγ = f/(H + ∂fᵀ Del ∂g), Δσ = Δγ Del ∂g, Δϵ += Del \ Δσ, σ −= Δσ while |f| > 1e-6 (:20-43).
// Returns 1 when the point yielded (ϵII is written to *ep1, as mpts.ϵpII[p] = ϵII at :45, the same
// row the J2 restatement writes), 0 when elastic, -1 after more than 1e4 iterations (the reference
// throws, :38-41).  Δλ is not written, as in the reference.
// ---------------------------------------------------------------------------
EP_HD double mc_tau(const double* s, double* sm) {
    *sm = 0.5 * (s[0] + s[1]);
    const double d = s[0] - s[1];
    return sqrt(0.25 * (d * d) + s[2] * s[2]);
}

EP_HD int mc_return(double* s, double ep2, double c0, double cr, double sphi, double cphi, double Hp,
                    const double* Del, const double* DelLU, const int* piv, double* ep1) {
    const double spsi = 0x1.1df37c4954c21p-7;        // sin(0.5*π/180.0), MCRetMap.jl:3
    const double H = cphi * Hp;
    const double e0 = ep2;
    double c = c0 + Hp * e0;
    if (c < cr) c = cr;
    double sm, tII = mc_tau(s, &sm);
    double f = (tII + sm * sphi) - c * cphi;
    if (!(f > 0.0)) return 0;
    double g = e0, de[3] = {0.0, 0.0, 0.0};
    int it = 0;
    while (fabs(f) > 1.0e-6) {
        it = it + 1;
        const double a = (s[0] - s[1]) / (4.0 * tII);
        const double df[3] = {a + sphi / 2.0, -(s[0] - s[1]) / (4.0 * tII) + sphi / 2.0, s[2] / tII};
        const double dg[3] = {a + spsi / 2.0, -(s[0] - s[1]) / (4.0 * tII) + spsi / 2.0, s[2] / tII};
        // ∂fᵀ Del ∂g as (∂fᵀ Del) ∂g
        double den = 0.0;
        for (int j = 0; j < 3; ++j) {
            const double r = (df[0] * Del[3 * j] + df[1] * Del[1 + 3 * j]) + df[2] * Del[2 + 3 * j];
            den = (j == 0) ? r * dg[0] : den + r * dg[j];
        }
        const double dgam = f / (H + den);
        double ds[3], x[3];
        for (int i = 0; i < 3; ++i)
            ds[i] = ((dgam * Del[i]) * dg[0] + (dgam * Del[i + 3]) * dg[1]) + (dgam * Del[i + 6]) * dg[2];
        lu_solve<3>(DelLU, piv, ds, x);
        for (int i = 0; i < 3; ++i) de[i] = de[i] + x[i];
        g = e0 + sqrt((2.0 / 3.0) * ((de[0] * de[0] + de[1] * de[1]) + 2.0 * (de[2] * de[2])));
        c = c0 + Hp * g;
        if (c < cr) c = cr;
        for (int i = 0; i < 3; ++i) s[i] = s[i] - ds[i];
        tII = mc_tau(s, &sm);
        f = (tII + sm * sphi) - c * cphi;
        if (it > 10000) return -1;
    }
    *ep1 = g;
    return 1;
}

// ---------------------------------------------------------------------------
// Modified Cam-Clay return (camC.zip: camC/camCmodRetMap.jl, after De Souza Neto, Perić & Owen 2008),
// the reference's archived Cam-Clay variant that its dispatcher names (plast.jl:28-29, commented
// out).  Constants as written there: χ = 3/2, Pt = Kc/10, a0 = Pt + Kc/10, β = 1, M from ϕcs = 20°,
// ζ = 0 (a = a0 exp(−ζ ϵpV)), at most 19 cutting-plane iterations while |f| > 1e-6.  Restated:
//  * the yield function is the ellipse f = (P − Pt + a)²/b² + (q/M)² − a² (b = β when P < Pt − a,
//    else 1) — the form the variant's derivative (∂f/∂P = 2(P − Pt + a)/b²) and its envelope plot
//    use; its camCYield writes (P + Pt − a), which puts the ellipse's centre on the tension side;
//  * P, q and n as camCParam forms them (2d: P = (σxx + σyy)/2, J2 with 2σxy²), the flow direction
//    ∂f/∂σ = ∂f/∂P/3 [1 1 (1) 0…] + √χ ∂f/∂q n as written (its 1/3 also in 2d);
//  * ϵpII and ϵpV of the Solid: γ starts from the softening input ϵpII[2,p] and is written to
//    *ep1 (the row the J2 and MC restatements write), ϵpV is read and written through *epV.
// Returns 1 when the point yielded, 0 when elastic.  Δλ is not written, as in the reference.
// ---------------------------------------------------------------------------
template <int NS>
EP_HD double camc_param(const double* s, double* q, double* n) {
    const double chi = 3.0 / 2.0;
    double P, J2, x[NS];
    if (NS == 3) {
        P = (s[0] + s[1]) / 2.0;
        x[0] = s[0] - P; x[1] = s[1] - P; x[2] = s[2] - 0.0;
        J2 = 0.5 * ((x[0] * x[0] + x[1] * x[1]) + 2.0 * (x[2] * x[2]));
    } else {
        P = ((s[0] + s[1]) + s[2]) / 3.0;
        for (int i = 0; i < 3; ++i) x[i] = s[i] - P;
        for (int i = 3; i < 6; ++i) x[i] = s[i] - 0.0;
        J2 = 0.5 * (((((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2]) + 2.0 * (x[3] * x[3])) + 2.0 * (x[4] * x[4])) +
                    2.0 * (x[5] * x[5]));
    }
    const double xn = sqrt(2.0 * J2);
    for (int i = 0; i < NS; ++i) n[i] = x[i] / xn;
    *q = sqrt(chi) * xn;
    return P;
}

EP_HD double camc_yield(double P, double q, double Pt, double a, double beta, double M, double* b) {
    *b = (P < Pt - a) ? beta : 1.0;
    const double u = P - Pt + a, w = q / M;
    return ((1.0 / ((*b) * (*b))) * (u * u) + w * w) - a * a;
}

template <int NS>
EP_HD int camc_return(double* s, double ep2, double* epV, double Kc, const double* Del, double* ep1) {
    const double sqchi = 0x1.3988e1409212ep+0;          // sqrt(3/2)
    const double Pt = Kc / 10.0;
    const double a0 = Pt + Kc / 10.0;
    const double beta = 1.0 / 1.0;
    const double M = 0x1.8b4b7e887abd4p-1;               // 6 sin ϕcs / (3 − sin ϕcs), ϕcs = 20.0*π/180.0
    const double zeta = 0.0;
    double a = a0 * ep_exp(-zeta * (*epV));
    double q, n[NS], b;
    double P = camc_param<NS>(s, &q, n);
    double f = camc_yield(P, q, Pt, a, beta, M, &b);
    if (!(f > 0.0)) return 0;
    double ev = *epV, g = ep2;
    int eta = 1;
    while (fabs(f) > 1.0e-6 && eta < 20) {
        const double dfdp = (2.0 / (b * b)) * (P - Pt + a);
        const double dfdq = (2.0 * q) / (M * M);
        double df[NS];
        for (int i = 0; i < NS; ++i) {
            const bool normal = i < (NS == 3 ? 2 : 3);
            df[i] = normal ? (dfdp * 1.0) / 3.0 + (sqchi * dfdq) * n[i] : (sqchi * dfdq) * n[i];
        }
        // Δλ = f / (∂fᵀ Del ∂f), (∂fᵀ Del) ∂f
        double den = 0.0;
        for (int j = 0; j < NS; ++j) {
            double r = df[0] * Del[NS * j];
            for (int i = 1; i < NS; ++i) r = r + df[i] * Del[i + NS * j];
            den = (j == 0) ? r * df[0] : den + r * df[j];
        }
        const double dl = f / den;
        for (int i = 0; i < NS; ++i) {
            double r = (dl * Del[i]) * df[0];
            for (int j = 1; j < NS; ++j) r = r + (dl * Del[i + NS * j]) * df[j];
            s[i] = s[i] - r;
        }
        ev = ev + dl * dfdp;
        g = g + dl * dfdq;
        a = a0 * ep_exp(-zeta * ev);
        P = camc_param<NS>(s, &q, n);
        f = camc_yield(P, q, Pt, a, beta, M, &b);
        eta = eta + 1;
    }
    *epV = ev;
    *ep1 = g;
    return 1;
}

// ϵ = tensor(Del \ σ, ½) after a return (MCRetMap.jl:44, camCmodRetMap.jl: mpD.ϵ = mutate(Del\σ, 0.5)).
template <int D>
EP_HD void strain_from_stress(const double* s, const double* DelLU, const int* piv, double* eps) {
    const int NS = (D == 2) ? 3 : 6;
    double x[NS];
    lu_solve<NS>(DelLU, piv, s, x);
    tensor_from_voigt<D>(x, 0.5, eps);
}

// Finite-strain elastic predictor (elast.jl:45-56): b <- ΔF b ΔF', ϵ = ½ log b,
// τ = Del voigt(ϵ, 2).
template <int D>
EP_HD void finite_elast(const double* dF, double* b, double* eps, double* tau, const double* Del) {
    const int NS = (D == 2) ? 3 : 6;
    double T[D * D], bn[D * D], lam[D], V[D * D], L[D], R[D * D], e[NS];
    matmul<D>(dF, b, T);
    matmul_bt<D>(T, dF, bn);
    for (int i = 0; i < D * D; ++i) b[i] = bn[i];
    eig_sym<D>(bn, lam, V);
    for (int i = 0; i < D; ++i) L[i] = ep_log(lam[i]);
    vdvt<D>(V, L, R);
    for (int i = 0; i < D * D; ++i) eps[i] = 0.5 * R[i];
    voigt_from_tensor<D>(eps, 2.0, e);
    matvec<NS>(Del, e, tau);
}

// After a finite-strain return: ϵ = tensor(Del \ τ, ½), b = V diag(exp 2λ) V' (DP.jl:63-66).
template <int D>
EP_HD void finite_rebuild_b(const double* tau, const double* DelLU, const int* piv, double* eps, double* b) {
    const int NS = (D == 2) ? 3 : 6;
    double x[NS], lam[D], V[D * D], E[D];
    lu_solve<NS>(DelLU, piv, tau, x);
    tensor_from_voigt<D>(x, 0.5, eps);
    if (D == 2) eig_sym2(eps[0], eps[2], eps[3], lam, V);
    else eig_sym3(eps, lam, V);
    for (int i = 0; i < D; ++i) E[i] = ep_exp(2.0 * lam[i]);
    vdvt<D>(V, E, b);
}

// Infinitesimal elastic predictor (elast.jl:69-80): ϵ = sym(ΔF) - I,
// ω = skew(ΔF), σJ = σ ω' + σ' ω (identically zero for symmetric σ),
// σ += Del voigt(ϵ, 2) + voigt(σJ, 1).  jaumann=1 adds ωσ - σω instead.
template <int D>
EP_HD void infinitesimal_elast(const double* dF, double* sig, double* eps, double* w, double* sJ,
                               const double* Del, int jaumann) {
    const int NS = (D == 2) ? 3 : 6;
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
            double a = dF[i + D * j], bt = dF[j + D * i];
            eps[i + D * j] = 0.5 * (a + bt) - (i == j ? 1.0 : 0.0);
            w[i + D * j] = 0.5 * (a - bt);
        }
    double S[D * D], A1[D * D], A2[D * D], e[NS], de[NS], sj[NS];
    tensor_from_voigt<D>(sig, 1.0, S);
    if (!jaumann) {
        matmul_bt<D>(S, w, A1);       // σ ω'
        matmul_at<D>(S, w, A2);       // σ' ω
    } else {
        matmul<D>(w, S, A1);          // ω σ
        matmul<D>(S, w, A2);
        for (int i = 0; i < D * D; ++i) A2[i] = -A2[i];
    }
    for (int i = 0; i < D * D; ++i) sJ[i] = A1[i] + A2[i];
    voigt_from_tensor<D>(eps, 2.0, e);
    matvec<NS>(Del, e, de);
    voigt_from_tensor<D>(sJ, 1.0, sj);
    for (int i = 0; i < NS; ++i) sig[i] = sig[i] + (de[i] + sj[i]);
}

}  // namespace ep
