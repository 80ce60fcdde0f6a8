// eporacle.cpp -- CPU FP64 restatement of ElastoPlasm's explicit MPM step.
//
// TEST INFRASTRUCTURE ONLY (the checker of the GPU library; see eporacle.h).
//
// One routine per reference kernel, in the reference's call order
// (workflow/worflow.jl:23-93), on Julia-layout column-major arrays:
//   tplgy      p2e2n_{2,3}d              workflow/shpfun/tplgy.jl:43-96
//   shpfun     bsmpm/gimpm/smpm_{2,3}d   workflow/shpfun/basis/*.jl, shpfun.jl:74-88
//   delta_np   Δnp_nd / Dij_nd           workflow/shpfun/misc.jl:1-28
//   p2n        transform + std/tpic/apic workflow/mapsto/p2n.jl:12-21, 135-296
//   Bij        APIC affine matrix        workflow/mapsto/Bij.jl:14-26 (called by n2p.jl:60-62, 72-74)
//   solve      euler                     workflow/mapsto/solve.jl:14-63
//   n2p        picflip_n2p + augm        workflow/mapsto/n2p.jl:14-76, augm.jl:13-53
//   update     deform/domain/ΔJ{n,s,p}   workflow/elastoplast/update/*.jl
//   elast      finite/infinitesimal      workflow/elastoplast/elast/elast.jl:45-124
//   plast      nonlocal + DP/J2/MC/camC  workflow/elastoplast/plast/{plast,nonlocal}.jl, retmap/*.jl (+ camC.zip)
//   run        get_dt/get_g/spacetime    program/utils/physics.jl:21-90, worflow.jl:27-39, 73-85
// The per-point constitutive arithmetic (eigen, log/exp, DP/J2 returns) is the
// shared header ep_scalar.h, which the GPU kernels compile too.
#include "eporacle.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../elastoplasm.jl_gb300/csrc/ep_scalar.h"

using std::vector;

struct eporacle {
    ep_cfg cfg;
    ep_cmpr cm;
    int dim, nstr, nn;
    int64_t nel[4], nno[4], Nn, Ne, Np;
    double h[3], x0[3];
    vector<double> xn;      // dim x Nn
    vector<double> xB;      // dim x 2
    vector<uint8_t> bcs;    // dim x Nn
    vector<int64_t> e2n;    // nn x Ne
    int nnel[3];
    // nodal
    vector<double> mi, oobf, a, pn, vn, dJn;
    // points
    vector<double> vmax, x, l0, l, n0, n, Om0, Om, dJ, J, u, v, pp, rho0, rho, c0, cr, phi, dlam,
        epII, epV, sig, tau, dv, du, dF, F, b, eps, w, sJ;
    vector<double> tphi, sphi, cphi;
    vector<int64_t> p2e, p2n;
    vector<double> phidphi;  // nn x Np x (dim+1)
    vector<double> dnp;      // nn x dim x Np
    vector<double> B, Dm;    // dim x dim x Np: APIC's Bᵢⱼ, Dᵢⱼ
    double DelLU[36];
    int piv[6];
    int threads = 1;
    int nonconverged = 0;   // a return map exceeded its iteration limit in the last retmap
    int err = 0;
    std::string msg;
};

static int fail(eporacle* o, int code, const char* m) {
    o->err = code;
    o->msg = m;
    return code;
}

// ---------------------------------------------------------------- e2n (e2n.jl:20-78)
static void build_e2n(eporacle* o) {
    const int64_t nn = o->nn;
    o->e2n.assign((size_t)nn * o->Ne, 0);
    if (o->dim == 2) {
        int64_t nx = o->nno[0], nz = o->nno[1];
        int64_t iel = 0;
        for (int64_t i0 = 1; i0 <= o->nel[0]; ++i0)
            for (int64_t j0 = 1; j0 <= o->nel[1]; ++j0) {
                int s = 0;
                for (int i = -1; i <= 2; ++i)
                    for (int j = -1; j <= 2; ++j) {
                        int64_t jj = j0 + j, ii = i0 + i;
                        int64_t id = (jj >= 1 && jj <= nz && ii >= 1 && ii <= nx) ? jj + nz * (ii - 1) : 0;
                        o->e2n[s + nn * iel] = id;
                        ++s;
                    }
                ++iel;
            }
    } else {
        int64_t nx = o->nno[0], ny = o->nno[1], nz = o->nno[2];
        int64_t iel = 0;
        for (int64_t k0 = 1; k0 <= o->nel[1]; ++k0)
            for (int64_t i0 = 1; i0 <= o->nel[0]; ++i0)
                for (int64_t j0 = 1; j0 <= o->nel[2]; ++j0) {
                    int s = 0;
                    for (int k = -1; k <= 2; ++k)
                        for (int i = -1; i <= 2; ++i)
                            for (int j = -1; j <= 2; ++j) {
                                int64_t jj = j0 + j, ii = i0 + i, kk = k0 + k;
                                bool ok = jj >= 1 && jj <= nz && ii >= 1 && ii <= nx && kk >= 1 && kk <= ny;
                                o->e2n[s + nn * iel] = ok ? jj + nz * (ii - 1) + nz * nx * (kk - 1) : 0;
                                ++s;
                            }
                    ++iel;
                }
    }
}

// ---------------------------------------------------------------- tplgy (tplgy.jl:43-96)
static int tplgy(eporacle* o) {
    const int d = o->dim;
    for (int64_t p = 0; p < o->Np; ++p) {
        double e[3];
        for (int i = 0; i < d; ++i) {
            // a non-finite position has no element (the reference's Int conversion throws there)
            if (!std::isfinite(o->x[i + d * p])) return fail(o, EP_ERR_NONFINITE, "non-finite point position");
            double f = ep::jfld(o->x[i + d * p] - o->x0[i], o->h[i]);
            double hi = (double)(o->nel[i] - 1);
            e[i] = f < 0.0 ? 0.0 : (f > hi ? hi : f);
        }
        int64_t el;
        if (d == 2) el = (int64_t)llround(1.0 + e[1] + (double)o->nel[1] * e[0]);
        else el = (int64_t)llround(1.0 + e[2] + (double)o->nel[2] * e[0] + (double)o->nel[2] * (double)o->nel[0] * e[1]);
        for (int k = 0; k < o->nn; ++k) o->p2n[k + o->nn * p] = o->e2n[k + o->nn * (el - 1)];
        o->p2e[p] = el;
    }
    return 0;
}

static inline double PHI(const eporacle* o, int k, int64_t p, int c) {
    return o->phidphi[k + (int64_t)o->nn * p + (int64_t)o->nn * o->Np * c];
}

// ---------------------------------------------------------------- shape functions
static int shpfun(eporacle* o) {
    const int d = o->dim, nn = o->nn;
    const int64_t Np = o->Np;
    std::fill(o->phidphi.begin(), o->phidphi.end(), 0.0);
    int bad = 0;
#pragma omp parallel for num_threads(o->threads) reduction(| : bad) schedule(static)
    for (int64_t p = 0; p < Np; ++p) {
        for (int k = 0; k < nn; ++k) {
            int64_t no = o->p2n[k + nn * p];
            if (no == 0) continue;
            double f[3], g[3];
            for (int i = 0; i < d; ++i) {
                double xp = o->x[i + d * p], xq = o->xn[i + d * (no - 1)];
                if (o->cfg.basis == EP_BASIS_BSMPM) {
                    double xi = (xp - xq) / o->h[i];
                    int cls = ep::bspline_class(xq, o->xB[i], o->xB[i + d], o->h[i]);
                    if (cls == ep::BS_INVALID) bad = 1;
                    ep::bspline(cls, xi, o->h[i], &f[i], &g[i]);
                } else if (o->cfg.basis == EP_BASIS_GIMPM) {
                    ep::gimp(xp - xq, o->h[i], o->l[i + d * p], &f[i], &g[i]);
                } else {
                    ep::hat(xp - xq, o->h[i], &f[i], &g[i]);
                }
            }
            double* P = &o->phidphi[0];
            const int64_t s1 = nn, s2 = (int64_t)nn * Np;
            if (d == 2) {
                P[k + s1 * p + s2 * 0] = f[0] * f[1];
                P[k + s1 * p + s2 * 1] = g[0] * f[1];
                P[k + s1 * p + s2 * 2] = f[0] * g[1];
            } else {
                P[k + s1 * p + s2 * 0] = f[0] * f[1] * f[2];
                P[k + s1 * p + s2 * 1] = g[0] * f[1] * f[2];
                P[k + s1 * p + s2 * 2] = f[0] * g[1] * f[2];
                P[k + s1 * p + s2 * 3] = f[0] * f[1] * g[2];
            }
        }
    }
    if (bad) return fail(o, EP_ERR_INVALID_POSITION, "Invalid position: B-spline node outside xB table");
    if (o->cfg.trsfr == EP_TRSFR_TPIC) {
        for (int64_t p = 0; p < Np; ++p)
            for (int k = 0; k < nn; ++k) {
                int64_t no = o->p2n[k + nn * p];
                if (no == 0) continue;
                for (int i = 0; i < d; ++i)
                    o->dnp[k + nn * i + (int64_t)nn * d * p] = o->xn[i + d * (no - 1)] - o->x[i + d * p];
            }
    } else if (o->cfg.trsfr == EP_TRSFR_APIC) {
        // Dij_nd (misc.jl:15-28): Δnp for every node, Dᵢⱼ assigned (not summed) node by node
        for (int64_t p = 0; p < Np; ++p)
            for (int k = 0; k < nn; ++k) {
                int64_t no = o->p2n[k + nn * p];
                if (no == 0) continue;
                double dl[3];
                for (int i = 0; i < d; ++i) {
                    dl[i] = o->xn[i + d * (no - 1)] - o->x[i + d * p];
                    o->dnp[k + nn * i + (int64_t)nn * d * p] = dl[i];
                }
                const double N = PHI(o, k, p, 0);
                for (int j = 0; j < d; ++j)
                    for (int i = 0; i < d; ++i) o->Dm[i + d * j + (int64_t)d * d * p] = N * (dl[i] * dl[j]);
            }
    }
    return 0;
}


#ifdef _OPENMP
#define ATOMIC_ADD(ref, val) _Pragma("omp atomic") ref += (val)
#else
#define ATOMIC_ADD(ref, val) ref += (val)
#endif

// ---------------------------------------------------------------- P2G (p2n.jl:135-191, 284-296)
static void p2n(eporacle* o, const double* g) {
    const int d = o->dim, nn = o->nn, ns = o->nstr;
    const int64_t Np = o->Np;
    if (o->cfg.deform == EP_DEFORM_FINITE)
        for (int64_t p = 0; p < Np; ++p)
            for (int c = 0; c < ns; ++c) o->sig[c + ns * p] = o->tau[c + ns * p] / o->J[p];
    std::fill(o->mi.begin(), o->mi.end(), 0.0);
    std::fill(o->pn.begin(), o->pn.end(), 0.0);
    std::fill(o->oobf.begin(), o->oobf.end(), 0.0);
    const bool tpic = o->cfg.trsfr == EP_TRSFR_TPIC, apic = o->cfg.trsfr == EP_TRSFR_APIC;
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p) {
        double ms = o->rho[p] * o->Om[p], Om = o->Om[p];
        const double* s = &o->sig[ns * p];
        const double* vp = &o->v[d * p];
        const double* gv = &o->dv[d * d * p];
        double C[9];   // APIC: Bᵢⱼ D⁻¹ (the same for every node of the point)
        if (apic) {
            if (d == 2) ep::apic_bdinv<2>(&o->B[4 * p], &o->Dm[4 * p], C);
            else ep::apic_bdinv<3>(&o->B[9 * p], &o->Dm[9 * p], C);
        }
        for (int k = 0; k < nn; ++k) {
            int64_t no = o->p2n[k + nn * p];
            if (no == 0) continue;
            int64_t q = no - 1;
            double N = PHI(o, k, p, 0);
            if (d == 2) {
                double Nx = PHI(o, k, p, 1), Ny = PHI(o, k, p, 2);
                double sxx = s[0], syy = s[1], sxy = s[2];
                ATOMIC_ADD(o->mi[q], N * ms);
                if (apic) {
                    const double dl[2] = {o->dnp[k + (int64_t)nn * 2 * p], o->dnp[k + nn + (int64_t)nn * 2 * p]};
                    ATOMIC_ADD(o->pn[0 + 2 * q], N * ms * (vp[0] + ep::apic_row<2>(C, 0, dl)));
                    ATOMIC_ADD(o->pn[1 + 2 * q], N * ms * (vp[1] + ep::apic_row<2>(C, 1, dl)));
                } else if (!tpic) {
                    double px = ms * vp[0], py = ms * vp[1];
                    ATOMIC_ADD(o->pn[0 + 2 * q], N * px);
                    ATOMIC_ADD(o->pn[1 + 2 * q], N * py);
                } else {
                    const double* D = &o->dnp[k + nn * 0 + (int64_t)nn * 2 * p];
                    double dx = D[0], dy = D[nn];
                    // ∇v[i,j] at gv[i + 2 j]
                    ATOMIC_ADD(o->pn[0 + 2 * q], N * ms * (vp[0] + gv[0] * dx + gv[2] * dy));
                    ATOMIC_ADD(o->pn[1 + 2 * q], N * ms * (vp[1] + gv[1] * dx + gv[3] * dy));
                }
                ATOMIC_ADD(o->oobf[0 + 2 * q], -(Om * (Nx * sxx + Ny * sxy)));
                ATOMIC_ADD(o->oobf[1 + 2 * q], -(Om * (Nx * sxy + Ny * syy) - N * (ms * g[1])));
            } else {
                double Nx = PHI(o, k, p, 1), Ny = PHI(o, k, p, 2), Nz = PHI(o, k, p, 3);
                double sxx = s[0], syy = s[1], szz = s[2], syx = s[5], szy = s[3], szx = s[4];
                ATOMIC_ADD(o->mi[q], N * ms);
                if (apic) {
                    const int64_t b = k + (int64_t)nn * 3 * p;
                    const double dl[3] = {o->dnp[b], o->dnp[b + nn], o->dnp[b + 2 * nn]};
                    ATOMIC_ADD(o->pn[0 + 3 * q], N * ms * (vp[0] + ep::apic_row<3>(C, 0, dl)));
                    ATOMIC_ADD(o->pn[1 + 3 * q], N * ms * (vp[1] + ep::apic_row<3>(C, 1, dl)));
                    ATOMIC_ADD(o->pn[2 + 3 * q], N * ms * (vp[2] + ep::apic_row<3>(C, 2, dl)));
                } else if (!tpic) {
                    double px = ms * vp[0], py = ms * vp[1], pz = ms * vp[2];
                    ATOMIC_ADD(o->pn[0 + 3 * q], N * px);
                    ATOMIC_ADD(o->pn[1 + 3 * q], N * py);
                    ATOMIC_ADD(o->pn[2 + 3 * q], N * pz);
                } else {
                    const double* D = &o->dnp[k + (int64_t)nn * 3 * p];
                    double dx = D[0], dy = D[nn], dz = D[2 * nn];
                    ATOMIC_ADD(o->pn[0 + 3 * q], N * ms * (vp[0] + gv[0] * dx + gv[3] * dy + gv[6] * dz));
                    ATOMIC_ADD(o->pn[1 + 3 * q], N * ms * (vp[1] + gv[1] * dx + gv[4] * dy + gv[7] * dz));
                    ATOMIC_ADD(o->pn[2 + 3 * q], N * ms * (vp[2] + gv[2] * dx + gv[5] * dy + gv[8] * dz));
                }
                ATOMIC_ADD(o->oobf[0 + 3 * q], -(Om * (Nx * sxx + Ny * syx + Nz * szx)));
                ATOMIC_ADD(o->oobf[1 + 3 * q], -(Om * (Nx * syx + Ny * syy + Nz * szy)));
                ATOMIC_ADD(o->oobf[2 + 3 * q], -(Om * (Nx * szx + Ny * szy + Nz * szz) - N * (ms * g[2])));
            }
        }
    }
}

// ---------------------------------------------------------------- grid update (solve.jl:14-63)
static void solve(eporacle* o, double dt) {
    const int d = o->dim;
    const double eta = o->cfg.damping;
    std::fill(o->a.begin(), o->a.end(), 0.0);
    std::fill(o->vn.begin(), o->vn.end(), 0.0);
    for (int64_t q = 0; q < o->Nn; ++q) {
        if (o->mi[q] == 0.0) continue;
        for (int i = 0; i < d; ++i) {
            if (o->bcs[i + d * q]) {
                o->a[i + d * q] = 0.0;
                o->vn[i + d * q] = 0.0;
            } else {
                double m = 1.0 / o->mi[q];
                double nrm = (d == 2) ? ep::jnorm<2>(&o->oobf[d * q]) : ep::jnorm<3>(&o->oobf[d * q]);
                double D = eta * nrm * ep::jsign(o->pn[i + d * q] * m);
                if (fabs(o->pn[i + d * q] * m) >= 1.0e-3) o->oobf[i + d * q] = o->oobf[i + d * q] - D;
                o->a[i + d * q] = o->oobf[i + d * q] * m;
                o->vn[i + d * q] = (o->pn[i + d * q] + dt * o->oobf[i + d * q]) * m;
            }
        }
    }
}

// ---------------------------------------------------------------- G2P (n2p.jl:14-76, augm.jl:13-53)
static void n2p(eporacle* o, double dt) {
    const int d = o->dim, nn = o->nn;
    const int64_t Np = o->Np;
    const double Cpf = o->cfg.C_pf;
    for (int i = 0; i < d; ++i) {
        double vm = o->vmax[i];
#pragma omp parallel for num_threads(o->threads) schedule(static) reduction(max : vm) if (o->threads > 1)
        for (int64_t p = 0; p < Np; ++p) {
            double vpic = 0.0;
            for (int k = 0; k < nn; ++k) {
                int64_t no = o->p2n[k + nn * p];
                if (no == 0) continue;
                vpic = vpic + PHI(o, k, p, 0) * o->vn[i + d * (no - 1)];
            }
            double aflip = 0.0;
            for (int k = 0; k < nn; ++k) {
                int64_t no = o->p2n[k + nn * p];
                if (no == 0) continue;
                aflip = aflip + PHI(o, k, p, 0) * o->a[i + d * (no - 1)];
            }
            double& vp = o->v[i + d * p];
            vp = Cpf * (vp + dt * aflip) + (1.0 - Cpf) * vpic;
            o->x[i + d * p] = o->x[i + d * p] + dt * vpic;
            double av = fabs(vp);
            if (!(vm >= av)) vm = av;   // max(vmax, |v|) with NaN propagation
        }
        o->vmax[i] = vm;
    }
    if (o->cfg.trsfr == EP_TRSFR_APIC) {
        // Bij (Bij.jl:14-26) from the grid velocities of the solve, before the mUSL re-projection
        // replaces them (n2p.jl:60-62); Δnp is the step-start offset of shpfun
        for (int64_t p = 0; p < Np; ++p) {
            double Bp[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int k = 0; k < nn; ++k) {
                int64_t no = o->p2n[k + nn * p];
                if (no == 0) continue;
                const double N = PHI(o, k, p, 0);
                for (int j = 0; j < d; ++j)
                    for (int i = 0; i < d; ++i)
                        Bp[i + d * j] = Bp[i + d * j] +
                                        N * (o->vn[i + d * (no - 1)] * o->dnp[k + nn * j + (int64_t)nn * d * p]);
            }
            for (int i = 0; i < d * d; ++i) o->B[i + (int64_t)d * d * p] = Bp[i];
        }
    }
    if (!o->cfg.musl) return;
    std::fill(o->pn.begin(), o->pn.end(), 0.0);
    std::fill(o->vn.begin(), o->vn.end(), 0.0);
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p)
        for (int i = 0; i < d; ++i)
            for (int k = 0; k < nn; ++k) {
                int64_t no = o->p2n[k + nn * p];
                if (no == 0) continue;
                ATOMIC_ADD(o->pn[i + d * (no - 1)], PHI(o, k, p, 0) * ((o->rho[p] * o->Om[p]) * o->v[i + d * p]));
            }
    for (int64_t q = 0; q < o->Nn; ++q) {
        if (o->mi[q] == 0.0) continue;
        for (int i = 0; i < d; ++i) {
            if (o->bcs[i + d * q]) o->vn[i + d * q] = 0.0;
            else o->vn[i + d * q] = o->pn[i + d * q] * (1.0 / o->mi[q]);
        }
    }
}

// ---------------------------------------------------------------- update (update.jl, deform.jl, domain.jl, volumetric.jl)
template <int D>
static void deform_point(eporacle* o, int64_t p, double dt) {
    const int nn = o->nn;
    double* gv = &o->dv[D * D * p];
    for (int i = 0; i < D * D; ++i) gv[i] = 0.0;
    for (int k = 0; k < nn; ++k) {
        int64_t no = o->p2n[k + nn * p];
        if (no == 0) continue;
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) gv[i + D * j] = gv[i + D * j] + PHI(o, k, p, j + 1) * o->vn[i + D * (no - 1)];
    }
    double* dF = &o->dF[D * D * p];
    double* F = &o->F[D * D * p];
    for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) dF[i + D * j] = (i == j ? 1.0 : 0.0) + dt * gv[i + D * j];
    double Fn[D * D];
    ep::matmul<D>(dF, F, Fn);
    for (int i = 0; i < D * D; ++i) F[i] = Fn[i];
    o->dJ[p] = ep::det_lu<D>(dF);
    o->J[p] = ep::det_lu<D>(F);
    o->Om[p] = o->J[p] * o->Om0[p];
    if (o->cfg.deform == EP_DEFORM_FINITE) {
        o->rho[p] = o->rho0[p] / o->J[p];
        o->n[p] = 1.0 - 1.0 / o->J[p] * (1.0 - o->n0[p]);
    }
    if (o->cfg.basis == EP_BASIS_GIMPM) {
        double* lp = &o->l[D * p];
        const double* l0 = &o->l0[D * p];
        switch (o->cfg.how) {
            case EP_HOW_UNDEFORMED:
                for (int i = 0; i < D; ++i) lp[i] = l0[i];
                break;
            case EP_HOW_DETFIJ: {
                double j = ep::det_lu<D>(F);
                for (int i = 0; i < D; ++i) lp[i] = l0[i] * j;
            } break;
            case EP_HOW_DETDFIJ: {
                double j = ep::det_lu<D>(dF);
                for (int i = 0; i < D; ++i) lp[i] = lp[i] * j;
            } break;
            case EP_HOW_FII:
                for (int i = 0; i < D; ++i) lp[i] = l0[i] * F[i + D * i];
                break;
            case EP_HOW_DFII:
                for (int i = 0; i < D; ++i) lp[i] = lp[i] * dF[i + D * i];
                break;
            case EP_HOW_UII:
            case EP_HOW_DUII: {
                const double* A = (o->cfg.how == EP_HOW_UII) ? F : dF;
                double C[D * D], lam[D], V[D * D], s[D], U[D * D];
                ep::matmul_at<D>(A, A, C);
                ep::eig_sym<D>(C, lam, V);
                for (int i = 0; i < D; ++i) s[i] = sqrt(lam[i]);
                ep::vdvt<D>(V, s, U);
                if (o->cfg.how == EP_HOW_UII)
                    for (int i = 0; i < D; ++i) lp[i] = U[i + D * i] * l0[i];
                else
                    for (int i = 0; i < D; ++i) lp[i] = U[i + D * i] * lp[i];
            } break;
            default: break;
        }
    }
}

static void update(eporacle* o, double dt) {
    const int d = o->dim, nn = o->nn;
    const int64_t Np = o->Np;
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p) {
        if (d == 2) deform_point<2>(o, p, dt);
        else deform_point<3>(o, p, dt);
    }
    if (!o->cfg.locking) return;
    std::fill(o->dJn.begin(), o->dJn.end(), 0.0);
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p)
        for (int k = 0; k < nn; ++k) {
            int64_t no = o->p2n[k + nn * p];
            if (no == 0) continue;
            ATOMIC_ADD(o->dJn[no - 1], PHI(o, k, p, 0) * ((o->rho[p] * o->Om[p]) * o->dJ[p]));
        }
    for (int64_t q = 0; q < o->Nn; ++q) {
        if (o->mi[q] == 0.0) o->dJn[q] = 0.0;
        else o->dJn[q] = o->dJn[q] / o->mi[q];
    }
    const double dimr = 1.0 / d;
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p) {
        double s = 0.0;
        for (int k = 0; k < nn; ++k) {
            int64_t no = o->p2n[k + nn * p];
            if (no == 0) continue;
            s = s + PHI(o, k, p, 0) * o->dJn[no - 1] / o->dJ[p];
        }
        double f = (d == 2) ? sqrt(s) : ep::ep_pow(s, dimr);
        for (int i = 0; i < d * d; ++i) o->dF[i + d * d * p] = o->dF[i + d * d * p] * f;
    }
}

// ---------------------------------------------------------------- elast (elast.jl:45-124)
static void elast(eporacle* o) {
    const int d = o->dim, ns = o->nstr;
    const int64_t Np = o->Np;
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p) {
        if (o->cfg.deform == EP_DEFORM_FINITE) {
            if (d == 2) ep::finite_elast<2>(&o->dF[4 * p], &o->b[4 * p], &o->eps[4 * p], &o->tau[3 * p], o->cm.Del);
            else ep::finite_elast<3>(&o->dF[9 * p], &o->b[9 * p], &o->eps[9 * p], &o->tau[6 * p], o->cm.Del);
        } else {
            if (d == 2)
                ep::infinitesimal_elast<2>(&o->dF[4 * p], &o->sig[ns * p], &o->eps[4 * p], &o->w[4 * p], &o->sJ[4 * p],
                                           o->cm.Del, o->cfg.jaumann);
            else
                ep::infinitesimal_elast<3>(&o->dF[9 * p], &o->sig[ns * p], &o->eps[9 * p], &o->w[9 * p], &o->sJ[9 * p],
                                           o->cm.Del, o->cfg.jaumann);
        }
    }
}

// ---------------------------------------------------------------- nonlocal (nonlocal.jl:18-47, plast.jl:51-59)
static void nonlocal(eporacle* o) {
    const int d = o->dim;
    const int64_t Np = o->Np;
    const double ls = o->cfg.nonloc_ls;
    // "tplgy": e2p[p, el] = p for el in the e2e neighbourhood of p's element
    // (e2e.jl:20-61: ±ceil(ls/h) elements per direction, clipped).  Column el
    // then lists, in ascending order, the points whose neighbourhood holds el.
    vector<vector<int64_t>> e2p((size_t)o->Ne);
    for (int64_t p = 0; p < Np; ++p) {
        int64_t el = o->p2e[p] - 1;
        int64_t c[3];
        if (d == 2) {
            c[0] = el / o->nel[1];            // x index
            c[1] = el % o->nel[1];            // z index
        } else {
            int64_t nzx = o->nel[2] * o->nel[0];
            c[1] = el / nzx;                  // y
            int64_t r = el % nzx;
            c[0] = r / o->nel[2];             // x
            c[2] = r % o->nel[2];             // z
        }
        // element id = z + nel_z x (+ nel_z nel_x y); enumerate in ascending id
        if (d == 2) {
            int64_t i0 = std::max<int64_t>(0, c[0] - o->nnel[0]), i1 = std::min<int64_t>(o->nel[0] - 1, c[0] + o->nnel[0]);
            int64_t j0 = std::max<int64_t>(0, c[1] - o->nnel[1]), j1 = std::min<int64_t>(o->nel[1] - 1, c[1] + o->nnel[1]);
            for (int64_t i = i0; i <= i1; ++i)
                for (int64_t j = j0; j <= j1; ++j) e2p[j + o->nel[1] * i].push_back(p);
        } else {
            int64_t ex = o->nel[0], ey = o->nel[1], ez = o->nel[2];
            int64_t i0 = std::max<int64_t>(0, c[0] - o->nnel[0]), i1 = std::min<int64_t>(ex - 1, c[0] + o->nnel[0]);
            int64_t k0 = std::max<int64_t>(0, c[1] - o->nnel[1]), k1 = std::min<int64_t>(ey - 1, c[1] + o->nnel[1]);
            int64_t j0 = std::max<int64_t>(0, c[2] - o->nnel[2]), j1 = std::min<int64_t>(ez - 1, c[2] + o->nnel[2]);
            for (int64_t k = k0; k <= k1; ++k)
                for (int64_t i = i0; i <= i1; ++i)
                    for (int64_t j = j0; j <= j1; ++j) e2p[j + ez * i + ez * ex * k].push_back(p);
        }
    }
    for (int64_t p = 0; p < Np; ++p) o->epII[1 + 2 * p] = 0.0;
    vector<double> W((size_t)Np, 0.0);
    std::unordered_map<uint64_t, double> w;
    vector<vector<int64_t>> p2p((size_t)Np);
    auto key = [&](int64_t a, int64_t b2) { return (uint64_t)a * (uint64_t)Np + (uint64_t)b2; };
    auto wget = [&](int64_t a, int64_t b2) {
        auto it = w.find(key(a, b2));
        return it == w.end() ? 0.0 : it->second;
    };
    // "p->q"
    for (int64_t p = 0; p < Np; ++p) {
        if (o->dlam[p] == 0.0) continue;
        for (int64_t q : e2p[o->p2e[p] - 1]) {
            double xi = o->x[0 + d * p] - o->x[0 + d * q], et = o->x[1 + d * p] - o->x[1 + d * q];
            double dd = sqrt(xi * xi + et * et);
            if (wget(p, q) == 0.0) {
                double r = dd / ls;
                double om = dd / ls * ep::ep_exp(-(r * r));
                if (om != 0.0) {
                    w[key(p, q)] = om;
                    w[key(q, p)] = om;
                }
                W[p] = W[p] + om;
                W[q] = W[q] + om;
                p2p[p].push_back(q);     // p2p[q,p] = q: column p gains row q
            }
        }
    }
    // "p<-q"
    for (int64_t p = 0; p < Np; ++p) {
        if (o->dlam[p] == 0.0) continue;
        if (!(W[p] > 1e-16)) {
            o->epII[1 + 2 * p] = o->epII[0 + 2 * p];
        } else {
            for (int64_t q : p2p[p])
                o->epII[1 + 2 * p] = o->epII[1 + 2 * p] + (wget(p, q) / W[p]) * o->epII[0 + 2 * q];
        }
    }
}

// ---------------------------------------------------------------- return maps (DP.jl, J2.jl)
static void retmap(eporacle* o) {
    const int d = o->dim, ns = o->nstr;
    const int64_t Np = o->Np;
    const bool fin = o->cfg.deform == EP_DEFORM_FINITE;
#pragma omp parallel for num_threads(o->threads) schedule(static) if (o->threads > 1)
    for (int64_t p = 0; p < Np; ++p) {
        double* s = fin ? &o->tau[ns * p] : &o->sig[ns * p];
        double ep1 = o->epII[0 + 2 * p], ep2 = o->epII[1 + 2 * p];
        if (o->cfg.constitutive == EP_CONS_DP) {
            double dl;
            if (d == 2) dl = ep::dp_return<3>(s, ep2, o->c0[p], o->cr[p], o->tphi[p], 0.0, 0.0, o->cm.Hp, o->cm.Kc, o->cm.Gc, &ep1);
            else dl = ep::dp_return<6>(s, ep2, o->c0[p], o->cr[p], 0.0, o->sphi[p], o->cphi[p], o->cm.Hp, o->cm.Kc, o->cm.Gc, &ep1);
            o->dlam[p] = dl;
            o->epII[0 + 2 * p] = ep1;
            if (fin) {
                if (d == 2) ep::finite_rebuild_b<2>(s, o->DelLU, o->piv, &o->eps[4 * p], &o->b[4 * p]);
                else ep::finite_rebuild_b<3>(s, o->DelLU, o->piv, &o->eps[9 * p], &o->b[9 * p]);
            }
        } else if (o->cfg.constitutive == EP_CONS_MC || o->cfg.constitutive == EP_CONS_CAMC) {
            // MCRetMap.jl:1-54 (2d) and camC/camCmodRetMap.jl, restated as in ep_scalar.h; a yielded
            // point takes ϵ = tensor(Del \ σ, ½) and, in finite strain, b_e = exp(2ϵ)
            int y;
            if (o->cfg.constitutive == EP_CONS_MC) {
                y = ep::mc_return(s, ep2, o->c0[p], o->cr[p], o->sphi[p], o->cphi[p], o->cm.Hp, o->cm.Del, o->DelLU,
                                  o->piv, &ep1);
                if (y < 0) o->nonconverged = 1;
            } else {
                double ev = o->epV[p];
                y = (d == 2) ? ep::camc_return<3>(s, ep2, &ev, o->cm.Kc, o->cm.Del, &ep1)
                             : ep::camc_return<6>(s, ep2, &ev, o->cm.Kc, o->cm.Del, &ep1);
                if (y > 0) o->epV[p] = ev;
            }
            if (y > 0) {
                o->epII[0 + 2 * p] = ep1;
                if (fin) {
                    if (d == 2) ep::finite_rebuild_b<2>(s, o->DelLU, o->piv, &o->eps[4 * p], &o->b[4 * p]);
                    else ep::finite_rebuild_b<3>(s, o->DelLU, o->piv, &o->eps[9 * p], &o->b[9 * p]);
                } else if (d == 2) {
                    ep::strain_from_stress<2>(s, o->DelLU, o->piv, &o->eps[4 * p]);
                } else {
                    ep::strain_from_stress<3>(s, o->DelLU, o->piv, &o->eps[9 * p]);
                }
            }
        } else {
            int y = (d == 2) ? ep::j2_return<3>(s, ep2, o->c0[p], o->cr[p], o->cm.Hp, o->cm.Del, &ep1)
                             : ep::j2_return<6>(s, ep2, o->c0[p], o->cr[p], o->cm.Hp, o->cm.Del, &ep1);
            if (y) {
                o->epII[0 + 2 * p] = ep1;
                if (fin) {
                    if (d == 2) ep::finite_rebuild_b<2>(s, o->DelLU, o->piv, &o->eps[4 * p], &o->b[4 * p]);
                    else ep::finite_rebuild_b<3>(s, o->DelLU, o->piv, &o->eps[9 * p], &o->b[9 * p]);
                }
            }
        }
    }
}

static void plast(eporacle* o) {
    if (o->cfg.nonloc) nonlocal(o);
    else
        for (int64_t p = 0; p < o->Np; ++p) o->epII[1 + 2 * p] = o->epII[0 + 2 * p];
    o->nonconverged = 0;
    retmap(o);
    if (o->nonconverged) fail(o, EP_ERR_NONCONVERGED, "CPA: return map iteration limit exceeded (MCRetMap.jl:38-41)");
}

// ---------------------------------------------------------------- API
extern "C" {

eporacle* eporacle_create(const ep_cfg* cfg, const ep_cmpr* cmpr, const ep_mesh_view* mesh, int64_t nmp) {
    if (!cfg || !cmpr || !mesh || nmp < 0) return nullptr;
    if (cfg->dim != 2 && cfg->dim != 3) return nullptr;
    eporacle* o = new eporacle();
    o->cfg = *cfg;
    o->cm = *cmpr;
    o->dim = cfg->dim;
    o->nstr = cfg->dim == 2 ? 3 : 6;
    o->nn = cfg->dim == 2 ? 16 : 64;
    for (int i = 0; i < 4; ++i) { o->nel[i] = mesh->nel[i]; o->nno[i] = mesh->nno[i]; }
    o->Ne = mesh->nel[o->dim];
    o->Nn = mesh->nno[o->dim];
    o->Np = nmp;
    const int d = o->dim;
    for (int i = 0; i < 3; ++i) { o->h[i] = mesh->h[i]; o->x0[i] = mesh->x0[i]; }
    o->xn.assign(mesh->x, mesh->x + d * o->Nn);
    o->xB.assign(mesh->xB, mesh->xB + 2 * d);
    o->bcs.assign(mesh->bcs, mesh->bcs + d * o->Nn);
    for (int i = 0; i < d; ++i) o->nnel[i] = (int)ceil(cfg->nonloc_ls / o->h[i]);
    build_e2n(o);
    const int64_t Nn = o->Nn, Np = o->Np;
    o->mi.assign(Nn, 0.0);
    o->oobf.assign(d * Nn, 0.0); o->a.assign(d * Nn, 0.0); o->pn.assign(d * Nn, 0.0);
    o->vn.assign(d * Nn, 0.0); o->dJn.assign(Nn, 0.0);
    o->vmax.assign(d, 0.0);
    auto V = [&](vector<double>& a, int64_t n) { a.assign(n, 0.0); };
    V(o->x, d * Np); V(o->l0, d * Np); V(o->l, d * Np); V(o->n0, Np); V(o->n, Np); V(o->Om0, Np);
    V(o->Om, Np); V(o->dJ, Np); V(o->J, Np); V(o->u, d * Np); V(o->v, d * Np); V(o->pp, d * Np);
    V(o->rho0, Np); V(o->rho, Np); V(o->c0, Np); V(o->cr, Np); V(o->phi, Np); V(o->dlam, Np);
    V(o->epII, 2 * Np); V(o->epV, Np); V(o->sig, o->nstr * Np); V(o->tau, o->nstr * Np);
    V(o->dv, d * d * Np); V(o->du, d * d * Np); V(o->dF, d * d * Np); V(o->F, d * d * Np);
    V(o->b, d * d * Np); V(o->eps, d * d * Np); V(o->w, d * d * Np); V(o->sJ, d * d * Np);
    V(o->B, d * d * Np); V(o->Dm, d * d * Np);
    V(o->tphi, Np); V(o->sphi, Np); V(o->cphi, Np);
    o->p2e.assign(Np, 0);
    o->p2n.assign((size_t)o->nn * Np, 0);
    o->phidphi.assign((size_t)o->nn * Np * (d + 1), 0.0);
    if (cfg->trsfr == EP_TRSFR_TPIC || cfg->trsfr == EP_TRSFR_APIC) o->dnp.assign((size_t)o->nn * d * Np, 0.0);
    const int ns = o->nstr;
    for (int i = 0; i < ns * ns; ++i) o->DelLU[i] = cmpr->Del[i];
    if (ns == 3) ep::lu_factor<3>(o->DelLU, o->piv);
    else ep::lu_factor<6>(o->DelLU, o->piv);
    return o;
}

static void cpy_in(vector<double>& dst, const double* src) {
    if (src) std::memcpy(dst.data(), src, dst.size() * sizeof(double));
}
static void cpy_out(const vector<double>& src, double* dst) {
    if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(double));
}

int eporacle_upload(eporacle* o, const ep_mpts_view* m) {
    if (!o || !m || m->nmp != o->Np || m->ndim != o->dim) return EP_ERR_ARG;
    if (m->vmax) o->vmax.assign(m->vmax, m->vmax + o->dim);
    cpy_in(o->x, m->x); cpy_in(o->l0, m->l0); cpy_in(o->l, m->l); cpy_in(o->n0, m->n0); cpy_in(o->n, m->n);
    cpy_in(o->Om0, m->Omega0); cpy_in(o->Om, m->Omega); cpy_in(o->dJ, m->dJ); cpy_in(o->J, m->J);
    cpy_in(o->u, m->u); cpy_in(o->v, m->v); cpy_in(o->pp, m->p); cpy_in(o->rho0, m->rho0); cpy_in(o->rho, m->rho);
    cpy_in(o->c0, m->c0); cpy_in(o->cr, m->cr); cpy_in(o->phi, m->phi); cpy_in(o->dlam, m->dlam);
    cpy_in(o->epII, m->epII); cpy_in(o->epV, m->epV); cpy_in(o->sig, m->sig); cpy_in(o->tau, m->tau);
    cpy_in(o->dv, m->dvij); cpy_in(o->du, m->duij); cpy_in(o->dF, m->dFij); cpy_in(o->F, m->Fij);
    cpy_in(o->b, m->bij); cpy_in(o->eps, m->eij); cpy_in(o->w, m->wij); cpy_in(o->sJ, m->sJij);
    cpy_in(o->B, m->Bij); cpy_in(o->Dm, m->Dij);
    for (int64_t p = 0; p < o->Np; ++p) {
        o->tphi[p] = tan(o->phi[p]);
        o->sphi[p] = sin(o->phi[p]);
        o->cphi[p] = cos(o->phi[p]);
    }
    return 0;
}

int eporacle_step(eporacle* o, int32_t phase, double dt, const double* g, double* vmax_out) {
    if (!o || !g) return EP_ERR_ARG;
    for (int i = 0; i < o->dim; ++i) o->vmax[i] = 0.0;
    int e = tplgy(o);
    if (e) return e;
    e = shpfun(o);
    if (e) return e;
    p2n(o, g);
    solve(o, dt);
    n2p(o, dt);
    update(o, dt);
    elast(o);
    if (phase == EP_PHASE_ELASTOPLASTIC) {
        plast(o);
        if (o->nonconverged) return EP_ERR_NONCONVERGED;
    }
    if (vmax_out)
        for (int i = 0; i < o->dim; ++i) vmax_out[i] = o->vmax[i];
    return 0;
}

int eporacle_run(eporacle* o, int32_t phase, double T, double tg, double* t_inout, int64_t* nsteps_out) {
    if (!o || !t_inout) return EP_ERR_ARG;
    double t = *t_inout;
    int64_t it = 0;
    const int d = o->dim;
    while (T > t) {
        double cm = -INFINITY;
        for (int i = 0; i < d; ++i) {
            double c = o->h[i] / (o->vmax[i] + o->cm.c);
            if (i == 0 || c > cm || c != c) cm = c;
        }
        double a = 0.5 * cm, bnd = T - t;
        double dt = (a < bnd) ? a : bnd;
        for (int i = 0; i < d; ++i) o->vmax[i] = 0.0;
        double g[3] = {0.0, 0.0, 0.0};
        double G = 9.81;
        if (phase == EP_PHASE_ELASTODYNAMIC && t <= tg) G = 9.81 * t / tg;
        g[d - 1] = -G;
        int e = eporacle_step(o, phase, dt, g, nullptr);
        if (e) { *t_inout = t; if (nsteps_out) *nsteps_out = it; return e; }
        t = t + dt;
        ++it;
    }
    *t_inout = t;
    if (nsteps_out) *nsteps_out = it;
    return 0;
}

int eporacle_download(eporacle* o, ep_mpts_view* m) {
    if (!o || !m) return EP_ERR_ARG;
    if (m->vmax) for (int i = 0; i < o->dim; ++i) m->vmax[i] = o->vmax[i];
    cpy_out(o->x, m->x); cpy_out(o->l0, m->l0); cpy_out(o->l, m->l); cpy_out(o->n0, m->n0); cpy_out(o->n, m->n);
    cpy_out(o->Om0, m->Omega0); cpy_out(o->Om, m->Omega); cpy_out(o->dJ, m->dJ); cpy_out(o->J, m->J);
    cpy_out(o->u, m->u); cpy_out(o->v, m->v); cpy_out(o->pp, m->p); cpy_out(o->rho0, m->rho0); cpy_out(o->rho, m->rho);
    cpy_out(o->c0, m->c0); cpy_out(o->cr, m->cr); cpy_out(o->phi, m->phi); cpy_out(o->dlam, m->dlam);
    cpy_out(o->epII, m->epII); cpy_out(o->epV, m->epV); cpy_out(o->sig, m->sig); cpy_out(o->tau, m->tau);
    cpy_out(o->dv, m->dvij); cpy_out(o->du, m->duij); cpy_out(o->dF, m->dFij); cpy_out(o->F, m->Fij);
    cpy_out(o->b, m->bij); cpy_out(o->eps, m->eij); cpy_out(o->w, m->wij); cpy_out(o->sJ, m->sJij);
    cpy_out(o->B, m->Bij); cpy_out(o->Dm, m->Dij);
    if (m->p2e) std::memcpy(m->p2e, o->p2e.data(), o->p2e.size() * sizeof(int64_t));
    if (m->p2n) std::memcpy(m->p2n, o->p2n.data(), o->p2n.size() * sizeof(int64_t));
    return 0;
}

int eporacle_download_mesh(eporacle* o, ep_mesh_fields* f) {
    if (!o || !f) return EP_ERR_ARG;
    cpy_out(o->mi, f->mi); cpy_out(o->pn, f->p); cpy_out(o->vn, f->v); cpy_out(o->a, f->a);
    cpy_out(o->oobf, f->oobf); cpy_out(o->dJn, f->dJ);
    return 0;
}

int eporacle_e2n(eporacle* o, int64_t* out) {
    if (!o || !out) return EP_ERR_ARG;
    std::memcpy(out, o->e2n.data(), o->e2n.size() * sizeof(int64_t));
    return 0;
}

void eporacle_set_threads(eporacle* o, int threads) {
    if (o) o->threads = threads < 1 ? 1 : threads;
}

const char* eporacle_last_error(eporacle* o) { return o ? o->msg.c_str() : "null oracle"; }

void eporacle_destroy(eporacle* o) { delete o; }

}  // extern "C"

// ---------------------------------------------------------------- scalar kernels exposed for unit tests
extern "C" {

double eporacle_exp(double x) { return ep::ep_exp(x); }
double eporacle_log(double x) { return ep::ep_log(x); }

void eporacle_eig_sym(int D, const double* A, double* lam, double* V) {
    if (D == 2) ep::eig_sym<2>(A, lam, V);
    else ep::eig_sym<3>(A, lam, V);
}

double eporacle_det(int D, const double* A) { return D == 2 ? ep::det_lu<2>(A) : ep::det_lu<3>(A); }

// basis: 0 bsmpm (cls, xi, dx), 1 gimpm (delta, h, lp), 2 smpm (delta, h)
void eporacle_shape(int basis, int cls, double a, double h, double lp, double* f, double* df) {
    if (basis == 0) ep::bspline(cls, a, h, f, df);
    else if (basis == 1) ep::gimp(a, h, lp, f, df);
    else ep::hat(a, h, f, df);
}

int eporacle_bspline_class(double xn, double xB0, double xB1, double dx) { return ep::bspline_class(xn, xB0, xB1, dx); }

// Drucker-Prager on one Voigt stress s[NS] (NS = 3 or 6), returns Δλ, updates s and ep1
double eporacle_dp(int NS, double* s, double ep2, double c0, double cr, double phi, double Hp, double Kc, double Gc,
                   double* ep1) {
    if (NS == 3) return ep::dp_return<3>(s, ep2, c0, cr, tan(phi), 0.0, 0.0, Hp, Kc, Gc, ep1);
    return ep::dp_return<6>(s, ep2, c0, cr, 0.0, sin(phi), cos(phi), Hp, Kc, Gc, ep1);
}

int eporacle_j2(int NS, double* s, double ep2, double c0, double cr, double Hp, const double* Del, double* ep1) {
    if (NS == 3) return ep::j2_return<3>(s, ep2, c0, cr, Hp, Del, ep1);
    return ep::j2_return<6>(s, ep2, c0, cr, Hp, Del, ep1);
}

double eporacle_jfld(double a, double h) { return ep::jfld(a, h); }

}  // extern "C"
